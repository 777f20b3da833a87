"""The oracle's quadrilateral path pinned by dgfem's own tests, restated:

* LegendreBasis: (p+1)^2 functions; values and gradients at the origin (p=2); corner
  values (p=1); Gram matrix on the tensor Gauss-Legendre rule (tests/basis/legendre_test.cpp);
* bilinear mapping: unit square centre, Jacobian and inverse, corners, a distorted quad
  (tests/reference/quad_test.cpp, tests/reference/mapping_test.cpp:176-196);
* quad face points on the edges y=-1, x=1, y=1, x=-1 and unit outward normals
  (tests/reference/quad_test.cpp:194-264);
plus properties of the quad residual: free stream preserved and discrete conservation on
periodic bilinear meshes, and 4 faces per element in the connectivity.
"""

import numpy as np
import pytest

import oracle as O
from meshes import PERIODIC_PAIRS, isentropic_vortex, primitive_to_conserved, quad_rectangle


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_legendre_count(p):
    assert O.n_basis(p, O.LEGENDRE) == (p + 1) ** 2
    assert len(O.basis_eval(O.LEGENDRE, p, 0.3, -0.2)) == (p + 1) ** 2


def test_legendre_values_and_gradients_at_origin():
    v = O.basis_eval(O.LEGENDRE, 2, 0.0, 0.0)
    assert np.allclose(v, [1.0, 0.0, -0.5, 0.0, 0.0, 0.0, -0.5, 0.0, 0.25], atol=1e-12)
    g = O.basis_grad(O.LEGENDRE, 2, 0.0, 0.0)
    ref = np.zeros((9, 2))
    ref[1] = (1.0, 0.0)
    ref[3] = (0.0, 1.0)
    ref[5] = (0.0, -0.5)
    ref[7] = (-0.5, 0.0)
    assert np.allclose(g, ref, atol=1e-12)


@pytest.mark.parametrize("x,y", [(-1, -1), (1, -1), (1, 1), (-1, 1)])
def test_legendre_corner_values(x, y):
    assert np.allclose(O.basis_eval(O.LEGENDRE, 1, x, y), [1.0, x, y, x * y], atol=1e-12)


def test_legendre_orthogonality_on_tensor_rule():
    pts, w = O.gl_rule(3)
    G = np.zeros((9, 9))
    for j in range(3):
        for i in range(3):
            phi = O.basis_eval(O.LEGENDRE, 2, pts[i], pts[j])
            G += w[i] * w[j] * np.outer(phi, phi)
    exp = np.diag([(2 / (2 * (k % 3) + 1)) * (2 / (2 * (k // 3) + 1)) for k in range(9)])
    assert np.allclose(G, exp, atol=1e-10)


@pytest.mark.parametrize("p", [1, 2, 3, 4])
def test_legendre_gradient_numerically(p):
    h = 1e-6
    for x, y in [(0.3, -0.4), (-0.7, 0.8), (0.99, 0.1)]:
        g = O.basis_grad(O.LEGENDRE, p, x, y)
        gx = (O.basis_eval(O.LEGENDRE, p, x + h, y) - O.basis_eval(O.LEGENDRE, p, x - h, y)) / (2 * h)
        gy = (O.basis_eval(O.LEGENDRE, p, x, y + h) - O.basis_eval(O.LEGENDRE, p, x, y - h)) / (2 * h)
        assert np.allclose(g[:, 0], gx, atol=1e-5) and np.allclose(g[:, 1], gy, atol=1e-5)


def test_bilinear_mapping_unit_square():
    V = [[0, 0], [1, 0], [1, 1], [0, 1]]
    x, d, A = O.compute_mapping(V, 0.0, 0.0)
    assert np.allclose(x, [0.5, 0.5]) and np.isclose(d, 0.25)
    assert np.allclose(A, [[2, 0], [0, 2]], atol=1e-10)
    for xi, X in [((-1, -1), (0, 0)), ((1, -1), (1, 0)), ((1, 1), (1, 1)), ((-1, 1), (0, 1))]:
        assert np.allclose(O.compute_mapping(V, *xi)[0], X, atol=1e-10)


def test_bilinear_mapping_distorted_quad():
    V = np.array([[0.0, 0.0], [2.0, 0.2], [2.1, 2.0], [0.1, 1.9]])
    x, d, A = O.compute_mapping(V, 0.0, 0.0)
    assert np.linalg.norm(x - V.mean(axis=0)) < 0.1 and d > 0
    # dxi_dx is the inverse of J_T = (dx/dxi)^T (mapping.cpp:22-50): A^T inverts the map's
    # Jacobian, checked by finite differences
    h = 1e-6
    J = np.column_stack([(O.compute_mapping(V, h, 0)[0] - O.compute_mapping(V, -h, 0)[0]) / (2 * h),
                         (O.compute_mapping(V, 0, h)[0] - O.compute_mapping(V, 0, -h)[0]) / (2 * h)])
    assert np.allclose(A.T @ J, np.eye(2), atol=1e-8)


def test_quad_face_points_lie_on_their_edges():
    pts, _ = O.gl_rule(3)
    checks = {0: lambda xi: abs(xi[1] + 1), 1: lambda xi: abs(xi[0] - 1), 2: lambda xi: abs(xi[1] - 1),
              3: lambda xi: abs(xi[0] + 1)}
    for f, c in checks.items():
        for s in pts:
            assert c(O.map_face_point(f, s, nv=4)) < 1e-10


def make(n, order, distort=0.0):
    v, e, b = quad_rectangle(n, distort=distort, seed=3)
    return O.OracleMesh(v, e, b, order=order, basis=O.LEGENDRE, periodic=PERIODIC_PAIRS)


def test_quad_connectivity_and_face_data():
    m = make(4, 2, distort=0.2)
    assert len(m.interior_faces()) == 2 * 16 and len(m.boundary_faces()) == 0
    nb = m.neighbors()
    assert nb.shape == (16, 4, 2) and np.all(nb[:, :, 0] >= 0)
    for e in range(m.ne):
        for f in range(4):
            r, fr = nb[e, f]
            assert nb[r, fr, 0] == e and nb[r, fr, 1] == f
            fd = m.face_data(e, f)
            assert np.isclose(np.linalg.norm(fd["normal"]), 1.0)
    d = m.element_data(0)["J_det_vol"]
    assert np.all(d > 0) and np.ptp(d) > 0  # bilinear: the Jacobian varies over the element


@pytest.mark.parametrize("order", [1, 2, 3])
def test_quad_free_stream_preservation(order):
    m = make(4, order, distort=0.2)
    U = primitive_to_conserved([1.0, 0.5, -0.2, 1.0])
    u = m.project(np.broadcast_to(U, m.quad_points().shape[:-1] + (4,)).copy())
    R = m.residual(O.euler(), u)
    scale = np.abs(m.volume_residual(O.euler(), 0, u)).max()
    assert np.abs(R).max() < 1e-11 * max(scale, 1.0)


def test_quad_discrete_conservation():
    m = make(5, 2, distort=0.2)
    u = m.project(isentropic_vortex(m.quad_points(), beta=5.0))
    R = m.residual(O.euler(), u)
    # phi_0 = P_0 P_0 = 1: the constant test function sees only cancelling face terms
    total = R[:, 0, :].sum(axis=0)
    assert np.abs(total).max() < 1e-12 * max(1.0, np.abs(R).max())
