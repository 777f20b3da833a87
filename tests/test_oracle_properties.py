"""Property tests of the oracle's inviscid Euler path (dgfem has no Euler KAT).

* periodic N x N x 2 meshes have 1.5 E interior faces and no boundary face;
* free stream is preserved (residual ~ 0);
* discrete conservation: the constant test function sees only cancelling face terms;
* the thread count does not change a single bit of the residual;
* the isentropic vortex converges to the exact advected solution.
"""

import numpy as np
import pytest

import oracle as O
from meshes import PERIODIC_PAIRS, isentropic_vortex, periodic_rectangle, primitive_to_conserved


def make(n, order, basis):
    v, e, b = periodic_rectangle(n)
    return O.OracleMesh(v, e, b, order=order, basis=basis, periodic=PERIODIC_PAIRS)


@pytest.mark.parametrize("n", [2, 3, 8])
def test_periodic_structure(n):
    m = make(n, 1, O.MONOMIAL)
    assert len(m.interior_faces()) == 3 * n * n
    assert len(m.boundary_faces()) == 0
    nb = m.neighbors()
    assert np.all(nb[:, :, 0] >= 0)
    # neighbour relation is symmetric
    for e in range(m.ne):
        for f in range(3):
            r, fr = nb[e, f]
            assert nb[r, fr, 0] == e and nb[r, fr, 1] == f


def project(m, fn):
    return m.project(fn(m.quad_points()))


@pytest.mark.parametrize("basis", [O.MONOMIAL, O.DUBINER])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_free_stream_preservation(basis, order):
    m = make(4, order, basis)
    U = primitive_to_conserved([1.0, 0.5, -0.2, 1.0])
    u = project(m, lambda x: np.broadcast_to(U, x.shape[:-1] + (4,)))
    R = m.residual(O.euler(), u)
    # round-off only: relative to the size of a single volume-term contribution
    scale = np.abs(m.volume_residual(O.euler(), 0, u)).max()
    assert np.abs(R).max() < 1e-12 * max(scale, 1.0)


@pytest.mark.parametrize("basis", [O.MONOMIAL, O.DUBINER])
def test_discrete_conservation(basis):
    m = make(6, 2, basis)
    u = project(m, lambda x: isentropic_vortex(x, beta=5.0))
    R = m.residual(O.euler(), u)
    # coefficients c with sum_i c_i phi_i == 1
    c = np.linalg.lstsq(m.tables()["phi_vol"], np.ones(m.nq), rcond=None)[0]
    total = np.einsum("i,eiv->v", c, R)
    assert np.abs(total).max() < 1e-12 * max(1.0, np.abs(R).max())


def test_thread_count_is_bitwise_neutral():
    m = make(8, 3, O.DUBINER)
    u = project(m, lambda x: isentropic_vortex(x, beta=5.0, xc=0.7, yc=-0.3))
    O.set_threads(1)
    R1 = m.residual(O.euler(), u)
    O.set_threads(4)
    R4 = m.residual(O.euler(), u)
    O.set_threads(1)
    assert np.array_equal(R1, R4)


def test_vortex_converges_to_exact():
    errs = []
    for n in (8, 16):
        m = make(n, 2, O.DUBINER)
        u = project(m, lambda x: isentropic_vortex(x))
        dt, steps = 0.02 * 16 / n, int(round(0.4 / (0.02 * 16 / n)))
        u = m.rk3_step(O.euler(), u, dt, steps)
        ex = project(m, lambda x: isentropic_vortex(x, t=dt * steps))
        errs.append(np.sqrt(np.mean((u - ex) ** 2)))
    assert errs[1] < errs[0] / 3.0
