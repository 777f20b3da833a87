"""dgfem's own known-answer tests, re-run against the CPU oracle (pins the oracle).

Each test names the dgfem test it restates.  Tolerances are dgfem's.
"""

import math

import numpy as np
import pytest

import oracle as O
from meshes import two_triangle_mesh, primitive_to_conserved

# ------------------------------------------------------------------ quadrature
# tests/quadrature/factory_test.cpp


def _exact_tri(a, b):
    return math.factorial(a) * math.factorial(b) / math.factorial(a + b + 2)


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_dunavant_degree_of_precision(order):
    """QuadratureFactoryTest.DegreeOfPrecision (factory_test.cpp:202-249)."""
    p, w = O.tri_rule(order)
    for td in range(order + 1):
        for a in range(td + 1):
            b = td - a
            num = float(np.sum(w * p[:, 0] ** a * p[:, 1] ** b))
            assert abs(num - _exact_tri(a, b)) < 1e-10


@pytest.mark.parametrize("order", [2, 4, 6, 8])
def test_dunavant_rules_used_by_the_space(order):
    """The 2p rules DGSpace uses (space.cpp:40-41) are exact to degree 2p (the degree-8
    rule is tabulated to 15 digits, so its tolerance is looser); weights sum to 1/2."""
    p, w = O.tri_rule(order)
    assert abs(w.sum() - 0.5) < 1e-12
    assert np.all(p[:, 0] >= -1e-12) and np.all(p[:, 1] >= -1e-12)
    assert np.all(p.sum(1) <= 1 + 1e-12)
    tol = 1e-13 if order <= 6 else 1e-12
    for td in range(order + 1):
        for a in range(td + 1):
            b = td - a
            num = float(np.sum(w * p[:, 0] ** a * p[:, 1] ** b))
            assert abs(num - _exact_tri(a, b)) < tol, (order, a, b)


def test_dunavant_integration_accuracy():
    """QuadratureFactoryTest.IntegrationAccuracy (factory_test.cpp:107-146)."""
    for order in range(2, 6):
        p, w = O.tri_rule(order)
        a, b = order - 2, 1
        num = float(np.sum(w * p[:, 0] ** a * p[:, 1] ** b))
        assert abs(num - _exact_tri(a, b)) < 1e-12


def test_weight_positivity():
    """QuadratureFactoryTest.WeightPositivity (factory_test.cpp:151-200)."""
    for n in range(1, 9):
        _, w = O.gl_rule(n)
        assert np.all(w > 0)
    for order in (1, 2):
        assert np.all(O.tri_rule(order)[1] > 0)
    assert np.any(O.tri_rule(3)[1] < 0)


def test_gauss_legendre_symmetry_and_exactness():
    """QuadratureFactoryTest.GaussLegendreSymmetry (factory_test.cpp:251-...) plus the
    2n-1 exactness that DGSpace relies on (space.cpp:43-46)."""
    for n in range(1, 9):
        x, w = O.gl_rule(n)
        assert abs(w.sum() - 2.0) < 1e-12
        for i in range(n // 2):
            assert abs(x[i] + x[n - 1 - i]) < 1e-12
            assert abs(w[i] - w[n - 1 - i]) < 1e-12
        for d in range(2 * n):
            exact = 0.0 if d % 2 else 2.0 / (d + 1)
            assert abs(float(np.sum(w * x ** d)) - exact) < 1e-12


# ------------------------------------------------------------------ bases
# tests/basis/monomial_test.cpp


def test_monomial_values():
    """MonomialBasisTriangleTest.EvaluateAtPoint (monomial_test.cpp:32-49)."""
    v = O.basis_eval(O.MONOMIAL, 1, 2.0, 3.0)
    assert np.allclose(v, [1.0, 3.0, 2.0], atol=1e-12)


def test_monomial_gradients():
    """EvaluateGradientAtOrigin / EvaluateGradientAtPoint (monomial_test.cpp:51-104)."""
    g = O.basis_grad(O.MONOMIAL, 2, 0.0, 0.0)
    exp = np.zeros((6, 2))
    exp[1] = [0, 1]
    exp[2] = [1, 0]
    assert np.allclose(g, exp, atol=1e-12)
    g = O.basis_grad(O.MONOMIAL, 2, 2.0, 3.0)
    assert np.allclose(g[3:], [[0, 6], [3, 2], [4, 0]], atol=1e-12)


def test_monomial_high_order_and_completeness():
    """HighOrderEvaluation / PolynomialCompleteness (monomial_test.cpp:106-160)."""
    x, y = 0.4, 0.3
    v = O.basis_eval(O.MONOMIAL, 3, x, y)
    assert len(v) == 10
    assert abs(v[0] - 1) < 1e-12 and abs(v[1] - y) < 1e-12 and abs(v[2] - x) < 1e-12
    assert abs(v[6] - y ** 3) < 1e-12 and abs(v[9] - x ** 3) < 1e-12
    c = np.array([3.0, 2.0, 4.0, -1.0, 2.0, 3.0])
    for x, y in [(0.1, 0.2), (0.5, 0.3), (0.2, 0.6)]:
        exact = 3 + 2 * y + 4 * x - y * y + 2 * x * y + 3 * x * x
        assert abs(c @ O.basis_eval(O.MONOMIAL, 2, x, y) - exact) < 1e-12


@pytest.mark.parametrize("basis", [O.MONOMIAL, O.DUBINER])
def test_basis_numerical_gradient(basis):
    """NumericalGradientVerification (monomial_test.cpp:162-190, dubiner_test.cpp:219-255)."""
    h = 1e-7
    pt = (0.35, 0.45) if basis == O.MONOMIAL else (0.3, 0.4)
    g = O.basis_grad(basis, 2, *pt)
    for k in range(6):
        gx = (O.basis_eval(basis, 2, pt[0] + h, pt[1])[k] - O.basis_eval(basis, 2, pt[0] - h, pt[1])[k]) / (2 * h)
        gy = (O.basis_eval(basis, 2, pt[0], pt[1] + h)[k] - O.basis_eval(basis, 2, pt[0], pt[1] - h)[k]) / (2 * h)
        assert abs(g[k, 0] - gx) < 1e-5 and abs(g[k, 1] - gy) < 1e-5


# tests/basis/dubiner_test.cpp


def test_dubiner_orthonormality():
    """DubinerBasisTest.OrthonormalityVerification (dubiner_test.cpp:132-177)."""
    p, w = O.tri_rule(5)
    G = np.zeros((6, 6))
    for q in range(len(w)):
        phi = O.basis_eval(O.DUBINER, 2, *p[q])
        G += w[q] * np.outer(phi, phi)
    G *= 0.5
    assert np.allclose(G, np.eye(6), atol=1e-10)


def test_dubiner_completeness_and_singularity():
    """PolynomialCompleteness, SingularityHandling, EvaluateGradientAtOrigin
    (dubiner_test.cpp:179-217, 93-104, 61-91)."""
    def poly(x, y):
        return 1 + 2 * x + 3 * y + x * x + x * y + y * y
    p, w = O.tri_rule(5)
    c = np.zeros(6)
    for q in range(len(w)):
        c += w[q] * poly(*p[q]) * O.basis_eval(O.DUBINER, 2, *p[q])
    c *= 0.5
    for pt in [(0.2, 0.3), (0.5, 0.2), (0.1, 0.6)]:
        assert abs(c @ O.basis_eval(O.DUBINER, 2, *pt) - poly(*pt)) < 1e-10
    assert np.all(np.isfinite(O.basis_eval(O.DUBINER, 2, 0.0, 1.0)))
    assert np.all(np.isfinite(O.basis_grad(O.DUBINER, 2, 0.0, 1.0)))
    g = O.basis_grad(O.DUBINER, 1, 0.0, 0.0)
    assert abs(g[0, 0]) < 1e-12 and abs(g[0, 1]) < 1e-12
    for i in (1, 2):
        assert 0 < np.hypot(*g[i]) < 100


# ------------------------------------------------------------------ mapping
# tests/reference/mapping_test.cpp


def test_mapping_unit_triangle():
    """GeometricMappingTest.ComputeMapping (mapping_test.cpp:98-127)."""
    x, d, A = O.compute_mapping([[0, 0], [1, 0], [0, 1]], 1 / 3, 1 / 3)
    assert np.allclose(x, [1 / 3, 1 / 3], atol=1e-12)
    assert abs(d - 1.0) < 1e-12
    assert np.allclose(A, np.eye(2), atol=1e-12)


def test_mapping_singular_and_affine():
    """SingularJacobian / AffineMappingTriangle (mapping_test.cpp:129-176)."""
    with pytest.raises(RuntimeError):
        O.compute_mapping([[0, 0], [0, 0], [0, 1]], 1 / 3, 1 / 3)
    V = np.array([[1.0, 2.0], [3.0, 2.0], [1.0, 4.0]])
    for xi in [(0, 0), (1, 0), (0, 1), (0.5, 0.25)]:
        x, _, _ = O.compute_mapping(V, *xi)
        N = np.array([1 - xi[0] - xi[1], xi[0], xi[1]])
        assert np.linalg.norm(x - N @ V) < 1e-12


# ------------------------------------------------------------------ face integrals
# tests/reference/face_integral_test.cpp


def _face_int(face, fn):
    s, w = O.gl_rule(3)  # DGSpace("triangle", 2) uses p+1 = 3 points
    ref = np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]])
    e = [(0, 1), (1, 2), (2, 0)][face]
    L = np.linalg.norm(ref[e[1]] - ref[e[0]])
    return sum(fn(O.map_face_point(face, s[q])) * w[q] * L / 2.0 for q in range(3))


def test_face_integrals():
    """TriangleFaceIntegralConstant/Linear/Quadratic (face_integral_test.cpp:44-100)."""
    one = lambda x: 1.0
    assert abs(_face_int(0, one) - 1) < 1e-12
    assert abs(_face_int(1, one) - math.sqrt(2)) < 1e-12
    assert abs(_face_int(2, one) - 1) < 1e-12
    fx = lambda x: x[0]
    assert abs(_face_int(0, fx) - 0.5) < 1e-12
    assert abs(_face_int(1, fx) - math.sqrt(2) / 2) < 1e-11
    assert abs(_face_int(2, fx)) < 1e-12
    assert abs(_face_int(0, lambda x: x[0] ** 2) - 1 / 3) < 1e-12
    assert abs(_face_int(1, lambda x: x[0] * x[1]) - math.sqrt(2) / 6) < 1e-11


# ------------------------------------------------------------------ Navier-Stokes KATs
# tests/solver/navier_stokes_weak_formulation_test.cpp

GAMMA = 1.4


def test_penalty_parameter_scaling():
    """PenaltyParameterScaling (navier_stokes_weak_formulation_test.cpp:185-200)."""
    ph = O.navier_stokes(GAMMA, 1.0e-2, 0.72, 7.5)
    assert O.penalty(ph, 2, 0.125) == 7.5 * 1.0e-2 * 3 * 3 / 0.125
    assert O.penalty(ph, 2, 1e-14) == 7.5 * 1.0e-2 * 3 * 3 / 1e-12


def _two_tri(order=1):
    v, e, b = two_triangle_mesh()
    return O.OracleMesh(v, e, b, order=order, basis=O.MONOMIAL)


def _constant_coeffs(m, U):
    u = np.zeros((m.ne, m.np, 4))
    u[:, 0, :] = U
    return u


def test_two_triangle_mesh_structure():
    """create_test_mesh (tests/test_helpers.h:11-51): one interior face, four boundary
    faces; the boundary-edge list is read as vertex pairs, so two faces carry tag 0."""
    m = _two_tri()
    f = m.interior_faces()
    assert f.tolist() == [[0, 1, 2, 0, 1]]
    b = m.boundary_faces()
    assert b.tolist() == [[0, 0, 2], [0, 1, 3], [1, 1, 0], [1, 2, 0]]


def test_uniform_flow_has_zero_viscous_residual():
    """UniformFlowHasZeroResidual (:202-260), far-field BC on every named tag."""
    m = _two_tri()
    U = primitive_to_conserved([1.0, 0.5, 0.0, 1.0], GAMMA)
    for tag in (1, 2, 3, 4):
        m.set_bc(tag, O.FAR_FIELD, value=U)
    ph = O.navier_stokes(GAMMA, 1.0e-3, 0.72, 5.0)
    u = _constant_coeffs(m, U)
    for e in range(m.ne):
        assert np.abs(m.volume_residual(ph, e, u, viscous=True)).max() < 1e-12
    for k in range(len(m.interior_faces())):
        RL, RR = m.interior_face_residual(ph, k, u, viscous=True)
        assert np.abs(RL).max() < 1e-12 and np.abs(RR).max() < 1e-12
    for k in range(len(m.boundary_faces())):
        assert np.abs(m.boundary_face_residual(ph, k, u, viscous=True)).max() < 1e-12


def _analytic_viscous_flux(U, gU, gamma, mu, pr):
    """AnalyticViscousFlux (:59-121), an independent restatement inside dgfem's test."""
    rho = U[0]
    rho_safe = max(rho, 1e-12)
    u, v = U[1] / rho, U[2] / rho
    p = (gamma - 1) * (U[3] - 0.5 * rho * (u * u + v * v))
    grho, grhou, grhov, gE = gU[0], gU[1], gU[2], gU[3]
    gu = (grhou - u * grho) / rho_safe
    gv = (grhov - v * grho) / rho_safe
    ksq = u * u + v * v
    gp = (gamma - 1) * (gE - 0.5 * ksq * grho - rho * (u * gu + v * gv))
    rho_sq = max(rho * rho, 1e-24)
    gT = (rho * gp - p * grho) / rho_sq
    div = gu[0] + gv[1]
    lam = -2 * mu / 3
    txx = 2 * mu * gu[0] + lam * div
    tyy = 2 * mu * gv[1] + lam * div
    txy = mu * (gu[1] + gv[0])
    kappa = mu * gamma / (pr * (gamma - 1))
    qx, qy = -kappa * gT[0], -kappa * gT[1]
    return (np.array([0, txx, txy, u * txx + v * txy + qx]),
            np.array([0, txy, tyy, u * txy + v * tyy + qy]))


def _shear_setup():
    """make_shear_flow_setup (:123-183): rho=1, rho*u=y, rho*v=0, p=1 in the P1 monomial
    basis [1, eta, xi] from vertex values."""
    m = _two_tri()
    u = np.zeros((m.ne, 3, 4))
    for e in range(m.ne):
        X = m.vertices[m.elements[e]]
        for var, fn in enumerate([lambda x: 1.0, lambda x: x[1], lambda x: 0.0,
                                  lambda x: 1.0 / (GAMMA - 1) + 0.5 * x[1] ** 2]):
            vals = [fn(X[k]) for k in range(3)]
            u[e, :, var] = [vals[0], vals[2] - vals[0], vals[1] - vals[0]]
    return m, u


MU, PR = 5.0e-2, 0.72


def test_shear_flow_volume_residual_matches_analytic():
    """ShearFlowVolumeResidualMatchesAnalytic (:262-324)."""
    m, u = _shear_setup()
    ph = O.navier_stokes(GAMMA, MU, PR, 5.0)
    qp, qw = O.tri_rule(2)
    kappa = MU * GAMMA / (PR * (GAMMA - 1))
    for e in range(m.ne):
        comp = m.volume_residual(ph, e, u, viscous=True)
        d = m.element_data(e)
        J, D = d["J_det_vol"], d["dphi_dx_vol"]
        grhou = sum(u[e, i, 1] * D[i] for i in range(3))
        gE = sum(u[e, i, 3] * D[i] for i in range(3))
        exp = np.zeros((3, 4))
        V = m.vertices[m.elements[e]]
        for q in range(len(qw)):
            w = qw[q] * abs(J[q])
            xi = qp[q]
            y = (np.array([1 - xi[0] - xi[1], xi[0], xi[1]]) @ V)[1]
            for i in range(3):
                g = D[q * 3 + i]
                exp[i, 1] -= w * MU * g[1]
                exp[i, 2] -= w * MU * g[0]
                gpy = (GAMMA - 1) * (gE[1] - y * grhou[1])
                exp[i, 3] -= w * (MU * y - kappa * gpy) * g[1]
        assert np.abs(comp[:, 0]).max() < 1e-12
        assert np.abs(comp[:, 1:] - exp[:, 1:]).max() < 1e-10


def test_shear_flow_interior_face_residual_matches_analytic():
    """ShearFlowInteriorFaceResidualMatchesAnalytic (:326-405)."""
    m, u = _shear_setup()
    ph = O.navier_stokes(GAMMA, MU, PR, 5.0)
    L, R, fL, fR, rev = m.interior_faces()[0]
    cL, cR = m.interior_face_residual(ph, 0, u, viscous=True)
    t = m.tables()
    dL, dR = m.face_data(L, fL), m.face_data(R, fR)
    n, hF = dL["normal"], dL["length"]
    eL, eR = np.zeros((3, 4)), np.zeros((3, 4))
    for q in range(m.nfq):
        w = t["face_w"][q] * hF * 0.5
        qR = m.nfq - 1 - q if rev else q
        pL, pR = t["phi_face"][fL, q], t["phi_face"][fR, qR]
        UL, UR = pL @ u[L], pR @ u[R]
        gUL = np.zeros((4, 2))
        gUR = np.zeros((4, 2))
        for i in range(3):
            gUL += np.outer(u[L, i], dL["dphi_dx_face"][q * 3 + i])
            gUR += np.outer(u[R, i], dR["dphi_dx_face"][qR * 3 + i])
        FL, GL = _analytic_viscous_flux(UL, gUL, GAMMA, MU, PR)
        FR, GR = _analytic_viscous_flux(UR, gUR, GAMMA, MU, PR)
        Fn = 0.5 * (FL * n[0] + GL * n[1]) + 0.5 * (FR * -n[0] + GR * -n[1])
        eL -= w * np.outer(pL, Fn)
        eR += w * np.outer(pR, Fn)
    assert np.abs(cL - eL).max() < 1e-10
    assert np.abs(cR - eR).max() < 1e-10


def test_shear_flow_boundary_face_residual_matches_analytic():
    """ShearFlowBoundaryFaceResidualMatchesAnalytic (:407-503): far-field functor BC
    (1, y, 0, 1) on every named tag; tag-0 faces keep U_bc = U_L."""
    m, u = _shear_setup()
    bcfn = lambda x, y: primitive_to_conserved([1.0, y, 0.0, 1.0], GAMMA)
    for tag in (1, 2, 3, 4):
        m.set_bc(tag, O.FAR_FIELD, fn=bcfn)
    ph = O.navier_stokes(GAMMA, MU, PR, 5.0)
    t = m.tables()
    bf = m.boundary_faces()
    assert len(bf) > 0
    for k, (e, f, tag) in enumerate(bf):
        comp = m.boundary_face_residual(ph, k, u, viscous=True)
        d = m.face_data(e, f)
        n, hF, qpf = d["normal"], d["length"], d["quad_points"]
        sigma = O.penalty(ph, 1, hF)
        exp = np.zeros((3, 4))
        for q in range(m.nfq):
            w = t["face_w"][q] * hF * 0.5
            phi = t["phi_face"][f, q]
            UL = phi @ u[e]
            gU = sum(np.outer(u[e, i], d["dphi_dx_face"][q * 3 + i]) for i in range(3))
            Fv, Gv = _analytic_viscous_flux(UL, gU, GAMMA, MU, PR)
            Ub = bcfn(qpf[q], qpf[q + m.nfq]) if tag in (1, 2, 3, 4) else UL
            Fn = (Fv * n[0] + Gv * n[1]) - sigma * (Ub - UL)
            exp -= w * np.outer(phi, Fn)
        assert np.abs(comp - exp).max() < 1e-10


def test_no_slip_boundary_generates_residual():
    """NoSlipBoundaryGeneratesResidual (:505-536), through the full assembler."""
    m = _two_tri()
    U = primitive_to_conserved([1.0, 0.5, 0.0, 1.0], GAMMA)
    for tag in (1, 2, 3, 4):
        m.set_bc(tag, O.NO_SLIP_WALL, value=[1.0, 0.0, 0.0, 1.0])
    ph = O.navier_stokes(GAMMA, 1.0e-3, 0.72, 5.0)
    R = m.residual(ph, _constant_coeffs(m, U))
    assert sum(np.linalg.norm(R[e]) for e in range(m.ne)) > 1e-6


# ------------------------------------------------------------------ Euler (commented-out in dgfem)
# tests/solver/weak_form_test.cpp:350-384


def test_conserved_primitive_roundtrip_and_rusanov_antisymmetry():
    """ConservedPrimitiveConversion / RusanovFlux (weak_form_test.cpp:355-384)."""
    UL = np.array([1.0, 0.0, 0.0, 2.5])
    UR = np.array([0.125, 0.0, 0.0, 0.25])
    n = np.array([1.0, 0.0])
    H = O.rusanov(1.4, UL, UR, n)
    Hn = O.rusanov(1.4, UR, UL, -n)
    assert np.all(np.abs(H + Hn) <= 1e-12)
    rng = np.random.default_rng(7)
    for _ in range(50):
        W1 = [rng.uniform(0.5, 2), rng.normal(), rng.normal(), rng.uniform(0.5, 2)]
        W2 = [rng.uniform(0.5, 2), rng.normal(), rng.normal(), rng.uniform(0.5, 2)]
        a = primitive_to_conserved(W1)
        b = primitive_to_conserved(W2)
        t = rng.uniform(0, 2 * np.pi)
        nn = np.array([np.cos(t), np.sin(t)])
        # bitwise antisymmetry: the element-centric GPU face kernel relies on it
        assert np.array_equal(O.rusanov(1.4, a, b, nn), -O.rusanov(1.4, b, a, -nn))
