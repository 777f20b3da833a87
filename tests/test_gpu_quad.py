"""GPU parity of the quadrilateral path (DGSpace("quad", p), LegendreBasis, bilinear
elements) against the CPU oracle, through the C ABI.

Tolerances (relative L2 over all entries):
  FP64 residual                                   <= 1e-12
  FP64 M_K^-1 R, projection and SSP-RK3 steps     <= 1e-11
  double-float (df64) residual                    <= 1e-11
  mixed (FP32 arithmetic) residual                <= 2e-5
  mixed M_K^-1 R                                  <= 5e-5 (M_K^-1 lifts the high modes)
  mixed SSP-RK3, 5 steps                          <= 1e-6
The element mass inverse is applied as D^-1 Phi^T diag(w/|J|) Phi D^-1 on the GPU and as
dgfem's LU inverse of the assembled M_K in the oracle: equal in exact arithmetic.
"""

import numpy as np
import pytest

import oracle as O
from meshes import PERIODIC_PAIRS, TAGS, isentropic_vortex, primitive_to_conserved, quad_rectangle

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dg():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import dgfem_gb300 as d
    return d


def rel(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_pair(dg, v, e, b, order, periodic, bcs=()):
    om = O.OracleMesh(v, e, b, order=order, basis=O.LEGENDRE, periodic=PERIODIC_PAIRS if periodic else ())
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    pm = dg.DGMesh(v, e, None, dict(TAGS), edges)
    if periodic:
        pm.set_periodic_boundaries("Left", "Right")
        pm.set_periodic_boundaries("Bottom", "Top")
    for name, tag, typ, val in bcs:
        om.set_bc(tag, typ, value=val)
        pm.set_boundary_condition_euler(name, dg.BoundaryConditionEuler(typ, val))
    return om, pm


def physics(dg, visc, mu=0.05, pr=0.72, s0=5.0):
    if visc:
        return O.navier_stokes(1.4, mu, pr, s0), dg.NavierStokesWeakFormulation(1.4, mu, pr, s0)
    return O.euler(1.4), dg.EulerWeakFormulation(1.4)


def vortex_state(om, seed=0, noise=1e-3):
    u = om.project(isentropic_vortex(om.quad_points(), beta=5.0, xc=0.3, yc=-0.2))
    rng = np.random.default_rng(seed)
    return u + noise * rng.standard_normal(u.shape) * np.abs(u).max()


@pytest.mark.parametrize("visc", [False, True])
@pytest.mark.parametrize("distort", [0.0, 0.2])
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_quad_residual_fp64_periodic(dg, order, distort, visc):
    v, e, b = quad_rectangle(6, distort=distort, seed=order)
    om, pm = make_pair(dg, v, e, b, order, True)
    oph, wf = physics(dg, visc)
    u = vortex_state(om)
    ctx = dg.DGContext(pm, dg.DGSpace("quad", order), wf, "fp64")
    assert ctx.shape == (36, (order + 1) ** 2, 4)
    R_gpu = ctx.residual(torch.tensor(u, device="cuda")).cpu().numpy()
    R_orc = om.residual(oph, u)
    assert rel(R_gpu, R_orc) <= 1e-12
    assert rel(ctx.residual(u), R_orc) <= 1e-12  # host-pointer entry point


@pytest.mark.parametrize("order", [3, 4])
@pytest.mark.parametrize("visc", [False, True])
def test_quad_residual_fp64_boundaries(dg, visc, order):
    """Slip wall, far field and no-slip wall faces on a distorted, element-permuted mesh."""
    rng = np.random.default_rng(5)
    v, e, b = quad_rectangle(7, 0.0, 1.0, 0.0, 1.0, distort=0.2, seed=3)
    e = e[rng.permutation(len(e))]
    U_inf = primitive_to_conserved([1.0, 0.4, 0.1, 1.0])
    bcs = [("Bottom", 2, O.SLIP_WALL, [0, 0, 0, 0]),
           ("Right", 3, O.FAR_FIELD, U_inf),
           ("Top", 4, O.NO_SLIP_WALL, [1.0, 0.0, 0.0, 1.0]),
           ("Left", 5, O.FAR_FIELD, U_inf)]
    om, pm = make_pair(dg, v, e, b, order, False, bcs=bcs)
    oph, wf = physics(dg, visc)
    u = om.project(np.broadcast_to(U_inf, om.quad_points().shape[:-1] + (4,)).copy())
    u = u + 1e-2 * np.random.default_rng(1).standard_normal(u.shape) * np.abs(u).max()
    ctx = dg.DGContext(pm, dg.DGSpace("quad", order), wf, "fp64")
    R_gpu = ctx.residual(torch.tensor(u, device="cuda")).cpu().numpy()
    assert rel(R_gpu, om.residual(oph, u)) <= 1e-12


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_quad_rhs_and_mass_inverse_fp64(dg, order):
    v, e, b = quad_rectangle(5, distort=0.25, seed=11)
    om, pm = make_pair(dg, v, e, b, order, True)
    oph, wf = physics(dg, False)
    u = vortex_state(om)
    ctx = dg.DGContext(pm, dg.DGSpace("quad", order), wf, "fp64")
    ut = torch.tensor(u, device="cuda")
    assert rel(ctx.rhs(ut).cpu().numpy(), om.rhs(oph, u)) <= 1e-11
    R = om.residual(oph, u)
    assert rel(ctx.apply_mass_inv(torch.tensor(R, device="cuda")).cpu().numpy(), om.apply_mass_inv(R)) <= 1e-11


@pytest.mark.parametrize("visc", [False, True])
@pytest.mark.parametrize("order", [2, 3, 4])
def test_quad_rk3_steps_fp64(dg, order, visc):
    v, e, b = quad_rectangle(6, distort=0.15, seed=2)
    om, pm = make_pair(dg, v, e, b, order, True)
    oph, wf = physics(dg, visc, mu=0.01)
    u0 = vortex_state(om, noise=0.0)
    # at CFL 0.1 the p=4 Navier-Stokes step diverges in the oracle itself (NaN within 4 steps)
    dt = (0.05 if order == 4 else 0.1) / om.max_cfl(1.4, u0, 1.0)
    ref = om.rk3_step(oph, u0, dt, 4)
    assert np.isfinite(ref).all()
    ctx = dg.DGContext(pm, dg.DGSpace("quad", order), wf, "fp64")
    ut = torch.tensor(u0, device="cuda")
    ctx.rk3_step(ut, dt, 2)
    ctx.rk3_step(ut, dt, 2)  # graph replay
    assert rel(ut.cpu().numpy(), ref) <= 1e-11
    assert rel(ctx.rk3_step(u0, dt, 4), ref) <= 1e-11


@pytest.mark.parametrize("order", [3, 4])
def test_quad_monitors_and_projection(dg, order):
    v, e, b = quad_rectangle(8, distort=0.2, seed=4)
    om, pm = make_pair(dg, v, e, b, order, True)
    ctx = dg.DGContext(pm, dg.DGSpace("quad", order), dg.EulerWeakFormulation(), "fp64")
    xq = ctx.quad_points()
    assert rel(xq, om.quad_points()) <= 1e-15
    uq = isentropic_vortex(xq, beta=5.0)
    u = ctx.project(torch.tensor(uq, device="cuda"))
    u_ref = om.project(uq)
    assert rel(u.cpu().numpy(), u_ref) <= 1e-11
    cfl = om.max_cfl(1.4, u_ref, 0.01)
    assert abs(ctx.max_cfl(u, 0.01) - cfl) <= 1e-11 * cfl
    lo, hi = ctx.density_range(u)
    rlo, rhi = om.density_range(u_ref)
    assert abs(lo - rlo) <= 1e-11 and abs(hi - rhi) <= 1e-11
    neg = u.clone()
    neg[3, 0, 0] = -1.0
    assert ctx.max_cfl(neg, 0.01) == float("inf")


def test_quad_solver_api_conserves_mass(dg):
    """EulerDGSolver on a uniform periodic quad mesh: on equal squares the Legendre mode 0
    carries the element mean, so the total mass is sum_e u[e, 0, 0] up to a constant."""
    v, e, b = quad_rectangle(8)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    m = dg.DGMesh(v, e, None, dict(TAGS), edges)
    m.set_periodic_boundaries("Left", "Right")
    m.set_periodic_boundaries("Bottom", "Top")
    s = dg.EulerDGSolver(m, dg.DGSpace("quad", 2))
    frames = s.solve(lambda x: isentropic_vortex(x), 0.1, 0.02, save_every=2)
    assert len(frames) >= 3 and all(np.isfinite(f).all() for f in frames)
    m0 = [f.reshape(64, 9, 4)[:, 0, 0].sum() for f in frames]
    assert abs(m0[-1] - m0[0]) <= 1e-12 * abs(m0[0])


def test_quad_unsupported_forms_fail_loudly(dg):
    v, e, b = quad_rectangle(3)
    m = dg.DGMesh(v, e, None, dict(TAGS), {})
    with pytest.raises(dg.DGXError):
        dg.DGContext(m, dg.DGSpace("quad", 5), dg.EulerWeakFormulation(), "fp64")
    tri = dg.DGMesh.rectangle(2, 2, 0, 1, 0, 1)
    with pytest.raises(dg.DGXError):
        dg.DGContext(tri, dg.DGSpace("quad", 2), dg.EulerWeakFormulation(), "fp64")
    ctx = dg.DGContext(m, dg.DGSpace("quad", 2), dg.EulerWeakFormulation(), "fp64")
    u = torch.zeros(ctx.shape, dtype=torch.float64, device="cuda")
    with pytest.raises(dg.DGXError):
        ctx.residual_vjp(u, u)


@pytest.mark.parametrize("visc", [False, True])
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_quad_residual_mixed_and_df64(dg, order, visc):
    v, e, b = quad_rectangle(6, distort=0.2, seed=order)
    om, pm = make_pair(dg, v, e, b, order, True)
    oph, wf = physics(dg, visc)
    u = vortex_state(om)
    R_orc = om.residual(oph, u)
    ut = torch.tensor(u, device="cuda")
    mixed = dg.DGContext(pm, dg.DGSpace("quad", order), wf, "mixed")
    R_mx = mixed.residual(ut).cpu().numpy()
    assert rel(R_mx, R_orc) <= 2e-5
    df = dg.DGContext(pm, dg.DGSpace("quad", order), wf, "df64")
    assert rel(df.residual(ut).cpu().numpy(), R_orc) <= 1e-11
    # the rhs entry of the FP32 form applies M_K^-1 in FP64 to its FP32 residual
    rhs_mx = mixed.rhs(ut).cpu().numpy()
    assert rel(rhs_mx, om.apply_mass_inv(R_mx)) <= 1e-11
    # M_K^-1 scales Legendre mode (i, j) by about (2i+1)(2j+1)/4 (up to 20 at p=4), which lifts
    # the FP32 residual's relative error in the high modes: 5e-5 of the oracle's M_K^-1 R
    assert rel(rhs_mx, om.rhs(oph, u)) <= 5e-5


@pytest.mark.parametrize("visc", [False, True])
@pytest.mark.parametrize("order", [2, 3, 4])
def test_quad_rk3_mixed_precision_vs_oracle(dg, order, visc):
    """FP32 residual and stage increment, FP64 state and RK3 combination: after 5 steps
    within 1e-6 relative L2 of the FP64 oracle; the update itself to FP32 level."""
    v, e, b = quad_rectangle(8, distort=0.15, seed=9)
    om, pm = make_pair(dg, v, e, b, order, True)
    oph, wf = physics(dg, visc, mu=0.01)
    u0 = vortex_state(om, noise=0.0)
    # CFL 0.02: at 0.1 the p=3 Navier-Stokes step is unstable in the oracle itself (a 1e-7
    # perturbation of u0 grows 80x in 5 steps), which would amplify FP32 rounding alike
    dt = 0.02 / om.max_cfl(1.4, u0, 1.0)
    ref = om.rk3_step(oph, u0, dt, 5)
    ctx = dg.DGContext(pm, dg.DGSpace("quad", order), wf, "mixed")
    ut = torch.tensor(u0, device="cuda")
    ctx.rk3_step(ut, dt, 3)
    ctx.rk3_step(ut, dt, 2)
    out = ut.cpu().numpy()
    assert rel(out, ref) <= 1e-6
    assert rel(out - u0, ref - u0) <= 1e-4
