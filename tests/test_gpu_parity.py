"""GPU parity of the dgx path against the CPU oracle, through the C ABI.

Tolerances (relative L2 over all entries, the state's own scale):
  FP64 residual (DGAssembler::assemble_euler_residual)      <= 1e-12
  FP64 M^-1 R and SSP-RK3 steps                              <= 1e-11 (Dubiner), 1e-10 (monomial)
  mixed-precision residual (FP32 arithmetic)                 <= 2e-5
"""

import numpy as np
import pytest

import oracle as O
from meshes import PERIODIC_PAIRS, TAGS, isentropic_vortex, periodic_rectangle, primitive_to_conserved, two_triangle_mesh

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


def make_pair(dg, v, e, b, order, basis, periodic, tags=TAGS, bcs=()):
    om = O.OracleMesh(v, e, b, order=order, basis=basis, periodic=PERIODIC_PAIRS if periodic else ())
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    pm = dg.DGMesh(v, e, None, dict(tags), edges)
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


BASES = {"monomial": O.MONOMIAL, "dubiner": O.DUBINER}


@pytest.mark.parametrize("visc", [False, True])
@pytest.mark.parametrize("basis", ["monomial", "dubiner"])
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_residual_fp64_periodic(dg, order, basis, visc):
    v, e, b = periodic_rectangle(6)
    om, pm = make_pair(dg, v, e, b, order, BASES[basis], True)
    oph, wf = physics(dg, visc)
    u = vortex_state(om)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", order, basis), wf, "fp64")
    R_gpu = ctx.residual(torch.tensor(u, device="cuda")).cpu().numpy()
    R_orc = om.residual(oph, u)
    assert rel(R_gpu, R_orc) <= 1e-12
    # the host-pointer entry point gives the same numbers
    assert rel(ctx.residual(u), R_orc) <= 1e-12


@pytest.mark.parametrize("visc", [False, True])
def test_residual_fp64_unstructured_with_boundaries(dg, visc):
    rng = np.random.default_rng(11)
    v, e, b = periodic_rectangle(7, 0.0, 1.0, 0.0, 1.0)
    inner = (v[:, 0] > 0) & (v[:, 0] < 1) & (v[:, 1] > 0) & (v[:, 1] < 1)
    v = v.copy()
    v[inner] += rng.uniform(-0.03, 0.03, size=(inner.sum(), 2))
    e = e[rng.permutation(len(e))]
    U_inf = primitive_to_conserved([1.0, 0.4, 0.1, 1.0])
    bcs = [("Bottom", 2, O.SLIP_WALL, [0, 0, 0, 0]),
           ("Right", 3, O.FAR_FIELD, U_inf),
           ("Top", 4, O.NO_SLIP_WALL, [1.0, 0.0, 0.0, 1.0]),
           ("Left", 5, O.FAR_FIELD, U_inf)]
    om, pm = make_pair(dg, v, e, b, 3, O.DUBINER, False, bcs=bcs)
    oph, wf = physics(dg, visc)
    u = om.project(np.broadcast_to(U_inf, om.quad_points().shape[:-1] + (4,)).copy())
    u = u + 1e-2 * np.random.default_rng(1).standard_normal(u.shape) * np.abs(u).max()
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 3, "dubiner"), wf, "fp64")
    R_gpu = ctx.residual(torch.tensor(u, device="cuda")).cpu().numpy()
    assert rel(R_gpu, om.residual(oph, u)) <= 1e-12


def test_residual_two_triangle_navier_stokes(dg):
    """dgfem's NoSlipBoundaryGeneratesResidual setup (navier_stokes_weak_formulation_test.cpp:505-536)."""
    v, e, b = two_triangle_mesh()
    tags = {"bottom": 1, "right": 2, "top": 3, "left": 4}
    bcs = [(n, t, O.NO_SLIP_WALL, [1.0, 0.0, 0.0, 1.0]) for n, t in tags.items()]
    om, pm = make_pair(dg, v, e, b, 1, O.MONOMIAL, False, tags=tags, bcs=bcs)
    oph, wf = physics(dg, True, mu=1e-3)
    U = primitive_to_conserved([1.0, 0.5, 0.0, 1.0])
    u = np.zeros((2, 3, 4))
    u[:, 0, :] = U
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 1, "monomial"), wf, "fp64")
    R_gpu = ctx.residual(u)
    R_orc = om.residual(oph, u)
    assert sum(np.linalg.norm(R_gpu[k]) for k in range(2)) > 1e-6
    assert rel(R_gpu, R_orc) <= 1e-12


@pytest.mark.parametrize("basis,tol", [("dubiner", 1e-11), ("monomial", 1e-10)])
@pytest.mark.parametrize("order", [2, 3, 4])
def test_rhs_and_mass_inverse_fp64(dg, order, basis, tol):
    v, e, b = periodic_rectangle(5)
    om, pm = make_pair(dg, v, e, b, order, BASES[basis], True)
    oph, wf = physics(dg, False)
    u = vortex_state(om)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", order, basis), wf, "fp64")
    ut = torch.tensor(u, device="cuda")
    assert rel(ctx.rhs(ut).cpu().numpy(), om.rhs(oph, u)) <= tol
    R = om.residual(oph, u)
    assert rel(ctx.apply_mass_inv(torch.tensor(R, device="cuda")).cpu().numpy(), om.apply_mass_inv(R)) <= tol


@pytest.mark.parametrize("visc", [False, True])
@pytest.mark.parametrize("order,basis", [(2, "dubiner"), (3, "dubiner"), (3, "monomial")])
def test_rk3_steps_fp64(dg, order, basis, visc):
    v, e, b = periodic_rectangle(6)
    om, pm = make_pair(dg, v, e, b, order, BASES[basis], True)
    oph, wf = physics(dg, visc, mu=0.01)
    u0 = vortex_state(om, noise=0.0)
    dt = 0.02
    ref = om.rk3_step(oph, u0, dt, 4)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", order, basis), wf, "fp64")
    ut = torch.tensor(u0, device="cuda")
    ctx.rk3_step(ut, dt, 2)
    ctx.rk3_step(ut, dt, 2)  # graph replay
    tol = 1e-11 if basis == "dubiner" else 1e-10
    assert rel(ut.cpu().numpy(), ref) <= tol
    # host entry point
    assert rel(ctx.rk3_step(u0, dt, 4), ref) <= tol


@pytest.mark.parametrize("visc", [False, True])
@pytest.mark.parametrize("order", [2, 3, 4])
def test_residual_mixed_precision(dg, order, visc):
    v, e, b = periodic_rectangle(6)
    om, pm = make_pair(dg, v, e, b, order, O.DUBINER, True)
    oph, wf = physics(dg, visc)
    u = vortex_state(om)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", order, "dubiner"), wf, "mixed")
    R = ctx.residual(torch.tensor(u, device="cuda")).cpu().numpy()
    assert rel(R, om.residual(oph, u)) <= 2e-5


def test_monitors_projection_and_nan(dg):
    v, e, b = periodic_rectangle(8)
    om, pm = make_pair(dg, v, e, b, 3, O.DUBINER, True)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(), "fp64")
    xq = ctx.quad_points()
    assert rel(xq, om.quad_points()) <= 1e-15
    uq = isentropic_vortex(xq, beta=5.0)
    u = ctx.project(torch.tensor(uq, device="cuda"))
    u_ref = om.project(uq)
    assert rel(u.cpu().numpy(), u_ref) <= 1e-12
    assert abs(ctx.max_cfl(u, 0.01) - om.max_cfl(1.4, u_ref, 0.01)) <= 1e-12 * om.max_cfl(1.4, u_ref, 0.01)
    lo, hi = ctx.density_range(u)
    rlo, rhi = om.density_range(u_ref)
    assert abs(lo - rlo) <= 1e-12 and abs(hi - rhi) <= 1e-12
    assert not ctx.has_nan(u)
    bad = u.clone()
    bad[5, 2, 1] = float("nan")
    assert ctx.has_nan(bad)
    neg = u.clone()
    neg[3, 0, 0] = -1.0  # negative density: CFL is +inf, as in compute_max_cfl
    assert ctx.max_cfl(neg, 0.01) == float("inf")


def test_solver_api_runs_and_conserves(dg):
    m = dg.DGMesh.rectangle(8, 8, -5, 5, -5, 5, periodic=True)
    s = dg.EulerDGSolver(m, dg.DGSpace("triangle", 2, "dubiner"))
    frames = s.solve(lambda x: isentropic_vortex(x), 0.1, 0.02, save_every=2)
    assert len(frames) >= 3 and all(np.isfinite(f).all() for f in frames)
    # mass (Dubiner mode 0 carries the mean): conserved to round-off
    m0 = [f.reshape(128, 6, 4)[:, 0, 0].sum() for f in frames]
    assert abs(m0[-1] - m0[0]) <= 1e-12 * abs(m0[0])


@pytest.mark.parametrize("visc", [False, True])
@pytest.mark.parametrize("order", [2, 3, 4])
def test_rk3_mixed_precision_vs_oracle(dg, order, visc):
    """FP32 increments + FP64 accumulation: after 5 steps (one 2-step replay pair and a
    single step), within 1e-6 relative L2 of the FP64 oracle."""
    v, e, b = periodic_rectangle(8)
    om, pm = make_pair(dg, v, e, b, order, O.DUBINER, True)
    oph, wf = physics(dg, visc, mu=0.01)
    u0 = vortex_state(om, noise=0.0)
    dt = 0.02 / om.max_cfl(1.4, u0, 1.0)
    ref = om.rk3_step(oph, u0, dt, 5)
    assert np.isfinite(ref).all()
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", order, "dubiner"), wf, "mixed")
    ut = torch.tensor(u0, device="cuda")
    ctx.rk3_step(ut, dt, 3)
    ctx.rk3_step(ut, dt, 2)
    err = rel(ut.cpu().numpy(), ref)
    assert err <= 1e-6, err
    # the update itself (u^5 - u^0) is accurate to FP32 level
    assert rel(ut.cpu().numpy() - u0, ref - u0) <= 1e-4


def test_config1_vortex_200_steps_fp64(dg):
    """The plain-form workload: periodic [-5,5]^2, 16x16x2 = 512 triangles, Dubiner p=2,
    beta = 5 vortex at the origin on the free stream (1, 0.5, 0, 1), CFL 0.1 under dgfem's
    definition, 200 SSP-RK3 steps.  The 512x6x4 FP64 state equals the oracle's to 1e-10
    after 200 steps (rounding accumulates over 600 RHS evaluations), and both carry the
    same error against the exactly advected vortex."""
    v, e, b = periodic_rectangle(16)
    om, pm = make_pair(dg, v, e, b, 2, O.DUBINER, True)
    u0 = om.project(isentropic_vortex(om.quad_points(), beta=5.0))
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 2, "dubiner"), dg.EulerWeakFormulation(1.4), "fp64")
    ut = torch.tensor(u0, device="cuda")
    dt_gpu = 0.1 / ctx.max_cfl(ut, 1.0)
    dt = 0.1 / om.max_cfl(1.4, u0, 1.0)
    assert abs(dt_gpu - dt) <= 1e-14 * dt
    ref = om.rk3_step(O.euler(1.4), u0, dt, 200)
    ctx.rk3_step(ut, dt, 200)
    out = ut.cpu().numpy()
    assert out.shape == (512, 6, 4)
    assert rel(out, ref) <= 1e-10
    exact = om.project(isentropic_vortex(om.quad_points(), t=200 * dt, beta=5.0))
    assert abs(rel(out, exact) - rel(ref, exact)) <= 1e-8
    assert rel(out, exact) < 2e-3


def test_quad_points_on_device_equal_host_points(dg):
    """dgx_quad_points_device writes the points dgx_quad_points returns (the initial condition
    can then be evaluated on the GPU before dgx_project)."""
    m = dg.DGMesh.rectangle(9, 7, -5.0, 5.0, -3.0, 4.0, periodic=True)
    ctx = dg.DGContext(m, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), "fp64")
    xd = ctx.quad_points_device()
    torch.cuda.synchronize()
    assert np.array_equal(xd.cpu().numpy(), ctx.quad_points())
