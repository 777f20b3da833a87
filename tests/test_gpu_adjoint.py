"""Differentiation of the FP64 path: tangent-linear (dual numbers) and hand-written adjoint.

* JVP of the residual against central differences of the oracle residual;
* adjoint identity <J v, w> = <v, J^T w> for the residual (periodic and with far-field /
  no-slip faces) and for SSP-RK3 steps (tangent-linear vs adjoint);
* dJ/du0 of the kinetic energy after n steps (checkpointed adjoint) against FP64 central
  differences (h = 1e-6) and against the tangent-linear model;
* the torch.autograd binding.
"""

import numpy as np
import pytest

import oracle as O
from meshes import PERIODIC_PAIRS, TAGS, isentropic_vortex, periodic_rectangle, primitive_to_conserved

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dg():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import dgfem_gb300 as d
    return d


def make(dg, n=6, order=3, visc=False, bcs=False):
    if bcs:
        v, e, b = periodic_rectangle(n, 0.0, 1.0, 0.0, 1.0)
    else:
        v, e, b = periodic_rectangle(n)
    om = O.OracleMesh(v, e, b, order=order, basis=O.DUBINER, periodic=() if bcs else PERIODIC_PAIRS)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    pm = dg.DGMesh(v, e, None, dict(TAGS), edges)
    U_inf = primitive_to_conserved([1.0, 0.4, 0.1, 1.0])
    if bcs:
        spec = [("Bottom", 2, O.NO_SLIP_WALL, [1.0, 0.0, 0.0, 1.0]), ("Right", 3, O.FAR_FIELD, U_inf),
                ("Top", 4, O.NO_SLIP_WALL, [1.0, 0.0, 0.0, 1.0]), ("Left", 5, O.FAR_FIELD, U_inf)]
        for name, tag, typ, val in spec:
            om.set_bc(tag, typ, value=val)
            pm.set_boundary_condition_euler(name, dg.BoundaryConditionEuler(typ, val))
    else:
        pm.set_periodic_boundaries("Left", "Right")
        pm.set_periodic_boundaries("Bottom", "Top")
    wf = dg.NavierStokesWeakFormulation(1.4, 0.01, 0.72, 5.0) if visc else dg.EulerWeakFormulation(1.4)
    ph = O.navier_stokes(1.4, 0.01, 0.72, 5.0) if visc else O.euler(1.4)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", order, "dubiner"), wf, "fp64")
    if bcs:
        u = om.project(np.broadcast_to(U_inf, om.quad_points().shape[:-1] + (4,)).copy())
        u = u + 1e-3 * np.random.default_rng(5).standard_normal(u.shape)
    else:
        u = om.project(isentropic_vortex(om.quad_points(), beta=5.0, xc=0.3))
    return om, ctx, ph, u


def T(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def dot(a, b):
    return float(torch.sum(a * b))


@pytest.mark.parametrize("visc", [False, True])
def test_residual_jvp_matches_oracle_differences(dg, visc):
    om, ctx, ph, u = make(dg, visc=visc)
    v = np.random.default_rng(1).standard_normal(u.shape) * 1e-2
    jv = ctx.residual_jvp(T(u), T(v)).cpu().numpy()
    h = 1e-6
    fd = (om.residual(ph, u + h * v) - om.residual(ph, u - h * v)) / (2 * h)
    assert np.linalg.norm(jv - fd) / np.linalg.norm(fd) <= 1e-6


@pytest.mark.parametrize("bcs", [False, True])
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_residual_adjoint_identity(dg, order, bcs):
    om, ctx, ph, u = make(dg, order=order, bcs=bcs)
    rng = np.random.default_rng(order)
    v = T(rng.standard_normal(u.shape))
    w = T(rng.standard_normal(u.shape))
    ut = T(u)
    lhs = dot(ctx.residual_jvp(ut, v), w)
    rhs = dot(v, ctx.residual_vjp(ut, w))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)


def test_rk3_adjoint_identity(dg):
    om, ctx, ph, u = make(dg, n=8, order=3)
    dt = 0.05 / om.max_cfl(1.4, u, 1.0)
    rng = np.random.default_rng(2)
    du0 = T(rng.standard_normal(u.shape))
    w = T(rng.standard_normal(u.shape))
    n = 3
    ut, dut = T(u), du0.clone()
    ctx.rk3_step_tlm(ut, dut, dt, n)
    # the state the tangent-linear model carries is the forward solution
    ref = om.rk3_step(ph, u, dt, n)
    assert np.linalg.norm(ut.cpu().numpy() - ref) / np.linalg.norm(ref) <= 1e-11
    states = [T(u)]
    for _ in range(n - 1):
        s = states[-1].clone()
        ctx.rk3_step(s, dt, 1)
        states.append(s)
    ubar = w.clone()
    for k in range(n - 1, -1, -1):
        ctx.rk3_step_adjoint(states[k], ubar, dt)
    lhs, rhs = dot(dut, w), dot(du0, ubar)
    assert abs(lhs - rhs) <= 1e-11 * abs(lhs)


def test_kinetic_energy_gradient_fd_and_tlm(dg):
    om, ctx, ph, u = make(dg, n=8, order=3)
    dt = 0.05 / om.max_cfl(1.4, u, 1.0)
    n, ce = 20, 7
    J, g = ctx.kinetic_energy_gradient(T(u), dt, n, ce)
    # J itself against the oracle trajectory
    uT = om.rk3_step(ph, u, dt, n)
    assert abs(J - ctx.kinetic_energy(T(uT))) <= 1e-10 * abs(J)
    rng = np.random.default_rng(16)
    h = 1e-6
    for k in range(4):
        d = rng.standard_normal(u.shape)
        d /= np.linalg.norm(d)
        jp = ctx.kinetic_energy(ctx.rk3_step(T(u + h * d), dt, n))
        jm = ctx.kinetic_energy(ctx.rk3_step(T(u - h * d), dt, n))
        fd = (jp - jm) / (2 * h)
        adj = dot(g, T(d))
        assert abs(adj - fd) <= 1e-6 * max(abs(fd), 1e-8), (k, adj, fd)
        # tangent-linear: dJ = <dJ/du(T), du(T)>
        ut, dut = T(u), T(d)
        ctx.rk3_step_tlm(ut, dut, dt, n)
        _, gT = ctx.kinetic_energy(ut, grad=True)
        tlm = dot(gT, dut)
        assert abs(adj - tlm) <= 1e-10 * max(abs(tlm), 1e-12), (k, adj, tlm)


def test_torch_autograd_binding(dg):
    om, ctx, ph, u = make(dg, n=6, order=2)
    dt = 0.05 / om.max_cfl(1.4, u, 1.0)
    u0 = T(u).requires_grad_(True)
    J = dg.kinetic_energy(dg.rk3_trajectory(u0, ctx, dt, 9, checkpoint_every=4), ctx)
    J.backward()
    J2, g = ctx.kinetic_energy_gradient(T(u), dt, 9, 4)
    assert abs(J.item() - J2) <= 1e-12 * abs(J2)
    assert torch.linalg.vector_norm(u0.grad - g) <= 1e-11 * torch.linalg.vector_norm(g)


def test_adjoint_rejects_unsupported_contexts(dg):
    v, e, b = periodic_rectangle(4)
    m = dg.DGMesh.rectangle(4, 4, -5, 5, -5, 5, periodic=True)
    mixed = dg.DGContext(m, dg.DGSpace("triangle", 2, "dubiner"), dg.EulerWeakFormulation(), "mixed")
    u = torch.ones(mixed.shape, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        mixed.residual_vjp(u, u)
    ns = dg.DGContext(m, dg.DGSpace("triangle", 2, "dubiner"), dg.NavierStokesWeakFormulation(), "fp64")
    with pytest.raises(ValueError):
        ns.residual_vjp(u, u)


def binomial_optimum(n, snapshots):
    """Griewank and Walther's minimal forward-step count for reversing n steps with c = snapshots + 1
    checkpoints (the start state included): t n - C(c + t, t - 1), C(c + t - 1, t - 1) < n <= C(c + t, t)."""
    from math import comb
    if n <= 1:
        return 0
    c = snapshots + 1
    t = 0
    while comb(c + t, t) < n:
        t += 1
    return t * n - comb(c + t, t - 1)


@pytest.mark.parametrize("n,snapshots", [(1, 3), (2, 0), (9, 0), (20, 1), (20, 3), (33, 2), (20, 40)])
def test_binomial_checkpointing_equals_uniform(dg, n, snapshots):
    """The gradient with binomial checkpointing equals the uniform-checkpoint gradient bit for bit
    (the same forward states, the same adjoint steps in the same order); the forward steps it
    recomputes are the published optimum for its memory."""
    om, ctx, ph, u = make(dg, n=6, order=3)
    dt = 0.05 / om.max_cfl(1.4, u, 1.0)
    J1, g1 = ctx.kinetic_energy_gradient(T(u), dt, n, 7)
    J2, g2, st = ctx.kinetic_energy_gradient_binomial(T(u), dt, n, snapshots)
    assert J1 == J2
    assert torch.equal(g1, g2)
    s = min(snapshots, n - 1)
    assert st["states_held"] == s + 1
    assert st["recomputed_steps"] == st["optimal_recomputed_steps"]
    want = n * (n - 1) // 2 if s == 0 else binomial_optimum(n, s)
    assert st["optimal_recomputed_steps"] == want


def test_binomial_checkpointing_long_run(dg):
    """500 steps with 10 snapshots: 11 states instead of the uniform scheme's ~70, the gradient
    still equal bit for bit."""
    om, ctx, ph, u = make(dg, n=4, order=2)
    dt = 0.05 / om.max_cfl(1.4, u, 1.0)
    J1, g1 = ctx.kinetic_energy_gradient(T(u), dt, 500, 23)
    J2, g2, st = ctx.kinetic_energy_gradient_binomial(T(u), dt, 500, 10)
    assert J1 == J2 and torch.equal(g1, g2)
    assert st["recomputed_steps"] == binomial_optimum(500, 10)
    assert st["recomputed_steps"] <= 4 * 500
