"""Element partitions on the GPU: FP64 contexts on the parts' meshes, stepped stage by stage with
dgx_rk3_stage and the halo rows exchanged between stages in one process (one GPU holds every
part; across GPUs the exchange is torch.distributed point-to-point, tested on gloo ranks in
test_partition.py).  Five steps on 2 and 4 parts equal dgx_rk3_step on the whole mesh bit for
bit, and three dgx_rk3_stage calls equal one dgx_rk3_step."""

import numpy as np
import pytest

from test_partition import TAGS, case, edges_of, make_plan
from meshes import isentropic_vortex

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dg():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import dgfem_gb300 as d
    return d


def whole_context(dg, kind):
    v, e, b, periodic, bcs, phys, order = case(kind)
    m = dg.DGMesh(v, e, None, TAGS, edges_of(b))
    for t1, t2 in periodic:
        m.set_periodic_boundaries(t1, t2)
    for name, (t, val) in bcs.items():
        m.set_boundary_condition_euler(name, dg.BoundaryConditionEuler(t, val))
    wf = (dg.NavierStokesWeakFormulation(1.4, 0.02, 0.72, 5.0) if phys.viscous else dg.EulerWeakFormulation(1.4))
    return m, dg.DGSpace("triangle", order, "dubiner"), wf


@pytest.mark.parametrize("n_parts", [2, 4])
@pytest.mark.parametrize("kind", ["euler", "ns", "walls", "channel"])
def test_partitioned_gpu_run_equals_whole_mesh(dg, kind, n_parts):
    from dgfem_gb300.partition import step_local
    m, space, wf = whole_context(dg, kind)
    ctx = dg.DGContext(m, space, wf, "fp64")
    u0 = ctx.project(torch.tensor(isentropic_vortex(ctx.quad_points(), beta=4.0, xc=0.4, yc=-0.3, uinf=0.4),
                                  device="cuda"))
    dt = 0.02 / ctx.max_cfl(u0, 1.0)
    whole = u0.clone()
    ctx.rk3_step(whole, dt, 5)
    v, e, b, periodic, bcs, _, _ = case(kind)
    plan = make_plan(dg, v, e, b, periodic, bcs, n_parts)
    ctxs = [dg.DGContext(plan.mesh(dg, r), space, wf, "fp64") for r in range(n_parts)]
    states = [torch.tensor(s, device="cuda") for s in plan.scatter(u0.cpu().numpy())]
    step_local(plan, ctxs, states, dt, 5)
    torch.cuda.synchronize()
    got = plan.gather([s.cpu().numpy() for s in states])
    ref = whole.cpu().numpy()
    assert np.isfinite(ref).all() and np.linalg.norm(ref - u0.cpu().numpy()) > 0
    assert np.array_equal(got, ref), np.abs(got - ref).max()


def test_three_stages_equal_one_step(dg):
    m, space, wf = whole_context(dg, "euler")
    ctx = dg.DGContext(m, space, wf, "fp64")
    u0 = ctx.project(torch.tensor(isentropic_vortex(ctx.quad_points(), beta=4.0), device="cuda"))
    dt = 0.02 / ctx.max_cfl(u0, 1.0)
    a = u0.clone()
    ctx.rk3_step(a, dt, 1)
    u, w1, w2 = u0.clone(), torch.empty_like(u0), torch.empty_like(u0)
    ctx.rk3_stage(u, u, w1, dt, 1)
    ctx.rk3_stage(u, w1, w2, dt, 2)
    ctx.rk3_stage(u, w2, u, dt, 3)
    torch.cuda.synchronize()
    assert torch.equal(u, a)
    mixed = dg.DGContext(m, space, wf, "mixed")
    with pytest.raises(ValueError):
        mixed.rk3_stage(u, u, w1, dt, 1)
