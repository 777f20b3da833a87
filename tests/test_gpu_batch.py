"""Batched independent solves (dgx_batch_*) and the launch-shape autotuner, on the GPU.

* every instance of a batch (uneven meshes, orders 1..4, its own time step) ends where the
  same instance run alone through a mixed-precision context ends (same FP32 stage code,
  same rounding: <= 1e-12 relative), and within the mixed tolerance of the FP64 oracle;
* batches with boundary faces (far-field / no-slip next to periodic instances);
* Navier-Stokes batches (shared viscous parameters) against single viscous solves;
* the grid the autotuner picks is one of its candidates; DGX_AUTOTUNE=0 keeps one CTA per
  tile.
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


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


U_INF = primitive_to_conserved([1.0, 0.4, 0.1, 1.0])
WALLS = [("Bottom", 2, O.NO_SLIP_WALL, [1.0, 0.0, 0.0, 1.0]), ("Right", 3, O.FAR_FIELD, U_INF),
         ("Top", 4, O.FAR_FIELD, U_INF), ("Left", 5, O.FAR_FIELD, U_INF)]


def instance(dg, n, order, beta, xc, yc, uinf, walls=False):
    v, e, b = periodic_rectangle(n)
    om = O.OracleMesh(v, e, b, order=order, basis=O.DUBINER, periodic=() if walls else PERIODIC_PAIRS)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    pm = dg.DGMesh(v, e, None, dict(TAGS), edges)
    if walls:
        for name, tag, typ, val in WALLS:
            om.set_bc(tag, typ, value=val)
            pm.set_boundary_condition_euler(name, dg.BoundaryConditionEuler(typ, val))
    else:
        pm.set_periodic_boundaries("Left", "Right")
        pm.set_periodic_boundaries("Bottom", "Top")
    u0 = om.project(isentropic_vortex(om.quad_points(), beta=beta, xc=xc, yc=yc, uinf=uinf))
    dt = 0.02 / om.max_cfl(1.4, u0, 1.0)
    return om, pm, u0, dt


SPECS = [  # n, order, beta, xc, yc, u_inf: uneven sizes, orders 1..4, several per order
    (4, 1, 2.0, 0.5, -1.0, 0.3), (10, 2, 4.5, -1.5, 0.2, 0.7), (5, 3, 1.5, 1.0, 1.0, 0.2),
    (9, 2, 3.0, 0.0, -2.0, 0.5), (3, 4, 2.5, -0.5, 0.5, 0.6), (7, 3, 5.0, 1.8, -0.3, 0.4),
    (12, 3, 3.5, -1.0, 1.5, 0.8), (6, 1, 1.2, 0.2, 0.2, 0.25),
]


def build(dg, specs, walls=()):
    """[(oracle mesh, product mesh, u0, dt)] and the orders, one entry per spec."""
    return [instance(dg, *sp, walls=(k in walls)) for k, sp in enumerate(specs)], [sp[1] for sp in specs]


def run_batch(dg, insts, orders, steps=(3, 2), wf=None):
    batch = dg.DGBatch([i[1] for i in insts], [dg.DGSpace("triangle", p, "dubiner") for p in orders], wf)
    for k, (om, pm, u0, dt) in enumerate(insts):
        batch.state(k).copy_(torch.tensor(u0, device="cuda"))
    dts = [i[3] for i in insts]
    for n in steps:
        batch.rk3_step(dts, n)
    torch.cuda.synchronize()
    return batch, [batch.state(k).cpu().numpy() for k in range(len(insts))]


def single(dg, om, pm, u0, dt, order, steps=(3, 2), wf=None):
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", order, "dubiner"), wf or dg.EulerWeakFormulation(1.4), "mixed")
    u = torch.tensor(u0, device="cuda")
    for n in steps:
        ctx.rk3_step(u, dt, n)
    return u.cpu().numpy()


@pytest.mark.parametrize("walls", [(), (1, 4, 6)])
def test_batch_face_trace_form_equals_batched_kernel(dg, monkeypatch, walls):
    """An Euler batch run by the single context's face-trace kernel (one launch per order and
    stage, DGX_STAGE_KERNEL=trace32s) equals the batched row-form kernel (=rows) bit for bit after
    steps (3, 2): one call's first, middle and last steps, and a call of two.  Uneven sizes and
    orders 1..4, so each order's range ends in a partial 32-element tile.  With walls, instances
    1, 4 and 6 have far-field and no-slip sides: their orders' trace buffers end in ghost blocks,
    the other orders' do not."""
    insts, orders = build(dg, SPECS, walls)
    monkeypatch.setenv("DGX_STAGE_KERNEL", "rows")
    brows, rows = run_batch(dg, insts, orders)
    assert brows.stage_form() == "batched rows"
    monkeypatch.setenv("DGX_STAGE_KERNEL", "trace32s")
    batch, trace = run_batch(dg, insts, orders)
    assert batch.stage_form() == "traces per order"
    grid, tiles = batch.launch_shape()
    assert grid == tiles
    for k in range(len(insts)):
        assert np.isfinite(trace[k]).all() and np.abs(trace[k] - insts[k][2]).max() > 0
        assert np.array_equal(rows[k], trace[k]), k


@pytest.mark.parametrize("walls", [(), (1, 4, 6)])
def test_batch_matches_single_solves_and_oracle(dg, monkeypatch, walls):
    # the single solves run a CUDA-core form, which the batched kernel equals bit for bit (the
    # tensor-core form rounds differently)
    monkeypatch.setenv("DGX_STAGE_KERNEL", "trace")
    insts, orders = build(dg, SPECS, walls)
    batch, outs = run_batch(dg, insts, orders)
    for k, ((om, pm, u0, dt), order) in enumerate(zip(insts, orders)):
        alone = single(dg, om, pm, u0, dt, order)
        assert rel(outs[k], alone) <= 1e-12, (k, rel(outs[k], alone))
        ref = om.rk3_step(O.euler(1.4), u0, dt, 5)
        assert np.isfinite(ref).all()
        assert rel(outs[k], ref) <= 1e-6, (k, rel(outs[k], ref))
        assert rel(outs[k] - u0, ref - u0) <= 1e-4


@pytest.mark.parametrize("walls", [(), (0, 3)])
def test_batch_navier_stokes_matches_single_solves_and_oracle(dg, walls):
    """Navier-Stokes instances (shared mu, Prandtl, sigma0) of orders 1..4: each equals its
    mixed-precision context run alone (the same viscous stage code) and stays within the mixed
    tolerance of the FP64 oracle."""
    mu, pr, s0 = 0.01, 0.72, 5.0
    wf = dg.NavierStokesWeakFormulation(1.4, mu, pr, s0)
    specs = [(5, 1, 2.0, 0.5, -1.0, 0.3), (6, 2, 3.0, -1.0, 0.2, 0.5), (4, 3, 2.5, 1.0, 1.0, 0.2),
             (3, 4, 2.0, -0.5, 0.5, 0.4), (7, 3, 4.0, 0.3, -0.6, 0.6)]
    insts, orders = build(dg, specs, walls)
    batch, outs = run_batch(dg, insts, orders, wf=wf)
    for k, ((om, pm, u0, dt), order) in enumerate(zip(insts, orders)):
        alone = single(dg, om, pm, u0, dt, order, wf=wf)
        assert rel(outs[k], alone) <= 1e-12, (k, rel(outs[k], alone))
        ref = om.rk3_step(O.navier_stokes(1.4, mu, pr, s0), u0, dt, 5)
        assert np.isfinite(ref).all()
        assert rel(outs[k], ref) <= 1e-6, (k, rel(outs[k], ref))
        assert rel(outs[k] - u0, ref - u0) <= 1e-4


def test_batch_state_views_and_shapes(dg):
    insts, orders = build(dg, SPECS[:3])
    batch = dg.DGBatch([i[1] for i in insts], [dg.DGSpace("triangle", p, "dubiner") for p in orders])
    for k, (om, pm, u0, dt) in enumerate(insts):
        assert batch.shapes[k] == u0.shape
        s = batch.state(k)
        assert s.shape == u0.shape and s.dtype == torch.float64 and s.is_cuda
        assert float(torch.abs(s).max()) == 0.0  # zero after creation
        s.copy_(torch.tensor(u0, device="cuda"))
    for k, (om, pm, u0, dt) in enumerate(insts):  # views alias the batch's memory
        assert np.array_equal(batch.state(k).cpu().numpy(), u0)
    with pytest.raises(IndexError):
        batch.state(len(insts))
    with pytest.raises(ValueError):
        batch.rk3_step([0.01] * len(insts[:-1]) + [0.0])


def test_batch_launch_shape_is_a_candidate(dg):
    # with a 120 x 120 x 2 instance there are more tiles than SMs, so candidates differ
    insts, orders = build(dg, SPECS + [(120, 2, 3.0, 0.0, 0.0, 0.5)])
    batch, _ = run_batch(dg, insts, orders, steps=(1,))
    grid, tiles = batch.launch_shape()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    # the instances of one order share one element range, cut into 128-element tiles
    per_order = {}
    for (_, pm, _, _), p in zip(insts, orders):
        per_order[p] = per_order.get(p, 0) + pm.get_n_elements()
    assert tiles == sum(-(-ne // 128) for ne in per_order.values())
    assert grid == tiles or (grid % sms == 0 and sms <= grid < tiles), (grid, tiles)


def test_context_autotuner_and_switch(dg, monkeypatch):
    # element counts no other test uses, so the tuner sees new keys; more tiles than SMs
    om, pm, u0, dt = instance(dg, 111, 2, 3.0, 0.0, 0.0, 0.5)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 2, "dubiner"), dg.EulerWeakFormulation(1.4), "mixed")
    assert ctx.launch_shape()[0] == 0
    u = torch.tensor(u0, device="cuda")
    ctx.rk3_step(u, dt, 2)
    grid, tiles, _ = ctx.launch_shape()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    assert grid == tiles or (grid % sms == 0 and grid < tiles)
    ref = om.rk3_step(O.euler(1.4), u0, dt, 2)
    assert rel(u.cpu().numpy(), ref) <= 1e-6
    # with the tuner off, a fresh key gets one CTA per tile
    monkeypatch.setenv("DGX_AUTOTUNE", "0")
    om2, pm2, _, _ = instance(dg, 113, 2, 3.0, 0.0, 0.0, 0.5)
    ctx2 = dg.DGContext(pm2, dg.DGSpace("triangle", 2, "dubiner"), dg.EulerWeakFormulation(1.4), "mixed")
    u2 = torch.tensor(om2.project(isentropic_vortex(om2.quad_points(), beta=3.0)), device="cuda")
    ctx2.rk3_step(u2, dt, 1)
    g2, t2, tc2 = ctx2.launch_shape()
    assert g2 == t2 and not tc2
