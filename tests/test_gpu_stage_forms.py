"""The CUDA-core forms of the mixed-precision Euler stage, through the C ABI:
DGX_STAGE_KERNEL=rows (neighbour coefficient rows per face), =trace (face traces through
HBM; =trace64 / =trace32 keep its kernel at 64- or 32-element tiles, =trace32s at 32-element
tiles with each element's neighbour trace blocks copied into shared memory) and =pipe (the trace
kernel whose CTAs copy their next tile's inputs while computing a tile).  They perform the same FP32 operations in the same order, so their states agree bit
for bit, p = 1..4, periodic and with far-field / no-slip / slip faces, over step counts that
exercise the one-step and two-step graphs; both stay within the mixed-precision bar of the
FP64 oracle.  With a condition on every boundary face the trace form writes ghost blocks and
runs its kernel without the boundary branch; with faces that have no condition ("skip") it
runs the kernel with it.  Without the variable the autotuner times both and reports its
choice."""

import numpy as np
import pytest

import oracle as O
from meshes import PERIODIC_PAIRS, TAGS, isentropic_vortex, periodic_rectangle
from test_gpu_tensor_core import U_INF, case, rel

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dg():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import dgfem_gb300 as d
    return d


def run(dg, monkeypatch, pm, order, u0, dt, kernel, steps=(3, 2)):
    if kernel:
        monkeypatch.setenv("DGX_STAGE_KERNEL", kernel)
    else:
        monkeypatch.delenv("DGX_STAGE_KERNEL", raising=False)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", order, "dubiner"), dg.EulerWeakFormulation(1.4), "mixed")
    u = torch.tensor(u0, device="cuda")
    for n in steps:
        ctx.rk3_step(u, dt, n)
    torch.cuda.synchronize()
    return u.cpu().numpy(), ctx.stage_form()


@pytest.mark.parametrize("walls", [False, True, "skip"])
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_trace_form_equals_row_form(dg, monkeypatch, order, walls):
    om, pm, u0, dt = case(dg, 9, order, walls)
    ref = om.rk3_step(O.euler(1.4), u0, dt, 5)
    rows, f1 = run(dg, monkeypatch, pm, order, u0, dt, "rows")
    trace, f2 = run(dg, monkeypatch, pm, order, u0, dt, "trace")
    pipe, f3 = run(dg, monkeypatch, pm, order, u0, dt, "pipe")
    assert f1 == "rows" and f2 in ("traces", "traces pipelined")
    # the pipelined kernel needs every boundary face to have a condition (ghost blocks)
    assert f3 == ("rows" if walls == "skip" else "traces pipelined")
    assert np.array_equal(rows, trace)
    assert np.array_equal(rows, pipe)
    assert rel(trace, ref) <= 1e-6
    # 162 elements: 6 tiles of 32 and 3 of 64, the last one partial
    for kernel, tile in (("trace64", 64), ("trace32", 32), ("trace32s", 32)):
        small, form, t, shared = run_tile(dg, monkeypatch, pm, order, u0, dt, kernel)
        assert form == "traces" and t == tile
        # the shared-memory copies need every face to be an interior or a ghost face
        assert shared == (kernel == "trace32s" and walls != "skip")
        assert np.array_equal(rows, small)


def run_tile(dg, monkeypatch, pm, order, u0, dt, kernel):
    monkeypatch.setenv("DGX_STAGE_KERNEL", kernel)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", order, "dubiner"), dg.EulerWeakFormulation(1.4), "mixed")
    u = torch.tensor(u0, device="cuda")
    for n in (3, 2):
        ctx.rk3_step(u, dt, n)
    torch.cuda.synchronize()
    return u.cpu().numpy(), ctx.stage_form(), ctx.stage_tile(), ctx.stage_nbr_shared()


@pytest.mark.parametrize("walls", [False, True])
def test_small_tiles_equal_row_form_many_tiles(dg, monkeypatch, walls):
    """200 x 200 x 2 elements at 64- and 32-element tiles (1250 and 2500 CTAs), the latter also
    with the neighbour blocks through shared memory: bit for bit the row form's state after
    steps (3, 2)."""
    _, pm, u0, dt = case(dg, 200, 3, walls)
    rows, _ = run(dg, monkeypatch, pm, 3, u0, dt, "rows")
    for kernel, tile in (("trace64", 64), ("trace32", 32), ("trace32s", 32)):
        small, form, t, shared = run_tile(dg, monkeypatch, pm, 3, u0, dt, kernel)
        assert form == "traces" and t == tile and shared == (kernel == "trace32s")
        assert np.array_equal(rows, small)


@pytest.mark.parametrize("walls", [False, True])
def test_pipelined_form_equals_row_form_many_tiles(dg, monkeypatch, walls):
    """200 x 200 x 2 elements, 625 tiles: every CTA of the pipelined kernel (2 or 3 per SM)
    walks two to four tiles, each tile's inputs copied while the tile before it is computed.
    The states equal the row form's bit for bit after steps (3, 2) (one call's first, middle and
    last steps, and a call of two)."""
    _, pm, u0, dt = case(dg, 200, 3, walls)
    rows, _ = run(dg, monkeypatch, pm, 3, u0, dt, "rows")
    pipe, form = run(dg, monkeypatch, pm, 3, u0, dt, "pipe")
    assert form == "traces pipelined"
    assert np.isfinite(pipe).all() and np.abs(pipe - u0).max() > 0
    assert np.array_equal(rows, pipe)


def test_pipelined_form_bounded_wait_runs_out_and_reports(dg, monkeypatch):
    """With one poll per wait, the first wait of every CTA of the pipelined kernel gives up
    (its bulk copy cannot have landed yet): the CTA flags a timeout, waits for the copy in
    flight and returns.  dgx_step_status reports DGX_ERR_TIMEOUT; a new context then steps
    correctly."""
    om, pm, u0, dt = case(dg, 8, 3, False)
    monkeypatch.setenv("DGX_TRACE_WAIT_LIMIT", "1")
    monkeypatch.setenv("DGX_STAGE_KERNEL", "pipe")
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), "mixed")
    u = torch.tensor(u0, device="cuda")
    ctx.rk3_step(u, dt, 1)
    torch.cuda.synchronize()
    assert ctx.stage_form() == "traces pipelined"
    with pytest.raises(dg.DGXError) as ex:
        ctx.step_nonfinite()
    assert ex.value.code == dg._lib.ERR_TIMEOUT
    monkeypatch.delenv("DGX_TRACE_WAIT_LIMIT")
    ctx2 = dg.DGContext(pm, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), "mixed")
    u2 = torch.tensor(u0, device="cuda")
    ctx2.rk3_step(u2, dt, 2)
    assert not ctx2.step_nonfinite()
    assert rel(u2.cpu().numpy(), om.rk3_step(O.euler(1.4), u0, dt, 2)) <= 1e-6


@pytest.mark.parametrize("order", [2, 3])
def test_trace_form_equals_row_form_channel(dg, monkeypatch, order):
    """Periodic in x, a slip wall below and far field above: periodic pairs and ghost blocks
    in one mesh."""
    v, e, b = periodic_rectangle(9)
    om = O.OracleMesh(v, e, b, order=order, basis=O.DUBINER, periodic=(PERIODIC_PAIRS[0],))
    om.set_bc(TAGS["Bottom"], O.SLIP_WALL, value=[0.0] * 4)
    om.set_bc(TAGS["Top"], O.FAR_FIELD, value=U_INF)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    pm = dg.DGMesh(v, e, None, dict(TAGS), edges)
    pm.set_periodic_boundaries("Left", "Right")
    pm.set_boundary_condition_euler("Bottom", dg.BoundaryConditionEuler(O.SLIP_WALL, [0.0] * 4))
    pm.set_boundary_condition_euler("Top", dg.BoundaryConditionEuler(O.FAR_FIELD, U_INF))
    u0 = om.project(isentropic_vortex(om.quad_points(), beta=4.0, xc=0.4, yc=-0.3, uinf=0.4))
    dt = 0.02 / om.max_cfl(1.4, u0, 1.0)
    ref = om.rk3_step(O.euler(1.4), u0, dt, 5)
    rows, f1 = run(dg, monkeypatch, pm, order, u0, dt, "rows")
    trace, f2 = run(dg, monkeypatch, pm, order, u0, dt, "trace")
    pipe, f3 = run(dg, monkeypatch, pm, order, u0, dt, "pipe")
    assert f1 == "rows" and f2 in ("traces", "traces pipelined") and f3 == "traces pipelined"
    assert np.array_equal(rows, trace)
    assert np.array_equal(rows, pipe)
    assert rel(trace, ref) <= 1e-6
    small, form, tile, shared = run_tile(dg, monkeypatch, pm, order, u0, dt, "trace32s")
    assert form == "traces" and tile == 32 and shared
    # run_tile makes steps (3, 2) like run
    assert np.array_equal(rows, small)


def test_autotuner_reports_a_form(dg, monkeypatch):
    om, pm, u0, dt = case(dg, 24, 3, False)  # 1152 elements, 9 tiles
    u, form = run(dg, monkeypatch, pm, 3, u0, dt, None, steps=(1,))
    assert form in ("rows", "traces", "traces pipelined", "tensor cores")
    assert rel(u, om.rk3_step(O.euler(1.4), u0, dt, 1)) <= 1e-6
    monkeypatch.delenv("DGX_STAGE_KERNEL", raising=False)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), "mixed")
    assert ctx.stage_tile() == 0
    ctx.rk3_step(torch.tensor(u0, device="cuda"), dt, 1)
    assert ctx.stage_tile() in (128, 64, 32)
    assert ctx.stage_tile() == 128 or ctx.stage_form() == "traces"


@pytest.mark.parametrize("walls", [False, True, "skip"])
@pytest.mark.parametrize("kernel,n", [("rows", 1), ("trace", 1), ("trace", 3), ("pipe", 1), ("pipe", 3),
                                      ("trace64", 1), ("trace32", 3), ("trace32s", 1), ("trace32s", 3),
                                      ("tc", 1), ("tc", 3)])
def test_host_pointer_step_equals_device_step(dg, monkeypatch, kernel, n, walls):
    """dgx_rk3_step_host runs its last step's stage 3 in tile ranges, each copied back to the
    host while the next range computes; the state equals the device-pointer step's bit for bit."""
    om, pm, u0, dt = case(dg, 24, 3, walls)  # 1152 elements: 9 tiles, 4 ranges
    monkeypatch.setenv("DGX_STAGE_KERNEL", kernel)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), "mixed")
    u = torch.tensor(u0, device="cuda")
    ctx.rk3_step(u, dt, n)
    uh = ctx.rk3_step(u0, dt, n)
    assert np.array_equal(u.cpu().numpy(), uh)
    assert rel(uh, om.rk3_step(O.euler(1.4), u0, dt, n)) <= 1e-6


@pytest.mark.parametrize("n", [1, 2])
def test_host_pointer_step_tensor_core_form(dg, monkeypatch, n):
    """The host-pointer step with the tensor-core form (stage 3 in tile ranges, each copied
    back while the next computes) equals the device-pointer step bit for bit."""
    om, pm, u0, dt = case(dg, 24, 3, False)
    monkeypatch.setenv("DGX_STAGE_KERNEL", "tc")
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), "mixed")
    u = torch.tensor(u0, device="cuda")
    ctx.rk3_step(u, dt, n)
    assert ctx.stage_form() == "tensor cores"
    assert np.array_equal(u.cpu().numpy(), ctx.rk3_step(u0, dt, n))


def test_host_pointer_step_quadrilaterals(dg):
    """Mixed quadrilaterals take the host-pointer step without the range-wise overlap; it equals
    the device-pointer step bit for bit."""
    from meshes import PERIODIC_PAIRS, TAGS, quad_rectangle
    v, e, b = quad_rectangle(12, distort=0.2)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    pm = dg.DGMesh(v, e, None, dict(TAGS), edges)
    pm.set_periodic_boundaries("Left", "Right")
    pm.set_periodic_boundaries("Bottom", "Top")
    om = O.OracleMesh(v, e, b, order=3, basis=O.LEGENDRE, periodic=PERIODIC_PAIRS)
    from meshes import isentropic_vortex
    u0 = om.project(isentropic_vortex(om.quad_points(), beta=5.0))
    dt = 0.05 / om.max_cfl(1.4, u0, 1.0)
    ctx = dg.DGContext(pm, dg.DGSpace("quad", 3), dg.EulerWeakFormulation(1.4), "mixed")
    u = torch.tensor(u0, device="cuda")
    ctx.rk3_step(u, dt, 3)
    assert np.array_equal(u.cpu().numpy(), ctx.rk3_step(u0, dt, 3))
