"""The two CUDA-core forms of the mixed-precision Euler stage, through the C ABI:
DGX_STAGE_KERNEL=rows (neighbour coefficient rows per face) and =trace (face traces through
HBM).  They perform the same FP32 operations in the same order, so their states agree bit
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
    assert (f1, f2) == ("rows", "traces")
    assert np.array_equal(rows, trace)
    assert rel(trace, ref) <= 1e-6


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
    assert (f1, f2) == ("rows", "traces")
    assert np.array_equal(rows, trace)
    assert rel(trace, ref) <= 1e-6


def test_autotuner_reports_a_form(dg, monkeypatch):
    om, pm, u0, dt = case(dg, 24, 3, False)  # 1152 elements, 9 tiles
    u, form = run(dg, monkeypatch, pm, 3, u0, dt, None, steps=(1,))
    assert form in ("rows", "traces")
    assert rel(u, om.rk3_step(O.euler(1.4), u0, dt, 1)) <= 1e-6


@pytest.mark.parametrize("walls", [False, True, "skip"])
@pytest.mark.parametrize("kernel,n", [("rows", 1), ("trace", 1), ("trace", 3), ("tc", 1), ("tc", 3)])
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
