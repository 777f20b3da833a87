"""The tensor-core (3xTF32 tcgen05) form of the mixed-precision Euler stage, through the
C ABI.  DGX_STAGE_KERNEL=tc makes the autotuner take it (orders 1-3, meshes whose faces are
all interior faces or boundary faces with a condition); =trace keeps the CUDA-core
face-trace form.

* p = 1..3, periodic and with far-field / no-slip / slip faces: 5 RK3 steps within 1e-6
  relative L2 of the FP64 oracle (the mixed-precision bar) and within 1e-6 of the CUDA-core
  form; the increments within 1e-4;
* the bench workload at t_final: 512 x 512 x 2 triangles, Dubiner p=3, 500 steps at CFL 0.05:
  within 1e-6 relative L2 of the FP64 path (the target of the mixed-precision form);
* a mesh with more tiles than SMs (each CTA walks several tiles, two in flight);
* no tensor-core form at p = 4, on meshes with faces that take no part, and for
  Navier-Stokes: the choice falls back to CUDA cores;
* a bounded wait that runs out (DGX_TC_WAIT_LIMIT=1 poll): the kernels report
  DGX_ERR_TIMEOUT through dgx_step_status, return, and the context works afterwards.
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


def case(dg, n, order, walls):
    v, e, b = periodic_rectangle(n)
    if walls:  # perturb interior vertices: unstructured, non-uniform elements
        rng = np.random.default_rng(3)
        inner = (np.abs(v[:, 0]) < 4.99) & (np.abs(v[:, 1]) < 4.99)
        v = v.copy()
        v[inner] += 0.15 * (10.0 / n) * rng.uniform(-1, 1, (inner.sum(), 2))
    om = O.OracleMesh(v, e, b, order=order, basis=O.DUBINER, periodic=() if walls else PERIODIC_PAIRS)
    edges = {}
    for t, a, c in b:
        edges.setdefault(int(t), []).append((int(a), int(c)))
    pm = dg.DGMesh(v, e, None, dict(TAGS), edges)
    if walls:
        spec = [("Bottom", 2, O.NO_SLIP_WALL, [1.0, 0.0, 0.0, 1.0]), ("Right", 3, O.FAR_FIELD, U_INF),
                ("Top", 4, O.SLIP_WALL, [0.0, 0.0, 0.0, 0.0]), ("Left", 5, O.FAR_FIELD, U_INF)]
        for name, tag, typ, val in spec:
            if walls == "skip" and name == "Top":  # no condition: both sides skip these faces
                continue
            om.set_bc(tag, typ, value=val)
            pm.set_boundary_condition_euler(name, dg.BoundaryConditionEuler(typ, val))
    else:
        pm.set_periodic_boundaries("Left", "Right")
        pm.set_periodic_boundaries("Bottom", "Top")
    u0 = om.project(isentropic_vortex(om.quad_points(), beta=4.0, xc=0.4, yc=-0.3, uinf=0.4))
    dt = 0.02 / om.max_cfl(1.4, u0, 1.0)
    return om, pm, u0, dt


def run(dg, monkeypatch, pm, order, u0, dt, kernel, steps=(3, 2), wf=None):
    monkeypatch.setenv("DGX_STAGE_KERNEL", kernel)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", order, "dubiner"), wf or dg.EulerWeakFormulation(1.4), "mixed")
    u = torch.tensor(u0, device="cuda")
    for n in steps:
        ctx.rk3_step(u, dt, n)
    torch.cuda.synchronize()
    assert not ctx.step_nonfinite()
    return u.cpu().numpy(), ctx.launch_shape()


@pytest.mark.parametrize("walls", [False, True])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_tensor_core_stage_vs_oracle(dg, monkeypatch, order, walls):
    om, pm, u0, dt = case(dg, 7, order, walls)
    ref = om.rk3_step(O.euler(1.4), u0, dt, 5)
    assert np.isfinite(ref).all()
    u_tc, (grid, tiles, tc) = run(dg, monkeypatch, pm, order, u0, dt, "tc")
    assert tc and grid == tiles
    u_cc, (_, _, tc2) = run(dg, monkeypatch, pm, order, u0, dt, "trace")
    assert not tc2
    assert rel(u_tc, ref) <= 1e-6, rel(u_tc, ref)
    assert rel(u_tc - u0, ref - u0) <= 1e-4, rel(u_tc - u0, ref - u0)
    assert rel(u_tc, u_cc) <= 1e-6


def test_tensor_core_stage_walks_several_tiles(dg, monkeypatch):
    om, pm, u0, dt = case(dg, 111, 2, False)  # 24,642 elements: 193 tiles, more than SMs
    ref = om.rk3_step(O.euler(1.4), u0, dt, 3)
    u_tc, (grid, tiles, tc) = run(dg, monkeypatch, pm, 2, u0, dt, "tc", steps=(3,))
    assert tc and grid < tiles
    assert rel(u_tc, ref) <= 1e-6


def test_tensor_core_form_at_t_final(dg, monkeypatch):
    """The bench workload: 500 steps from the seeded vortex, tensor-core form against the FP64
    path (which equals the oracle to its rounding floor per RHS, test_gpu_full_size.py)."""
    monkeypatch.setenv("DGX_STAGE_KERNEL", "tc")
    mesh = dg.DGMesh.rectangle(512, 512, -5.0, 5.0, -5.0, 5.0, periodic=True)
    space, wf = dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4)
    c64 = dg.DGContext(mesh, space, wf, "fp64")
    ctc = dg.DGContext(mesh, space, wf, "mixed")
    xc, yc = np.random.default_rng(0).uniform(-2.0, 2.0, size=2)
    u0 = c64.project(torch.tensor(isentropic_vortex(c64.quad_points(), beta=5.0, xc=xc, yc=yc), device="cuda"))
    dt = 0.05 / c64.max_cfl(u0, 1.0)
    u64, utc = u0.clone(), u0.clone()
    c64.rk3_step(u64, dt, 500)
    ctc.rk3_step(utc, dt, 500)
    torch.cuda.synchronize()
    assert ctc.stage_form() == "tensor cores"
    assert not ctc.step_nonfinite()
    err = float(torch.linalg.vector_norm(utc - u64) / torch.linalg.vector_norm(u64))
    assert err <= 1e-6, err


@pytest.mark.parametrize("what", ["p4", "skip", "navier_stokes"])
def test_no_tensor_core_form_falls_back(dg, monkeypatch, what):
    order = 4 if what == "p4" else 2
    om, pm, u0, dt = case(dg, 5, order, "skip" if what == "skip" else False)
    wf = dg.NavierStokesWeakFormulation(1.4, 0.01, 0.72, 5.0) if what == "navier_stokes" else None
    u, (grid, tiles, tc) = run(dg, monkeypatch, pm, order, u0, dt, "tc", steps=(1,), wf=wf)
    assert not tc and grid > 0
    if wf is None:
        assert rel(u, om.rk3_step(O.euler(1.4), u0, dt, 1)) <= 1e-6


def test_default_choice_is_timed_and_accurate(dg, monkeypatch):
    om, pm, u0, dt = case(dg, 9, 3, False)
    monkeypatch.delenv("DGX_STAGE_KERNEL", raising=False)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), "mixed")
    u = torch.tensor(u0, device="cuda")
    ctx.rk3_step(u, dt, 2)
    grid, tiles, tc = ctx.launch_shape()
    assert grid > 0
    assert rel(u.cpu().numpy(), om.rk3_step(O.euler(1.4), u0, dt, 2)) <= 1e-6


def test_bounded_wait_runs_out_and_reports(dg, monkeypatch):
    """With one poll per wait, the first wait of every CTA gives up (its bulk copy cannot have
    landed yet): the kernels flag a timeout, drain their copies and MMAs, free TMEM and return.
    dgx_step_status reports DGX_ERR_TIMEOUT; a new context then steps correctly."""
    om, pm, u0, dt = case(dg, 8, 3, False)
    monkeypatch.setenv("DGX_TC_WAIT_LIMIT", "1")
    monkeypatch.setenv("DGX_STAGE_KERNEL", "tc")
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), "mixed")
    u = torch.tensor(u0, device="cuda")
    ctx.rk3_step(u, dt, 1)
    torch.cuda.synchronize()
    assert ctx.launch_shape()[2]
    with pytest.raises(dg.DGXError) as ex:
        ctx.step_nonfinite()
    assert ex.value.code == dg._lib.ERR_TIMEOUT
    monkeypatch.delenv("DGX_TC_WAIT_LIMIT")
    ctx2 = dg.DGContext(pm, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), "mixed")
    u2 = torch.tensor(u0, device="cuda")
    ctx2.rk3_step(u2, dt, 2)
    torch.cuda.synchronize()
    assert not ctx2.step_nonfinite()
    assert rel(u2.cpu().numpy(), om.rk3_step(O.euler(1.4), u0, dt, 2)) <= 1e-6
