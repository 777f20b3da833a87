"""The tensor-core (3xTF32 tcgen05) form of the mixed-precision Euler stage, through the
C ABI: DGX_STAGE_KERNEL=tc makes the autotuner take it; unset, the CUDA-core form runs.

* p = 1..4, periodic and with far-field / no-slip / slip faces: 5 RK3 steps within 1e-6
  relative L2 of the FP64 oracle (the mixed-precision bar), and within 1e-6 of the
  CUDA-core form;
* a mesh with more tiles than SMs, so each CTA walks several tiles;
* Navier-Stokes has no tensor-core form: the choice falls back to CUDA cores.
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
    if kernel:
        monkeypatch.setenv("DGX_STAGE_KERNEL", kernel)
    else:
        monkeypatch.delenv("DGX_STAGE_KERNEL", raising=False)
    ctx = dg.DGContext(pm, dg.DGSpace("triangle", order, "dubiner"), wf or dg.EulerWeakFormulation(1.4), "mixed")
    u = torch.tensor(u0, device="cuda")
    for n in steps:
        ctx.rk3_step(u, dt, n)
    torch.cuda.synchronize()
    return u.cpu().numpy(), ctx.launch_shape()


@pytest.mark.parametrize("walls", [False, True])
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_tensor_core_stage_vs_oracle(dg, monkeypatch, order, walls):
    om, pm, u0, dt = case(dg, 7, order, walls)
    ref = om.rk3_step(O.euler(1.4), u0, dt, 5)
    assert np.isfinite(ref).all()
    u_tc, (grid, tiles, tc) = run(dg, monkeypatch, pm, order, u0, dt, "tc")
    assert tc and grid == tiles
    u_cc, (_, _, tc2) = run(dg, monkeypatch, pm, order, u0, dt, "")
    assert not tc2
    assert rel(u_tc, ref) <= 1e-6, rel(u_tc, ref)
    assert rel(u_tc - u0, ref - u0) <= 1e-4
    assert rel(u_tc, u_cc) <= 1e-6


def test_tensor_core_stage_walks_several_tiles(dg, monkeypatch):
    om, pm, u0, dt = case(dg, 111, 2, False)  # 24,642 elements: 193 tiles, more than SMs
    ref = om.rk3_step(O.euler(1.4), u0, dt, 3)
    u_tc, (grid, tiles, tc) = run(dg, monkeypatch, pm, 2, u0, dt, "tc", steps=(3,))
    assert tc and grid < tiles
    assert rel(u_tc, ref) <= 1e-6


def test_navier_stokes_keeps_cuda_cores(dg, monkeypatch):
    om, pm, u0, dt = case(dg, 5, 2, False)
    _, (grid, tiles, tc) = run(dg, monkeypatch, pm, 2, u0, dt, "tc", steps=(1,),
                               wf=dg.NavierStokesWeakFormulation(1.4, 0.01, 0.72, 5.0))
    assert not tc and grid > 0


def test_auto_mode_times_both_forms(dg, monkeypatch):
    om, pm, u0, dt = case(dg, 9, 3, False)
    u, (grid, tiles, tc) = run(dg, monkeypatch, pm, 3, u0, dt, "auto", steps=(2,))
    ref = om.rk3_step(O.euler(1.4), u0, dt, 2)
    assert grid > 0 and rel(u, ref) <= 1e-6
