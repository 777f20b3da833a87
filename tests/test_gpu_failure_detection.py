"""Failure detection without a GPU fault: the failure is made on the host (a NaN, or a
negative density, written into the input state), and the status the stage kernels raise
is read back through the C ABI (dgx_step_status -> DGX_ERR_NONFINITE), as dgfem's per-step
NaN check would stop the run (compressible_solver_base.cpp:290-301)."""

import ctypes as C

import numpy as np
import pytest

from meshes import isentropic_vortex

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def dg():
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import dgfem_gb300 as d
    return d


def vortex(xy):
    return isentropic_vortex(xy, beta=5.0)


def vortex_ctx(dg, precision):
    m = dg.DGMesh.rectangle(12, 12, -5, 5, -5, 5, periodic=True)
    ctx = dg.DGContext(m, dg.DGSpace("triangle", 2, "dubiner"), dg.EulerWeakFormulation(1.4), precision)
    u = ctx.project(torch.tensor(vortex(ctx.quad_points()), device="cuda"))
    return ctx, u


@pytest.mark.parametrize("precision", ["fp64", "mixed", "df64"])
def test_clean_steps_report_ok(dg, precision):
    ctx, u = vortex_ctx(dg, precision)
    ctx.rk3_step(u, 0.01, 3)
    assert not ctx.step_nonfinite()


@pytest.mark.parametrize("precision", ["fp64", "mixed", "df64"])
def test_injected_nan_is_reported_and_cleared(dg, precision):
    ctx, u = vortex_ctx(dg, precision)
    u[17, 0, 3] = float("nan")  # the failure, made on the host side of the call
    ctx.rk3_step(u, 0.01, 2)
    assert ctx.step_nonfinite()
    assert not ctx.step_nonfinite()  # read clears the flag
    from dgfem_gb300 import _lib as L
    f = C.c_int()
    u2 = torch.nan_to_num(u) * 0
    u2[..., 0, 0] = 1.0
    u2[..., 0, 3] = 2.5
    ctx.rk3_step(u2, 0.01, 1)
    assert L.load().dgx_step_status(ctx._h, C.byref(f), None) == L.OK and f.value == 0


def test_negative_density_blows_up_and_is_reported(dg):
    ctx, u = vortex_ctx(dg, "fp64")
    u[5, 0, 0] = -abs(float(u[5, 0, 0]))  # negative mean density: pressure and sound speed go non-real
    assert ctx.max_cfl(u, 0.01) == float("inf")  # dgfem's compute_max_cfl guard
    ctx.rk3_step(u, 0.01, 1)
    assert ctx.step_nonfinite()


def test_solver_loop_stops_on_nonfinite(dg):
    m = dg.DGMesh.rectangle(8, 8, -5, 5, -5, 5, periodic=True)
    solver = dg.EulerDGSolver(m, dg.DGSpace("triangle", 2, "dubiner"))

    def ic(xy):
        U = vortex(xy)
        U[3, 2, 1] = np.nan
        return U
    frames = solver.solve(ic, T_final=1.0, dt=0.01, save_every=10)
    assert solver.telemetry["steps_completed"] == 1  # stopped after the first step
    assert len(frames) == 2
