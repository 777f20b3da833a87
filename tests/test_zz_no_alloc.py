"""The allocation-free SSP-RK3 entry point (dgx_rk3_step_static) against dgx_rk3_step.

dgx_rk3_step_static serves callers that may not allocate device memory while they run (a
host framework whose own pool owns all device memory, a loop that must never enter the
CUDA allocator): it takes its stage buffers from a static device array of the library
instead of the context's allocations.  These tests call both entry points through the C
ABI on the same state and compare the results after each of two calls in a row, for the
FP64 and the mixed-precision paths; check that the device's free memory does not change
across the first calls on a fresh context (lazy module loading left at CUDA's default);
and check that a state above the array's limit is refused.  This file is collected last so
a failure here does not hide the other tests.
"""

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


def rel(a, b):
    a = a.double().cpu().numpy()
    b = b.double().cpu().numpy()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_static_step_matches_context_step(dg, monkeypatch, precision):
    # the context's mixed step is pinned to a CUDA-core form: the allocation-free entry point
    # runs the neighbour-row form, which that form equals bit for bit
    monkeypatch.setenv("DGX_STAGE_KERNEL", "trace")
    lib = dg.load()
    mesh = dg.DGMesh.rectangle(16, 16, -5.0, 5.0, -5.0, 5.0, periodic=True)
    ctx = dg.DGContext(mesh, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), precision)
    u0 = ctx.project(torch.tensor(isentropic_vortex(ctx.quad_points(), beta=5.0), device="cuda"))
    dt = 0.05 / ctx.max_cfl(u0, 1.0)
    a = u0.clone()
    b = u0.clone()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for n_steps in (3, 2):  # two calls in a row, odd and even step counts
        dg._lib.check(lib.dgx_rk3_step(ctx._h, C.c_void_p(a.data_ptr()), dt, n_steps, stream))
        dg._lib.check(lib.dgx_rk3_step_static(ctx._h, C.c_void_p(b.data_ptr()), dt, n_steps, stream))
        torch.cuda.synchronize()
        assert torch.isfinite(b).all()
        # the same kernels on the same inputs (mixed: the neighbour-row and face-trace forms
        # of the stage give the same numbers bit for bit), so the states are equal
        assert torch.equal(b, a), rel(b, a)
    assert rel(b, u0) > 1e-6  # the state did move


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_static_step_allocates_no_device_memory(dg, precision):
    """Free device memory is the same before the first two calls on a new context and after
    them.  The scratch array and the kernels are loaded when the context is created."""
    import os
    assert os.environ.get("CUDA_MODULE_LOADING", "LAZY") == "LAZY"
    lib = dg.load()
    mesh = dg.DGMesh.rectangle(12, 12, -5.0, 5.0, -5.0, 5.0, periodic=True)
    ctx = dg.DGContext(mesh, dg.DGSpace("triangle", 2, "dubiner"), dg.EulerWeakFormulation(1.4), precision)
    u = ctx.project(torch.tensor(isentropic_vortex(ctx.quad_points(), beta=5.0), device="cuda"))
    dt = 0.05 / ctx.max_cfl(u, 1.0)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for n_steps in (1, 2):
        dg._lib.check(lib.dgx_rk3_step_static(ctx._h, C.c_void_p(u.data_ptr()), dt, n_steps, stream))
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert torch.isfinite(u).all()


def test_static_step_rejects_states_above_the_limit(dg):
    lib = dg.load()
    # 128 x 128 x 2 elements, p=3: 1,310,720 values > DGX_STATIC_MAX_STATE = 1,048,576
    mesh = dg.DGMesh.rectangle(128, 128, 0.0, 1.0, 0.0, 1.0, periodic=True)
    ctx = dg.DGContext(mesh, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(1.4), "fp64")
    assert ctx.n_elements * ctx.n_basis * 4 > dg._lib.STATIC_MAX_STATE
    u = torch.ones(ctx.shape, dtype=torch.float64, device="cuda")
    rc = lib.dgx_rk3_step_static(ctx._h, C.c_void_p(u.data_ptr()), 1e-3, 1,
                                 C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == dg._lib.ERR_INVALID
    assert b"DGX_STATIC_MAX_STATE" in lib.dgx_last_error()
    assert torch.equal(u, torch.ones_like(u))  # nothing ran
