// dgx_rk3_step_static: SSP-RK3 steps whose stage buffers live in a fixed, file-scope
// device array instead of memory the library allocates.
//
// Who needs it: code that drives the solver from a place where it may not call
// cudaMalloc -- a host framework that owns all device memory through its own pool and
// forbids the libraries it loads from allocating, or a real-time loop that must never
// enter the CUDA allocator.  Such a caller creates the context once during set-up and
// then advances the state with this entry point, which allocates nothing.
//
// Limits and behaviour:
//  * the scratch is one static __device__ array of 2 * DGX_STATIC_MAX_STATE doubles
//    (16 MiB).  Under lazy module loading (CUDA's default) the array is placed on a device
//    when its module is loaded there; dgx_create does that for its device (with the device
//    current), together with the kernels this entry point launches, so the steps themselves
//    allocate nothing.  A device keeps the array until the process exits;
//  * states larger than DGX_STATIC_MAX_STATE values are rejected with DGX_ERR_INVALID;
//  * all calls share the array.  Stage buffers are written in full before they are read,
//    so nothing has to start at zero, but two calls whose work overlaps on the GPU (other
//    streams, other host threads) race on it;
//  * the array's device address is looked up once per device, at dgx_create; creating the
//    context before any stream capture keeps that lookup out of a capture.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "dgx_context.h"
#include "dgx_internal.h"

using namespace dgx;

// FP64 / double-float contexts: two FP64 stage states; mixed: five FP32 arrays (the two FP32
// copies of u^n, the two increments and the low parts of the double-float state)
static __device__ __align__(256) double g_rk3_scratch[(5 * (size_t)DGX_STATIC_MAX_STATE + 1) / 2];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_rk3_scratch on the current device `dev` (host code may not use the
// symbol itself as an address).  The first lookup on a device loads the array's module
// there; later calls return the cached address.
int scratch_for_device(int dev, double** out) {
    if (dev < 0 || dev >= kMaxDevices) return dgx::set_error(DGX_ERR_CUDA, "device index out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_rk3_scratch);
        if (e != cudaSuccess)
            return dgx::set_error(DGX_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        g_scratch_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_ptr[dev];
    return DGX_OK;
}
}  // namespace

int dgx::static_scratch_setup(int dev) {
    double* p = nullptr;
    if (int rc = scratch_for_device(dev, &p)) return rc;
    if (prepare_f64_to_f32())
        return dgx::set_error(DGX_ERR_CUDA, std::string("loading the FP64->FP32 conversion kernel: ") +
                                                cudaGetErrorString(cudaGetLastError()));
    return DGX_OK;
}

extern "C" int dgx_rk3_step_static(dgx_ctx* c, double* u, double dt, int n_steps, void* stream) {
    if (c && c->nvpe == 4) return dgx::set_error(DGX_ERR_INVALID, "dgx_rk3_step_static: triangle meshes only");
    if (!c || (c->ne && !u) || n_steps < 0) return dgx::set_error(DGX_ERR_INVALID, "dgx_rk3_step_static: bad argument");
    if (c->nstate > (size_t)DGX_STATIC_MAX_STATE)
        return dgx::set_error(DGX_ERR_INVALID,
                              "dgx_rk3_step_static: the state has " + std::to_string(c->nstate) +
                                  " values, above the static scratch limit DGX_STATIC_MAX_STATE = " +
                                  std::to_string((long long)DGX_STATIC_MAX_STATE));
    if (c->ne == 0 || n_steps == 0) return DGX_OK;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev != c->device)
        return dgx::set_error(DGX_ERR_CUDA, "dgx_rk3_step_static: the context's device must be current");
    double* scratch = nullptr;
    int rc = scratch_for_device(dev, &scratch);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const bool visc = c->prm.physics == DGX_NAVIER_STOKES;

    if (c->prm.precision != DGX_MIXED) {
        // u1 = u + dt L(u); u2 = 3/4 u + 1/4 (u1 + dt L(u1)); u <- 1/3 u + 2/3 (u2 + dt L(u2))
        double* u1 = scratch;
        double* u2 = scratch + c->nstate;
        StepArgs a{};
        a.ne = c->ne;
        a.geom = c->d_geom;
        a.conn = c->d_conn;
        a.bc = c->d_bc;
        a.gamma = c->prm.gamma;
        a.mu = c->prm.mu;
        a.prandtl = c->prm.prandtl;
        a.sigma0 = c->prm.sigma0;
        a.order = c->prm.order;
        a.minv_diag = c->minv_diag;
        a.mode = MODE_STAGE;
        a.dt = dt;
        a.status = c->d_status;
        auto launch = [&](const StepArgs& x) {
            return c->prm.precision == DGX_DF64 ? launch_element_df64(c->prm.order, visc, x, c->ops, s)
                                                : launch_element_fp64(c->prm.order, visc, x, c->ops, s);
        };
        for (int n = 0; n < n_steps && !rc; ++n) {
            a.u = u; a.un = nullptr; a.out = u1; a.a = 0.0; a.b = 1.0;
            rc = launch(a);
            a.u = u1; a.un = u; a.out = u2; a.a = 0.75; a.b = 0.25;
            if (!rc) rc = launch(a);
            a.u = u2; a.un = u; a.out = u; a.a = 1.0 / 3.0; a.b = 2.0 / 3.0;
            if (!rc) rc = launch(a);
        }
    } else {
        // FP32 copies of u^n (ping-ponged) and the two FP32 stage increments: 4 * nstate
        // floats, the same bytes as two FP64 states.
        float* f = reinterpret_cast<float*>(scratch);
        float* uhi[2] = {f, f + c->nstate};
        float* d1 = f + 2 * c->nstate;
        float* d2 = f + 3 * c->nstate;
        float* ulo = f + 4 * c->nstate;
        if (launch_f64_to_f32(c->nstate, u, uhi[0], s))
            return dgx::set_error(DGX_ERR_CUDA, std::string("dgx_rk3_step_static: conversion launch failed: ") +
                                                    launch_error_text());
        StageArgs a{};
        a.status = c->d_status;
        a.ne = c->ne;
        a.geom = c->d_geomf;
        a.conn = c->d_conn;
        a.bc = c->d_bc;
        a.dt = (float)dt;
        a.gamma = (float)c->prm.gamma;
        a.mu = (float)c->prm.mu;
        a.kappa = visc ? (float)(c->prm.mu * c->prm.gamma / (c->prm.prandtl * (c->prm.gamma - 1.0))) : 0.0f;
        a.sigma0 = (float)c->prm.sigma0;
        a.boundary = c->boundary;
        a.u64 = u;
        a.ulo = ulo;
        for (int n = 0; n < n_steps && !rc; ++n) {
            const int src = n & 1;
            a.uhi = uhi[src];
            a.uhi_out = uhi[1 - src];
            set_step_kind(a, step_kind(n, n_steps));
            a.stage = 1; a.din = nullptr; a.dout = d1;
            rc = launch_stage_mixed(c->prm.order, visc, a, c->ops, s);
            a.stage = 2; a.din = d1; a.dout = d2;
            if (!rc) rc = launch_stage_mixed(c->prm.order, visc, a, c->ops, s);
            a.stage = 3; a.din = d2; a.dout = nullptr;
            if (!rc) rc = launch_stage_mixed(c->prm.order, visc, a, c->ops, s);
        }
    }
    if (rc)
        return dgx::set_error(DGX_ERR_CUDA, std::string("dgx_rk3_step_static: kernel launch failed: ") +
                                                launch_error_text());
    return DGX_OK;
}
