// The device-resident solver context behind include/dgx.h's dgx_ctx (internal).
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/dgx.h"
#include "dgx_internal.h"

struct dgx_ctx {
    int device = 0;
    dgx_params prm{};
    int ne = 0, np = 0, nq = 0, nfq = 0;
    size_t nstate = 0;  // ne*np*4
    dgx::OpsHost ops{};
    std::vector<double> xq;  // physical volume points
    dgx::ElemGeom* d_geom = nullptr;
    dgx::ElemGeomF* d_geomf = nullptr;  // FP32 rounding of d_geom (mixed precision)
    dgx::ElemConn* d_conn = nullptr;
    dgx::BCSlot* d_bc = nullptr;
    double* d_u1 = nullptr;
    double* d_u2 = nullptr;
    double* d_hu = nullptr;   // host-variant staging
    double* d_hr = nullptr;
    double* d_mon = nullptr;  // [4]
    int* d_flag = nullptr;
    float* d_uhi[2] = {nullptr, nullptr};  // FP32 copies of u^n (mixed RK3), ping-ponged
    float* d_d1 = nullptr;                  // FP32 stage increments (mixed RK3)
    float* d_d2 = nullptr;
    int minv_diag = 0;
    int boundary = 0;  // some face is a boundary face or takes no part
    int has_slip_wall = 0;
    double* d_adj[3] = {nullptr, nullptr, nullptr};  // adjoint scratch (allocated on first use)
    cudaStream_t cap = nullptr;  // capture stream
    cudaGraphExec_t graph = nullptr;   // one step (FP64) or two steps (mixed)
    cudaGraphExec_t graph1 = nullptr;  // mixed: one step
    const double* graph_u = nullptr;
    double graph_dt = 0.0;
};

namespace dgx {
// Records the message returned by dgx_last_error() on this thread and returns `code`.
int set_error(int code, const std::string& msg);
}  // namespace dgx
