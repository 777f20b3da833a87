// The device-resident solver context behind include/dgx.h's dgx_ctx (internal).
#pragma once

#include <cuda_runtime.h>

#include <functional>
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
    mutable std::vector<double> xq;  // physical volume points (host copy, filled on first use)
    double* d_xq = nullptr;          // physical volume points on the device [ne][nq][2]
    dgx::ElemGeom* d_geom = nullptr;
    dgx::ElemGeomF* d_geomf = nullptr;  // FP32 rounding of d_geom (mixed precision)
    dgx::ElemConn* d_conn = nullptr;
    int nvpe = 3;                        // 4: quadrilateral mesh (d_qgeom/d_qconn replace d_geom/d_conn)
    dgx::QuadGeom* d_qgeom = nullptr;
    dgx::QuadConn* d_qconn = nullptr;
    dgx::QuadGeomF* d_qgeomf = nullptr;  // FP32 rounding of d_qgeom (mixed precision)
    dgx::BCSlot* d_bc = nullptr;
    double* d_u1 = nullptr;
    double* d_u2 = nullptr;
    double* d_hu = nullptr;   // host-variant staging
    double* d_hr = nullptr;
    double* d_mon = nullptr;  // [4]
    int* d_flag = nullptr;
    int* d_status = nullptr;  // bit 0: an RK3 step produced a non-finite value (dgx_step_status)
    float* d_uhi[2] = {nullptr, nullptr};  // FP32 copies of u^n (mixed RK3), ping-ponged
    float* d_ulo = nullptr;                 // low parts of the double-float state (mixed RK3)
    float* d_tr[2] = {nullptr, nullptr};    // face traces of the stage states (mixed Euler, trace form)
    // trace form with ghost blocks (every boundary face has a condition): the connectivity with
    // boundary face k pointing at block ne + k of d_tr, and each ghost block's condition slot
    dgx::ElemConn* d_tconn = nullptr;
    int* d_ghost_bc = nullptr;
    float* d_d1 = nullptr;                  // FP32 stage increments (mixed RK3)
    float* d_d2 = nullptr;
    int minv_diag = 0;
    int boundary = 0;  // some face is a boundary face or takes no part
    int has_slip_wall = 0;
    double* d_adj[3] = {nullptr, nullptr, nullptr};  // adjoint scratch (allocated on first use)
    double* d_kin = nullptr;  // objective partial sums (allocated on first use)
    cudaStream_t cap = nullptr;  // capture stream
    cudaStream_t host_out = nullptr;          // host-pointer step: copies back (dgx_rk3_step_host)
    cudaEvent_t host_ev[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaGraphExec_t graph = nullptr;                         // FP64 / double-float: one step
    cudaGraphExec_t mgraph[dgx::N_STEP_GRAPHS] = {};         // mixed: the StepGraph replays
    int stage_grid = 0;  // mixed: stage-kernel grid picked by the autotuner (0: not yet)
    const double* graph_u = nullptr;
    double graph_dt = 0.0;
};

namespace dgx {
// Records the message returned by dgx_last_error() on this thread and returns `code`.
int set_error(int code, const std::string& msg);

// Host copy of a mesh's device geometry: per-element affine map, face normals and lengths,
// face connectivity, boundary-condition slots and the physical volume quadrature points.
struct HostGeometry {
    std::vector<ElemGeom> geom;   // triangles
    std::vector<ElemConn> conn;
    std::vector<QuadGeom> qgeom;  // quadrilaterals
    std::vector<QuadConn> qconn;
    std::vector<BCSlot> slots;
    std::vector<double> xq;
    int boundary = 0;       // some face is a boundary face or takes no part
    int has_slip_wall = 0;
};
// Returns a DGX status code; on failure the message is set for dgx_last_error().
int build_geometry(const dgx_mesh* m, const OpsHost& ops, HostGeometry& g);
// build_geometry's connectivity and boundary slots only (nf: faces per element of the space)
int build_topology(const dgx_mesh* m, int nf, HostGeometry& g);
// FP32 rounding of an element's geometry; `instance` is stored in the spare slot.
ElemGeomF geom_to_f32(const ElemGeom& g, int instance);
// Checks that a CUDA device of compute capability 10.3 is current; returns its ordinal.
int check_device(int* dev);

// Autotuner (dgx_tune.cpp): launch(grid, stream) enqueues one kernel launch with that grid.
using GridLaunch = std::function<int(int grid, cudaStream_t s)>;
// Candidate persistent grid sizes for a kernel over `ntiles` tiles: ntiles first (one CTA
// per tile), then the multiples of the SM count below it.
std::vector<int> grid_candidates(int ntiles);
// Picks the fastest candidate grid by timing on stream s (cached per key).
int tune_grid(const std::string& key, const std::vector<int>& candidates, const GridLaunch& launch, cudaStream_t s,
              int* best);
}  // namespace dgx
