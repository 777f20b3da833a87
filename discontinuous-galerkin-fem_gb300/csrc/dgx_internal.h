// Internal layouts shared by the host side (dgx_host.cpp) and the kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>

namespace dgx {

// Status of the kernel launch just made: 0, or -1 with the CUDA error kept in a thread-local
// slot, because reading it with cudaGetLastError() also clears it and the caller reports it
// later (launch_error_text()).
inline cudaError_t& last_launch_error() {
    static thread_local cudaError_t e = cudaSuccess;
    return e;
}
inline int launch_status() {
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return 0;
    last_launch_error() = e;
    return -1;
}
// Text of the error behind the last failed launch on this thread (then cleared), or of the
// pending CUDA error when no launch failed.
inline const char* launch_error_text() {
    cudaError_t e = last_launch_error();
    last_launch_error() = cudaSuccess;
    if (e == cudaSuccess) e = cudaGetLastError();
    return cudaGetErrorString(e);
}

// Bounded waits inside the kernels that wait on bulk copies or tensor-core work: by default up
// to 2^16 polls that may each sleep up to 20 us (about 1.3 s in all, far beyond any wait in a
// healthy launch).  The environment variable `env` = n makes it n plain polls (a test makes the
// waits run out on purpose and checks the status the kernels report).
inline void kernel_wait_bounds(const char* env, long long* limit, unsigned* hint_ns) {
    *limit = 1LL << 16;
    *hint_ns = 20000;
    const char* v = std::getenv(env);
    if (v && *v) {
        const long long x = std::atoll(v);
        if (x > 0) {
            *limit = x;
            *hint_ns = 0;
        }
    }
}

constexpr int NV = 4;      // conserved variables (rho, rho u, rho v, E), assembler.cpp:154
constexpr int MAX_P = 4;   // orders with compiled kernels
constexpr int TILE = 128;  // elements per CTA in the element kernels (one per thread)

__host__ __device__ constexpr int n_basis(int p) { return (p + 1) * (p + 2) / 2; }
// volume points of the degree-2p triangle rule DGSpace uses (space.cpp:40-41)
__host__ __device__ constexpr int n_quad(int p) {
    return p == 1 ? 3 : p == 2 ? 6 : p == 3 ? 12 : p == 4 ? 16 : 0;
}

// Per-element geometry, 128 B, one record per element in element order.
struct alignas(128) ElemGeom {
    double A[4];      // dxi/dx = inverse(J_T), row-major (mapping.cpp:33-47)
    double detJ;      // |det J_T|
    double h[3];      // face length; the L side's length for interior faces
    double n[3][2];   // face normal as seen from this element (= +/- the L side's normal)
    double pad[2];    // pad[0]: shortest vertex distance (compute_max_cfl's h_elem)
};
static_assert(sizeof(ElemGeom) == 128, "ElemGeom must stay 128 B");

// Quadrilaterals (DGSpace("quad", p), LegendreBasis): orders with compiled kernels,
// (p+1)^2 modes and (p+1)^2 tensor Gauss-Legendre volume points.
constexpr int MAX_P_QUAD = 4;
__host__ __device__ constexpr int n_basis_quad(int p) { return (p + 1) * (p + 1); }

// Per-element geometry of a bilinear quadrilateral, 192 B.  The map is not affine, so
// the metric terms are evaluated at each point from the shape-function derivatives of
// ReferenceQuad (src/reference/elements.cpp:92-111):
//   dx/dxi = jx[0] + jx[2] eta,  dx/deta = jx[1] + jx[2] xi,  and y likewise with jy.
struct alignas(64) QuadGeom {
    double jx[3];
    double jy[3];
    double h[4];     // face length; the L side's length for interior faces
    double n[4][2];  // face normal as seen from this element (= +/- the L side's normal)
    double hmin;     // shortest distance between two vertices (compute_max_cfl's h_elem)
    double pad[5];
};
static_assert(sizeof(QuadGeom) == 192, "QuadGeom must stay 192 B");

// The same record rounded once to FP32 (96 B) for the mixed-precision stage on
// quadrilaterals, whose arithmetic is FP32 (conversions from FP64 would use the FP64 pipe).
struct alignas(32) QuadGeomF {
    float jx[3];
    float jy[3];
    float h[4];
    float n[4][2];
    float hmin;
    float pad[5];
};
static_assert(sizeof(QuadGeomF) == 96, "QuadGeomF must stay 96 B");

// Face connectivity of a quadrilateral, ElemConn's encoding over four faces.
struct alignas(32) QuadConn {
    int nbr[4];
    int flags;
    int pad[3];
};

// The same record rounded once to FP32 (64 B) for the mixed-precision stage kernel,
// whose arithmetic is FP32: it holds exactly the values that kernel would obtain by
// converting ElemGeom on load.
struct alignas(64) ElemGeomF {
    float A[4];
    float detJ;
    float h[3];
    float n[3][2];
    float hmin;
    float pad;
};
static_assert(sizeof(ElemGeomF) == 64, "ElemGeomF must stay 64 B");

// Per-element face connectivity, 16 B.
//   nbr[f] >= 0       interior face: neighbour element
//   nbr[f] = -1 - s   boundary face with boundary-condition slot s
//   nbr[f] = SKIP     face that takes no part in the residual (no BC set)
// flags, 4 bits per face f at bit 4f: [1:0] neighbour's face, [2] reversed point order,
// [3] this element is the L side of the face in dgfem's face list.
struct alignas(16) ElemConn {
    int nbr[3];
    int flags;
};
constexpr int NBR_SKIP = -0x40000000;

struct BCSlot {
    int type;  // DGX_BC_*
    int pad;
    double value[4];
};
constexpr int MAX_BC = 64;

// Reference-element operators for order P, stored in precision T.
template <int P, typename T>
struct Ops {
    static constexpr int NP = n_basis(P), NQ = n_quad(P), NFQ = P + 1;
    T phi[NQ][NP];        // basis at volume points
    T dr[NQ][NP];         // d/dxi at volume points
    T ds[NQ][NP];         // d/deta at volume points
    T phif[3][NFQ][NP];   // basis at face points (face f, point q)
    T drf[3][NFQ][NP];    // d/dxi at face points
    T dsf[3][NFQ][NP];    // d/deta at face points
    T wq[NQ];             // volume weights
    T wf[NFQ];            // Gauss-Legendre weights on [-1, 1]
    T minv[NP][NP];       // inverse of the reference mass matrix sum_q w_q phi phi^T
};

// Host copy of all operators in double precision, sized for MAX_P triangles (15 modes, 16
// points) and MAX_P_QUAD quadrilaterals (25 modes, 25 points).
constexpr int OPS_MAX_NP = 25, OPS_MAX_NQ = 25, OPS_MAX_NFQ = 5;
struct OpsHost {
    int p, np, nq, nfq;
    int nf;            // faces per element: 3 (triangles) or 4 (quadrilaterals)
    double phi[OPS_MAX_NQ][OPS_MAX_NP], dr[OPS_MAX_NQ][OPS_MAX_NP], ds[OPS_MAX_NQ][OPS_MAX_NP];
    double phif[4][OPS_MAX_NFQ][OPS_MAX_NP], drf[4][OPS_MAX_NFQ][OPS_MAX_NP], dsf[4][OPS_MAX_NFQ][OPS_MAX_NP];
    double wq[OPS_MAX_NQ], wf[OPS_MAX_NFQ];
    double minv[OPS_MAX_NP][OPS_MAX_NP];
    double qp[OPS_MAX_NQ][2];         // volume points on the reference element
    double fp[OPS_MAX_NFQ];           // face points on [-1, 1]
    double fxi[4][OPS_MAX_NFQ][2];    // face points on the reference element, face f, point q
};

// Reference operators of order p in the given basis (returns nonzero on failure; dgx_host.cpp).
int make_ops(int p, int basis, OpsHost& o);

template <int P, typename T>
inline void fill_ops(const OpsHost& h, Ops<P, T>& o) {
    constexpr int NP = Ops<P, T>::NP, NQ = Ops<P, T>::NQ, NFQ = Ops<P, T>::NFQ;
    for (int q = 0; q < NQ; ++q)
        for (int i = 0; i < NP; ++i) {
            o.phi[q][i] = (T)h.phi[q][i];
            o.dr[q][i] = (T)h.dr[q][i];
            o.ds[q][i] = (T)h.ds[q][i];
        }
    for (int f = 0; f < 3; ++f)
        for (int q = 0; q < NFQ; ++q)
            for (int i = 0; i < NP; ++i) {
                o.phif[f][q][i] = (T)h.phif[f][q][i];
                o.drf[f][q][i] = (T)h.drf[f][q][i];
                o.dsf[f][q][i] = (T)h.dsf[f][q][i];
            }
    for (int q = 0; q < NQ; ++q) o.wq[q] = (T)h.wq[q];
    for (int q = 0; q < NFQ; ++q) o.wf[q] = (T)h.wf[q];
    for (int i = 0; i < NP; ++i)
        for (int j = 0; j < NP; ++j) o.minv[i][j] = (T)h.minv[i][j];
}

enum Mode { MODE_RESIDUAL = 0, MODE_RHS = 1, MODE_STAGE = 2 };

// Arguments of one element-kernel launch.
struct StepArgs {
    int ne;
    int mode;              // Mode
    const double* u;       // stage state (neighbours are read from it)
    const double* un;      // u^n for MODE_STAGE (own element only); may be null when a == 0
    double* out;           // residual, M^-1 R, or the next stage state
    const ElemGeom* geom;
    const ElemConn* conn;
    const BCSlot* bc;
    double dt, a, b;       // MODE_STAGE: out = a*un + b*(u + dt*du); a == 0: out = u + dt*du
    double gamma, mu, prandtl, sigma0;
    int order;
    int minv_diag;         // 1 when M_ref^-1 is diagonal (Dubiner): scale instead of a dense product
    int* status;           // device flag: bit 0 set when a non-finite value was produced
};

// Arguments of the mixed-precision SSP-RK3 stage kernel.  The stage state is uhi + d,
// uhi the FP32 rounding of u^n and d an FP32 increment:
//   stage 1: d1 = dt L(u^n)
//   stage 2: d2 = 1/4 (d1 + dt L(u^n + d1))
//   stage 3: u^{n+1} = u^n + 2/3 (d2 + dt L(u^n + d2))      (this add in FP64)
// which is SSP_RK::step_rk3 (include/dgfem/solver/time_stepping.hpp:39-55) written in
// increments: u1 = u^n + d1, u2 = 3/4 u^n + 1/4 (u1 + dt L(u1)) = u^n + d2, and
// u^{n+1} = 1/3 u^n + 2/3 (u2 + dt L(u2)) = u^n + 2/3 (d2 + dt L(u2)).
struct StageArgs {
    int ne, stage;
    const float* uhi;   // FP32 u^n (neighbours read it)
    const float* din;   // increment of the stage state (null in stage 1)
    float* dout;        // next increment (stages 1, 2)
    // The state between the steps of one call is the double-float pair uhi + ulo (both FP32,
    // |ulo| <= ulp(uhi) / 2: a 48-bit significand); the caller's FP64 state u64 is read by the
    // first step of a call and written by its last (stage 3 only):
    //   u64_in:  u^n = u64 (else uhi + ulo);  u64_out: u^{n+1} -> u64 (else -> uhi_out + ulo)
    double* u64;        // the caller's FP64 state
    float* ulo;         // low part of the double-float state, updated in place in stage 3
    int u64_in, u64_out;
    float* uhi_out;     // FP32 rounding of u^{n+1} (stage 3; not the buffer uhi points to)
    const ElemGeomF* geom;
    const ElemConn* conn;
    const BCSlot* bc;
    float dt, gamma, mu, kappa, sigma0;
    int boundary;       // 1 when some face is a boundary or skipped face
    const float* dt_inst;  // batched solves: dt per instance, instance id in ElemGeomF::pad (else null)
    int grid;           // persistent grid size (0: one CTA per tile)
    int* status;        // device flag: bit 0 set when stage 3 produced a non-finite value
    const QuadGeomF* qgeom;  // quadrilateral meshes: their records (geom and conn are then null)
    const QuadConn* qconn;
    const float* tin;   // face-trace form: traces of this stage's state (dg_stage_trace.cuh)
    float* tout;        // face-trace form: traces of the next stage's state
    int tile0, ntile;   // CUDA-core forms: the tiles [tile0, tile0 + ntile) only (ntile = 0: all)
    // face-trace form on a mesh whose every boundary face has a condition (null otherwise): its
    // connectivity, in which boundary face k points at the ghost block ne + k of the trace
    // buffers, and the condition slot of each ghost block
    const ElemConn* tconn;
    const int* ghost_bc;
    // bounded waits of the pipelined trace kernel: polls, and the sleep hint of each poll (ns)
    long long wait_limit;
    unsigned wait_hint_ns;
};

// The steps of one mixed-precision call: the first reads the caller's FP64 state, the last
// writes it back, the ones between carry the double-float pair (StageArgs::u64_in / u64_out of
// stage 3); a call of one step reads and writes FP64.
enum StepKind { STEP_ONLY = 0, STEP_FIRST = 1, STEP_MID = 2, STEP_LAST = 3 };
inline StepKind step_kind(int k, int n) {
    return n == 1 ? STEP_ONLY : k == 0 ? STEP_FIRST : k == n - 1 ? STEP_LAST : STEP_MID;
}
inline void set_step_kind(StageArgs& a, StepKind kind) {
    a.u64_in = kind == STEP_ONLY || kind == STEP_FIRST;
    a.u64_out = kind == STEP_ONLY || kind == STEP_LAST;
}
// A call of n steps as replays of at most six captured graphs; step k reads the FP32 copy
// uhi[k & 1]:  ONLY (src 0) | FIRST (src 0), MID2 (src 1, 0) ..., MID (src 1)?, LAST0/LAST1.
enum StepGraph { G_ONLY = 0, G_FIRST, G_MID2, G_MID, G_LAST0, G_LAST1, N_STEP_GRAPHS };
struct GraphStep {
    int src;
    StepKind kind;
};
inline int graph_steps(int g, GraphStep out[2]) {
    switch (g) {
    case G_ONLY: out[0] = {0, STEP_ONLY}; return 1;
    case G_FIRST: out[0] = {0, STEP_FIRST}; return 1;
    case G_MID2: out[0] = {1, STEP_MID}; out[1] = {0, STEP_MID}; return 2;
    case G_MID: out[0] = {1, STEP_MID}; return 1;
    case G_LAST0: out[0] = {0, STEP_LAST}; return 1;
    default: out[0] = {1, STEP_LAST}; return 1;
    }
}
template <class F>
inline int for_step_graphs(int n, F&& f) {
    if (n <= 0) return 0;
    if (n == 1) return f(G_ONLY);
    if (int rc = f(G_FIRST)) return rc;
    const int m = n - 2;
    for (int i = 0; i + 1 < m; i += 2)
        if (int rc = f(G_MID2)) return rc;
    if (m & 1)
        if (int rc = f(G_MID)) return rc;
    return f(((n - 1) & 1) ? G_LAST1 : G_LAST0);
}

// Launchers (one translation unit per precision).
int launch_element_fp64(int p, bool viscous, const StepArgs& a, const OpsHost& ops, cudaStream_t s);
int launch_element_mixed(int p, bool viscous, const StepArgs& a, const OpsHost& ops, cudaStream_t s);
int configure_element_fp64(int p, bool viscous);
int configure_element_mixed(int p, bool viscous);
// double-float form of the FP64 element kernel (dgx_kernels_df64.cu)
int launch_element_df64(int p, bool viscous, const StepArgs& a, const OpsHost& ops, cudaStream_t s);
int configure_element_df64(int p, bool viscous);
int launch_stage_mixed(int p, bool viscous, const StageArgs& a, const OpsHost& ops, cudaStream_t s);
// Tensor-core form of the mixed Euler stage (dgx_kernels_tc.cu), orders 1..3, meshes whose
// faces are all interior or ghost faces (StageArgs::tconn).  A StageArgs::grid with STAGE_TC
// set selects it; the low bits are its grid (<= 0: one CTA per tile).  It exchanges face
// traces like the face-trace form (tin / tout), and launch_tc_trace_init writes the traces of
// uhi with its own operations (the CUDA-core trace kernel's would differ in rounding).
constexpr int STAGE_TC = 1 << 30;
int launch_stage_tc(int p, const StageArgs& a, const OpsHost& ops, int grid, cudaStream_t s);
int launch_tc_trace_init(int p, const StageArgs& a, const OpsHost& ops, int grid, cudaStream_t s);
int configure_stage_tc(int p);
bool stage_tc_supported(int p);
// Face-trace form of the mixed Euler stage (dgx_kernels_trace.cu).  A StageArgs::grid with
// STAGE_TRACE set selects it; the low bits are its grid.  launch_trace_init writes the traces
// of uhi to tout (the state a step starts from).
constexpr int STAGE_TRACE = 1 << 28;
// With STAGE_TRACE: the pipelined persistent trace kernel (stage_trace_pipe_kernel), which
// bulk-copies the next tile's inputs while a tile is computed; periodic or ghost-block meshes.
constexpr int STAGE_PIPE = 1 << 27;
// With STAGE_TRACE: the face-trace kernel at 64- or 32-element tiles, one CTA per tile (the
// low bits are then ignored); dgx_kernels_trace_small.cu.
constexpr int STAGE_T64 = 1 << 26;
constexpr int STAGE_T32 = 1 << 25;
// With STAGE_T32: each thread copies its element's neighbour trace blocks into shared memory
// by cp.async during staging (meshes whose faces are all interior or ghost faces).
constexpr int STAGE_NBS = 1 << 24;
constexpr int STAGE_FLAGS = STAGE_TC | STAGE_TRACE | STAGE_PIPE | STAGE_T64 | STAGE_T32 | STAGE_NBS;
int launch_stage_trace_small(int p, int tile, bool nbs, const StageArgs& a, const OpsHost& ops, cudaStream_t s);
int launch_stage_trace_nbs(int p, const StageArgs& a, const OpsHost& ops, cudaStream_t s);
int launch_stage_trace(int p, const StageArgs& a, const OpsHost& ops, int grid, cudaStream_t s);
int launch_trace_init(int p, const StageArgs& a, const OpsHost& ops, cudaStream_t s);
int configure_stage_trace(int p);
size_t trace_floats_per_element(int p);
int stage_tc_ctas_per_sm(int p);
// Batched solves (dgx_batch.cu): one launch of the stage over the element ranges of
// orders 1..MAX_P (per_order[p-1], ne = 0 for an absent order), grid <= 0: one CTA per tile.
int launch_batch_stage(const StageArgs* per_order, const OpsHost* ops, int boundary, bool visc, int grid,
                       cudaStream_t s);
int batch_tiles(const StageArgs* per_order);
int configure_batch_stage(bool visc);

// Device-side set-up (dgx_setup.cu).  device_face_pairs: the face-slot pairing of a mesh's
// connectivity, nbr[2 s], nbr[2 s + 1] = element and face paired with face slot s, -1 when none
// (host arrays; returns nonzero on a CUDA failure).  launch_device_geometry: per-element
// geometry (ElemGeom or QuadGeom, and their FP32 roundings when geomf is non-null) and the
// physical volume points; err bit 0: singular Jacobian, bit 1: degenerate edge.
int device_face_pairs(int ne, int K, const int* elems_host, long long nv, int* nbr_host);
int launch_device_geometry(int ne, int nvpe, const OpsHost& ops, const double* d_verts, const int* d_elems,
                           const void* d_conn, void* d_geom, void* d_geomf, double* d_xq, int* d_err,
                           cudaStream_t s);

// Small FP64 utility kernels (dgx_misc.cu).
int launch_mass_inv(int ne, int p, const OpsHost& ops, const ElemGeom* geom, const double* in,
                    double* out, cudaStream_t s);
int launch_project(int ne, int p, const OpsHost& ops, const ElemGeom* geom, const double* uq,
                   double* u, cudaStream_t s);
int launch_monitor(int ne, int p, const OpsHost& ops, const ElemGeom* geom, const double* u,
                   double dt, double gamma, double* d_out /*[4]*/, cudaStream_t s);
int launch_has_nan(size_t n, const double* u, int* d_flag, cudaStream_t s);
// Basis evaluation at reference points (dgx_misc.cu), at most EVAL_MAX_POINTS points.
constexpr int EVAL_MAX_POINTS = 128;
int launch_eval_points(int ne, int np, int npts, const double* phi, const double* u, double* out, cudaStream_t s);
int launch_f64_to_f32(size_t n, const double* in, float* out, cudaStream_t s);
// Loads the conversion kernel on the current device (lazy module loading otherwise loads
// it, and allocates its code, at its first launch).
int prepare_f64_to_f32();
// Set-up of the allocation-free stepping entry point (dgx_static.cu) for the current
// device: looks up, and so loads, the static scratch array and the kernels that entry point
// launches besides the context's element or stage kernels.  Called by dgx_create.
int static_scratch_setup(int dev);

// Quadrilateral kernels (dgx_quad.cu; the double-float element kernel in
// dgx_kernels_df64.cu), orders 1..MAX_P_QUAD, precision DGX_FP64 / DGX_MIXED / DGX_DF64.
// StepArgs::geom and StepArgs::conn are not used; the quadrilateral records are passed
// beside them.
int launch_quad_element(int p, bool viscous, int precision, const StepArgs& a, const QuadGeom* geom,
                        const QuadConn* conn, const OpsHost& ops, cudaStream_t s);
int configure_quad_element(int p, bool viscous, int precision);
int launch_quad_element_df64(int p, bool viscous, const StepArgs& a, const QuadGeom* geom, const QuadConn* conn,
                             const OpsHost& ops, cudaStream_t s);
int configure_quad_element_df64(int p, bool viscous);
// the mixed-precision increment-form stage on quadrilaterals (StageArgs::qgeom / qconn set)
int launch_quad_stage(int p, bool viscous, const StageArgs& a, const OpsHost& ops, cudaStream_t s);
int configure_quad_stage(int p, bool viscous);
int launch_quad_mass_inv(int ne, int p, const OpsHost& ops, const QuadGeom* geom, const double* in, double* out,
                         cudaStream_t s);
int launch_quad_project(int ne, int p, const OpsHost& ops, const QuadGeom* geom, const double* uq, double* u,
                        cudaStream_t s);
int launch_quad_monitor(int ne, int p, const OpsHost& ops, const QuadGeom* geom, const double* u, double dt,
                        double gamma, double* d_out, cudaStream_t s);

}  // namespace dgx
