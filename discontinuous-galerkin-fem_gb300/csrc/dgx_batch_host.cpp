// Batched independent solves behind include/dgx.h's dgx_batch_* entry points.
//
// dgfem advances one mesh per solver object (CompressibleDGSolverBase::solve,
// src/solver/compressible_solver_base.cpp:236-312); an ensemble is a loop over solver
// objects.  Here an ensemble of mixed-precision Euler (or Navier-Stokes) solves shares one
// device layout:
// the instances of each order are concatenated into one element range (geometry in FP32
// with the instance number in the spare slot, connectivity and boundary slots offset into
// the range), every RK3 stage of every instance is one launch of the batched stage kernel
// (dgx_batch.cu), and a step is a CUDA graph of three such launches.  Periodic Euler batches
// may instead run each stage as one launch per order of the single context's face-trace kernel
// (32-element tiles, neighbour blocks in shared memory, dg_stage_trace.cuh), on each order's
// concatenated range with its own trace buffers; the autotuner keeps whichever is faster.  Euler
// batches with boundary faces take that form too when every boundary face has a condition: each
// order's trace buffers then end in one ghost block per boundary face, as a single context's do.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "dgx_context.h"

using namespace dgx;

namespace {
struct Group {  // the instances of one order, concatenated
    int ne = 0;
    size_t nstate = 0;  // ne * np * 4
    ElemGeomF* geomf = nullptr;
    ElemConn* conn = nullptr;
    BCSlot* bc = nullptr;
    double* u = nullptr;                  // FP64 state of every instance of this order
    float* uhi[2] = {nullptr, nullptr};   // FP32 copies of u^n, ping-ponged
    float* ulo = nullptr;                 // low parts of the double-float state
    float* d1 = nullptr;                  // FP32 stage increments
    float* d2 = nullptr;
    float* tr[2] = {nullptr, nullptr};    // face traces (face-trace form), ping-ponged
    ElemConn* tconn = nullptr;            // face-trace form with ghost blocks: boundary faces as interior
    int* ghost_bc = nullptr;              //   faces to ghost blocks ne + k, and block k's condition slot
    int nghost = 0;
};
}  // namespace

struct dgx_batch {
    int device = 0;
    int n_inst = 0;
    dgx_params prm{};
    Group grp[MAX_P];
    OpsHost ops[MAX_P] = {};                         // reference operators of each order present
    std::vector<int> inst_order, inst_e0, inst_ne;  // per instance: order, first element in its group, elements
    float* d_dt = nullptr;                           // per-instance time step (FP32, as the stage arithmetic)
    std::vector<float> dt_uploaded;
    int boundary = 0;
    int grid = 0;  // stage-kernel grid picked by the autotuner (0: not yet); with STAGE_TRACE the face-trace form
    bool trace_ok = false;  // Euler without skipped faces: every group has trace buffers (and ghost blocks)
    cudaStream_t cap = nullptr;
    cudaGraphExec_t graph[N_STEP_GRAPHS] = {};  // the StepGraph replays (dgx_internal.h)
};

static void free_batch(dgx_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    for (cudaGraphExec_t g : b->graph)
        if (g) cudaGraphExecDestroy(g);
    for (Group& g : b->grp) {
        cudaFree(g.geomf);
        cudaFree(g.conn);
        cudaFree(g.bc);
        cudaFree(g.u);
        cudaFree(g.uhi[0]);
        cudaFree(g.uhi[1]);
        cudaFree(g.ulo);
        cudaFree(g.d1);
        cudaFree(g.d2);
        cudaFree(g.tr[0]);
        cudaFree(g.tr[1]);
        cudaFree(g.tconn);
        cudaFree(g.ghost_bc);
    }
    cudaFree(b->d_dt);
    if (b->cap) cudaStreamDestroy(b->cap);
    delete b;
}

extern "C" void dgx_batch_destroy(dgx_batch* b) { free_batch(b); }

extern "C" int dgx_batch_create(int n_inst, const dgx_mesh* const* meshes, const dgx_params* params, dgx_batch** out) {
    if (!out) return set_error(DGX_ERR_INVALID, "dgx_batch_create: null argument");
    *out = nullptr;
    if (n_inst < 1 || !meshes || !params) return set_error(DGX_ERR_INVALID, "dgx_batch_create: no instances");
    const dgx_params& p0 = params[0];
    for (int i = 0; i < n_inst; ++i) {
        const dgx_params& p = params[i];
        const std::string at = " (instance " + std::to_string(i) + ")";
        if (!meshes[i]) return set_error(DGX_ERR_INVALID, "dgx_batch_create: null mesh" + at);
        int nvpe = 0;
        if (dgx_mesh_vertices_per_element(meshes[i], &nvpe) != DGX_OK || nvpe != 3)
            return set_error(DGX_ERR_INVALID, "batched solves run on triangle meshes" + at);
        if (p.order < 1 || p.order > MAX_P)
            return set_error(DGX_ERR_INVALID, "Element order must be between 1 and 4 for the GPU kernels" + at);
        if (p.physics != DGX_EULER && p.physics != DGX_NAVIER_STOKES)
            return set_error(DGX_ERR_INVALID, "unknown physics" + at);
        if (p.precision != DGX_MIXED)
            return set_error(DGX_ERR_INVALID, "batched solves run in mixed precision" + at);
        if (p.basis != p0.basis || p.gamma != p0.gamma || p.physics != p0.physics)
            return set_error(DGX_ERR_INVALID, "batched instances must share the basis, gamma and physics" + at);
        if (p.physics == DGX_NAVIER_STOKES) {  // NavierStokesWeakFormulation ctor checks (:22-33)
            if (p.mu != p0.mu || p.prandtl != p0.prandtl || p.sigma0 != p0.sigma0)
                return set_error(DGX_ERR_INVALID, "batched Navier-Stokes instances must share mu, Prandtl and sigma0" + at);
            if (!(p.mu > 0.0))
                return set_error(DGX_ERR_INVALID, "Dynamic viscosity must be positive for Navier-Stokes weak formulation" + at);
            if (!(p.prandtl > 0.0))
                return set_error(DGX_ERR_INVALID, "Prandtl number must be positive for Navier-Stokes weak formulation" + at);
            if (!(p.sigma0 > 0.0))
                return set_error(DGX_ERR_INVALID, "Penalty prefactor must be positive for Navier-Stokes weak formulation" + at);
        }
        if (p.basis != DGX_BASIS_MONOMIAL && p.basis != DGX_BASIS_DUBINER)
            return set_error(DGX_ERR_INVALID, "unknown basis" + at);
    }
    int dev = 0;
    if (int rc = check_device(&dev)) return rc;
    const bool visc = p0.physics == DGX_NAVIER_STOKES;
    if (configure_batch_stage(visc)) return set_error(DGX_ERR_CUDA, "could not configure the batched stage kernel");

    auto* b = new dgx_batch;
    b->device = dev;
    b->n_inst = n_inst;
    b->prm = p0;
    b->inst_order.resize(n_inst);
    b->inst_e0.resize(n_inst);
    b->inst_ne.resize(n_inst);
    bool have[MAX_P] = {};
    for (int i = 0; i < n_inst; ++i) have[params[i].order - 1] = true;
    for (int p = 1; p <= MAX_P; ++p)
        if (have[p - 1] && make_ops(p, p0.basis, b->ops[p - 1])) {
            free_batch(b);
            return set_error(DGX_ERR_RUNTIME, "could not build reference operators");
        }

    // per order: concatenated FP32 geometry, connectivity and boundary slots
    std::vector<ElemGeomF> gf[MAX_P];
    std::vector<ElemConn> cn[MAX_P];
    std::vector<BCSlot> bs[MAX_P];
    for (int i = 0; i < n_inst; ++i) {
        const int pi = params[i].order - 1;
        HostGeometry hg;
        if (int rc = build_geometry(meshes[i], b->ops[pi], hg)) {
            free_batch(b);
            return set_error(rc, std::string(dgx_last_error()) + " (instance " + std::to_string(i) + ")");
        }
        const int e0 = (int)gf[pi].size(), s0 = (int)bs[pi].size();
        const int ne = (int)hg.geom.size();
        b->inst_order[i] = pi + 1;
        b->inst_e0[i] = e0;
        b->inst_ne[i] = ne;
        if (hg.boundary) b->boundary = 1;
        for (int e = 0; e < ne; ++e) {
            gf[pi].push_back(geom_to_f32(hg.geom[e], i));
            ElemConn c = hg.conn[e];
            for (int f = 0; f < 3; ++f) {
                if (c.nbr[f] == NBR_SKIP) continue;
                c.nbr[f] = c.nbr[f] >= 0 ? c.nbr[f] + e0 : c.nbr[f] - s0;  // -1 - slot -> -1 - (slot + s0)
            }
            cn[pi].push_back(c);
        }
        if (!hg.boundary) continue;
        bs[pi].insert(bs[pi].end(), hg.slots.begin(), hg.slots.end());
    }
    auto up = [](void** dst, const void* src, size_t bytes) {
        if (cudaMalloc(dst, bytes ? bytes : 16) != cudaSuccess) return false;
        return !bytes || cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    for (int p = 0; p < MAX_P; ++p) {
        Group& g = b->grp[p];
        g.ne = (int)gf[p].size();
        if (g.ne == 0) continue;
        if (bs[p].empty()) bs[p].push_back(BCSlot{});
        g.nstate = (size_t)g.ne * n_basis(p + 1) * NV;
        if (!up((void**)&g.geomf, gf[p].data(), gf[p].size() * sizeof(ElemGeomF)) ||
            !up((void**)&g.conn, cn[p].data(), cn[p].size() * sizeof(ElemConn)) ||
            !up((void**)&g.bc, bs[p].data(), bs[p].size() * sizeof(BCSlot)) ||
            cudaMalloc((void**)&g.u, g.nstate * sizeof(double)) != cudaSuccess ||
            cudaMemset(g.u, 0, g.nstate * sizeof(double)) != cudaSuccess ||
            cudaMalloc((void**)&g.uhi[0], g.nstate * sizeof(float)) != cudaSuccess ||
            cudaMalloc((void**)&g.uhi[1], g.nstate * sizeof(float)) != cudaSuccess ||
            cudaMalloc((void**)&g.ulo, g.nstate * sizeof(float)) != cudaSuccess ||
            cudaMalloc((void**)&g.d1, g.nstate * sizeof(float)) != cudaSuccess ||
            cudaMalloc((void**)&g.d2, g.nstate * sizeof(float)) != cudaSuccess) {
            cudaGetLastError();
            free_batch(b);
            return set_error(DGX_ERR_CUDA, "cudaMalloc / upload failed for the batched state");
        }
    }
    // face-trace form for Euler batches whose faces are all interior or boundary faces with a
    // condition: two trace buffers per order, each with one ghost block per boundary face after
    // the order's elements (the single context's trace-form connectivity, dgx_create)
    b->trace_ok = !visc;
    std::vector<ElemConn> tc[MAX_P];
    std::vector<int> gb[MAX_P];
    for (int p = 0; p < MAX_P && b->trace_ok; ++p) {
        const int ne = b->grp[p].ne;
        if (ne == 0 || !b->boundary) continue;
        tc[p] = cn[p];
        for (int e = 0; e < ne && b->trace_ok; ++e)
            for (int f = 0; f < 3; ++f) {
                const int nb = cn[p][e].nbr[f];
                if (nb == NBR_SKIP) {
                    b->trace_ok = false;  // a face without a condition: the batched kernel only
                    break;
                }
                if (nb < 0) {
                    tc[p][e].nbr[f] = ne + (int)gb[p].size();
                    tc[p][e].flags &= ~(7 << (4 * f));  // the block's face 0, points in this face's order
                    gb[p].push_back(-1 - nb);
                }
            }
    }
    for (int p = 0; p < MAX_P && b->trace_ok; ++p) {
        Group& g = b->grp[p];
        if (g.ne == 0) continue;
        g.nghost = (int)gb[p].size();
        const size_t bytes = ((size_t)g.ne + g.nghost) * trace_floats_per_element(p + 1) * sizeof(float);
        if (cudaMalloc((void**)&g.tr[0], bytes) != cudaSuccess || cudaMalloc((void**)&g.tr[1], bytes) != cudaSuccess ||
            (g.nghost && (!up((void**)&g.tconn, tc[p].data(), tc[p].size() * sizeof(ElemConn)) ||
                          !up((void**)&g.ghost_bc, gb[p].data(), gb[p].size() * sizeof(int))))) {
            cudaGetLastError();
            free_batch(b);
            return set_error(DGX_ERR_CUDA, "cudaMalloc failed for the batched face traces");
        }
    }
    if (cudaMalloc((void**)&b->d_dt, n_inst * sizeof(float)) != cudaSuccess ||
        cudaMemset(b->d_dt, 0, n_inst * sizeof(float)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        free_batch(b);
        return set_error(DGX_ERR_CUDA, "cudaMalloc failed for the batched time steps");
    }
    b->dt_uploaded.assign(n_inst, 0.0f);
    *out = b;
    return DGX_OK;
}

extern "C" int dgx_batch_info(const dgx_batch* b, int inst, int* ne, int* np, double** u) {
    if (!b) return set_error(DGX_ERR_INVALID, "null batch");
    if (inst < 0 || inst >= b->n_inst) return set_error(DGX_ERR_RANGE, "instance index out of range");
    const int p = b->inst_order[inst];
    if (ne) *ne = b->inst_ne[inst];
    if (np) *np = n_basis(p);
    if (u) *u = b->grp[p - 1].u + (size_t)b->inst_e0[inst] * n_basis(p) * NV;
    return DGX_OK;
}

extern "C" int dgx_batch_launch_shape(const dgx_batch* b, int* grid, int* tiles) {
    if (!b) return set_error(DGX_ERR_INVALID, "null batch");
    int t = 0;
    for (const Group& g : b->grp) t += (g.ne + TILE - 1) / TILE;
    if (grid) *grid = b->grid & ~STAGE_FLAGS;
    if (tiles) *tiles = t;
    return DGX_OK;
}

extern "C" int dgx_batch_stage_form(const dgx_batch* b, int* form) {
    if (!b || !form) return set_error(DGX_ERR_INVALID, "null argument");
    *form = b->grid == 0 ? 0 : (b->grid & STAGE_TRACE) ? 2 : 1;
    return DGX_OK;
}

// Stage arguments of every order for one step reading uhi[src], in place `kind` of its call.
static void batch_stage_args(const dgx_batch* b, int src, int stage, StepKind kind, StageArgs* a) {
    for (int p = 0; p < MAX_P; ++p) {
        const Group& g = b->grp[p];
        StageArgs& s = a[p];
        s = StageArgs{};
        s.ne = g.ne;
        if (!g.ne) continue;
        s.stage = stage;
        s.uhi = g.uhi[src];
        s.din = stage == 1 ? nullptr : stage == 2 ? g.d1 : g.d2;
        s.dout = stage == 1 ? g.d1 : stage == 2 ? g.d2 : nullptr;
        s.u64 = g.u;
        s.ulo = g.ulo;
        set_step_kind(s, kind);
        s.uhi_out = g.uhi[1 - src];
        s.geom = g.geomf;
        s.conn = g.conn;
        s.bc = g.bc;
        s.dt = 0.0f;
        s.gamma = (float)b->prm.gamma;
        if (b->prm.physics == DGX_NAVIER_STOKES) {
            s.mu = (float)b->prm.mu;
            s.kappa = (float)(b->prm.mu * b->prm.gamma / (b->prm.prandtl * (b->prm.gamma - 1.0)));
            s.sigma0 = (float)b->prm.sigma0;
        }
        // the batched kernel takes the batch's boundary flag as its own argument; the face-trace form
        // needs each order's: with ghost blocks, the order has boundary faces iff it has ghosts
        s.boundary = b->trace_ok ? (g.nghost > 0) : b->boundary;
        s.tconn = g.tconn;  // read by the face-trace form only
        s.ghost_bc = g.ghost_bc;
        s.dt_inst = b->d_dt;
        s.grid = b->grid;
    }
}

// The face-trace form of one stage: one launch per order.  A step starting from uhi[src] reads
// the traces in tr[src], tr[1-src], tr[src] and writes tr[1-src], tr[src], tr[1-src] (the single
// context's order), so the next step starts from uhi[1-src] with its traces in tr[1-src].
static int launch_batch_trace_stage(const dgx_batch* b, StageArgs* a, int src, int grid, cudaStream_t s) {
    for (int p = 0; p < MAX_P; ++p) {
        const Group& g = b->grp[p];
        if (!g.ne) continue;
        const int stage = a[p].stage;
        a[p].tin = g.tr[stage == 2 ? 1 - src : src];
        a[p].tout = g.tr[stage == 2 ? src : 1 - src];
        a[p].grid = grid;
        if (launch_stage_trace(p + 1, a[p], b->ops[p], grid & ~STAGE_TRACE, s)) return -1;
    }
    return 0;
}

// the traces of the start state uhi[0] of every order into tr[0]
static int launch_batch_trace_init(const dgx_batch* b, cudaStream_t s) {
    StageArgs a[MAX_P];
    batch_stage_args(b, 0, 1, STEP_ONLY, a);
    for (int p = 0; p < MAX_P; ++p) {
        const Group& g = b->grp[p];
        if (!g.ne) continue;
        a[p].tout = g.tr[0];
        if (launch_trace_init(p + 1, a[p], b->ops[p], s)) return -1;
    }
    return 0;
}

static int enqueue_batch_step(dgx_batch* b, int src, StepKind kind, cudaStream_t s) {
    for (int stage = 1; stage <= 3; ++stage) {
        StageArgs a[MAX_P];
        batch_stage_args(b, src, stage, kind, a);
        const int rc = (b->grid & STAGE_TRACE)
                           ? launch_batch_trace_stage(b, a, src, b->grid, s)
                           : launch_batch_stage(a, b->ops, b->boundary, b->prm.physics == DGX_NAVIER_STOKES, b->grid, s);
        if (rc)
            return set_error(DGX_ERR_CUDA, std::string("batched stage launch failed: ") +
                                               launch_error_text());
    }
    return DGX_OK;
}

static int capture_batch(dgx_batch* b, cudaGraphExec_t* out, int which) {
    cudaGraph_t g;
    GraphStep gs[2];
    const int steps = graph_steps(which, gs);
    if (cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
        return set_error(DGX_ERR_CUDA, "graph capture could not start");
    int rc = DGX_OK;
    for (int k = 0; k < steps && !rc; ++k) rc = enqueue_batch_step(b, gs[k].src, gs[k].kind, b->cap);
    const cudaError_t ec = cudaStreamEndCapture(b->cap, &g);
    if (rc) return rc;
    if (ec != cudaSuccess) return set_error(DGX_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
    const cudaError_t ei = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        *out = nullptr;
        return set_error(DGX_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
    }
    return DGX_OK;
}

extern "C" int dgx_batch_rk3_step(dgx_batch* b, const double* dt, int n_steps, void* stream) {
    if (!b || !dt || n_steps < 0) return set_error(DGX_ERR_INVALID, "dgx_batch_rk3_step: bad argument");
    for (int i = 0; i < b->n_inst; ++i)
        if (!(dt[i] > 0.0) || !std::isfinite(dt[i]))
            return set_error(DGX_ERR_INVALID, "dgx_batch_rk3_step: time step of instance " + std::to_string(i) +
                                                  " must be positive and finite");
    if (n_steps == 0) return DGX_OK;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<float> dtf(b->n_inst);
    for (int i = 0; i < b->n_inst; ++i) dtf[i] = (float)dt[i];
    if (dtf != b->dt_uploaded) {  // pageable source: the copy has read it when the call returns
        if (cudaMemcpyAsync(b->d_dt, dtf.data(), dtf.size() * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess)
            return set_error(DGX_ERR_CUDA, "time-step upload failed");
        b->dt_uploaded = dtf;
    }
    for (const Group& g : b->grp)
        if (g.ne && launch_f64_to_f32(g.nstate, g.u, g.uhi[0], s))
            return set_error(DGX_ERR_CUDA, "conversion launch failed");
    // the face-trace form's traces of the start state (its timed launches below read them too)
    if (b->trace_ok && (b->grid == 0 || (b->grid & STAGE_TRACE)) && launch_batch_trace_init(b, s))
        return set_error(DGX_ERR_CUDA, std::string("batched trace launch failed: ") + launch_error_text());
    if (b->grid == 0) {
        // launch shape: timed on stage 1, which writes only the increment scratch (and, in the
        // face-trace form, the traces in tr[1]); candidates: the batched kernel at each grid and,
        // for Euler batches without skipped faces, the face-trace form (DGX_STAGE_KERNEL=rows keeps
        // the first)
        std::string key = "batch";
        for (int p = 0; p < MAX_P; ++p) key += " p" + std::to_string(p + 1) + ":" + std::to_string(b->grp[p].ne);
        if (b->boundary) key += " bnd";
        const bool visc = b->prm.physics == DGX_NAVIER_STOKES;
        if (visc) key += " ns";
        const char* mode = std::getenv("DGX_STAGE_KERNEL");
        const bool rows_only = mode && std::strcmp(mode, "rows") == 0;
        const bool trace_only = mode && std::strcmp(mode, "trace32s") == 0;
        StageArgs a[MAX_P];
        batch_stage_args(b, 0, 1, STEP_ONLY, a);
        const OpsHost* ops = b->ops;
        std::vector<int> cands;
        if (!(trace_only && b->trace_ok)) cands = grid_candidates(batch_tiles(a));
        if (b->trace_ok && !rows_only) {
            cands.push_back(STAGE_TRACE | STAGE_T32 | STAGE_NBS | batch_tiles(a));
            key += " trace";
        }
        if (mode) key += std::string(" ") + mode;
        int grid = 0;
        const int rc = tune_grid(key, cands, [&](int g, cudaStream_t ts) {
            if (g & STAGE_TRACE) {
                StageArgs t[MAX_P];
                std::memcpy(t, a, sizeof(t));
                return launch_batch_trace_stage(b, t, 0, g, ts);
            }
            return launch_batch_stage(a, ops, b->boundary, visc, g, ts);
        }, s, &grid);
        if (rc) return rc;
        b->grid = grid;
    }
    return for_step_graphs(n_steps, [&](int g) {
        if (!b->graph[g])
            if (int rc = capture_batch(b, &b->graph[g], g)) return rc;
        if (cudaGraphLaunch(b->graph[g], s) != cudaSuccess)
            return set_error(DGX_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(cudaGetLastError()));
        return (int)DGX_OK;
    });
}
