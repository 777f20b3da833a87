// Launchers of the tensor-core (3xTF32 tcgen05) form of the mixed-precision Euler stage,
// orders 1..3 (dg_stage_tc.cuh).
#include <cstdlib>

#include "dg_stage_tc.cuh"

namespace dgx {

// Bounded waits inside the kernels (kernel_wait_bounds); DGX_TC_WAIT_LIMIT=n: n plain polls.
static void tc_wait_bounds(long long* limit, unsigned* hint_ns) { kernel_wait_bounds("DGX_TC_WAIT_LIMIT", limit, hint_ns); }

template <int P>
static int configure_tc_t() {
    const int b = Tc<P>::SMEM;
    const auto set = [b](const void* f) {
        return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, b) == cudaSuccess;
    };
    return set((const void*)stage_tc_kernel<P, false>) && set((const void*)stage_tc_kernel<P, true>) &&
                   set((const void*)tc_trace_init_kernel<P, false>) && set((const void*)tc_trace_init_kernel<P, true>)
               ? 0
               : -1;
}

bool stage_tc_supported(int p) { return p >= 1 && p <= 3; }

int configure_stage_tc(int p) {
    switch (p) {
    case 1: return configure_tc_t<1>();
    case 2: return configure_tc_t<2>();
    case 3: return configure_tc_t<3>();
    default: return 0;  // no tensor-core form at this order; nothing to configure
    }
}

int stage_tc_ctas_per_sm(int) { return 1; }

template <int P>
static int launch_tc_t(const StageArgs& a, const OpsHost& oh, int grid, bool init, cudaStream_t st) {
    TcArgs<P> k;
    std::memset(&k, 0, sizeof(k));
    k.s = a;
    if (a.tconn) k.s.conn = a.tconn;  // boundary faces as interior faces to ghost blocks
    if (!fill_tc_ops<P>(oh, k)) return -1;
    tc_wait_bounds(&k.wait_limit, &k.wait_hint_ns);
    const int ntiles = a.ntile > 0 ? a.ntile : (a.ne + TILE - 1) / TILE;
    if (ntiles == 0) return 0;
    if (grid <= 0 || grid > ntiles) grid = ntiles;
    const bool ghost = a.tconn != nullptr;
    if (init) {
        if (ghost) tc_trace_init_kernel<P, true><<<grid, Tc<P>::THREADS, Tc<P>::SMEM, st>>>(k);
        else tc_trace_init_kernel<P, false><<<grid, Tc<P>::THREADS, Tc<P>::SMEM, st>>>(k);
    } else {
        if (ghost) stage_tc_kernel<P, true><<<grid, Tc<P>::THREADS, Tc<P>::SMEM, st>>>(k);
        else stage_tc_kernel<P, false><<<grid, Tc<P>::THREADS, Tc<P>::SMEM, st>>>(k);
    }
    return launch_status();
}

static int dispatch(int p, const StageArgs& a, const OpsHost& ops, int grid, bool init, cudaStream_t s) {
    // the tensor-core form covers meshes whose faces are all interior or ghost faces
    if (a.boundary && !a.tconn) return -1;
    switch (p) {
    case 1: return launch_tc_t<1>(a, ops, grid, init, s);
    case 2: return launch_tc_t<2>(a, ops, grid, init, s);
    case 3: return launch_tc_t<3>(a, ops, grid, init, s);
    default: return -1;
    }
}

int launch_stage_tc(int p, const StageArgs& a, const OpsHost& ops, int grid, cudaStream_t s) {
    return dispatch(p, a, ops, grid, false, s);
}

int launch_tc_trace_init(int p, const StageArgs& a, const OpsHost& ops, int grid, cudaStream_t s) {
    return dispatch(p, a, ops, grid, true, s);
}

}  // namespace dgx
