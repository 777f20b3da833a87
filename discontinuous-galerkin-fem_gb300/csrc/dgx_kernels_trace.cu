// Face-trace form of the mixed Euler stage (dg_stage_trace.cuh).
#include "dg_stage_trace.cuh"

namespace dgx {

#define DGX_TRACE_P(FN, ARGS)          \
    switch (p) {                       \
    case 1: return FN<1> ARGS;         \
    case 2: return FN<2> ARGS;         \
    case 3: return FN<3> ARGS;         \
    case 4: return FN<4> ARGS;         \
    default: return -1;                \
    }

int launch_stage_trace(int p, const StageArgs& a, const OpsHost& ops, int grid, cudaStream_t s) {
    if (grid & (STAGE_T64 | STAGE_T32))
        return launch_stage_trace_small(p, (grid & STAGE_T64) ? 64 : 32, (grid & STAGE_NBS) != 0, a, ops, s);
    DGX_TRACE_P(launch_stage_trace_t, (a, ops, grid, s))
}

int launch_trace_init(int p, const StageArgs& a, const OpsHost& ops, cudaStream_t s) {
    DGX_TRACE_P(launch_trace_init_t, (a, ops, s))
}

int configure_stage_trace(int p) { DGX_TRACE_P(configure_stage_trace_t, ()) }

size_t trace_floats_per_element(int p) { return (size_t)3 * (p + 1) * NV; }

}  // namespace dgx
