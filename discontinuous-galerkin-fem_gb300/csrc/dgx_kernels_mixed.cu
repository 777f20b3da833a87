// Mixed-precision element kernels: FP32 flux and contraction arithmetic, FP64 geometry,
// FP64 inverse mass matrix and FP64 RK3 state accumulation.
#include "dg_stage.cuh"

namespace dgx {

int launch_element_mixed(int p, bool viscous, const StepArgs& a, const OpsHost& ops, cudaStream_t s) {
#define ARGS (a, ops, s)
    DGX_ELEMENT_DISPATCH(launch_element_t, float)
#undef ARGS
}

int launch_stage_mixed(int p, bool viscous, const StageArgs& a, const OpsHost& ops, cudaStream_t s) {
    if (a.qgeom) return launch_quad_stage(p, viscous, a, ops, s);
    if (a.grid & STAGE_TRACE) {
        if (viscous) return -1;
        return launch_stage_trace(p, a, ops, a.grid & ~STAGE_TRACE, s);
    }
    if (a.grid & STAGE_TC) {
        if (viscous) return -1;
        return launch_stage_tc(p, a, ops, a.grid & ~STAGE_TC, s);
    }
#define ARGS (a, ops, s)
    DGX_ELEMENT_DISPATCH(launch_stage_t, float)
#undef ARGS
}

static int configure_stage(int p, bool viscous) {
#define ARGS ()
    DGX_ELEMENT_DISPATCH(configure_stage_t, float)
#undef ARGS
}

int configure_element_mixed(int p, bool viscous) {
    if (configure_stage(p, viscous)) return -1;
#define ARGS ()
    DGX_ELEMENT_DISPATCH(configure_element_t, float)
#undef ARGS
}

}  // namespace dgx
