// Element kernels in double-float arithmetic (df64.cuh): the FP64 path's algorithm and
// FP64 state, geometry, M^-1 and RK3 combination, with the residual's arithmetic on the
// FP32 pipe in pairs of floats.
#include "df64.cuh"
#include "dg_element.cuh"
#include "dg_quad.cuh"

namespace dgx {

template <>
__device__ __forceinline__ f2 rcp_<f2>(f2 x) { return f2(1.0f, 0.0f) / x; }
template <>
__device__ __forceinline__ f2 sqrt_<f2>(f2 x) { return df_sqrt(x); }

int launch_element_df64(int p, bool viscous, const StepArgs& a, const OpsHost& ops, cudaStream_t s) {
#define ARGS (a, ops, s)
    DGX_ELEMENT_DISPATCH(launch_element_t, f2)
#undef ARGS
}

int launch_quad_element_df64(int p, bool viscous, const StepArgs& a, const QuadGeom* geom, const QuadConn* conn,
                             const OpsHost& ops, cudaStream_t s) {
    DGX_QUAD_DISPATCH(launch_quad_t, f2, (a, geom, conn, ops, s))
}

int configure_quad_element_df64(int p, bool viscous) { DGX_QUAD_DISPATCH(configure_quad_t, f2, ()) }

int configure_element_df64(int p, bool viscous) {
#define ARGS ()
    DGX_ELEMENT_DISPATCH(configure_element_t, f2)
#undef ARGS
}

}  // namespace dgx
