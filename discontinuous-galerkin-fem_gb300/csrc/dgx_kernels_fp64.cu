// FP64 element kernels: the plain form of the path, parity target <= 1e-12 against dgfem.
#include "dg_element.cuh"

namespace dgx {

int launch_element_fp64(int p, bool viscous, const StepArgs& a, const OpsHost& ops, cudaStream_t s) {
#define ARGS (a, ops, s)
    DGX_ELEMENT_DISPATCH(launch_element_t, double)
#undef ARGS
}

int configure_element_fp64(int p, bool viscous) {
#define ARGS ()
    DGX_ELEMENT_DISPATCH(configure_element_t, double)
#undef ARGS
}

}  // namespace dgx
