// Launchers of the tensor-core (3xTF32 tcgen05) form of the mixed-precision Euler stage.
#include "dg_stage_tc.cuh"

namespace dgx {

template <int P>
static int configure_tc_t() {
    const int b = (int)stage_tc_smem_bytes<P>();
    return cudaFuncSetAttribute(stage_tc_kernel<P, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ==
                       cudaSuccess &&
                   cudaFuncSetAttribute(stage_tc_kernel<P, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ==
                       cudaSuccess
               ? 0
               : -1;
}

int configure_stage_tc(int p) {
    switch (p) {
    case 1: return configure_tc_t<1>();
    case 2: return configure_tc_t<2>();
    case 3: return configure_tc_t<3>();
    case 4: return configure_tc_t<4>();
    default: return -1;
    }
}

int stage_tc_ctas_per_sm(int p) {
    switch (p) {
    case 1: return TcShape<1>::COLS == 512 ? 1 : 2;
    case 2: return TcShape<2>::COLS == 512 ? 1 : 2;
    case 3: return TcShape<3>::COLS == 512 ? 1 : 2;
    default: return TcShape<4>::COLS == 512 ? 1 : 2;
    }
}

template <int P>
static int launch_tc_t(const StageArgs& a, const OpsHost& oh, int grid, cudaStream_t st) {
    TArgs<P> k;
    k.s = a;
    fill_tc_ops<P>(oh, k);
    const int ntiles = (a.ne + TILE - 1) / TILE;
    if (ntiles == 0) return 0;
    if (grid <= 0 || grid > ntiles) grid = ntiles;
    const size_t smem = stage_tc_smem_bytes<P>();
    if (a.boundary)
        stage_tc_kernel<P, true><<<grid, TcShape<P>::THREADS, smem, st>>>(k);
    else
        stage_tc_kernel<P, false><<<grid, TcShape<P>::THREADS, smem, st>>>(k);
    return launch_status();
}

int launch_stage_tc(int p, const StageArgs& a, const OpsHost& ops, int grid, cudaStream_t s) {
    switch (p) {
    case 1: return launch_tc_t<1>(a, ops, grid, s);
    case 2: return launch_tc_t<2>(a, ops, grid, s);
    case 3: return launch_tc_t<3>(a, ops, grid, s);
    case 4: return launch_tc_t<4>(a, ops, grid, s);
    default: return -1;
    }
}

}  // namespace dgx
