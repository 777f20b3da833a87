// Face-trace form of the mixed Euler stage at 32-element tiles with each element's neighbour
// trace blocks copied into shared memory during staging (dg_stage_trace.cuh,
// stage_trace_kernel<P, false, GHOST, 32, true, SK>), one CTA per tile, on meshes whose faces
// are all interior or ghost faces.  Each stage runs the instantiation specialised for it:
// stage 1, stage 2, stage 3 of a step between the first and the last of a call (double-float
// state in and out), or the general one (stage 3 of a call's first or last step, which reads or
// writes the FP64 state).  Stages 1 and 2 apart measured 0.7 % faster than one kernel for both.  The host's tile range (StageArgs::tile0, ntile, counted in 128-element
// tiles) is converted to 32-element tiles here.
#include "dg_stage_trace.cuh"

namespace dgx {

template <int P, int SK>
static int launch_nbs_t(const StageArgs& a, const OpsHost& oh, cudaStream_t st) {
    constexpr int T = 32, K = TILE / T;
    if (a.boundary && !a.tconn) return -1;  // faces without a condition: no neighbour block to copy
    SArgs<P, false> ka;
    ka.s = a;
    if (a.tconn) ka.s.conn = a.tconn;  // boundary faces as interior faces to ghost blocks
    fill_ops<P, float>(oh, ka.o);
    fill_lift<P, float>(oh, ka.l);
    const int all = (a.ne + T - 1) / T;
    const int t0 = a.tile0 * K;
    const int nt = a.ntile > 0 ? std::min(a.ntile * K, all - t0) : all - t0;
    if (nt <= 0) return 0;
    ka.s.tile0 = t0;
    ka.s.ntile = nt;
    const size_t smem = stage_trace_smem_bytes<P, T, true>();
    if (a.tconn)
        stage_trace_kernel<P, false, true, T, true, SK><<<nt, T, smem, st>>>(ka);
    else
        stage_trace_kernel<P, false, false, T, true, SK><<<nt, T, smem, st>>>(ka);
    return launch_status();
}

template <int P>
static int launch_nbs_p(const StageArgs& a, const OpsHost& oh, cudaStream_t st) {
    if (a.stage == 1) return launch_nbs_t<P, SK_1>(a, oh, st);
    if (a.stage == 2) return launch_nbs_t<P, SK_2>(a, oh, st);
    if (!a.u64_in && !a.u64_out) return launch_nbs_t<P, SK_3DF>(a, oh, st);
    return launch_nbs_t<P, SK_ANY>(a, oh, st);
}

int launch_stage_trace_nbs(int p, const StageArgs& a, const OpsHost& ops, cudaStream_t s) {
    switch (p) {
    case 1: return launch_nbs_p<1>(a, ops, s);
    case 2: return launch_nbs_p<2>(a, ops, s);
    case 3: return launch_nbs_p<3>(a, ops, s);
    case 4: return launch_nbs_p<4>(a, ops, s);
    default: return -1;
    }
}

}  // namespace dgx
