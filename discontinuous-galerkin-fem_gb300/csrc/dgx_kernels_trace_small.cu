// Face-trace form of the mixed Euler stage at 64- and 32-element tiles (dg_stage_trace.cuh,
// stage_trace_kernel<P, BND, GHOST, T>), in a translation unit of its own so that it compiles
// beside the 128-element kernels.  One CTA per tile; the host's tile range (StageArgs::tile0,
// ntile, counted in 128-element tiles) is converted to T-element tiles here.  The 32-element
// kernels that copy the neighbours' trace blocks into shared memory are in
// dgx_kernels_trace_nbs.cu.
#include "dg_stage_trace.cuh"

namespace dgx {

template <int P, int T>
static int launch_small_t(const StageArgs& a, const OpsHost& oh, cudaStream_t st) {
    static_assert(TILE % T == 0, "tiles of T elements split the 128-element tiles");
    constexpr int K = TILE / T;
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
    const size_t smem = stage_trace_smem_bytes<P, T>();
    if (a.tconn)
        stage_trace_kernel<P, false, true, T><<<nt, T, smem, st>>>(ka);
    else if (a.boundary)
        stage_trace_kernel<P, true, false, T><<<nt, T, smem, st>>>(ka);
    else
        stage_trace_kernel<P, false, false, T><<<nt, T, smem, st>>>(ka);
    return launch_status();
}

int launch_stage_trace_small(int p, int tile, bool nbs, const StageArgs& a, const OpsHost& ops, cudaStream_t s) {
    const bool t64 = tile == 64;
    if (!t64 && tile != 32) return -1;
    if (nbs) return t64 ? -1 : launch_stage_trace_nbs(p, a, ops, s);
    switch (p) {
    case 1: return t64 ? launch_small_t<1, 64>(a, ops, s) : launch_small_t<1, 32>(a, ops, s);
    case 2: return t64 ? launch_small_t<2, 64>(a, ops, s) : launch_small_t<2, 32>(a, ops, s);
    case 3: return t64 ? launch_small_t<3, 64>(a, ops, s) : launch_small_t<3, 32>(a, ops, s);
    case 4: return t64 ? launch_small_t<4, 64>(a, ops, s) : launch_small_t<4, 32>(a, ops, s);
    default: return -1;
    }
}

}  // namespace dgx
