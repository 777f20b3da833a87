// Batched mixed-precision SSP-RK3 stage kernel: many independent Euler or Navier-Stokes
// solves, of uneven sizes and orders 1..4, advanced by one persistent launch per stage.
//
// The instances of one order are concatenated into one element range (their own
// connectivity, offset into the range), so a tile of 128 elements holds one order only.
// Tiles of order 1 come first, then order 2, ...; each CTA loads the neighbour-face
// operators of every order once, then walks the tiles with a grid stride and runs the
// order's tile body (dg_stage.cuh) on each.  Each element carries its instance number in
// ElemGeomF::pad and takes its time step from a per-instance table.  The physics (and its
// parameters) is the batch's: VISC selects the Navier-Stokes tile body for every order.
#include <cstring>

#include "dg_stage.cuh"

namespace dgx {

template <bool VISC>
struct BatchArgs {
    SArgs<1, VISC> a1;
    SArgs<2, VISC> a2;
    SArgs<3, VISC> a3;
    SArgs<4, VISC> a4;
    int tile_end[MAX_P];  // tiles of orders 1..p, cumulative
};
static_assert(sizeof(BatchArgs<false>) <= 32764 && sizeof(BatchArgs<true>) <= 32764,
              "batched stage arguments exceed the kernel parameter limit");

template <int P, bool VISC>
__device__ __forceinline__ const SArgs<P, VISC>& batch_order(const BatchArgs<VISC>& b) {
    if constexpr (P == 1) return b.a1;
    else if constexpr (P == 2) return b.a2;
    else if constexpr (P == 3) return b.a3;
    else return b.a4;
}

// first shared-memory float of order p's neighbour-face operators (16-byte aligned)
template <bool VISC>
__host__ __device__ constexpr int batch_op_off(int p) {
    int s = 0;
    for (int q = 1; q < p; ++q) s += (VISC ? 3 : 1) * 3 * n_basis(q) * ((q + 1 + 3) & ~3);
    return s;
}

template <int P, int PMAX, bool VISC, bool BND>
__device__ __forceinline__ void batch_tile(const BatchArgs<VISC>& ka, const float* sOp, float* sU, float* sDt, int t) {
    if constexpr (P < PMAX) {
        if (t >= ka.tile_end[P - 1]) {
            batch_tile<P + 1, PMAX, VISC, BND>(ka, sOp, sU, sDt, t);
            return;
        }
    }
    const int t0 = P > 1 ? ka.tile_end[P - 2] : 0;
    stage_tile<P, VISC, BND>(batch_order<P>(ka), sOp + batch_op_off<VISC>(P), sU, sDt, t - t0);
}

template <int P, int PMAX, bool VISC>
__device__ __forceinline__ void batch_load_ops(const BatchArgs<VISC>& ka, float* sOp) {
    constexpr int OPF = stage_op_floats<P, VISC>();
    const float* src = &batch_order<P>(ka).nb.phi[0][0][0];
    for (int k = threadIdx.x; k < OPF; k += TILE) sOp[batch_op_off<VISC>(P) + k] = src[k];
    if constexpr (P < PMAX) batch_load_ops<P + 1, PMAX>(ka, sOp);
}

template <int PMAX, bool VISC, bool BND>
__global__ void __launch_bounds__(TILE, stage_min_blocks(PMAX, VISC))
    batch_stage_kernel(const __grid_constant__ BatchArgs<VISC> ka) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sOp = reinterpret_cast<float*>(smem_raw);
    float* sDt = sOp + batch_op_off<VISC>(PMAX + 1);
    float* sU = sDt + TILE;
    batch_load_ops<1, PMAX>(ka, sOp);
    __syncthreads();
    const int ntiles = ka.tile_end[PMAX - 1];
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) batch_tile<1, PMAX, VISC, BND>(ka, sOp, sU, sDt, t);
}

template <int PMAX, bool VISC>
constexpr size_t batch_smem_bytes() {
    return (size_t)(batch_op_off<VISC>(PMAX + 1) + TILE + TILE * stage_stride<PMAX>()) * sizeof(float);
}

template <int PMAX, bool VISC>
static int configure_batch_t() {
    const int b = (int)batch_smem_bytes<PMAX, VISC>();
    return cudaFuncSetAttribute(batch_stage_kernel<PMAX, VISC, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                b) == cudaSuccess &&
                   cudaFuncSetAttribute(batch_stage_kernel<PMAX, VISC, false>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, b) == cudaSuccess
               ? 0
               : -1;
}

template <bool VISC>
static int configure_batch_v() {
    return configure_batch_t<1, VISC>() || configure_batch_t<2, VISC>() || configure_batch_t<3, VISC>() ||
                   configure_batch_t<4, VISC>()
               ? -1
               : 0;
}

int configure_batch_stage(bool visc) { return visc ? configure_batch_v<true>() : configure_batch_v<false>(); }

template <int P, bool VISC>
static SArgs<P, VISC>& order_slot(BatchArgs<VISC>& b) {
    if constexpr (P == 1) return b.a1;
    else if constexpr (P == 2) return b.a2;
    else if constexpr (P == 3) return b.a3;
    else return b.a4;
}

template <int P, bool VISC>
static void fill_order(BatchArgs<VISC>& b, const StageArgs& a, const OpsHost& oh) {
    SArgs<P, VISC>& k = order_slot<P>(b);
    k.s = a;
    if (a.ne == 0) return;
    fill_ops<P, float>(oh, k.o);
    fill_lift<P, float>(oh, k.l);
    fill_nbr_ops<P>(oh, k.nb);
}

template <int PMAX, bool VISC>
static int launch_batch_t(const BatchArgs<VISC>& b, bool boundary, int grid, cudaStream_t st) {
    if (boundary)
        batch_stage_kernel<PMAX, VISC, true><<<grid, TILE, batch_smem_bytes<PMAX, VISC>(), st>>>(b);
    else
        batch_stage_kernel<PMAX, VISC, false><<<grid, TILE, batch_smem_bytes<PMAX, VISC>(), st>>>(b);
    return launch_status();
}

int batch_tiles(const StageArgs* per_order) {
    int n = 0;
    for (int p = 0; p < MAX_P; ++p) n += (per_order[p].ne + TILE - 1) / TILE;
    return n;
}

template <bool VISC>
static int launch_batch_v(const StageArgs* per_order, const OpsHost* ops, int boundary, int grid, cudaStream_t s) {
    static_assert(MAX_P == 4, "batched stage kernel covers orders 1..4");
    BatchArgs<VISC> b;
    std::memset(&b, 0, sizeof(b));
    fill_order<1>(b, per_order[0], ops[0]);
    fill_order<2>(b, per_order[1], ops[1]);
    fill_order<3>(b, per_order[2], ops[2]);
    fill_order<4>(b, per_order[3], ops[3]);
    int pmax = 0, tiles = 0;
    for (int p = 0; p < MAX_P; ++p) {
        tiles += (per_order[p].ne + TILE - 1) / TILE;
        b.tile_end[p] = tiles;
        if (per_order[p].ne > 0) pmax = p + 1;
    }
    if (tiles == 0) return 0;
    if (grid <= 0 || grid > tiles) grid = tiles;
    switch (pmax) {
    case 1: return launch_batch_t<1>(b, boundary != 0, grid, s);
    case 2: return launch_batch_t<2>(b, boundary != 0, grid, s);
    case 3: return launch_batch_t<3>(b, boundary != 0, grid, s);
    default: return launch_batch_t<4>(b, boundary != 0, grid, s);
    }
}

int launch_batch_stage(const StageArgs* per_order, const OpsHost* ops, int boundary, bool visc, int grid,
                       cudaStream_t s) {
    return visc ? launch_batch_v<true>(per_order, ops, boundary, grid, s)
                : launch_batch_v<false>(per_order, ops, boundary, grid, s);
}

}  // namespace dgx
