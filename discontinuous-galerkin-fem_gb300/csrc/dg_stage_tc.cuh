// Tensor-core form of the mixed-precision SSP-RK3 stage (Euler): the basis<->point
// contractions run as 3xTF32 tcgen05 GEMMs with FP32 accumulation in TMEM.
//
// Same discretisation, increment form and stage combination as stage_kernel
// (dg_stage.cuh); only where the contractions run changes.  Per tile of 128 elements
// (M = 128 rows, element e = TMEM lane e), for each conserved variable v:
//   GEMM1  D1_v[e, n] = sum_i U[e, i, v] Psi[n, i]          interpolation to the NQ volume
//          points and the 3 * NFQ face points of the element's own faces;
//   GEMM2  D2_v[e, i] = sum_m A2_v[e, m] W[i, m]            projection back to the basis:
//          A2_v = [Fr(q) | Fs(q) | H'(f, j)], W = [pr | ps | pf] (M_ref^-1 folded in, as
//          LiftOps), so D2 = M^-1-scaled residual R[e, i, v].
// Each product is split 3xTF32 (a = a_hi + a_lo; a*b ~ a_hi b_hi + a_hi b_lo + a_lo b_hi),
// which keeps FP32-level accuracy.  Between the GEMMs, CUDA cores evaluate the Euler
// fluxes at the points, the neighbour traces and the Rusanov fluxes; they read D1 from
// TMEM and write A2 to TMEM (tcgen05.ld / tcgen05.st, each thread its element's lane).
//
// Operands: A1 (the tile's state, split) and the constant B operands sit in shared memory
// in the K-major no-swizzle layout of tc_ptx.cuh; A2 is read from TMEM.  TMEM holds
// D1 (4 x N1 columns; D2 reuses them), A2 hi and A2 lo (4 x K2 each): 192 to 512 columns.
//
// A CTA has 256 threads: two per element (TMEM lane e is reachable from warps e/32 and
// e/32 + 4).  Half 0 does the volume points and face 0, half 1 faces 1 and 2.  One
// thread issues the MMAs; completion is tracked by mbarriers whose waits are bounded.
#pragma once

#include <cstring>

#include "dg_stage.cuh"
#include "tc_ptx.cuh"

namespace dgx {

template <int P>
struct TcShape {
    static constexpr int NP = n_basis(P), NQ = n_quad(P), NFQ = P + 1, NB = NP * NV;
    static constexpr int NQ4 = (NQ + 3) & ~3;             // volume slots, padded to 4
    static constexpr int FQ = 3 * NFQ;                    // face points of the three faces
    static constexpr int FQ4 = (FQ + 3) & ~3;
    static constexpr int KP = (NP + 7) & ~7;              // GEMM1 K (basis)
    static constexpr int N1 = (NQ4 + FQ4 + 15) & ~15;     // GEMM1 N per variable (points)
    static constexpr int K2 = (2 * NQ4 + FQ4 + 7) & ~7;   // GEMM2 K per variable (flux slots)
    static constexpr int N2 = 16;                         // GEMM2 N per variable (basis, padded)
    static constexpr int A2 = 4 * N1;                     // TMEM column of A2 hi; lo follows at +4*K2
    static constexpr int COLS_USED = A2 + 8 * K2;
    static constexpr int COLS = COLS_USED <= 256 ? 256 : 512;
    static constexpr int THREADS = 2 * TILE;
};
static_assert(TcShape<4>::COLS_USED <= 512, "TMEM budget");
static_assert(TcShape<1>::N2 >= n_basis(1) && TcShape<4>::N2 >= n_basis(4), "GEMM2 N covers the basis");

template <int P>
struct TArgs {
    using S = TcShape<P>;
    StageArgs s;
    NbrOps<P> nb;
    float b1[2][S::N1 * S::KP];  // GEMM1 B, hi and lo: row n = point slot, k = basis function
    float b2[2][S::N2 * S::K2];  // GEMM2 B, hi and lo: row i = basis function, k = flux slot
    float wq[S::NQ];
    float wf[S::NFQ];
};

// shared memory: A1 [2][4][TILE * KP] | B1 [2][N1 * KP] | B2 [2][N2 * K2] | staged inputs
//                [2][TILE * NB] (uhi, d; bulk-copied) | U tile [TILE][STR] | neighbour-face
//                operators | dt [TILE] | 3 mbarriers | TMEM address
template <int P>
__host__ __device__ constexpr int tc_smem_floats() {
    using S = TcShape<P>;
    return 8 * TILE * S::KP + 2 * S::N1 * S::KP + 2 * S::N2 * S::K2 + 2 * TILE * S::NB + TILE * stage_stride<P>() +
           stage_op_floats<P, false>() + TILE + 8;
}

static __device__ int g_tc_timeout;  // set when a bounded mbarrier wait gave up (never expected)

// Traces of face f's neighbour at this face's points, from the neighbour's coefficients
// (independent of GEMM1, so they are formed while it runs).
template <int P, bool BND>
__device__ __forceinline__ void tc_face_nbr(const TArgs<P>& ka, const float* sOp, const ElemConn& C, int f,
                                            float (&Un)[P + 1][4]) {
    using S = TcShape<P>;
    constexpr int NP = S::NP, NFQ = S::NFQ, NB = S::NB, NFQP = NbrOps<P>::NFQP;
    const StageArgs& s = ka.s;
#pragma unroll
    for (int k = 0; k < NFQ; ++k)
#pragma unroll
        for (int v = 0; v < NV; ++v) Un[k][v] = 0.f;
    const int nb = C.nbr[f];
    if (BND && nb < 0) return;
    const int fl = (C.flags >> (4 * f)) & 15;
    const int nf = fl & 3;
    const bool rev = (fl >> 2) & 1;
    const float* op = sOp + nf * NP * NFQP;
#pragma unroll
    for (int i = 0; i < NP; ++i) {
        float c[4];
        load_row_f32<NB>(s.uhi, s.din, nb, i, c);
        float w[NFQP];
#pragma unroll
        for (int k4 = 0; k4 < NFQP; k4 += 4) {
            const float4 t = *reinterpret_cast<const float4*>(op + i * NFQP + k4);
            w[k4] = t.x; w[k4 + 1] = t.y; w[k4 + 2] = t.z; w[k4 + 3] = t.w;
        }
#pragma unroll
        for (int k = 0; k < NFQ; ++k) fma4(w[k], c, Un[k]);
    }
#pragma unroll
    for (int j = 0; j < NFQ / 2; ++j)
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            const float a = Un[j][v], b = Un[NFQ - 1 - j][v];
            Un[j][v] = rev ? b : a;
            Un[NFQ - 1 - j][v] = rev ? a : b;
        }
}

// H' = -(w_j h_F / (2|J|)) * numerical flux at the points of face f, written to A2 (hi, lo).
// Own traces come from D1; Un are the neighbour traces (unused on boundary faces).
template <int P, bool BND>
__device__ __forceinline__ void tc_face_flux(const TArgs<P>& ka, uint32_t tl, const ElemGeomF& G, const ElemConn& C,
                                             int f, const float (&Un)[P + 1][4]) {
    using S = TcShape<P>;
    constexpr int NFQ = S::NFQ;
    const StageArgs& s = ka.s;
    float Uo[NFQ][4];
#pragma unroll
    for (int j = 0; j < NFQ; ++j)
#pragma unroll
        for (int v = 0; v < NV; ++v) tc::ld1(tl + v * S::N1 + S::NQ4 + f * NFQ + j, Uo[j][v]);
    const int nb = C.nbr[f];
    const float nx = G.n[f][0], ny = G.n[f][1], hF = G.h[f];
    const float gamma = s.gamma;
    const bool interior = !BND || nb >= 0;
    tc::wait_ld();
    const float inv_j = __frcp_rn(G.detJ);
    float Hh[NFQ][4], Hl[NFQ][4];
#pragma unroll
    for (int j = 0; j < NFQ; ++j) {
        float H[4] = {0.f, 0.f, 0.f, 0.f};
        if (interior) {
            rusanov<float>(Uo[j], Un[j], nx, ny, gamma, H);
        } else if (nb != NBR_SKIP) {
            const BCSlot bc = s.bc[-1 - nb];
            float Ub[4];
            if (inviscid_ghost<float>(bc, Uo[j], nx, ny, gamma, Ub)) rusanov<float>(Uo[j], Ub, nx, ny, gamma, H);
        }
        const float w = -ka.wf[j] * hF * 0.5f * inv_j;
#pragma unroll
        for (int v = 0; v < NV; ++v) tc::split3(w * H[v], Hh[j][v], Hl[j][v]);
    }
    __syncwarp();
#pragma unroll
    for (int j = 0; j < NFQ; ++j)
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            const uint32_t col = 2 * S::NQ4 + f * NFQ + j;
            tc::st1(tl + S::A2 + v * S::K2 + col, Hh[j][v]);
            tc::st1(tl + S::A2 + (4 + v) * S::K2 + col, Hl[j][v]);
        }
}

template <int P, bool BND>
__global__ void __launch_bounds__(2 * TILE, 1) stage_tc_kernel(const __grid_constant__ TArgs<P> ka) {
    using S = TcShape<P>;
    constexpr int NP = S::NP, NQ = S::NQ, NB = S::NB, KP = S::KP, STR = stage_stride<P>(), NB4 = NB / 4;
    constexpr int OPF = stage_op_floats<P, false>();
    constexpr long WAIT_LIMIT = 1L << 24;
    const StageArgs& s = ka.s;
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    float* sA1 = reinterpret_cast<float*>(tc_smem_raw);
    float* sB1 = sA1 + 8 * TILE * KP;
    float* sB2 = sB1 + 2 * S::N1 * KP;
    float* sIn = sB2 + 2 * S::N2 * S::K2;  // [2][TILE * NB]: the next tile's uhi and d, bulk-copied
    float* sU = sIn + 2 * TILE * NB;
    float* sOp = sU + TILE * STR;
    float* sDt = sOp + OPF;
    uint64_t* mbar = reinterpret_cast<uint64_t*>(sDt + TILE);  // GEMM1, GEMM2, input copy
    uint32_t* tslot = reinterpret_cast<uint32_t*>(mbar + 3);

    const int t = threadIdx.x, warp = t >> 5;
    const int e = t & (TILE - 1), half = t >> 7;  // element (= TMEM lane), half
    for (int k = t; k < 2 * S::N1 * KP; k += S::THREADS) sB1[k] = (&ka.b1[0][0])[k];
    for (int k = t; k < 2 * S::N2 * S::K2; k += S::THREADS) sB2[k] = (&ka.b2[0][0])[k];
    for (int k = t; k < OPF; k += S::THREADS) sOp[k] = (&ka.nb.phi[0][0][0])[k];
    if (t == 0) {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        tc::mbar_init(&mbar[2], 1);
    }
    if (warp == 0) tc::tmem_alloc(tslot, S::COLS);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tm = *tslot;
    const uint32_t tl = tm + ((uint32_t)(32 * (warp & 3)) << 16);  // this warp's lane quadrant
    // A2 columns past the last flux slot are read by GEMM2 and never written per tile
    for (int c = 2 * S::NQ4 + S::FQ + half; c < S::K2; c += 2)
#pragma unroll
        for (int v = 0; v < 8; ++v) tc::st1(tl + S::A2 + v * S::K2 + c, 0.f);
    tc::wait_st();

    uint32_t phase = 0;
    bool failed = false;
    const int ntiles = (s.ne + TILE - 1) / TILE;
    // bulk copy of a tile's inputs into sIn, completing on mbar[2]
    auto stage_in = [&](int tile) {
        const int n0 = tile * TILE, nn = min(TILE, s.ne - n0);
        const uint32_t bytes = (uint32_t)(nn * NB * sizeof(float));
        tc::mbar_expect_tx(&mbar[2], s.din ? 2 * bytes : bytes);
        tc::bulk_g2s(sIn, s.uhi + (size_t)n0 * NB, bytes, &mbar[2]);
        if (s.din) tc::bulk_g2s(sIn + TILE * NB, s.din + (size_t)n0 * NB, bytes, &mbar[2]);
    };
    if (t == 0 && (int)blockIdx.x < ntiles) stage_in(blockIdx.x);
    bool copy_pending = (int)blockIdx.x < ntiles;
    uint32_t copy_parity = 0;  // the phase of mbar[2] the pending copy completes
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, phase ^= 1) {
        const int e0 = tile * TILE;
        const int nloc = min(TILE, s.ne - e0);
        const bool active = e < nloc;
        const int ee = active ? e0 + e : e0;  // inactive lanes work on a valid element; results unused
        if (t == 0 && s.stage == 3)  // this tile's FP64 state, read in the stage combination
            tc::prefetch_l2(s.u64 + (size_t)e0 * NB, (uint32_t)(nloc * NB * sizeof(double)));
        // the tile's inputs, bulk-copied into sIn while the previous tile was computed
        const bool okin = tc::mbar_wait(&mbar[2], phase, WAIT_LIMIT);
        if (__syncthreads_or(!okin)) {
            failed = true;
            break;
        }
        copy_pending = false;
        {   // stage state of the tile, rows = elements
            const float4* uh = reinterpret_cast<const float4*>(sIn);
            const float4* dd = s.din ? reinterpret_cast<const float4*>(sIn + TILE * NB) : nullptr;
            for (int g = t; g < nloc * NB4; g += S::THREADS) {
                float4 a = uh[g];
                if (dd) {
                    const float4 b = dd[g];
                    a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w;
                }
                const int le = g / NB4, k = 4 * (g - le * NB4);
                *reinterpret_cast<float4*>(sU + le * STR + k) = a;
            }
        }
        __syncthreads();
        if (tile + (int)gridDim.x < ntiles) {  // sIn is free: start the next tile's copy
            if (t == 0) {
                tc::fence_async_smem();
                stage_in(tile + gridDim.x);
            }
            copy_pending = true;
            copy_parity = phase ^ 1;
        }
        // A1: the split state in the K-major operand layout, variables 2*half and 2*half + 1
#pragma unroll
        for (int vv = 0; vv < 2; ++vv) {
            const int v = 2 * half + vv;
#pragma unroll
            for (int k4 = 0; k4 < KP; k4 += 4) {
                float hi[4], lo[4];
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int i = k4 + c;
                    const float x = (i < NP && active) ? sU[e * STR + i * NV + v] : 0.f;
                    tc::split3(x, hi[c], lo[c]);
                }
                const int off = tc::canon_off(e, k4, KP);
                *reinterpret_cast<float4*>(sA1 + v * TILE * KP + off) = make_float4(hi[0], hi[1], hi[2], hi[3]);
                *reinterpret_cast<float4*>(sA1 + (4 + v) * TILE * KP + off) = make_float4(lo[0], lo[1], lo[2], lo[3]);
            }
        }
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        if (t == 0) {  // GEMM1: per variable, KP/8 steps of three TF32 products
            tc::fence_after();
            constexpr uint32_t id = tc::idesc_tf32(128, S::N1);
            constexpr uint32_t SBO = (KP / 4) * 128;
            const uint32_t b_hi = tc::smem_u32(sB1), b_lo = tc::smem_u32(sB1 + S::N1 * KP);
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                const uint32_t a_hi = tc::smem_u32(sA1 + v * TILE * KP), a_lo = tc::smem_u32(sA1 + (4 + v) * TILE * KP);
#pragma unroll
                for (int ks = 0; ks < KP / 8; ++ks) {
                    const uint32_t d = tm + v * S::N1;
                    tc::mma_ss(d, tc::smem_desc(a_lo + ks * 256, 128, SBO), tc::smem_desc(b_hi + ks * 256, 128, SBO), id, ks > 0);
                    tc::mma_ss(d, tc::smem_desc(a_hi + ks * 256, 128, SBO), tc::smem_desc(b_lo + ks * 256, 128, SBO), id, true);
                    tc::mma_ss(d, tc::smem_desc(a_hi + ks * 256, 128, SBO), tc::smem_desc(b_hi + ks * 256, 128, SBO), id, true);
                }
            }
            tc::commit(&mbar[0]);
        }
        // neighbour traces while GEMM1 runs: half 0 face 0, half 1 faces 1 and 2
        const ElemGeomF G = s.geom[ee];
        const ElemConn C = s.conn[ee];
        float UnA[P + 1][4], UnB[P + 1][4];
        if (half == 0) {
            tc_face_nbr<P, BND>(ka, sOp, C, 0, UnA);
        } else {
            tc_face_nbr<P, BND>(ka, sOp, C, 1, UnA);
            tc_face_nbr<P, BND>(ka, sOp, C, 2, UnB);
        }
        const bool ok1 = tc::mbar_wait(&mbar[0], phase, WAIT_LIMIT);
        if (__syncthreads_or(!ok1)) {
            failed = true;
            break;
        }
        tc::fence_after();

        // ---- fluxes between the GEMMs
        if (half == 0) {
            if (active && s.dt_inst) sDt[e] = s.dt_inst[__float_as_int(G.pad)];
            __syncwarp();
            const float A00 = G.A[0], A01 = G.A[1], A10 = G.A[2], A11 = G.A[3];
#pragma unroll
            for (int q0 = 0; q0 < S::NQ4; q0 += 4) {
                float Uv[4][4];
#pragma unroll
                for (int v = 0; v < NV; ++v) tc::ld4(tl + v * S::N1 + q0, Uv[v]);
                tc::wait_ld();
                float rh[4][4], rl[4][4], sh[4][4], sl[4][4];  // [variable][point]
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int q = q0 + j;
                    if (q < NQ) {
                        const float U[4] = {Uv[0][j], Uv[1][j], Uv[2][j], Uv[3][j]};
                        float F[4], Gf[4], u, vv, pp, ri;
                        euler_flux<float>(U, s.gamma - 1.0f, F, Gf, u, vv, pp, ri);
#pragma unroll
                        for (int v = 0; v < NV; ++v) {
                            tc::split3(ka.wq[q] * (A00 * F[v] + A10 * Gf[v]), rh[v][j], rl[v][j]);
                            tc::split3(ka.wq[q] * (A01 * F[v] + A11 * Gf[v]), sh[v][j], sl[v][j]);
                        }
                    } else {
#pragma unroll
                        for (int v = 0; v < NV; ++v) rh[v][j] = rl[v][j] = sh[v][j] = sl[v][j] = 0.f;
                    }
                }
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    tc::st4(tl + S::A2 + v * S::K2 + q0, rh[v]);
                    tc::st4(tl + S::A2 + (4 + v) * S::K2 + q0, rl[v]);
                    tc::st4(tl + S::A2 + v * S::K2 + S::NQ4 + q0, sh[v]);
                    tc::st4(tl + S::A2 + (4 + v) * S::K2 + S::NQ4 + q0, sl[v]);
                }
            }
            tc_face_flux<P, BND>(ka, tl, G, C, 0, UnA);
        } else {
            tc_face_flux<P, BND>(ka, tl, G, C, 1, UnA);
            tc_face_flux<P, BND>(ka, tl, G, C, 2, UnB);
        }
        __syncwarp();
        tc::wait_st();
        tc::fence_before();
        __syncthreads();
        if (t == 0) {  // GEMM2: A from TMEM, per variable, K2/8 steps of three TF32 products
            tc::fence_after();
            constexpr uint32_t id = tc::idesc_tf32(128, S::N2);
            constexpr uint32_t SBO = (S::K2 / 4) * 128;
            const uint32_t b_hi = tc::smem_u32(sB2), b_lo = tc::smem_u32(sB2 + S::N2 * S::K2);
#pragma unroll
            for (int v = 0; v < 4; ++v) {
                const uint32_t d = tm + v * S::N2;
#pragma unroll
                for (int ks = 0; ks < S::K2 / 8; ++ks) {
                    const uint32_t a_hi = tm + S::A2 + v * S::K2 + ks * 8, a_lo = tm + S::A2 + (4 + v) * S::K2 + ks * 8;
                    tc::mma_ts(d, a_lo, tc::smem_desc(b_hi + ks * 256, 128, SBO), id, ks > 0);
                    tc::mma_ts(d, a_hi, tc::smem_desc(b_lo + ks * 256, 128, SBO), id, true);
                    tc::mma_ts(d, a_hi, tc::smem_desc(b_hi + ks * 256, 128, SBO), id, true);
                }
            }
            tc::commit(&mbar[1]);
        }
        const bool ok2 = tc::mbar_wait(&mbar[1], phase, WAIT_LIMIT);
        if (__syncthreads_or(!ok2)) {
            failed = true;
            break;
        }
        tc::fence_after();
        {   // residual (M^-1 applied) of variables 2*half, 2*half + 1 into the tile rows
            float r0[16], r1[16];
            __syncwarp();
            tc::ld16(tl + (2 * half) * S::N2, r0);
            tc::ld16(tl + (2 * half + 1) * S::N2, r1);
            tc::wait_ld();
            if (active) {
#pragma unroll
                for (int i = 0; i < NP; ++i)
                    *reinterpret_cast<float2*>(sU + e * STR + i * NV + 2 * half) = make_float2(r0[i], r1[i]);
            }
        }
        tc::fence_before();
        __syncthreads();
        stage_combine<NB, STR, S::THREADS, (TILE * NB4 + S::THREADS - 1) / S::THREADS>(s, sU, sDt, e0, nloc,
                                                                                       [](int le) { return le; });
        __syncthreads();
    }
    if (failed) {  // a wait gave up: flag it, let outstanding MMAs and copies drain
        if (t == 0) atomicExch(&g_tc_timeout, 1);
        tc::mbar_wait(&mbar[0], phase, WAIT_LIMIT);
        tc::mbar_wait(&mbar[1], phase, WAIT_LIMIT);
    }
    if (copy_pending) tc::mbar_wait(&mbar[2], copy_parity, WAIT_LIMIT);
    tc::fence_before();
    __syncthreads();
    if (warp == 0) {
        tc::fence_after();
        tc::tmem_dealloc(tm, S::COLS);
    }
}

// host: tf32 rounding (nearest, ties to even) of a finite float
inline float tf32_round_host(float x) {
    uint32_t b;
    std::memcpy(&b, &x, 4);
    if ((b & 0x7f800000u) == 0x7f800000u) return x;
    b += 0xFFFu + ((b >> 13) & 1u);
    b &= 0xFFFFE000u;
    std::memcpy(&x, &b, 4);
    return x;
}
inline void split3_host(double x, float& hi, float& lo) {
    hi = tf32_round_host((float)x);
    lo = tf32_round_host((float)(x - (double)hi));
}

template <int P>
inline void fill_tc_ops(const OpsHost& h, TArgs<P>& k) {
    using S = TcShape<P>;
    constexpr int NP = S::NP, NQ = S::NQ, NFQ = S::NFQ;
    fill_nbr_ops<P>(h, k.nb);
    for (int n = 0; n < S::N1; ++n)
        for (int i = 0; i < S::KP; ++i) {
            double x = 0.0;
            if (i < NP) {
                if (n < NQ) x = h.phi[n][i];
                else if (n >= S::NQ4 && n < S::NQ4 + S::FQ) x = h.phif[(n - S::NQ4) / NFQ][(n - S::NQ4) % NFQ][i];
            }
            const int off = tc::canon_off(n, i, S::KP);
            split3_host(x, k.b1[0][off], k.b1[1][off]);
        }
    for (int i = 0; i < S::N2; ++i)
        for (int m = 0; m < S::K2; ++m) {
            double x = 0.0;
            if (i < NP) {
                auto lift = [&](const double* op) {  // (M_ref^-1 op)_i for an operator row over the basis
                    double a = 0.0;
                    for (int kk = 0; kk < NP; ++kk) a += h.minv[i][kk] * op[kk];
                    return a;
                };
                if (m < NQ) x = lift(h.dr[m]);
                else if (m >= S::NQ4 && m < S::NQ4 + NQ) x = lift(h.ds[m - S::NQ4]);
                else if (m >= 2 * S::NQ4 && m < 2 * S::NQ4 + S::FQ)
                    x = lift(h.phif[(m - 2 * S::NQ4) / NFQ][(m - 2 * S::NQ4) % NFQ]);
            }
            const int off = tc::canon_off(i, m, S::K2);
            split3_host(x, k.b2[0][off], k.b2[1][off]);
        }
    for (int q = 0; q < NQ; ++q) k.wq[q] = (float)h.wq[q];
    for (int j = 0; j < NFQ; ++j) k.wf[j] = (float)h.wf[j];
}

template <int P>
inline size_t stage_tc_smem_bytes() {
    const size_t b = (size_t)tc_smem_floats<P>() * sizeof(float);
    // TMEM bounds the CTAs per SM (512 columns: one, 256: two); shared memory enforces it
    const size_t floor = TcShape<P>::COLS == 512 ? 120 * 1024 : 80 * 1024;
    return b < floor ? floor : b;
}

}  // namespace dgx
