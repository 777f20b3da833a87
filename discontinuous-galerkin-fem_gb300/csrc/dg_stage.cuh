// Mixed-precision SSP-RK3 stage kernel.
//
// Same discretisation as the FP64 element kernel (dg_element.cuh): volume flux
// integral, three faces with the Rusanov flux (plus the viscous terms for
// Navier-Stokes), M^-1 and the stage combination, one thread per element.  Here:
//  * arithmetic is FP32 and the stage state is uhi + d (StageArgs, dgx_internal.h);
//  * M_ref^-1 is folded into the lift operators (precomputed in FP64, rounded once);
//  * the volume and face-point loops are fully unrolled, so their operators are
//    immediate constant-bank operands; the loop over the three faces stays rolled (its
//    operators are read by face index), which keeps the code small enough for the
//    instruction cache and the registers within the cap;
//  * a neighbour's face operators depend on which of its faces is shared, a per-thread
//    value; they sit in shared memory as [face][basis][point] rows read as 16-byte
//    vectors.  Lower and upper triangles of a structured mesh share faces in a fixed
//    pattern, so threads are mapped to elements as (even elements, odd elements): the
//    neighbour face is then the same across a warp and the reads are broadcasts;
//  * a neighbour's traces at all face points are formed in one pass over its
//    coefficients, read through L1 (the tile was just loaded) or L2.
#pragma once

#include "dg_element.cuh"
#include "fp_bits.cuh"

namespace dgx {

// Shared-memory row stride (floats) of one element: 16-byte aligned, and stride/4 odd so
// that eight threads reading their rows with 16-byte loads hit disjoint banks.
template <int P>
__host__ __device__ constexpr int stage_stride() {
    return ((n_basis(P) * NV / 4) & 1) ? n_basis(P) * NV : n_basis(P) * NV + 4;
}

template <int P>
struct NbrOps {  // neighbour-face operators, [face][basis][point] with the point axis padded to 4
    static constexpr int NP = n_basis(P), NFQ = P + 1, NFQP = (NFQ + 3) & ~3;
    float phi[3][NP][NFQP];
    float dr[3][NP][NFQP];
    float ds[3][NP][NFQP];
};

template <int P, bool VISC>
struct SArgs {
    StageArgs s;
    Ops<P, float> o;
    LiftOps<P, float> l;
    NbrOps<P> nb;
};

template <int P>
inline void fill_nbr_ops(const OpsHost& h, NbrOps<P>& n) {
    constexpr int NP = n_basis(P), NFQ = P + 1, NFQP = NbrOps<P>::NFQP;
    for (int f = 0; f < 3; ++f)
        for (int i = 0; i < NP; ++i)
            for (int k = 0; k < NFQP; ++k) {
                n.phi[f][i][k] = k < NFQ ? (float)h.phif[f][k][i] : 0.0f;
                n.dr[f][i][k] = k < NFQ ? (float)h.drf[f][k][i] : 0.0f;
                n.ds[f][i][k] = k < NFQ ? (float)h.dsf[f][k][i] : 0.0f;
            }
}

// thread t of a 128-thread CTA works on local element el(t) = 2 (t mod 64) + t / 64;
// local element el lives in shared-memory row row(el) = (el mod 2) * 64 + el / 2 = t.
__device__ __forceinline__ int stage_row(int el) { return (el & 1) * (TILE / 2) + (el >> 1); }
__device__ __forceinline__ int stage_elem(int t) { return 2 * (t & (TILE / 2 - 1)) + t / (TILE / 2); }

// CTAs per SM the register allocation must allow.  Measured on GB300 for p=3 Euler (with
// the face loop unrolled): 4 CTAs (128 registers, 152 B of spills) beat the unconstrained
// 163 registers / 3 CTAs by 9%; with the rolled face loop 4 CTAs spill 12 B.
// DGX_STAGE_MIN_BLOCKS overrides it for experiments.
__host__ __device__ constexpr int stage_min_blocks(int p, bool visc) {
#ifdef DGX_STAGE_MIN_BLOCKS
    return DGX_STAGE_MIN_BLOCKS + 0 * p * visc;
#else
    return visc ? (p <= 2 ? 3 : 2) : (p <= 3 ? 4 : 3);
#endif
}

// acc[0..3] += s * c[0..3] as two packed FP32-pair FMAs (variables (0,1) and (2,3)); the
// same rounding as four fmaf, half the instructions on sm_100-family FP32 pipes.
__device__ __forceinline__ void fma4(float s, const float (&c)[4], float (&acc)[4]) {
    const float2 ss = make_float2(s, s);
    const float2 a = __ffma2_rn(ss, make_float2(c[0], c[1]), make_float2(acc[0], acc[1]));
    const float2 b = __ffma2_rn(ss, make_float2(c[2], c[3]), make_float2(acc[2], acc[3]));
    acc[0] = a.x;
    acc[1] = a.y;
    acc[2] = b.x;
    acc[3] = b.y;
}

// Double-float addition (hi, lo) + d -> (oh, ol), |lo| <= ulp(hi) / 2: Knuth's TwoSum of hi and
// d (exact), the low parts added, and a second TwoSum that renormalises, so oh is the FP32
// rounding of oh + ol and the result is within 2^-48 of the exact sum (relative).  Every
// operation is a rounded FP32 add (never contracted or reassociated).
__device__ __forceinline__ void df_add(float hi, float lo, float d, float& oh, float& ol) {
    const float s = __fadd_rn(hi, d);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(d, bp));
    const float t = __fadd_rn(lo, e);
    oh = __fadd_rn(s, t);
    const float bq = __fsub_rn(oh, s);
    ol = __fadd_rn(__fsub_rn(s, __fsub_rn(oh, bq)), __fsub_rn(t, bq));
}

// entry f of a three-entry array held in registers, for a face index known only at run time
// (indexing the array itself places it, and the whole record, in local memory: 15 local loads
// per element and stage in the face-trace kernel, whose stage went 2.5 % faster with these)
template <class T>
__device__ __forceinline__ T pick3(int f, T a, T b, T c) {
    return f == 0 ? a : (f == 1 ? b : c);
}

__device__ __forceinline__ bool finite_f32(float x) { return (__float_as_uint(x) & 0x7f800000u) != 0x7f800000u; }

// Stage 3 of one value: u^{n+1} = u^n + d.  u^n is un64 (M::in64: the caller's FP64 state, first
// step of a call) or the double-float pair hi + lo; u^{n+1} goes to r64 (M::out64: last step of a
// call; written by the caller) or to the pair (returned hi, lo_out).  A call of one step adds in
// FP64 exactly as before; the steps between the first and the last of a call add on the FP32
// pipe (GB300's FP64 pipe runs at a small fraction of its FP32 rate).  Returns the FP32 rounding
// of u^{n+1}; the conversions run on the integer pipe (fp_bits.cuh).  M says which case: an
// Rk3Mode fixes it at compile time (a loop per case, chosen once per tile by rk3_dispatch: the
// row form's scalar loop ran 4-7 % faster so), Rk3Runtime reads it from s per value (the float4
// combinations: four copies of those loops spill in the face-trace kernel).
template <bool IN64, bool OUT64>
struct Rk3Mode {
    static constexpr bool stage12 = false;
    __device__ static constexpr bool in64(const StageArgs&) { return IN64; }
    __device__ static constexpr bool out64(const StageArgs&) { return OUT64; }
};
struct Rk3Runtime {
    static constexpr bool stage12 = false;
    __device__ static bool in64(const StageArgs& s) { return s.u64_in != 0; }
    __device__ static bool out64(const StageArgs& s) { return s.u64_out != 0; }
};
struct Stage12Mode {  // stages 1 and 2 of stage_combine (no state update)
    static constexpr bool stage12 = true;
    __device__ static constexpr bool in64(const StageArgs&) { return false; }
    __device__ static constexpr bool out64(const StageArgs&) { return false; }
};

template <class M>
__device__ __forceinline__ float rk3_next_m(const StageArgs& s, double un64, float hi, float lo, float d,
                                            float& lo_out, double& r64, bool& bad) {
    if (M::in64(s)) {
        const double r = un64 + f32_to_f64_bits(d);
        const float h = f64_to_f32_bits(r);
        if (M::out64(s)) r64 = r;
        else lo_out = f64_to_f32_bits(r - f32_to_f64_bits(h));  // the difference is exact in FP64
        bad |= !finite_bits(r);
        return h;
    }
    float h, l;
    df_add(hi, lo, d, h, l);
    if (M::out64(s)) r64 = f32_to_f64_bits(h) + f32_to_f64_bits(l);  // exact: l lies below h's last bit
    else lo_out = l;
    bad |= !finite_f32(h);
    return h;
}

// f(Rk3Mode<s.u64_in, s.u64_out>{})
template <class F>
__device__ __forceinline__ void rk3_dispatch(const StageArgs& s, F&& f) {
    if (s.u64_in) {
        if (s.u64_out) f(Rk3Mode<true, true>{});
        else f(Rk3Mode<true, false>{});
    } else {
        if (s.u64_out) f(Rk3Mode<false, true>{});
        else f(Rk3Mode<false, false>{});
    }
}

// rk3_next_m with the case read from s (the tensor-core form's per-value combine)
__device__ __forceinline__ float rk3_next(const StageArgs& s, double un64, float hi, float lo, float d, float& lo_out,
                                          double& r64, bool& bad) {
    return rk3_next_m<Rk3Runtime>(s, un64, hi, lo, d, lo_out, r64, bad);
}

// Stage 3 of four consecutive values at float4 index i4 of the state arrays: reads u^n (u64 or
// the pair, loaded by the caller into un / hi / lo), writes u64 or ulo, and uhi_out; returns the
// FP32 rounding of u^{n+1}.
template <class M>
__device__ __forceinline__ float4 rk3_next4(const StageArgs& s, size_t i4, const double2 (&un)[2], float4 hi,
                                            float4 lo, const float (&d)[4], bool& bad) {
    const double u0[4] = {un[0].x, un[0].y, un[1].x, un[1].y};
    const float h0[4] = {hi.x, hi.y, hi.z, hi.w}, l0[4] = {lo.x, lo.y, lo.z, lo.w};
    float h[4], l[4];
    double r[4];
#pragma unroll
    for (int v = 0; v < 4; ++v) h[v] = rk3_next_m<M>(s, u0[v], h0[v], l0[v], d[v], l[v], r[v], bad);
    if (M::out64(s)) {
        reinterpret_cast<double2*>(s.u64)[2 * i4] = make_double2(r[0], r[1]);
        reinterpret_cast<double2*>(s.u64)[2 * i4 + 1] = make_double2(r[2], r[3]);
    } else {
        reinterpret_cast<float4*>(s.ulo)[i4] = make_float4(l[0], l[1], l[2], l[3]);
    }
    const float4 o = make_float4(h[0], h[1], h[2], h[3]);
    reinterpret_cast<float4*>(s.uhi_out)[i4] = o;
    return o;
}

// The stage-3 inputs of four values at float4 index i4: u64 (M::in64) or the pair uhi + ulo.
template <class M>
__device__ __forceinline__ void rk3_load4(const StageArgs& s, size_t i4, double2 (&un)[2], float4& hi, float4& lo) {
    if (M::in64(s)) {
        un[0] = reinterpret_cast<const double2*>(s.u64)[2 * i4];
        un[1] = reinterpret_cast<const double2*>(s.u64)[2 * i4 + 1];
    } else {
        hi = __ldg(reinterpret_cast<const float4*>(s.uhi) + i4);
        lo = reinterpret_cast<const float4*>(s.ulo)[i4];
    }
}

// rk3_load4 / rk3_next4 with the case read from s (the float4 stage combinations)
__device__ __forceinline__ void rk3_load4(const StageArgs& s, size_t i4, double2 (&un)[2], float4& hi, float4& lo) {
    rk3_load4<Rk3Runtime>(s, i4, un, hi, lo);
}
__device__ __forceinline__ float4 rk3_next4(const StageArgs& s, size_t i4, const double2 (&un)[2], float4 hi, float4 lo,
                                            const float (&d)[4], bool& bad) {
    return rk3_next4<Rk3Runtime>(s, i4, un, hi, lo, d, bad);
}

// Stage combination of one tile in the increment form, 16-byte accesses:
//   stage 1: dout = dt R;  stage 2: dout = (din + dt R) / 4;
//   stage 3: u^{n+1} = u^n + 2/3 (din + dt R) (rk3_next), uhi_out = its FP32 rounding.
// R (M^-1-scaled residual) of local element le is row rowof(le) of sR; the loads of CH
// consecutive float4 slots of a thread are issued before any of them is used.
template <int NB, int STR, int THREADS, int CH, typename RowOf>
__device__ __forceinline__ void stage_combine(const StageArgs& s, const float* sR, const float* sDt, int e0,
                                              int nloc, RowOf rowof) {
    constexpr int NB4 = NB / 4;
    const int n4 = nloc * NB4;
    const size_t b4 = (size_t)e0 * NB4;
    const int t = threadIdx.x;
    bool bad = false;
    for (int g0 = t; g0 < n4; g0 += CH * THREADS) {
        float4 dv[CH], hi[CH], lo[CH];
        double2 un[CH][2];
#pragma unroll
        for (int k = 0; k < CH; ++k) {
            const int g = g0 + k * THREADS;
            if (g < n4) {
                if (s.stage >= 2) dv[k] = __ldg(reinterpret_cast<const float4*>(s.din) + b4 + g);
                if (s.stage == 3) rk3_load4(s, b4 + g, un[k], hi[k], lo[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < CH; ++k) {
            const int g = g0 + k * THREADS;
            if (g >= n4) break;
            const int le = g / NB4, c = 4 * (g - le * NB4);
            const int row = rowof(le);
            const float4 du = *reinterpret_cast<const float4*>(sR + row * STR + c);
            const float dt = s.dt_inst ? sDt[row] : s.dt;
            if (s.stage == 1) {
                reinterpret_cast<float4*>(s.dout)[b4 + g] = make_float4(dt * du.x, dt * du.y, dt * du.z, dt * du.w);
            } else if (s.stage == 2) {
                reinterpret_cast<float4*>(s.dout)[b4 + g] =
                    make_float4(0.25f * (dv[k].x + dt * du.x), 0.25f * (dv[k].y + dt * du.y),
                                0.25f * (dv[k].z + dt * du.z), 0.25f * (dv[k].w + dt * du.w));
            } else {
                const float d[4] = {(2.0f / 3.0f) * (dv[k].x + dt * du.x), (2.0f / 3.0f) * (dv[k].y + dt * du.y),
                                    (2.0f / 3.0f) * (dv[k].z + dt * du.z), (2.0f / 3.0f) * (dv[k].w + dt * du.w)};
                rk3_next4(s, b4 + g, un[k], hi[k], lo[k], d, bad);
            }
        }
    }
    if (bad && s.status) atomicOr(s.status, 1);
}

// hint: bring [p, p + bytes) into L2 (bulk async prefetch; 16-byte aligned, bytes % 16 == 0)
__device__ __forceinline__ void prefetch_l2_bulk(const void* p, unsigned bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(p), "r"(bytes) : "memory");
}

// hint for stage 3: bring the tile's u^n (u64, or the low parts ulo) into L2
__device__ __forceinline__ void rk3_prefetch(const StageArgs& s, size_t v0, int nvals) {
    if (s.u64_in) prefetch_l2_bulk(s.u64 + v0, (unsigned)(nvals * sizeof(double)));
    else prefetch_l2_bulk(s.ulo + v0, (unsigned)(nvals * sizeof(float)));
}

// hint: bring the 128-byte line holding p into L2
__device__ __forceinline__ void prefetch_l2_line(const void* p) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// The stage state uhi + din of the tile starting at element e0 into shared memory, element
// le's row at row_of(le) * STR, by the T threads of a CTA of T-element tiles.  In a full tile a
// thread issues all of its 16-byte loads before it uses the first, so the tile costs one memory
// round trip instead of one per pass.
template <int NB, int STR, int T = TILE, typename RowOf>
__device__ __forceinline__ void stage_load_tile(const float* uhi, const float* din, float* sU, int e0, int nloc,
                                                RowOf row_of) {
    constexpr int NB4 = NB / 4;
    const int tl = threadIdx.x;
    const float4* uh = reinterpret_cast<const float4*>(uhi + (size_t)e0 * NB);
    const float4* dd = din ? reinterpret_cast<const float4*>(din + (size_t)e0 * NB) : nullptr;
    auto put = [&](int g, const float4& a) {
        const int le = g / NB4, k = 4 * (g - le * NB4);
        *reinterpret_cast<float4*>(sU + row_of(le) * STR + k) = a;
    };
    if (nloc == T) {
        float4 a[NB4];
        if (dd) {
            float4 b[NB4];
#pragma unroll
            for (int r = 0; r < NB4; ++r) {
                a[r] = __ldg(uh + tl + r * T);
                b[r] = __ldg(dd + tl + r * T);
            }
#pragma unroll
            for (int r = 0; r < NB4; ++r) {
                a[r].x += b[r].x; a[r].y += b[r].y; a[r].z += b[r].z; a[r].w += b[r].w;
            }
        } else {
#pragma unroll
            for (int r = 0; r < NB4; ++r) a[r] = __ldg(uh + tl + r * T);
        }
#pragma unroll
        for (int r = 0; r < NB4; ++r) put(tl + r * T, a[r]);
        return;
    }
    for (int g = tl; g < nloc * NB4; g += T) {
        float4 a = __ldg(uh + g);
        if (dd) {
            const float4 b = __ldg(dd + g);
            a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w;
        }
        put(g, a);
    }
}

// Floats of shared memory the neighbour-face operators take (16-byte rows).
template <int P, bool VISC>
__host__ __device__ constexpr int stage_op_floats() {
    return (VISC ? 3 : 1) * 3 * n_basis(P) * NbrOps<P>::NFQP;
}

// One tile of TILE elements: stage it, compute the element residuals, write the stage.
// sOp: the neighbour-face operators; sU: [TILE][stride] floats; sDt: [TILE] floats.
template <int P, bool VISC, bool BND>
__device__ __forceinline__ void stage_tile(const SArgs<P, VISC>& ka, const float* sOp, float* sU, float* sDt,
                                           int tile) {
    constexpr int NP = n_basis(P), NQ = n_quad(P), NFQ = P + 1, NB = NP * NV, STR = stage_stride<P>();
    constexpr int NFQP = NbrOps<P>::NFQP;
    const StageArgs& s = ka.s;
    const Ops<P, float>& o = ka.o;
    const LiftOps<P, float>& L = ka.l;

    const int e0 = tile * TILE;
    const int nloc = min(TILE, s.ne - e0);
    const int tl = threadIdx.x;
    const int el = stage_elem(tl);
    const bool active = el < nloc;
    const int e = e0 + el;
    if (tl == 0 && s.stage == 3)  // u^n is read back in the stage combination
        rk3_prefetch(s, (size_t)e0 * NB, nloc * NB);
    stage_load_tile<NB, STR>(s.uhi, s.din, sU, e0, nloc, [](int le) { return stage_row(le); });
    __syncthreads();

    float R[NP][NV];
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
        for (int v = 0; v < NV; ++v) R[i][v] = 0.0f;

    if (active) {
        const ElemGeomF G = s.geom[e];
        const float A00 = G.A[0], A01 = G.A[1], A10 = G.A[2], A11 = G.A[3];
        const float gamma = s.gamma, mu = s.mu, kappa = s.kappa;
        const float* Ue = sU + tl * STR;
        if (s.dt_inst) sDt[tl] = s.dt_inst[__float_as_int(G.pad)];  // batched: per-instance dt

        // ---------------- volume (EulerWeakFormulation::volume_residual :72-115,
        //                  NavierStokesWeakFormulation::viscous_volume_residual :100-140)
        // Navier-Stokes: two points per pass (fully unrolled, the viscous kernel's code outgrows the
        // instruction cache: 0.89 no-instruction stalls per issue at p=4; unrolled by 2 the step went
        // 0.490 -> 0.461 ms at 256x256x2, by 1 or 4 0.470 and 0.475)
#pragma unroll (VISC ? 2 : NQ)
        for (int q = 0; q < NQ; ++q) {
            float U[4] = {0.f, 0.f, 0.f, 0.f};
            float gr[4] = {0.f, 0.f, 0.f, 0.f}, gs[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                const float4 c4 = *reinterpret_cast<const float4*>(Ue + i * NV);
                const float c[4] = {c4.x, c4.y, c4.z, c4.w};
                fma4(o.phi[q][i], c, U);
                if (VISC) {
                    fma4(o.dr[q][i], c, gr);
                    fma4(o.ds[q][i], c, gs);
                }
            }
            float F[4], Gf[4], u, vv, pp, ri;
            euler_flux<float>(U, gamma - 1.0f, F, Gf, u, vv, pp, ri);
            if (VISC) {
                float gx[4], gy[4], Fv[4], Gv[4];
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    gx[v] = A00 * gr[v] + A01 * gs[v];
                    gy[v] = A10 * gr[v] + A11 * gs[v];
                }
                viscous_flux<float>(U, gx, gy, gamma, mu, kappa, Fv, Gv);
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    F[v] -= Fv[v];
                    Gf[v] -= Gv[v];
                }
            }
            float Fr[4], Fs[4];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                Fr[v] = o.wq[q] * (A00 * F[v] + A10 * Gf[v]);
                Fs[v] = o.wq[q] * (A01 * F[v] + A11 * Gf[v]);
            }
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                fma4(L.pr[q][i], Fr, R[i]);
                fma4(L.ps[q][i], Fs, R[i]);
            }
        }

        // ---------------- faces (interior_face_residual :117-175, boundary_face_residual
        //                  :177-250 and the viscous counterparts, NS :142-273)
        const ElemConn C = s.conn[e];
        const float inv_j = __frcp_rn(G.detJ);
        // one face body, walked three times: unrolled, the code missed the instruction cache and
        // spilled at the register cap (Euler p=3 0.646 -> 0.594 ms/step, NS p=4 0.676 -> 0.521)
#pragma unroll 1
        for (int f = 0; f < 3; ++f) {
            const int nb = C.nbr[f];
            if (BND && nb == NBR_SKIP) continue;
            const int fl = (C.flags >> (4 * f)) & 15;
            const int nf = fl & 3;
            const bool rev = (fl >> 2) & 1;
            const float sideL = ((fl >> 3) & 1) ? 1.0f : -1.0f;
            // indexed by the runtime face: the record goes to local memory (register selects, which
            // the face-trace kernel uses, measured 3 % slower here: they add register pressure)
            const float nx = G.n[f][0], ny = G.n[f][1], hF = G.h[f];
            // neighbour traces at its own points k, then reordered to this face's points
            float Un[NFQ][4], Nr[VISC ? NFQ : 1][4], Ns[VISC ? NFQ : 1][4];
#pragma unroll
            for (int k = 0; k < NFQ; ++k)
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    Un[k][v] = 0.f;
                    if (VISC) { Nr[k][v] = 0.f; Ns[k][v] = 0.f; }
                }
            BCSlot bc;
            bc.type = -1;
            float B00 = 0.f, B01 = 0.f, B10 = 0.f, B11 = 0.f;
            if (!BND || nb >= 0) {
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
                    if (VISC) {
                        const float* opr = op + 3 * NP * NFQP;
                        const float* ops = op + 6 * NP * NFQP;
#pragma unroll
                        for (int k4 = 0; k4 < NFQP; k4 += 4) {
                            const float4 t = *reinterpret_cast<const float4*>(opr + i * NFQP + k4);
                            w[k4] = t.x; w[k4 + 1] = t.y; w[k4 + 2] = t.z; w[k4 + 3] = t.w;
                        }
#pragma unroll
                        for (int k = 0; k < NFQ; ++k) fma4(w[k], c, Nr[k]);
#pragma unroll
                        for (int k4 = 0; k4 < NFQP; k4 += 4) {
                            const float4 t = *reinterpret_cast<const float4*>(ops + i * NFQP + k4);
                            w[k4] = t.x; w[k4 + 1] = t.y; w[k4 + 2] = t.z; w[k4 + 3] = t.w;
                        }
#pragma unroll
                        for (int k = 0; k < NFQ; ++k) fma4(w[k], c, Ns[k]);
                    }
                }
#pragma unroll
                for (int j = 0; j < NFQ / 2; ++j)
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        const float a = Un[j][v], b = Un[NFQ - 1 - j][v];
                        Un[j][v] = rev ? b : a;
                        Un[NFQ - 1 - j][v] = rev ? a : b;
                        if (VISC) {
                            const float c = Nr[j][v], d = Nr[NFQ - 1 - j][v];
                            Nr[j][v] = rev ? d : c;
                            Nr[NFQ - 1 - j][v] = rev ? c : d;
                            const float x = Ns[j][v], y = Ns[NFQ - 1 - j][v];
                            Ns[j][v] = rev ? y : x;
                            Ns[NFQ - 1 - j][v] = rev ? x : y;
                        }
                    }
                if (VISC) {
                    const ElemGeomF& GN = s.geom[nb];
                    B00 = GN.A[0]; B01 = GN.A[1]; B10 = GN.A[2]; B11 = GN.A[3];
                }
            } else {
                bc = s.bc[-1 - nb];
            }
            const float sigma = VISC ? s.sigma0 * mu * float((P + 1) * (P + 1)) / fmaxf(hF, 1e-12f) : 0.f;
#pragma unroll
            for (int j = 0; j < NFQ; ++j) {
                float Uo[4] = {0.f, 0.f, 0.f, 0.f};
                float gr[4] = {0.f, 0.f, 0.f, 0.f}, gs[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
                for (int i = 0; i < NP; ++i) {
                    const float4 c4 = *reinterpret_cast<const float4*>(Ue + i * NV);
                    const float c[4] = {c4.x, c4.y, c4.z, c4.w};
                    fma4(o.phif[f][j][i], c, Uo);
                    if (VISC) {
                        fma4(o.drf[f][j][i], c, gr);
                        fma4(o.dsf[f][j][i], c, gs);
                    }
                }
                float H[4];
                if (!BND || nb >= 0) {
                    rusanov<float>(Uo, Un[j], nx, ny, gamma, H);
                } else {
                    float Ub[4];
                    if (inviscid_ghost<float>(bc, Uo, nx, ny, gamma, Ub)) {
                        rusanov<float>(Uo, Ub, nx, ny, gamma, H);
                    } else {
#pragma unroll
                        for (int v = 0; v < 4; ++v) H[v] = 0.f;
                    }
                }
                if (VISC) {
                    float gx[4], gy[4], Fv[4], Gv[4];
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        gx[v] = A00 * gr[v] + A01 * gs[v];
                        gy[v] = A10 * gr[v] + A11 * gs[v];
                    }
                    viscous_flux<float>(Uo, gx, gy, gamma, mu, kappa, Fv, Gv);
                    if (!BND || nb >= 0) {
                        float hx[4], hy[4], Fn2[4], Gn2[4];
#pragma unroll
                        for (int v = 0; v < NV; ++v) {
                            hx[v] = B00 * Nr[j][v] + B01 * Ns[j][v];
                            hy[v] = B10 * Nr[j][v] + B11 * Ns[j][v];
                        }
                        viscous_flux<float>(Un[j], hx, hy, gamma, mu, kappa, Fn2, Gn2);
#pragma unroll
                        for (int v = 0; v < NV; ++v) {
                            const float jmp = 0.5f * ((Fv[v] * nx + Gv[v] * ny) - (Fn2[v] * nx + Gn2[v] * ny));
                            H[v] += sideL * jmp - sigma * (Un[j][v] - Uo[v]);
                        }
                    } else if (bc.type >= 0) {
                        float Ub[4];
                        viscous_ghost<float>(bc, gamma, Ub);
#pragma unroll
                        for (int v = 0; v < NV; ++v) H[v] += (Fv[v] * nx + Gv[v] * ny) - sigma * (Ub[v] - Uo[v]);
                    }
                }
                const float w = o.wf[j] * hF * 0.5f * inv_j;
#pragma unroll
                for (int i = 0; i < NP; ++i) fma4(-(w * L.pf[f][j][i]), H, R[i]);
            }
        }
    }
    __syncthreads();  // every neighbour read of sU is done
    if (active) {
#pragma unroll
        for (int i = 0; i < NP; ++i)
            *reinterpret_cast<float4*>(sU + tl * STR + i * NV) = make_float4(R[i][0], R[i][1], R[i][2], R[i][3]);
    }
    __syncthreads();
    // stage combination, one value per pass (the float4 form of stage_combine spills here); the
    // stage-3 variants (rk3_next's four cases) each get their own loop
    const size_t base = (size_t)e0 * NB;
    bool bad = false;
    auto du_of = [&](int g, float& du, float& dt) {
        const int le = g / NB;
        du = sU[stage_row(le) * STR + (g - le * NB)];
        dt = s.dt_inst ? sDt[stage_row(le)] : s.dt;
    };
    if (s.stage <= 2) {
        for (int g = tl; g < nloc * NB; g += TILE) {
            float du, dt;
            du_of(g, du, dt);
            s.dout[base + g] = s.stage == 1 ? dt * du : 0.25f * (__ldg(s.din + base + g) + dt * du);
        }
    } else {
        rk3_dispatch(s, [&](auto m) {
            using M = decltype(m);
            for (int g = tl; g < nloc * NB; g += TILE) {
                float du, dt;
                du_of(g, du, dt);
                const size_t i = base + g;
                const float d = (2.0f / 3.0f) * (__ldg(s.din + i) + dt * du);
                float l = 0.0f;
                double r = 0.0;
                const float h = M::in64(s) ? rk3_next_m<M>(s, s.u64[i], 0.0f, 0.0f, d, l, r, bad)
                                           : rk3_next_m<M>(s, 0.0, __ldg(s.uhi + i), s.ulo[i], d, l, r, bad);
                if (M::out64(s)) s.u64[i] = r;
                else s.ulo[i] = l;
                s.uhi_out[i] = h;
            }
        });
    }
    if (bad && s.status) atomicOr(s.status, 1);
    __syncthreads();  // the next tile reuses sU / sDt
}

// Persistent stage kernel: each CTA loads the neighbour-face operators once, then walks
// the tiles with a grid stride.  The grid size is picked by the autotuner.
template <int P, bool VISC, bool BND>
__global__ void __launch_bounds__(TILE, stage_min_blocks(P, VISC)) stage_kernel(const __grid_constant__ SArgs<P, VISC> ka) {
    constexpr int OPF = stage_op_floats<P, VISC>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sOp = reinterpret_cast<float*>(smem_raw);
    float* sDt = sOp + OPF;
    float* sU = sDt + TILE;
    {
        const float* src = &ka.nb.phi[0][0][0];
        for (int k = threadIdx.x; k < OPF; k += TILE) sOp[k] = src[k];
    }
    __syncthreads();
    const int ntiles = ka.s.ntile > 0 ? ka.s.ntile : (ka.s.ne + TILE - 1) / TILE;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) stage_tile<P, VISC, BND>(ka, sOp, sU, sDt, ka.s.tile0 + t);
}

template <int P, bool VISC>
inline size_t stage_smem_bytes() {
    return (size_t)(stage_op_floats<P, VISC>() + TILE + TILE * stage_stride<P>()) * sizeof(float);
}

template <int P, typename T, bool VISC>
inline int configure_stage_t() {
    const int b = (int)stage_smem_bytes<P, VISC>();
    return cudaFuncSetAttribute(stage_kernel<P, VISC, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ==
                       cudaSuccess &&
                   cudaFuncSetAttribute(stage_kernel<P, VISC, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        b) == cudaSuccess
               ? 0
               : -1;
}

template <int P, typename T, bool VISC>
inline int launch_stage_t(const StageArgs& a, const OpsHost& oh, cudaStream_t st) {
    SArgs<P, VISC> ka;
    ka.s = a;
    fill_ops<P, float>(oh, ka.o);
    fill_lift<P, float>(oh, ka.l);
    fill_nbr_ops<P>(oh, ka.nb);
    const int ntiles = a.ntile > 0 ? a.ntile : (a.ne + TILE - 1) / TILE;
    if (ntiles == 0) return 0;
    const int grid = a.grid > 0 && a.grid < ntiles ? a.grid : ntiles;
    if (a.boundary)
        stage_kernel<P, VISC, true><<<grid, TILE, stage_smem_bytes<P, VISC>(), st>>>(ka);
    else
        stage_kernel<P, VISC, false><<<grid, TILE, stage_smem_bytes<P, VISC>(), st>>>(ka);
    return launch_status();
}

}  // namespace dgx
