// Mixed-precision SSP-RK3 Euler stage with face traces exchanged through HBM.
//
// The stage kernel of dg_stage.cuh forms a neighbour's trace on the shared face itself: it
// reads the neighbour's Np coefficient rows of uhi and of the increment (2 Np 16-byte loads
// per face) and contracts them with the neighbour-face operators, so every face trace is
// formed twice per stage (once by each side) and the kernel waits on long chains of
// neighbour-row loads.  Here each element writes, at the end of a stage, the traces of its
// next stage state at the points of its three faces:
//   tr[e][f][j][v], face f, point j (the face's own order), variable v  (3 (p+1) 4 floats),
// and the next stage reads its neighbour's block (16 (p+1) contiguous bytes per face) instead
// of the neighbour's coefficient rows; its own traces it still forms from its staged
// coefficients (measured faster than reading them back).  Every trace is formed with the
// operators and the operation order of the face loop of dg_stage.cuh, so the two forms give
// the same numbers bit for bit.  The traces of the state a step starts from are written by
// trace_init_kernel; stage 3 writes those of the next step's start state (the FP32 copy of
// u^{n+1}), so the two ping-pong buffers carry the traces from stage to stage and step to step.
// On a mesh whose boundary faces all have a condition, the buffers hold one ghost block per
// boundary face after the elements' blocks; the owner fills it with the ghost states of its
// traces and the face loop reads it like a neighbour's block (GHOST kernels, no boundary
// branch).  Meshes with faces that take no part keep the boundary branch (BND kernels).
#pragma once

#include <type_traits>

#include "dg_stage.cuh"
#include "tc_ptx.cuh"

namespace dgx {

// Which stages a trace-kernel instantiation serves: any (the stage and, for stage 3, the state's
// case read from StageArgs), stages 1 and 2 (the stage read from StageArgs), stage 1 or stage 2
// alone, or stage 3 of a step between the first and the last of a call (double-float state in
// and out).  The specialised kernels leave out the code of the other stages, which the
// instruction cache then does not have to hold.
enum StageKind { SK_ANY = 0, SK_12 = 1, SK_3DF = 2, SK_1 = 3, SK_2 = 4 };

template <int P>
__host__ __device__ constexpr int trace_floats() { return 3 * (P + 1) * NV; }

// stage_combine (dg_stage.cuh), which in addition replaces each residual slot of sR with the
// next stage state: uhi + dout after stages 1 and 2 (what the next stage stages as uhi + din),
// the FP32 copy of u^{n+1} after stage 3.  SK: the stages served (StageKind).
template <int NB, int STR, int THREADS, int CH, int SK = SK_ANY, typename RowOf>
__device__ __forceinline__ void stage_combine_next(const StageArgs& s, float* sR, const float* sDt, int e0, int nloc,
                                                   RowOf rowof) {
    using M = typename std::conditional<SK == SK_3DF, Rk3Mode<false, false>, Rk3Runtime>::type;
    constexpr int NB4 = NB / 4;
    const int n4 = nloc * NB4;
    const size_t b4 = (size_t)e0 * NB4;
    const int t = threadIdx.x;
    const int stage = SK == SK_1 ? 1 : SK == SK_2 ? 2 : SK == SK_3DF ? 3 : s.stage;
    const bool st12 = SK == SK_12 || SK == SK_1 || SK == SK_2 || (SK == SK_ANY && stage <= 2);
    const bool with_din = SK == SK_3DF || SK == SK_2 || (SK != SK_1 && stage >= 2);
    bool bad = false;
    for (int g0 = t; g0 < n4; g0 += CH * THREADS) {
        float4 dv[CH], uh[CH], lo[CH];
        double2 un[CH][2];
#pragma unroll
        for (int k = 0; k < CH; ++k) {
            const int g = g0 + k * THREADS;
            if (g < n4) {
                if (with_din) dv[k] = __ldg(reinterpret_cast<const float4*>(s.din) + b4 + g);
                if (st12) uh[k] = __ldg(reinterpret_cast<const float4*>(s.uhi) + b4 + g);
                else rk3_load4<M>(s, b4 + g, un[k], uh[k], lo[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < CH; ++k) {
            const int g = g0 + k * THREADS;
            if (g >= n4) break;
            const int le = g / NB4, c = 4 * (g - le * NB4);
            const int row = rowof(le);
            float4* slot = reinterpret_cast<float4*>(sR + row * STR + c);
            const float4 du = *slot;
            const float dt = s.dt_inst ? sDt[row] : s.dt;
            if (st12) {
                const float4 o = stage == 1
                                     ? make_float4(dt * du.x, dt * du.y, dt * du.z, dt * du.w)
                                     : make_float4(0.25f * (dv[k].x + dt * du.x), 0.25f * (dv[k].y + dt * du.y),
                                                   0.25f * (dv[k].z + dt * du.z), 0.25f * (dv[k].w + dt * du.w));
                reinterpret_cast<float4*>(s.dout)[b4 + g] = o;
                // rounded add, never contracted with the product above: exactly uhi + din as staged
                *slot = make_float4(__fadd_rn(uh[k].x, o.x), __fadd_rn(uh[k].y, o.y), __fadd_rn(uh[k].z, o.z),
                                    __fadd_rn(uh[k].w, o.w));
            } else {
                const float d[4] = {(2.0f / 3.0f) * (dv[k].x + dt * du.x), (2.0f / 3.0f) * (dv[k].y + dt * du.y),
                                    (2.0f / 3.0f) * (dv[k].z + dt * du.z), (2.0f / 3.0f) * (dv[k].w + dt * du.w)};
                *slot = rk3_next4<M>(s, b4 + g, un[k], uh[k], lo[k], d, bad);
            }
        }
    }
    if (bad && s.status) atomicOr(s.status, 1);
}

// traces of the coefficient row block `c` (shared memory, rows NV floats apart) of element e
// on the three faces, written to tr (global, trace_floats<P>() floats)
// (one pass over the rows; each trace point still sums i = 0 .. Np-1 in order).  With ghost
// blocks (s.ghost_bc set, s.conn the trace-form connectivity) a boundary face's block gets the
// ghost state of each trace point (boundary_face_residual's, from the same trace value and
// the same operations as the boundary path of the face loop), so the next stage treats the
// face as an interior one.  GHOST = false leaves the ghost code out.
// ROLL: one face per pass (the 32-element-tile kernels, whose warps each run their own phase and
// so share less code in the instruction cache: unrolled over the faces they measured 2.4 %
// slower); otherwise all faces' points in one pass over the coefficients.  Each point sums
// i = 0 .. Np-1 in order either way.
template <int P, bool GHOST, bool ROLL = false>
__device__ __forceinline__ void write_traces(const Ops<P, float>& o, const float* c, float* tr, const StageArgs& s,
                                             int e) {
    constexpr int NP = n_basis(P), NFQ = P + 1;
    // ghost block nb of boundary face f from the face's trace values U
    auto ghost = [&](int f, int nb, const float (&U)[NFQ][4]) {
        const BCSlot bc = s.bc[s.ghost_bc[nb - s.ne]];
        const float nx = s.geom[e].n[f][0], ny = s.geom[e].n[f][1];
        float* g = s.tout + (size_t)nb * trace_floats<P>();
#pragma unroll
        for (int j = 0; j < NFQ; ++j) {
            float Ub[4];
            inviscid_ghost<float>(bc, U[j], nx, ny, s.gamma, Ub);
            *reinterpret_cast<float4*>(g + j * NV) = make_float4(Ub[0], Ub[1], Ub[2], Ub[3]);
        }
    };
    if constexpr (ROLL) {
        ElemConn C;
        if (GHOST && s.ghost_bc) C = s.conn[e];
#pragma unroll 1
        for (int f = 0; f < 3; ++f) {
            float U[NFQ][4];
#pragma unroll
            for (int j = 0; j < NFQ; ++j)
#pragma unroll
                for (int v = 0; v < NV; ++v) U[j][v] = 0.0f;
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                const float4 c4 = *reinterpret_cast<const float4*>(c + i * NV);
                const float cc[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
                for (int j = 0; j < NFQ; ++j) fma4(o.phif[f][j][i], cc, U[j]);
            }
#pragma unroll
            for (int j = 0; j < NFQ; ++j)
                *reinterpret_cast<float4*>(tr + (f * NFQ + j) * NV) = make_float4(U[j][0], U[j][1], U[j][2], U[j][3]);
            if (GHOST && s.ghost_bc) {
                const int nb = pick3(f, C.nbr[0], C.nbr[1], C.nbr[2]);
                if (nb >= s.ne) ghost(f, nb, U);
            }
        }
    } else {
        float U[3][NFQ][4];
#pragma unroll
        for (int f = 0; f < 3; ++f)
#pragma unroll
            for (int j = 0; j < NFQ; ++j)
#pragma unroll
                for (int v = 0; v < NV; ++v) U[f][j][v] = 0.0f;
#pragma unroll
        for (int i = 0; i < NP; ++i) {
            const float4 c4 = *reinterpret_cast<const float4*>(c + i * NV);
            const float cc[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
            for (int f = 0; f < 3; ++f)
#pragma unroll
                for (int j = 0; j < NFQ; ++j) fma4(o.phif[f][j][i], cc, U[f][j]);
        }
#pragma unroll
        for (int f = 0; f < 3; ++f)
#pragma unroll
            for (int j = 0; j < NFQ; ++j)
                *reinterpret_cast<float4*>(tr + (f * NFQ + j) * NV) = make_float4(U[f][j][0], U[f][j][1], U[f][j][2],
                                                                                  U[f][j][3]);
        if (GHOST && s.ghost_bc) {
            const ElemConn C = s.conn[e];
#pragma unroll
            for (int f = 0; f < 3; ++f)
                if (C.nbr[f] >= s.ne) ghost(f, C.nbr[f], U[f]);
        }
    }
}

// the neighbours' trace blocks of element e (64-byte aligned, one line each) into L2, while the
// volume terms are formed
template <int P, bool BND>
__device__ __forceinline__ void prefetch_neighbour_traces(const StageArgs& s, const ElemConn& C) {
    constexpr int NFQ = P + 1, TRF = trace_floats<P>();
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        const int nb = C.nbr[f];
        if (BND && nb < 0) continue;
        prefetch_l2_line(s.tin + (size_t)nb * TRF + ((C.flags >> (4 * f)) & 3) * NFQ * NV);
    }
}

// Thread t of a CTA of T-element tiles works on local element tile_elem<T>(t): the even elements
// (lower triangles of a structured mesh) on threads 0 .. T/2-1, the odd ones on the rest, so the
// threads of a warp read their face records in one pattern; the element's row in shared memory
// is tile_row<T>(tile_elem<T>(t)) = t.  For T = TILE these are stage_elem / stage_row.
template <int T>
__device__ __forceinline__ int tile_row(int el) { return (el & 1) * (T / 2) + (el >> 1); }
template <int T>
__device__ __forceinline__ int tile_elem(int t) { return 2 * (t & (T / 2 - 1)) + t / (T / 2); }

// Shared-memory row stride (floats) of an element's three neighbour trace blocks: 16-byte
// aligned, stride/4 odd (eight threads' 16-byte reads of their rows hit disjoint banks).
template <int P>
__host__ __device__ constexpr int nbr_trace_stride() {
    return ((trace_floats<P>() / 4) & 1) ? trace_floats<P>() : trace_floats<P>() + 4;
}

// 16-byte asynchronous copy global -> shared memory through L2 only (cp.async.cg: L1 is left to
// the stage combination's re-reads of the tile; caching the blocks in L1 too, .ca, measured
// 1.5 % slower), and the wait for all of this thread's copies
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// the neighbours' trace blocks of element e (every face interior or a ghost face) into the
// thread's row dst of shared memory, slot f holding the block the face loop reads for face f;
// the copies land while the volume terms are formed
template <int P>
__device__ __forceinline__ void copy_neighbour_traces(const StageArgs& s, const ElemConn& C, float* dst) {
    constexpr int NFQ = P + 1, TRF = trace_floats<P>();
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        const float* src = s.tin + (size_t)C.nbr[f] * TRF + ((C.flags >> (4 * f)) & 3) * NFQ * NV;
#pragma unroll
        for (int k = 0; k < NFQ; ++k) cp_async16(dst + (f * NFQ + k) * NV, src + k * NV);
    }
}

// One tile: `stage(G, C)` puts the stage state's rows into sU and the element's geometry and
// connectivity into G and C (the boundary variant reads G itself, after staging, short of
// registers) and ends with a barrier; then the residual, the stage combination and the next
// traces.  NBS: the neighbours' trace blocks were copied into the thread's row of sN by
// cp.async during staging (no boundary branch), and the face loop reads them there.
template <int P, bool BND, bool GHOST, int T, bool NBS = false, int SK = SK_ANY, class Stage>
__device__ __forceinline__ void stage_trace_tile_with(const SArgs<P, false>& ka, float* sU, float* sDt, int tile,
                                                      Stage&& stage, const float* sN = nullptr) {
    static_assert(!(NBS && BND), "neighbour traces in shared memory need every face interior or a ghost face");
    constexpr int NP = n_basis(P), NQ = n_quad(P), NFQ = P + 1, NB = NP * NV, STR = stage_stride<P>();
    constexpr int TRF = trace_floats<P>();
    const StageArgs& s = ka.s;
    const Ops<P, float>& o = ka.o;
    const LiftOps<P, float>& L = ka.l;

    const int e0 = tile * T;
    const int nloc = min(T, s.ne - e0);
    const int tl = threadIdx.x;
    const int el = tile_elem<T>(tl);
    const bool active = el < nloc;
    const int e = e0 + el;
    ElemGeomF G;
    ElemConn C;
    stage(G, C);

    float R[NP][NV];
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
        for (int v = 0; v < NV; ++v) R[i][v] = 0.0f;

    if (active) {
        if (BND) G = s.geom[e];
        const float A00 = G.A[0], A01 = G.A[1], A10 = G.A[2], A11 = G.A[3];
        const float gamma = s.gamma;
        const float* Ue = sU + tl * STR;
        if (s.dt_inst) sDt[tl] = s.dt_inst[__float_as_int(G.pad)];

        // ---------------- volume (EulerWeakFormulation::volume_residual :72-115)
        auto volume_point = [&](int q) {
            float U[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                const float4 c4 = *reinterpret_cast<const float4*>(Ue + i * NV);
                const float c[4] = {c4.x, c4.y, c4.z, c4.w};
                fma4(o.phi[q][i], c, U);
            }
            float F[4], Gf[4], u, vv, pp, ri;
            euler_flux<float>(U, gamma - 1.0f, F, Gf, u, vv, pp, ri);
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
        };
        if constexpr (T <= 32) {
            // three points per pass (fully unrolled, the code outgrew the instruction cache:
            // 0.406 -> 0.374 ms/step at 512x512x2 p=3 unrolled by 3, 0.373 by 2, 0.384 by 6)
#pragma unroll 3
            for (int q = 0; q < NQ; ++q) volume_point(q);
        } else {
            // fully unrolled (128-element tiles, whose four warps run one phase together, measured
            // 3.6 % slower rolled by 3)
#pragma unroll
            for (int q = 0; q < NQ; ++q) volume_point(q);
        }

        // ---------------- faces (interior_face_residual :117-175, boundary_face_residual :177-250)
        const float inv_j = __frcp_rn(G.detJ);
        if (NBS) cp_async_wait_all();  // this thread's copies of its neighbours' blocks
        // one face body, walked three times (the unrolled form measured 2.7 % slower: its
        // larger code missed the instruction cache and its registers spilled)
#pragma unroll 1
        for (int f = 0; f < 3; ++f) {
            const int nb = pick3(f, C.nbr[0], C.nbr[1], C.nbr[2]);
            if (BND && nb == NBR_SKIP) continue;
            const int fl = (C.flags >> (4 * f)) & 15;
            const int nf = fl & 3;
            const bool rev = (fl >> 2) & 1;
            const float nx = pick3(f, G.n[0][0], G.n[1][0], G.n[2][0]);
            const float ny = pick3(f, G.n[0][1], G.n[1][1], G.n[2][1]);
            const float hF = pick3(f, G.h[0], G.h[1], G.h[2]);
            float Uo[NFQ][4], Un[NFQ][4];
            // own traces from the staged coefficients: the same sums, in the same order, as the
            // previous stage's write_traces (the neighbours read those)
#pragma unroll
            for (int j = 0; j < NFQ; ++j)
#pragma unroll
                for (int v = 0; v < NV; ++v) Uo[j][v] = 0.f;
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                const float4 c4 = *reinterpret_cast<const float4*>(Ue + i * NV);
                const float cc[4] = {c4.x, c4.y, c4.z, c4.w};
#pragma unroll
                for (int j = 0; j < NFQ; ++j) fma4(o.phif[f][j][i], cc, Uo[j]);
            }
            BCSlot bc;
            bc.type = -1;
            // NBS: the neighbour's block in shared memory, read point by point in the loop below
            const float* nts = sN + tl * nbr_trace_stride<P>() + f * NFQ * NV;
            if (!NBS && (!BND || nb >= 0)) {
                const float* nt = s.tin + (size_t)nb * TRF + nf * NFQ * NV;
#pragma unroll
                for (int k = 0; k < NFQ; ++k) {
                    const float4 t = __ldg(reinterpret_cast<const float4*>(nt + k * NV));
                    Un[k][0] = t.x; Un[k][1] = t.y; Un[k][2] = t.z; Un[k][3] = t.w;
                }
#pragma unroll
                for (int j = 0; j < NFQ / 2; ++j)
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        const float a = Un[j][v], b = Un[NFQ - 1 - j][v];
                        Un[j][v] = rev ? b : a;
                        Un[NFQ - 1 - j][v] = rev ? a : b;
                    }
            } else if (BND && nb < 0) {
                bc = s.bc[-1 - nb];
            }
#pragma unroll
            for (int j = 0; j < NFQ; ++j) {
                float H[4];
                if (NBS) {
                    float un[4];
                    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                                 : "=f"(un[0]), "=f"(un[1]), "=f"(un[2]), "=f"(un[3])
                                 : "r"((unsigned)__cvta_generic_to_shared(nts + (rev ? NFQ - 1 - j : j) * NV)));
                    rusanov<float>(Uo[j], un, nx, ny, gamma, H);
                } else if (!BND || nb >= 0) {
                    rusanov<float>(Uo[j], Un[j], nx, ny, gamma, H);
                } else {
                    float Ub[4];
                    if (inviscid_ghost<float>(bc, Uo[j], nx, ny, gamma, Ub)) {
                        rusanov<float>(Uo[j], Ub, nx, ny, gamma, H);
                    } else {
#pragma unroll
                        for (int v = 0; v < 4; ++v) H[v] = 0.f;
                    }
                }
                const float w = o.wf[j] * hF * 0.5f * inv_j;
#pragma unroll
                for (int i = 0; i < NP; ++i) fma4(-(w * L.pf[f][j][i]), H, R[i]);
            }
        }
    }
    __syncthreads();  // every read of sU is done
    if (active) {
#pragma unroll
        for (int i = 0; i < NP; ++i)
            *reinterpret_cast<float4*>(sU + tl * STR + i * NV) = make_float4(R[i][0], R[i][1], R[i][2], R[i][3]);
    }
    __syncthreads();
    // stage combination; the next stage state (uhi + dout, or uhi_out after stage 3) replaces
    // each residual slot of sU
    stage_combine_next<NB, STR, T, 2, SK>(s, sU, sDt, e0, nloc, [](int le) { return tile_row<T>(le); });
    __syncthreads();
    if (active) write_traces<P, GHOST, (T <= 32)>(o, sU + tl * STR, s.tout + (size_t)e * TRF, s, e);
    __syncthreads();  // the next tile reuses sU / sDt
}

template <int P, bool BND, bool GHOST, int T, bool NBS, int SK>
__device__ __forceinline__ void stage_trace_tile(const SArgs<P, false>& ka, float* sU, float* sDt, float* sN,
                                                 int tile) {
    constexpr int NB = n_basis(P) * NV, STR = stage_stride<P>();
    const StageArgs& s = ka.s;
    stage_trace_tile_with<P, BND, GHOST, T, NBS, SK>(ka, sU, sDt, tile, [&](ElemGeomF& G, ElemConn& C) {
        const int e0 = tile * T, nloc = min(T, s.ne - e0);
        const int tl = threadIdx.x, el = tile_elem<T>(tl);
        // u^n is read back in the stage combination
        if (tl == 0 && (SK == SK_3DF || (SK == SK_ANY && s.stage == 3)))
            rk3_prefetch(s, (size_t)e0 * NB, nloc * NB);
        // the element's geometry and connectivity ride in the same round trip as the tile's state
        if (el < nloc) {
            if (!BND) G = s.geom[e0 + el];
            C = s.conn[e0 + el];
        }
        stage_load_tile<NB, STR, T>(s.uhi, SK == SK_1 ? nullptr : s.din, sU, e0, nloc,
                                    [](int le) { return tile_row<T>(le); });
        if (el < nloc) {
            if (NBS) copy_neighbour_traces<P>(s, C, sN + tl * nbr_trace_stride<P>());
            else prefetch_neighbour_traces<P, BND>(s, C);
        }
        __syncthreads();
    }, sN);
}

// CTAs per SM the register allocation must allow.  Measured on GB300 for p=3 (512x512x2):
// 3 CTAs (168 registers, no spills) 0.513 ms/step, 4 CTAs (128 registers) 0.544; the
// boundary-branch kernel, with the face loop still unrolled, ran 0.743 ms/step at 2 CTAs
// (255 registers) against 0.769 at 3 CTAs (580 B of spills).
__host__ __device__ constexpr int trace_min_blocks(int p, bool bnd) {
#ifdef DGX_TRACE_MIN_BLOCKS
    return DGX_TRACE_MIN_BLOCKS + 0 * p + 0 * bnd;
#else
    return (p <= 3 && !bnd) ? 3 : 2;
#endif
}

// Persistent form, grid from the autotuner.  BND: some faces are boundary or skipped faces
// (handled in the face loop); GHOST: boundary faces read ghost blocks, which this kernel writes.
// T: elements per tile and threads per CTA (TILE, or 64 or 32 at one CTA per tile: the same
// registers per thread and CTAs per SM in proportion, so the SM holds as many elements, in
// smaller groups whose barriers and load/compute phases are independent).  ka.s.tile0 and
// ka.s.ntile count T-element tiles.  NBS: neighbour trace blocks through shared memory (sN,
// after sU; every face interior or a ghost face).  SK: the stages served (StageKind).
template <int P, bool BND, bool GHOST, int T = TILE, bool NBS = false, int SK = SK_ANY>
__global__ void __launch_bounds__(T, trace_min_blocks(P, BND) * (TILE / T))
    stage_trace_kernel(const __grid_constant__ SArgs<P, false> ka) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sDt = reinterpret_cast<float*>(smem_raw);
    float* sU = sDt + T;
    float* sN = sU + T * stage_stride<P>();  // 16-byte aligned: T % 4 == 0, stride % 4 == 0
    const int ntiles = ka.s.ntile > 0 ? ka.s.ntile : (ka.s.ne + T - 1) / T;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x)
        stage_trace_tile<P, BND, GHOST, T, NBS, SK>(ka, sU, sDt, sN, ka.s.tile0 + t);
}

// Pipelined persistent form (Euler, no boundary branch: periodic meshes or ghost blocks).  Each
// CTA walks tiles blockIdx.x, + gridDim.x, ...; one thread bulk-copies (cp.async.bulk, completing
// on an mbarrier) the next tile's uhi and din rows, geometry and connectivity into a staging
// buffer as soon as the current tile has been staged from it, so a tile's loads run while the
// tile before it is computed.  The staged numbers and every operation after them are those of
// stage_trace_kernel.  Shared memory: sDt, sU, then the staging buffer and its barrier.
template <int P>
struct TracePipe {
    static constexpr int NB = n_basis(P) * NV;
    static constexpr int OFF_U = TILE * 4;
    static constexpr int OFF_HI = OFF_U + TILE * stage_stride<P>() * 4;
    static constexpr int OFF_DIN = OFF_HI + TILE * NB * 4;
    static constexpr int OFF_G = OFF_DIN + TILE * NB * 4;
    static constexpr int OFF_C = OFF_G + TILE * (int)sizeof(ElemGeomF);
    static constexpr int OFF_BAR = OFF_C + TILE * (int)sizeof(ElemConn);
    static constexpr int SMEM = OFF_BAR + 16;  // the barrier and the CTA's abort flag
    static_assert(OFF_HI % 16 == 0 && OFF_DIN % 16 == 0 && OFF_G % 16 == 0 && OFF_C % 16 == 0 && OFF_BAR % 8 == 0,
                  "bulk-copy destinations must be 16-byte aligned");
};

// bulk copies of tile `tile`'s inputs into the staging buffer (issuing thread only); every
// source starts on a 16-byte boundary (tile offsets are multiples of 128 elements) and every
// size is a multiple of 16 bytes
template <int P>
__device__ __forceinline__ void trace_pipe_issue(const StageArgs& s, unsigned char* sm, uint64_t* bar, int tile) {
    using TP = TracePipe<P>;
    const int e0 = tile * TILE, nloc = min(TILE, s.ne - e0);
    const uint32_t bs = (uint32_t)nloc * TP::NB * 4u, bd = s.din ? bs : 0u;
    const uint32_t bg = (uint32_t)nloc * (uint32_t)sizeof(ElemGeomF), bc = (uint32_t)nloc * (uint32_t)sizeof(ElemConn);
    tc::mbar_expect_tx(bar, bs + bd + bg + bc);
    tc::bulk_g2s(sm + TP::OFF_HI, s.uhi + (size_t)e0 * TP::NB, bs, bar);
    if (bd) tc::bulk_g2s(sm + TP::OFF_DIN, s.din + (size_t)e0 * TP::NB, bd, bar);
    tc::bulk_g2s(sm + TP::OFF_G, s.geom + e0, bg, bar);
    tc::bulk_g2s(sm + TP::OFF_C, s.conn + e0, bc, bar);
    if (s.stage == 3) rk3_prefetch(s, (size_t)e0 * TP::NB, nloc * TP::NB);
}

template <int P, bool GHOST>
__global__ void __launch_bounds__(TILE, 3) stage_trace_pipe_kernel(const __grid_constant__ SArgs<P, false> ka) {
    using TP = TracePipe<P>;
    constexpr int NB = TP::NB, NB4 = NB / 4, STR = stage_stride<P>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sDt = reinterpret_cast<float*>(smem_raw);
    float* sU = reinterpret_cast<float*>(smem_raw + TP::OFF_U);
    const float4* rHi = reinterpret_cast<const float4*>(smem_raw + TP::OFF_HI);
    const float4* rDin = reinterpret_cast<const float4*>(smem_raw + TP::OFF_DIN);
    const ElemGeomF* rG = reinterpret_cast<const ElemGeomF*>(smem_raw + TP::OFF_G);
    const ElemConn* rC = reinterpret_cast<const ElemConn*>(smem_raw + TP::OFF_C);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + TP::OFF_BAR);
    volatile int* abort = reinterpret_cast<volatile int*>(smem_raw + TP::OFF_BAR + 8);
    const StageArgs& s = ka.s;
    const int ntiles = s.ntile > 0 ? s.ntile : (s.ne + TILE - 1) / TILE;
    const int tl = threadIdx.x;
    if (tl == 0) {
        tc::mbar_init(bar, 1);
        *abort = 0;
    }
    __syncthreads();
    if (tl == 0 && (int)blockIdx.x < ntiles) trace_pipe_issue<P>(s, smem_raw, bar, s.tile0 + blockIdx.x);
    uint32_t parity = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const bool ok = tc::mbar_wait_or_abort(bar, parity, s.wait_limit, abort, s.wait_hint_ns);
        if (__syncthreads_or(!ok)) {
            // a copy did not complete in time: report it, let the copy in flight land, and stop
            if (tl == 0) {
                if (s.status) atomicOr(s.status, 2);
                // the copy in flight lands in this CTA's shared memory: wait for it (up to about
                // 1.3 s, whatever the configured limit) before the CTA exits
                for (int it = 0; it < (1 << 16) && !tc::mbar_test_sleep(bar, parity, 20000); ++it) {
                }
            }
            return;
        }
        parity ^= 1;
        const int tile = s.tile0 + t;
        stage_trace_tile_with<P, false, GHOST, TILE>(ka, sU, sDt, tile, [&](ElemGeomF& G, ElemConn& C) {
            const int e0 = tile * TILE, nloc = min(TILE, s.ne - e0);
            // the stage state uhi + din into sU (stage_load_tile's sums), the element's records
            for (int g = tl; g < nloc * NB4; g += TILE) {
                float4 a = rHi[g];
                if (s.din) {
                    const float4 b = rDin[g];
                    a.x += b.x; a.y += b.y; a.z += b.z; a.w += b.w;
                }
                const int le = g / NB4, k = 4 * (g - le * NB4);
                *reinterpret_cast<float4*>(sU + stage_row(le) * STR + k) = a;
            }
            const int el = stage_elem(tl);
            if (el < nloc) {
                G = rG[el];
                C = rC[el];
                prefetch_neighbour_traces<P, false>(s, C);
            }
            __syncthreads();  // the staging buffer has been read: the next tile's copies may land
            if (tl == 0 && t + (int)gridDim.x < ntiles) {
                tc::fence_async_smem();
                trace_pipe_issue<P>(s, smem_raw, bar, tile + gridDim.x);
            }
        });
    }
}

// The traces of the state u = uhi (+ din) a step starts from: one thread per element.
template <int P>
__global__ void __launch_bounds__(TILE) trace_init_kernel(const __grid_constant__ SArgs<P, false> ka) {
    constexpr int NB = n_basis(P) * NV, STR = stage_stride<P>(), NB4 = NB / 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sU = reinterpret_cast<float*>(smem_raw);
    const StageArgs& s = ka.s;
    const int e0 = (s.tile0 + blockIdx.x) * TILE;
    const int nloc = min(TILE, s.ne - e0);
    const float4* uh = reinterpret_cast<const float4*>(s.uhi + (size_t)e0 * NB);
    for (int g = threadIdx.x; g < nloc * NB4; g += TILE) {
        const int le = g / NB4, k = 4 * (g - le * NB4);
        *reinterpret_cast<float4*>(sU + le * STR + k) = __ldg(uh + g);
    }
    __syncthreads();
    if ((int)threadIdx.x < nloc)
        write_traces<P, true>(ka.o, sU + threadIdx.x * STR, s.tout + (size_t)(e0 + threadIdx.x) * trace_floats<P>(),
                              s, e0 + threadIdx.x);
}

template <int P, int T = TILE, bool NBS = false>
inline size_t stage_trace_smem_bytes() {
    return (size_t)(T + T * stage_stride<P>() + (NBS ? T * nbr_trace_stride<P>() : 0)) * sizeof(float);
}

template <int P>
inline int configure_stage_trace_t() {
    const int b = (int)stage_trace_smem_bytes<P>();
    return cudaFuncSetAttribute(stage_trace_kernel<P, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ==
                       cudaSuccess &&
                   cudaFuncSetAttribute(stage_trace_kernel<P, false, false>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, b) == cudaSuccess &&
                   cudaFuncSetAttribute(stage_trace_kernel<P, false, true>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, b) == cudaSuccess &&
                   cudaFuncSetAttribute(trace_init_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ==
                       cudaSuccess &&
                   cudaFuncSetAttribute(stage_trace_pipe_kernel<P, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        TracePipe<P>::SMEM) == cudaSuccess &&
                   cudaFuncSetAttribute(stage_trace_pipe_kernel<P, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        TracePipe<P>::SMEM) == cudaSuccess
               ? 0
               : -1;
}

template <int P>
inline int launch_stage_trace_t(const StageArgs& a, const OpsHost& oh, int grid, cudaStream_t st) {
    SArgs<P, false> ka;
    ka.s = a;
    if (a.tconn) ka.s.conn = a.tconn;  // boundary faces as interior faces to ghost blocks
    fill_ops<P, float>(oh, ka.o);
    fill_lift<P, float>(oh, ka.l);
    const int ntiles = a.ntile > 0 ? a.ntile : (a.ne + TILE - 1) / TILE;
    if (ntiles == 0) return 0;
    const bool pipe = (grid & STAGE_PIPE) != 0 && (a.tconn || !a.boundary);
    grid &= ~STAGE_PIPE;
    if (ka.s.wait_limit <= 0) kernel_wait_bounds("DGX_TRACE_WAIT_LIMIT", &ka.s.wait_limit, &ka.s.wait_hint_ns);
    if (grid <= 0 || grid > ntiles) grid = ntiles;
    if (pipe) {
        if (a.tconn)
            stage_trace_pipe_kernel<P, true><<<grid, TILE, TracePipe<P>::SMEM, st>>>(ka);
        else
            stage_trace_pipe_kernel<P, false><<<grid, TILE, TracePipe<P>::SMEM, st>>>(ka);
        return launch_status();
    }
    if (a.tconn)
        stage_trace_kernel<P, false, true><<<grid, TILE, stage_trace_smem_bytes<P>(), st>>>(ka);
    else if (a.boundary)
        stage_trace_kernel<P, true, false><<<grid, TILE, stage_trace_smem_bytes<P>(), st>>>(ka);
    else
        stage_trace_kernel<P, false, false><<<grid, TILE, stage_trace_smem_bytes<P>(), st>>>(ka);
    return launch_status();
}

template <int P>
inline int launch_trace_init_t(const StageArgs& a, const OpsHost& oh, cudaStream_t st) {
    SArgs<P, false> ka;
    ka.s = a;
    if (a.tconn) ka.s.conn = a.tconn;
    fill_ops<P, float>(oh, ka.o);
    const int ntiles = a.ntile > 0 ? a.ntile : (a.ne + TILE - 1) / TILE;
    if (ntiles == 0) return 0;
    trace_init_kernel<P><<<ntiles, TILE, stage_trace_smem_bytes<P>(), st>>>(ka);
    return launch_status();
}

}  // namespace dgx
