// Element kernels of the explicit DG path: volume flux integral, the three faces'
// numerical fluxes lifted to the element's modes, the inverse mass matrix and the
// SSP-RK3 stage combination, one thread per element, 128 elements per CTA.
//
// dgfem computes the same residual face-by-face (src/solver/assembler.cpp:137-279): every
// interior face evaluates the Rusanov flux once and adds -w*phi_L*H to the L element and
// +w*phi_R*H to the R element (src/weak_forms/euler_weak_formulation.cpp:117-175).  Here
// each element evaluates its own three faces with its own outward normal.  The Rusanov
// flux is exactly antisymmetric, H(U_L, U_R, n) == -H(U_R, U_L, -n) bit for bit, and the
// R side stores -n_L as its normal and the L side's face length, so the R side's
// contribution equals dgfem's up to summation order.  The viscous interior flux of
// dgfem is 1/2 (Fv_L - Fv_R).n - sigma (U_R - U_L) for both sides
// (src/weak_forms/navier_stokes_weak_formulation.cpp:189-202); its first term changes
// sign with the side, which is why each face slot records whether the element is the L
// side.
//
// Geometry is affine per element, so d(phi)/dx = A * d(phi)/d(xi) with A = inverse(J_T),
// and the volume integral is evaluated in contravariant form
//   sum_q w_q |J| (dphi/dx F + dphi/dy G) = sum_q (dphi/dxi Fr_q + dphi/deta Fs_q),
//   Fr = w|J| (A00 F + A10 G), Fs = w|J| (A01 F + A11 G),
// and M_K^-1 = M_ref^-1 / |J|.
//
// Data movement: a CTA stages its 128 elements' coefficients (one contiguous run in
// HBM) into shared memory with an odd row stride, so the one-element-per-thread reads
// are bank-conflict free; neighbours outside the tile are read through L1/L2.
#pragma once

#include "../../include/dgx.h"
#include "dg_physics.cuh"

namespace dgx {

template <int P, typename T, bool VISC>
struct KArgs {
    StepArgs s;
    Ops<P, T> o;
    double minv64[n_basis(P)][n_basis(P)];  // FP64 inverse reference mass matrix
};

// Projection/lift operators with the inverse reference mass matrix folded in:
// pr[q][i] = sum_k Minv[i][k] dr[q][k], ps likewise, pf[f][j][i] = sum_k Minv[i][k] phif[f][j][k].
template <int P, typename T>
struct LiftOps {
    static constexpr int NP = n_basis(P), NQ = n_quad(P), NFQ = P + 1;
    T pr[NQ][NP];
    T ps[NQ][NP];
    T pf[3][NFQ][NP];
};

template <int P, typename T>
inline void fill_lift(const OpsHost& h, LiftOps<P, T>& l) {
    constexpr int NP = n_basis(P), NQ = n_quad(P), NFQ = P + 1;
    for (int i = 0; i < NP; ++i) {
        for (int q = 0; q < NQ; ++q) {
            double a = 0.0, b = 0.0;
            for (int k = 0; k < NP; ++k) {
                a += h.minv[i][k] * h.dr[q][k];
                b += h.minv[i][k] * h.ds[q][k];
            }
            l.pr[q][i] = (T)a;
            l.ps[q][i] = (T)b;
        }
        for (int f = 0; f < 3; ++f)
            for (int j = 0; j < NFQ; ++j) {
                double a = 0.0;
                for (int k = 0; k < NP; ++k) a += h.minv[i][k] * h.phif[f][j][k];
                l.pf[f][j][i] = (T)a;
            }
    }
}

// One coefficient row (4 variables) of element `nb` from an FP64 state, converted to T.
template <typename T, int NB>
__device__ __forceinline__ void load_row_f64(const double* u, int nb, int i, T c[4]) {
    const double* p = u + (size_t)nb * NB + i * NV;
    const double2 a = __ldg(reinterpret_cast<const double2*>(p));
    const double2 b = __ldg(reinterpret_cast<const double2*>(p + 2));
    c[0] = (T)a.x;
    c[1] = (T)a.y;
    c[2] = (T)b.x;
    c[3] = (T)b.y;
}

// One coefficient row of element `nb` from uhi (+ d when d is not null), FP32.
template <int NB>
__device__ __forceinline__ void load_row_f32(const float* uhi, const float* d, int nb, int i, float c[4]) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(uhi + (size_t)nb * NB + i * NV));
    c[0] = a.x;
    c[1] = a.y;
    c[2] = a.z;
    c[3] = a.w;
    if (d) {
        const float4 b = __ldg(reinterpret_cast<const float4*>(d + (size_t)nb * NB + i * NV));
        c[0] += b.x;
        c[1] += b.y;
        c[2] += b.z;
        c[3] += b.w;
    }
}

// The residual (or, with FOLD, M_K^-1 times the residual) of one element, accumulated
// into R.  Ue: this element's coefficients (shared memory); sU/e0/nloc: the tile, for
// in-tile neighbours; getrow(nb, i, c): coefficient row i of an out-of-tile neighbour.
// NBREG keeps a neighbour's coefficients in registers across the face's points.  OT is
// the type the operators are stored in (T itself, or double when T carries derivatives).
template <int P, typename T, bool VISC, bool FOLD, bool NBREG, class GetRow, typename OT>
__device__ __forceinline__ void element_residual(const Ops<P, OT>& o, const LiftOps<P, OT>* L,
                                                 const T* Ue, const T* sU, int e0, int nloc,
                                                 const ElemGeom& G, const ElemConn& C,
                                                 const BCSlot* bcs, const ElemGeom* geoms,
                                                 T gamma, T mu, T kappa, T sigma0,
                                                 const GetRow& getrow, T R[n_basis(P)][NV]) {
    constexpr int NP = n_basis(P), NQ = n_quad(P), NFQ = P + 1, NB = NP * NV, STR = NB + 1;
    const T A00 = (T)G.A[0], A01 = (T)G.A[1], A10 = (T)G.A[2], A11 = (T)G.A[3];
    const T detJ = (T)G.detJ;

    // ---------------- volume: EulerWeakFormulation::volume_residual (:72-115)
    //                  + NavierStokesWeakFormulation::viscous_volume_residual (:100-140)
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
        T U[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
        for (int i = 0; i < NP; ++i)
#pragma unroll
            for (int v = 0; v < NV; ++v) U[v] = mac(U[v], o.phi[q][i], Ue[i * NV + v]);
#pragma unroll
        for (int v = 0; v < NV; ++v) U[v] = settle(U[v]);
        T F[4], Gf[4], u, vv, pp, ri;
        euler_flux<T>(U, gamma - T(1), F, Gf, u, vv, pp, ri);
        if (VISC) {
            T gr[4] = {T(0), T(0), T(0), T(0)}, gs[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
            for (int i = 0; i < NP; ++i)
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    gr[v] = mac(gr[v], o.dr[q][i], Ue[i * NV + v]);
                    gs[v] = mac(gs[v], o.ds[q][i], Ue[i * NV + v]);
                }
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                gr[v] = settle(gr[v]);
                gs[v] = settle(gs[v]);
            }
            T gx[4], gy[4], Fv[4], Gv[4];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                gx[v] = A00 * gr[v] + A01 * gs[v];
                gy[v] = A10 * gr[v] + A11 * gs[v];
            }
            viscous_flux<T>(U, gx, gy, gamma, mu, kappa, Fv, Gv);
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                F[v] -= Fv[v];
                Gf[v] -= Gv[v];
            }
        }
        const T w = FOLD ? o.wq[q] : o.wq[q] * detJ;
        T Fr[4], Fs[4];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            Fr[v] = w * (A00 * F[v] + A10 * Gf[v]);
            Fs[v] = w * (A01 * F[v] + A11 * Gf[v]);
        }
#pragma unroll
        for (int i = 0; i < NP; ++i) {
            const T a = FOLD ? L->pr[q][i] : o.dr[q][i];
            const T b = FOLD ? L->ps[q][i] : o.ds[q][i];
#pragma unroll
            for (int v = 0; v < NV; ++v) R[i][v] = mac(mac(R[i][v], a, Fr[v]), b, Fs[v]);
        }
    }

    // ---------------- faces: interior_face_residual (:117-175), boundary_face_residual
    //                  (:177-250) and their viscous counterparts (NS :142-273)
    const T inv_j = FOLD ? rcp_<T>(detJ) : T(1);
#pragma unroll 1
    for (int f = 0; f < 3; ++f) {
        const int nb = C.nbr[f];
        if (nb == NBR_SKIP) continue;
        const int fl = (C.flags >> (4 * f)) & 15;
        const int nf = fl & 3;
        const bool rev = (fl >> 2) & 1;
        const T sideL = ((fl >> 3) & 1) ? T(1) : T(-1);
        const T nx = (T)G.n[f][0], ny = (T)G.n[f][1];
        const T hF = (T)G.h[f];
        const T* Un_s = nullptr;
        T B00 = T(0), B01 = T(0), B10 = T(0), B11 = T(0);
        BCSlot bc;
        bc.type = -1;
        T Nc[NBREG ? NP : 1][NV];
        if (nb >= 0) {
            if (nb >= e0 && nb < e0 + nloc) Un_s = sU + (nb - e0) * STR;
            if (NBREG) {
#pragma unroll
                for (int i = 0; i < NP; ++i) {
                    if (Un_s) {
#pragma unroll
                        for (int v = 0; v < NV; ++v) Nc[i][v] = Un_s[i * NV + v];
                    } else {
                        getrow(nb, i, Nc[i]);
                    }
                }
            }
            if (VISC) {
                const ElemGeom& GN = geoms[nb];
                B00 = (T)GN.A[0]; B01 = (T)GN.A[1]; B10 = (T)GN.A[2]; B11 = (T)GN.A[3];
            }
        } else {
            bc = bcs[-1 - nb];
        }
        // NavierStokesWeakFormulation::compute_penalty_parameter (:275-278)
        const T sigma = VISC ? sigma0 * mu * T((P + 1) * (P + 1)) / (hF > T(1e-12) ? hF : T(1e-12)) : T(0);
#pragma unroll 1
        for (int j = 0; j < NFQ; ++j) {
            T Uo[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
            for (int i = 0; i < NP; ++i)
#pragma unroll
                for (int v = 0; v < NV; ++v) Uo[v] = mac(Uo[v], o.phif[f][j][i], Ue[i * NV + v]);
#pragma unroll
            for (int v = 0; v < NV; ++v) Uo[v] = settle(Uo[v]);
            T Un[4] = {T(0), T(0), T(0), T(0)};
            const int k = rev ? NFQ - 1 - j : j;
            if (nb >= 0) {
#pragma unroll
                for (int i = 0; i < NP; ++i) {
                    T c[4];
                    if (NBREG) {
#pragma unroll
                        for (int v = 0; v < NV; ++v) c[v] = Nc[i][v];
                    } else if (Un_s) {
#pragma unroll
                        for (int v = 0; v < NV; ++v) c[v] = Un_s[i * NV + v];
                    } else {
                        getrow(nb, i, c);
                    }
                    const T ph = o.phif[nf][k][i];
#pragma unroll
                    for (int v = 0; v < NV; ++v) Un[v] = mac(Un[v], ph, c[v]);
                }
#pragma unroll
                for (int v = 0; v < NV; ++v) Un[v] = settle(Un[v]);
            }
            T H[4];
            if (nb >= 0) {
                rusanov<T>(Uo, Un, nx, ny, gamma, H);
            } else {
                T Ub[4];
                if (inviscid_ghost<T>(bc, Uo, nx, ny, gamma, Ub)) {
                    rusanov<T>(Uo, Ub, nx, ny, gamma, H);
                } else {
#pragma unroll
                    for (int v = 0; v < 4; ++v) H[v] = T(0);
                }
            }
            if (VISC) {
                T gr[4] = {T(0), T(0), T(0), T(0)}, gs[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
                for (int i = 0; i < NP; ++i)
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        gr[v] = mac(gr[v], o.drf[f][j][i], Ue[i * NV + v]);
                        gs[v] = mac(gs[v], o.dsf[f][j][i], Ue[i * NV + v]);
                    }
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    gr[v] = settle(gr[v]);
                    gs[v] = settle(gs[v]);
                }
                T gx[4], gy[4], Fv[4], Gv[4];
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    gx[v] = A00 * gr[v] + A01 * gs[v];
                    gy[v] = A10 * gr[v] + A11 * gs[v];
                }
                viscous_flux<T>(Uo, gx, gy, gamma, mu, kappa, Fv, Gv);
                if (nb >= 0) {
                    T nr[4] = {T(0), T(0), T(0), T(0)}, ns[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
                    for (int i = 0; i < NP; ++i) {
                        T c[4];
                        if (NBREG) {
#pragma unroll
                            for (int v = 0; v < NV; ++v) c[v] = Nc[i][v];
                        } else if (Un_s) {
#pragma unroll
                            for (int v = 0; v < NV; ++v) c[v] = Un_s[i * NV + v];
                        } else {
                            getrow(nb, i, c);
                        }
#pragma unroll
                        for (int v = 0; v < NV; ++v) {
                            nr[v] = mac(nr[v], o.drf[nf][k][i], c[v]);
                            ns[v] = mac(ns[v], o.dsf[nf][k][i], c[v]);
                        }
                    }
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        nr[v] = settle(nr[v]);
                        ns[v] = settle(ns[v]);
                    }
                    T hx[4], hy[4], Fn2[4], Gn2[4];
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        hx[v] = B00 * nr[v] + B01 * ns[v];
                        hy[v] = B10 * nr[v] + B11 * ns[v];
                    }
                    viscous_flux<T>(Un, hx, hy, gamma, mu, kappa, Fn2, Gn2);
                    // own side L:  Fn = 1/2 (Fv_o - Fv_n).n - sigma (U_n - U_o)
                    // own side R:  dgfem adds +w phi Fn_L, i.e. -= w phi (-J - P)
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        const T jmp = T(0.5) * ((Fv[v] * nx + Gv[v] * ny) - (Fn2[v] * nx + Gn2[v] * ny));
                        H[v] += sideL * jmp - sigma * (Un[v] - Uo[v]);
                    }
                } else if (bc.type >= 0) {
                    T Ub[4];
                    viscous_ghost<T>(bc, gamma, Ub);
#pragma unroll
                    for (int v = 0; v < NV; ++v) H[v] += (Fv[v] * nx + Gv[v] * ny) - sigma * (Ub[v] - Uo[v]);
                }
            }
            const T w = o.wf[j] * hF * T(0.5) * inv_j;
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                const T sc = w * (FOLD ? L->pf[f][j][i] : o.phif[f][j][i]);
#pragma unroll
                for (int v = 0; v < NV; ++v) R[i][v] = mac(R[i][v], -sc, H[v]);
            }
        }
    }
}

// ---------------------------------------------------------------------------------
// Element kernel with FP64 input/output states: the FP64 path (T = double) and the
// mixed path's residual / rhs entry points (T = float).
// CTAs per SM the register allocation must allow (1: unconstrained).  DGX_ELEMENT_MIN_BLOCKS
// overrides it for experiments.
#ifndef DGX_ELEMENT_MIN_BLOCKS
#define DGX_ELEMENT_MIN_BLOCKS 1
#endif
template <int P, typename T, bool VISC>
__global__ void __launch_bounds__(TILE, DGX_ELEMENT_MIN_BLOCKS) element_kernel(const __grid_constant__ KArgs<P, T, VISC> ka) {
    constexpr int NP = n_basis(P), NB = NP * NV, STR = NB + 1;
    const StepArgs& s = ka.s;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* sU = reinterpret_cast<T*>(smem_raw);  // [TILE][STR], odd stride: conflict-free rows

    const int e0 = blockIdx.x * TILE;
    const int nloc = min(TILE, s.ne - e0);
    const int tl = threadIdx.x;
    const bool active = tl < nloc;
    const int e = e0 + tl;

    {   // stage the tile's coefficients: one contiguous run of nloc*NB doubles
        const double* ug = s.u + (size_t)e0 * NB;
        for (int g = tl; g < nloc * NB; g += TILE) {
            const int el = g / NB;
            sU[el * STR + (g - el * NB)] = (T)__ldg(ug + g);
        }
    }
    __syncthreads();

    T R[NP][NV];
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
        for (int v = 0; v < NV; ++v) R[i][v] = T(0);

    if (active) {
        const T mu = (T)s.mu;
        const T kappa = VISC ? (T)(s.mu * s.gamma / (s.prandtl * (s.gamma - 1.0))) : T(0);
        const double* ug = s.u;
        auto getrow = [ug](int nb, int i, T c[4]) { load_row_f64<T, NB>(ug, nb, i, c); };
        element_residual<P, T, VISC, false, false>(ka.o, (const LiftOps<P, T>*)nullptr, sU + tl * STR, sU, e0, nloc, s.geom[e],
                                                   s.conn[e], s.bc, s.geom, (T)s.gamma, mu, kappa,
                                                   (T)s.sigma0, getrow, R);
    }
    __syncthreads();  // all neighbour reads of sU are done

    // ---------------- epilogue: residual, or M^-1 R (apply_mass_inv,
    // compressible_solver_base.cpp:54-61) and the SSP-RK3 combination (time_stepping.hpp:39-55)
    double* sD = reinterpret_cast<double*>(smem_raw);  // [TILE][STR] doubles, reuses sU
    if (active) {
        if (s.mode == MODE_RESIDUAL) {
#pragma unroll
            for (int i = 0; i < NP; ++i)
#pragma unroll
                for (int v = 0; v < NV; ++v) sD[tl * STR + i * NV + v] = to_f64(R[i][v]);
        } else {
            const double ij = 1.0 / s.geom[e].detJ;
            if (s.minv_diag) {
#pragma unroll
                for (int i = 0; i < NP; ++i)
#pragma unroll
                    for (int v = 0; v < NV; ++v)
                        sD[tl * STR + i * NV + v] = ka.minv64[i][i] * to_f64(R[i][v]) * ij;
            } else {
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    double col[NP];
#pragma unroll
                    for (int i = 0; i < NP; ++i) {
                        double acc = 0.0;
#pragma unroll
                        for (int k = 0; k < NP; ++k) acc += ka.minv64[i][k] * to_f64(R[k][v]);
                        col[i] = acc * ij;
                    }
#pragma unroll
                    for (int i = 0; i < NP; ++i) sD[tl * STR + i * NV + v] = col[i];
                }
            }
        }
    }
    __syncthreads();
    double* og = s.out + (size_t)e0 * NB;
    const double* ug = s.u + (size_t)e0 * NB;
    const double* ung = s.un ? s.un + (size_t)e0 * NB : nullptr;
    bool bad = false;
    for (int g = tl; g < nloc * NB; g += TILE) {
        const int el = g / NB;
        const double d = sD[el * STR + (g - el * NB)];
        double r;
        if (s.mode != MODE_STAGE) {
            r = d;
        } else if (s.a == 0.0) {
            r = ug[g] + s.dt * d;
        } else {
            const double t = ug[g] + s.dt * d;
            r = s.a * __ldg(ung + g) + s.b * t;
        }
        bad |= !isfinite(r);
        og[g] = r;
    }
    if (bad && s.status) atomicOr(s.status, 1);
}

template <int P, typename T, bool VISC>
inline size_t element_smem_bytes() {
    return (size_t)TILE * (n_basis(P) * NV + 1) * sizeof(double);
}
// Raise the dynamic shared-memory limit once per context creation (never inside a
// stream capture).
template <int P, typename T, bool VISC>
inline int configure_element_t() {
    if (cudaFuncSetAttribute(element_kernel<P, T, VISC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)element_smem_bytes<P, T, VISC>()) != cudaSuccess)
        return -1;
    return 0;
}

template <int P, typename T, bool VISC>
inline int launch_element_t(const StepArgs& a, const OpsHost& oh, cudaStream_t st) {
    KArgs<P, T, VISC> ka;  // passed by value: every operator read is a constant-bank operand
    ka.s = a;
    fill_ops<P, T>(oh, ka.o);
    for (int i = 0; i < n_basis(P); ++i)
        for (int j = 0; j < n_basis(P); ++j) ka.minv64[i][j] = oh.minv[i][j];
    const int grid = (a.ne + TILE - 1) / TILE;
    if (grid == 0) return 0;
    element_kernel<P, T, VISC><<<grid, TILE, element_smem_bytes<P, T, VISC>(), st>>>(ka);
    return launch_status();
}

#define DGX_ELEMENT_DISPATCH(FN, T)                           \
    switch (p * 2 + (viscous ? 1 : 0)) {                      \
    case 2: return FN<1, T, false>ARGS;                       \
    case 3: return FN<1, T, true>ARGS;                        \
    case 4: return FN<2, T, false>ARGS;                       \
    case 5: return FN<2, T, true>ARGS;                        \
    case 6: return FN<3, T, false>ARGS;                       \
    case 7: return FN<3, T, true>ARGS;                        \
    case 8: return FN<4, T, false>ARGS;                       \
    case 9: return FN<4, T, true>ARGS;                        \
    default: return -1;                                       \
    }

}  // namespace dgx
