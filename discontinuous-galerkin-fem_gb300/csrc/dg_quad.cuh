// Element kernel for bilinear quadrilaterals (DGSpace("quad", p) with dgfem's LegendreBasis):
// volume flux integral, the four faces' numerical fluxes, the element's inverse mass
// matrix and the SSP-RK3 stage combination, one thread per element, 128 elements per CTA.
//
// The residual is dgfem's (src/solver/assembler.cpp:137-279 with
// src/weak_forms/euler_weak_formulation.cpp:72-250 and
// src/weak_forms/navier_stokes_weak_formulation.cpp:100-273), organised per element as in
// the triangle kernel: each element evaluates its own faces with its own outward normal,
// the R side of an interior face carrying -n_L and the L side's face length.
//
// Quadrilateral specifics:
//  * the bilinear map is not affine: J_T, |J| and A = inverse(J_T) are evaluated at every
//    volume and face point from six per-element coefficients (QuadGeom); no per-point
//    geometry is stored.  In the volume term |J| A needs no division:
//      |J| A = sign(det) [[J11, -J01], [-J10, J00]].
//  * M_K = Phi^T diag(w_q |J_q|) Phi with Phi the (p+1)^2 x (p+1)^2 matrix of basis values at
//    the tensor Gauss-Legendre points.  Phi is square and, because that rule integrates
//    the Legendre products exactly, Phi^T W Phi = D, the diagonal reference mass matrix.
//    Hence Phi^-1 = D^-1 Phi^T W and
//      M_K^-1 = D^-1 Phi^T diag(w_q / |J_q|) Phi D^-1,
//    two contractions with the interpolation table and a pointwise scaling, instead of
//    the dense per-element inverse dgfem stores
//    (CompressibleDGSolverBase::compute_mass_matrix_inverse_blocks,
//    src/solver/compressible_solver_base.cpp:41-61).
//
// T is the residual's arithmetic: double (DGX_FP64), float (DGX_MIXED) or f2 (DGX_DF64).
// The element kernel (residual, rhs and the FP64 / df64 RK3 stages) applies the element
// mass inverse in FP64 from FP64 tables (MassOps).  The mixed form's RK3 runs in the
// increment form of the triangle stage kernel (quad_stage_kernel): FP32 copies of u^n plus
// FP32 increments as the stage state, the increment dt M_K^-1 R in FP32 (a few percent of
// the state, so its FP32 rounding is a few 1e-9 of the state), and one FP64 add per value
// and step into the FP64 state.
#pragma once

#include <memory>

#include "../../include/dgx.h"
#include "dg_stage.cuh"

namespace dgx {

template <typename A, typename B>
struct is_same_type { static constexpr bool value = false; };
template <typename A>
struct is_same_type<A, A> { static constexpr bool value = true; };

template <int P, typename T>
struct QuadOps {
    static constexpr int N1 = P + 1, NP = N1 * N1, NQ = NP, NFQ = N1;
    T phi[NQ][NP];        // basis at volume points (q = j (p+1) + i at (x_i, x_j))
    T dr[NQ][NP];         // d/dxi at volume points
    T ds[NQ][NP];         // d/deta at volume points
    T phif[4][NFQ][NP];   // basis at face points
    T drf[4][NFQ][NP];
    T dsf[4][NFQ][NP];
    T wq[NQ];             // tensor Gauss-Legendre weights
    T xq[NQ][2];          // volume points (xi, eta)
    T wf[NFQ];            // Gauss-Legendre weights on [-1, 1]
    T xf[4][NFQ][2];      // face points on the reference square
    T dinv[NP];           // 1 / D_kk, D = sum_q w_q phi phi^T (diagonal)
};

template <int P, typename T>
inline void fill_quad_ops(const OpsHost& h, QuadOps<P, T>& o) {
    using Q = QuadOps<P, T>;
    for (int q = 0; q < Q::NQ; ++q) {
        for (int i = 0; i < Q::NP; ++i) {
            o.phi[q][i] = (T)h.phi[q][i];
            o.dr[q][i] = (T)h.dr[q][i];
            o.ds[q][i] = (T)h.ds[q][i];
        }
        o.wq[q] = (T)h.wq[q];
        o.xq[q][0] = (T)h.qp[q][0];
        o.xq[q][1] = (T)h.qp[q][1];
    }
    for (int f = 0; f < 4; ++f)
        for (int j = 0; j < Q::NFQ; ++j) {
            for (int i = 0; i < Q::NP; ++i) {
                o.phif[f][j][i] = (T)h.phif[f][j][i];
                o.drf[f][j][i] = (T)h.drf[f][j][i];
                o.dsf[f][j][i] = (T)h.dsf[f][j][i];
            }
            o.xf[f][j][0] = (T)h.fxi[f][j][0];
            o.xf[f][j][1] = (T)h.fxi[f][j][1];
        }
    for (int j = 0; j < Q::NFQ; ++j) o.wf[j] = (T)h.wf[j];
    for (int i = 0; i < Q::NP; ++i) o.dinv[i] = (T)h.minv[i][i];
}

// FP64 tables of the element mass inverse
template <int P>
struct MassOps {
    static constexpr int NP = (P + 1) * (P + 1), NQ = NP;
    double phi[NQ][NP];
    double wq[NQ];
    double xq[NQ][2];
    double dinv[NP];
};

template <int P>
inline void fill_mass_ops(const OpsHost& h, MassOps<P>& m) {
    for (int q = 0; q < MassOps<P>::NQ; ++q) {
        for (int i = 0; i < MassOps<P>::NP; ++i) m.phi[q][i] = h.phi[q][i];
        m.wq[q] = h.wq[q];
        m.xq[q][0] = h.qp[q][0];
        m.xq[q][1] = h.qp[q][1];
    }
    for (int i = 0; i < MassOps<P>::NP; ++i) m.dinv[i] = h.minv[i][i];
}

template <int P, typename T, bool VISC>
struct QKArgs {
    StepArgs s;  // s.geom and s.conn are not used
    const QuadGeom* geom;
    const QuadConn* conn;
    QuadOps<P, T> o;
    MassOps<P> m;
};

// Order 4: the operators (28 KB in FP64) and the FP64 mass-inverse tables (6 KB) exceed the
// 32 KB of kernel parameters together, so the mass-inverse tables live in constant memory.
// They depend on the order only (tensor Gauss-Legendre rule, Legendre basis), so one copy per
// device and translation unit, written when the kernel is configured, serves every context.
template <typename T, bool VISC>
struct QKArgs<4, T, VISC> {
    StepArgs s;
    const QuadGeom* geom;
    const QuadConn* conn;
    QuadOps<4, T> o;
};
static __constant__ MassOps<4> c_quad_mass4;

template <int P, typename T, bool VISC>
__device__ __forceinline__ const MassOps<P>& qk_mass(const QKArgs<P, T, VISC>& ka) {
    if constexpr (P == 4) return c_quad_mass4;
    else return ka.m;
}

// J_T at (xi, eta): rows (dx/dxi, dy/dxi) and (dx/deta, dy/deta) (mapping.cpp:22-50)
template <typename T, class QG>
__device__ __forceinline__ void quad_jacobian(const QG& G, T xi, T eta, T& J00, T& J01, T& J10, T& J11) {
    J00 = (T)G.jx[0] + (T)G.jx[2] * eta;
    J01 = (T)G.jy[0] + (T)G.jy[2] * eta;
    J10 = (T)G.jx[1] + (T)G.jx[2] * xi;
    J11 = (T)G.jy[1] + (T)G.jy[2] * xi;
}

// A = inverse(J_T) (mapping.cpp:33-47): dphi/dx = A0 dphi/dxi + A1 dphi/deta,
// dphi/dy = A2 dphi/dxi + A3 dphi/deta
template <typename T, class QG>
__device__ __forceinline__ void quad_inverse_map(const QG& G, T xi, T eta, T A[4]) {
    T J00, J01, J10, J11;
    quad_jacobian<T>(G, xi, eta, J00, J01, J10, J11);
    const T r = rcp_<T>(J00 * J11 - J10 * J01);
    A[0] = J11 * r;
    A[1] = -J01 * r;
    A[2] = -J10 * r;
    A[3] = J00 * r;
}

// Residual of one quadrilateral into R.  Ue: its coefficients (shared memory, rows STR
// apart); sU, e0, nloc: the tile, for in-tile neighbours; getrow(nb, i, c) reads row i of
// an out-of-tile neighbour from global memory.
template <int P, typename T, bool VISC, int STR, class GetRow, class QG>
__device__ __forceinline__ void quad_residual(const QuadOps<P, T>& o, const T* Ue, const T* sU, int e0, int nloc,
                                              const GetRow& getrow, const QG& G, const QuadConn& C,
                                              const BCSlot* bcs, const QG* geoms, T gamma, T mu,
                                              T kappa, T sigma0, T R[n_basis_quad(P)][NV]) {
    constexpr int NP = n_basis_quad(P), NQ = NP, NFQ = P + 1;

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
        T F[4], Gf[4], uu, vv, pp, ri;
        euler_flux<T>(U, gamma - T(1), F, Gf, uu, vv, pp, ri);
        T J00, J01, J10, J11;
        quad_jacobian<T>(G, o.xq[q][0], o.xq[q][1], J00, J01, J10, J11);
        const T det = J00 * J11 - J10 * J01;
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
            const T r = rcp_<T>(det);
            const T A0 = J11 * r, A1 = -J01 * r, A2 = -J10 * r, A3 = J00 * r;
            T gx[4], gy[4], Fv[4], Gv[4];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                gx[v] = A0 * gr[v] + A1 * gs[v];
                gy[v] = A2 * gr[v] + A3 * gs[v];
            }
            viscous_flux<T>(U, gx, gy, gamma, mu, kappa, Fv, Gv);
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                F[v] -= Fv[v];
                Gf[v] -= Gv[v];
            }
        }
        // w |J| (A0 F + A2 G) and w |J| (A1 F + A3 G), |J| A = sign(det) adj(J_T)
        const T w = det > T(0) ? o.wq[q] : -o.wq[q];
        T Fr[4], Fs[4];
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            Fr[v] = w * (J11 * F[v] - J10 * Gf[v]);
            Fs[v] = w * (J00 * Gf[v] - J01 * F[v]);
        }
#pragma unroll
        for (int i = 0; i < NP; ++i)
#pragma unroll
            for (int v = 0; v < NV; ++v) R[i][v] = mac(mac(R[i][v], o.dr[q][i], Fr[v]), o.ds[q][i], Fs[v]);
    }

    // ---------------- faces: interior_face_residual (:117-175), boundary_face_residual
    //                  (:177-250) and their viscous counterparts (NS :142-273)
#pragma unroll 1
    for (int f = 0; f < 4; ++f) {
        const int nb = C.nbr[f];
        if (nb == NBR_SKIP) continue;
        const int fl = (C.flags >> (4 * f)) & 15;
        const int nf = fl & 3;
        const bool rev = (fl >> 2) & 1;
        const T sideL = ((fl >> 3) & 1) ? T(1) : T(-1);
        const T nx = (T)G.n[f][0], ny = (T)G.n[f][1];
        const T hF = (T)G.h[f];
        const T* Un_s = nullptr;
        BCSlot bc;
        bc.type = -1;
        if (nb >= 0) {
            if (nb >= e0 && nb < e0 + nloc) Un_s = sU + (nb - e0) * STR;
        } else {
            bc = bcs[-1 - nb];
        }
        auto nrow = [&](int i, T c[4]) {
            if (Un_s) {
#pragma unroll
                for (int v = 0; v < NV; ++v) c[v] = Un_s[i * NV + v];
            } else {
                getrow(nb, i, c);
            }
        };
        // NavierStokesWeakFormulation::compute_penalty_parameter (:275-278)
        const T sigma = VISC ? sigma0 * mu * T((P + 1) * (P + 1)) / (hF > T(1e-12) ? hF : T(1e-12)) : T(0);
        // FP32: the neighbour's traces at all of its face points in one pass over its rows,
        // put in this face's point order (the face-point loop is then unrolled).  FP64 and
        // double-float: one pass per point, which keeps the register count (and spills) down.
        constexpr bool ONEPASS = is_same_type<T, float>::value;
        constexpr int JUNROLL = ONEPASS ? NFQ : 1;
        T Ut[ONEPASS ? NFQ : 1][4];
#pragma unroll
        for (int k = 0; k < (ONEPASS ? NFQ : 1); ++k)
#pragma unroll
            for (int v = 0; v < NV; ++v) Ut[k][v] = T(0);
        if (ONEPASS && nb >= 0) {
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                T c[4];
                nrow(i, c);
#pragma unroll
                for (int k = 0; k < NFQ; ++k) {
                    const T ph = o.phif[nf][k][i];
#pragma unroll
                    for (int v = 0; v < NV; ++v) Ut[k][v] = mac(Ut[k][v], ph, c[v]);
                }
            }
#pragma unroll
            for (int k = 0; k < NFQ; ++k)
#pragma unroll
                for (int v = 0; v < NV; ++v) Ut[k][v] = settle(Ut[k][v]);
#pragma unroll
            for (int j = 0; j < NFQ / 2; ++j)
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    const T a = Ut[j][v], b = Ut[NFQ - 1 - j][v];
                    Ut[j][v] = rev ? b : a;
                    Ut[NFQ - 1 - j][v] = rev ? a : b;
                }
        }
#pragma unroll JUNROLL
        for (int j = 0; j < NFQ; ++j) {
            T Uo[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
            for (int i = 0; i < NP; ++i)
#pragma unroll
                for (int v = 0; v < NV; ++v) Uo[v] = mac(Uo[v], o.phif[f][j][i], Ue[i * NV + v]);
#pragma unroll
            for (int v = 0; v < NV; ++v) Uo[v] = settle(Uo[v]);
            const int k = rev ? NFQ - 1 - j : j;
            if (!ONEPASS && nb >= 0) {
#pragma unroll
                for (int v = 0; v < NV; ++v) Ut[0][v] = T(0);
#pragma unroll
                for (int i = 0; i < NP; ++i) {
                    T c[4];
                    nrow(i, c);
                    const T ph = o.phif[nf][k][i];
#pragma unroll
                    for (int v = 0; v < NV; ++v) Ut[0][v] = mac(Ut[0][v], ph, c[v]);
                }
#pragma unroll
                for (int v = 0; v < NV; ++v) Ut[0][v] = settle(Ut[0][v]);
            }
            const T* Un = Ut[ONEPASS ? j : 0];
            T H[4] = {T(0), T(0), T(0), T(0)};
            if (nb >= 0) {
                rusanov<T>(Uo, Un, nx, ny, gamma, H);
            } else {
                T Ub[4];
                if (inviscid_ghost<T>(bc, Uo, nx, ny, gamma, Ub)) rusanov<T>(Uo, Ub, nx, ny, gamma, H);
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
                T A[4];
                quad_inverse_map<T>(G, o.xf[f][j][0], o.xf[f][j][1], A);
                T gx[4], gy[4], Fv[4], Gv[4];
#pragma unroll
                for (int v = 0; v < NV; ++v) {
                    gx[v] = A[0] * gr[v] + A[1] * gs[v];
                    gy[v] = A[2] * gr[v] + A[3] * gs[v];
                }
                viscous_flux<T>(Uo, gx, gy, gamma, mu, kappa, Fv, Gv);
                if (nb >= 0) {
                    T nr[4] = {T(0), T(0), T(0), T(0)}, ns[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
                    for (int i = 0; i < NP; ++i) {
                        T c[4];
                        nrow(i, c);
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
                    T B[4];
                    quad_inverse_map<T>(geoms[nb], o.xf[nf][k][0], o.xf[nf][k][1], B);
                    T hx[4], hy[4], Fn2[4], Gn2[4];
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        hx[v] = B[0] * nr[v] + B[1] * ns[v];
                        hy[v] = B[2] * nr[v] + B[3] * ns[v];
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
            const T w = o.wf[j] * hF * T(0.5);
#pragma unroll
            for (int i = 0; i < NP; ++i) {
                const T sc = w * o.phif[f][j][i];
#pragma unroll
                for (int v = 0; v < NV; ++v) R[i][v] = mac(R[i][v], -sc, H[v]);
            }
        }
    }
}

// M_K^-1 applied to the row r (this thread's NP x 4 values, overwritten) in arithmetic A
// from tables of type B: r <- D^-1 Phi^T diag(w_q / |J_q|) Phi D^-1 r, accumulated in acc.
template <int P, typename A, typename B, typename RT, class QG>
__device__ __forceinline__ void quad_mass_inv_row(const B (&phi)[n_basis_quad(P)][n_basis_quad(P)],
                                                  const B (&wq)[n_basis_quad(P)], const B (&xq)[n_basis_quad(P)][2],
                                                  const B (&dinv)[n_basis_quad(P)], const QG& G, RT* r,
                                                  A acc[n_basis_quad(P)][NV]) {
    constexpr int NP = n_basis_quad(P), NQ = NP;
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            r[i * NV + v] = (RT)((A)r[i * NV + v] * (A)dinv[i]);
            acc[i][v] = A(0);
        }
#pragma unroll 1
    for (int q = 0; q < NQ; ++q) {
        A y[4] = {A(0), A(0), A(0), A(0)};
#pragma unroll
        for (int k = 0; k < NP; ++k)
#pragma unroll
            for (int v = 0; v < NV; ++v) y[v] += (A)phi[q][k] * (A)r[k * NV + v];
        A J00, J01, J10, J11;
        quad_jacobian<A>(G, (A)xq[q][0], (A)xq[q][1], J00, J01, J10, J11);
        const A det = J00 * J11 - J10 * J01;
        const A s = (A)wq[q] / (det < A(0) ? -det : det);
#pragma unroll
        for (int i = 0; i < NP; ++i) {
            const A ph = (A)phi[q][i] * s;
#pragma unroll
            for (int v = 0; v < NV; ++v) acc[i][v] += ph * y[v];
        }
    }
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
        for (int v = 0; v < NV; ++v) r[i * NV + v] = (RT)((A)dinv[i] * acc[i][v]);
}

template <int P>
__device__ __forceinline__ void quad_mass_inv_row64(const MassOps<P>& m, const QuadGeom& G, double* r,
                                                    double acc[n_basis_quad(P)][NV]) {
    quad_mass_inv_row<P, double, double, double>(m.phi, m.wq, m.xq, m.dinv, G, r, acc);
}

template <int P, typename T, bool VISC>
__global__ void __launch_bounds__(TILE, 1) quad_element_kernel(const __grid_constant__ QKArgs<P, T, VISC> ka) {
    constexpr int NP = n_basis_quad(P), NB = NP * NV, STR = NB + 1;
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
        quad_residual<P, T, VISC, STR>(ka.o, sU + tl * STR, sU, e0, nloc, getrow, ka.geom[e], ka.conn[e], s.bc,
                                       ka.geom, (T)s.gamma, mu, kappa, (T)s.sigma0, R);
    }
    __syncthreads();  // all neighbour reads of sU are done

    // ---------------- epilogue: residual, or M_K^-1 R (apply_mass_inv,
    // compressible_solver_base.cpp:54-61) and the SSP-RK3 combination (time_stepping.hpp:39-55)
    double* sD = reinterpret_cast<double*>(smem_raw);  // [TILE][STR] doubles, reuses sU
    if (active) {
#pragma unroll
        for (int i = 0; i < NP; ++i)
#pragma unroll
            for (int v = 0; v < NV; ++v) sD[tl * STR + i * NV + v] = to_f64(R[i][v]);
        if (s.mode != MODE_RESIDUAL) {
            double acc[NP][NV];
            quad_mass_inv_row64<P>(qk_mass(ka), ka.geom[e], sD + tl * STR, acc);
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

template <int P, typename T>
inline size_t quad_smem_bytes() {
    return (size_t)TILE * (n_basis_quad(P) * NV + 1) * sizeof(double);
}

template <int P, typename T, bool VISC>
inline int configure_quad_t() {
    if (cudaFuncSetAttribute(quad_element_kernel<P, T, VISC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)quad_smem_bytes<P, T>()) != cudaSuccess)
        return -1;
    if constexpr (P == 4) {
        auto h = std::make_unique<OpsHost>();
        auto m = std::make_unique<MassOps<4>>();
        if (make_ops(4, DGX_BASIS_LEGENDRE, *h)) return -1;
        fill_mass_ops<4>(*h, *m);
        if (cudaMemcpyToSymbol(c_quad_mass4, m.get(), sizeof(MassOps<4>)) != cudaSuccess) return -1;
    }
    return 0;
}

template <int P, typename T, bool VISC>
inline int launch_quad_t(const StepArgs& a, const QuadGeom* geom, const QuadConn* conn, const OpsHost& oh,
                         cudaStream_t st) {
    static_assert(sizeof(QKArgs<P, T, VISC>) <= 32764, "quadrilateral kernel arguments exceed the parameter limit");
    QKArgs<P, T, VISC> ka;  // by value: operator reads are constant-bank operands
    ka.s = a;
    ka.geom = geom;
    ka.conn = conn;
    fill_quad_ops<P, T>(oh, ka.o);
    if constexpr (P < 4) fill_mass_ops<P>(oh, ka.m);
    const int grid = (a.ne + TILE - 1) / TILE;
    if (grid == 0) return 0;
    quad_element_kernel<P, T, VISC><<<grid, TILE, quad_smem_bytes<P, T>(), st>>>(ka);
    return launch_status();
}

#define DGX_QUAD_DISPATCH(FN, T, ARGS)               \
    switch (p * 2 + (viscous ? 1 : 0)) {             \
    case 2: return FN<1, T, false> ARGS;             \
    case 3: return FN<1, T, true> ARGS;              \
    case 4: return FN<2, T, false> ARGS;             \
    case 5: return FN<2, T, true> ARGS;              \
    case 6: return FN<3, T, false> ARGS;             \
    case 7: return FN<3, T, true> ARGS;              \
    case 8: return FN<4, T, false> ARGS;             \
    case 9: return FN<4, T, true> ARGS;              \
    default: return -1;                              \
    }

// ---------------------------------------------------------------------------------
// Mixed-precision SSP-RK3 stage on quadrilaterals, the increment form of StageArgs
// (dgx_internal.h): the stage state is uhi + din in FP32, stages 1 and 2 write FP32
// increments and stage 3 adds into the state (stage_combine, rk3_next).  No FP64 arithmetic or
// FP64 loads in stages 1 and 2: converting FP64 neighbour rows cost the element kernel's
// FP32 form more FP64-pipe time than its residual took FP32-pipe time.
template <int P>
__host__ __device__ constexpr int quad_stage_stride() {  // floats; a 16-byte row count that is odd
    return ((n_basis_quad(P) * NV / 4) & 1) ? n_basis_quad(P) * NV : n_basis_quad(P) * NV + 4;
}

template <int P, bool VISC>
struct QSArgs {
    StageArgs s;
    QuadOps<P, float> o;
};

template <int P, bool VISC>
__global__ void __launch_bounds__(TILE, 1) quad_stage_kernel(const __grid_constant__ QSArgs<P, VISC> ka) {
    constexpr int NP = n_basis_quad(P), NB = NP * NV, STR = quad_stage_stride<P>();
    const StageArgs& s = ka.s;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* sU = reinterpret_cast<float*>(smem_raw);  // [TILE][STR]
    float* sDt = sU + TILE * STR;                     // [TILE] (per-instance dt; unused here)

    const int e0 = blockIdx.x * TILE;
    const int nloc = min(TILE, s.ne - e0);
    const int tl = threadIdx.x;
    const bool active = tl < nloc;
    const int e = e0 + tl;
    if (tl == 0 && s.stage == 3)  // u^n is read back in the stage combination
        rk3_prefetch(s, (size_t)e0 * NB, nloc * NB);
    stage_load_tile<NB, STR>(s.uhi, s.din, sU, e0, nloc, [](int le) { return le; });
    __syncthreads();

    float R[NP][NV];
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
        for (int v = 0; v < NV; ++v) R[i][v] = 0.0f;
    if (active) {
        const float* uhi = s.uhi;
        const float* din = s.din;
        auto getrow = [uhi, din](int nb, int i, float c[4]) { load_row_f32<NB>(uhi, din, nb, i, c); };
        quad_residual<P, float, VISC, STR>(ka.o, sU + tl * STR, sU, e0, nloc, getrow, s.qgeom[e], s.qconn[e], s.bc,
                                           s.qgeom, s.gamma, s.mu, s.kappa, s.sigma0, R);
    }
    __syncthreads();  // all neighbour reads of sU are done
    if (active) {
#pragma unroll
        for (int i = 0; i < NP; ++i)
            *reinterpret_cast<float4*>(sU + tl * STR + i * NV) = make_float4(R[i][0], R[i][1], R[i][2], R[i][3]);
        float acc[NP][NV];
        quad_mass_inv_row<P, float, float, float>(ka.o.phi, ka.o.wq, ka.o.xq, ka.o.dinv, s.qgeom[e], sU + tl * STR,
                                                  acc);
    }
    __syncthreads();
    stage_combine<NB, STR, TILE, 2>(s, sU, sDt, e0, nloc, [](int le) { return le; });
}

template <int P, bool VISC>
inline size_t quad_stage_smem_bytes() {
    return (size_t)(TILE * quad_stage_stride<P>() + TILE) * sizeof(float);
}

template <int P, bool VISC>
inline int configure_quad_stage_t() {
    return cudaFuncSetAttribute(quad_stage_kernel<P, VISC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)quad_stage_smem_bytes<P, VISC>()) == cudaSuccess
               ? 0
               : -1;
}

template <int P, bool VISC>
inline int launch_quad_stage_t(const StageArgs& a, const OpsHost& oh, cudaStream_t st) {
    static_assert(sizeof(QSArgs<P, VISC>) <= 32764, "quadrilateral stage arguments exceed the parameter limit");
    QSArgs<P, VISC> ka;
    ka.s = a;
    fill_quad_ops<P, float>(oh, ka.o);
    const int grid = (a.ne + TILE - 1) / TILE;
    if (grid == 0) return 0;
    quad_stage_kernel<P, VISC><<<grid, TILE, quad_stage_smem_bytes<P, VISC>(), st>>>(ka);
    return launch_status();
}

}  // namespace dgx
