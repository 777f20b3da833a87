// Fused element kernel of the explicit DG path: volume flux integral, the three faces'
// numerical fluxes lifted to the element's modes, the inverse mass matrix and the
// SSP-RK3 stage combination, one thread per element.
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
#pragma once

#include "dgx_internal.h"

namespace dgx {

template <int P, typename T, bool VISC>
struct KArgs {
    StepArgs s;
    Ops<P, T> o;
    double minv64[n_basis(P)][n_basis(P)];  // FP64 inverse reference mass matrix
};

template <typename T>
__device__ __forceinline__ T rcp_(T x);
template <>
__device__ __forceinline__ double rcp_<double>(double x) { return 1.0 / x; }
template <>
__device__ __forceinline__ float rcp_<float>(float x) { return __frcp_rn(x); }
template <typename T>
__device__ __forceinline__ T sqrt_(T x);
template <>
__device__ __forceinline__ double sqrt_<double>(double x) { return sqrt(x); }
template <>
__device__ __forceinline__ float sqrt_<float>(float x) { return __fsqrt_rn(x); }

// get_fluxes_and_primitive, src/weak_forms/euler_weak_formulation.cpp:27-43
template <typename T>
__device__ __forceinline__ void euler_flux(const T U[4], T gm1, T F[4], T G[4], T& u, T& v, T& p,
                                           T& ri) {
    const T rho = U[0];
    ri = rcp_<T>(rho);
    u = U[1] * ri;
    v = U[2] * ri;
    p = gm1 * (U[3] - T(0.5) * rho * (u * u + v * v));
    const T ruv = rho * u * v;
    F[0] = U[1];
    F[1] = rho * u * u + p;
    F[2] = ruv;
    F[3] = u * (U[3] + p);
    G[0] = U[2];
    G[1] = ruv;
    G[2] = rho * v * v + p;
    G[3] = v * (U[3] + p);
}

// EulerWeakFormulation::rusanov_flux, src/weak_forms/euler_weak_formulation.cpp:51-70
template <typename T>
__device__ __forceinline__ void rusanov(const T UL[4], const T UR[4], T nx, T ny, T gamma, T H[4]) {
    T FL[4], GL[4], FR[4], GR[4], uL, vL, pL, riL, uR, vR, pR, riR;
    euler_flux<T>(UL, gamma - T(1), FL, GL, uL, vL, pL, riL);
    euler_flux<T>(UR, gamma - T(1), FR, GR, uR, vR, pR, riR);
    const T cL = sqrt_<T>(gamma * pL * riL);
    const T cR = sqrt_<T>(gamma * pR * riR);
    const T a = fabs(uL * nx + vL * ny) + cL;
    const T b = fabs(uR * nx + vR * ny) + cR;
    const T hs = T(0.5) * (a < b ? b : a);
#pragma unroll
    for (int v = 0; v < 4; ++v) {
        const T fnl = FL[v] * nx + GL[v] * ny;
        const T fnr = FR[v] * nx + GR[v] * ny;
        H[v] = T(0.5) * (fnl + fnr) - hs * (UR[v] - UL[v]);
    }
}

// NavierStokesWeakFormulation::compute_primitive_gradients + compute_viscous_fluxes,
// src/weak_forms/navier_stokes_weak_formulation.cpp:36-98 (gas constant 1).
// gx, gy: physical gradients of the conserved variables.
template <typename T>
__device__ __forceinline__ void viscous_flux(const T U[4], const T gx[4], const T gy[4], T gamma,
                                             T mu, T kappa, T Fv[4], T Gv[4]) {
    const T rho = U[0];
    const T ri = rcp_<T>(rho);
    const T ri_safe = rcp_<T>(rho > T(1e-12) ? rho : T(1e-12));
    const T u = U[1] * ri, v = U[2] * ri;
    const T p = (gamma - T(1)) * (U[3] - T(0.5) * rho * (u * u + v * v));
    const T gux = (gx[1] - u * gx[0]) * ri_safe, guy = (gy[1] - u * gy[0]) * ri_safe;
    const T gvx = (gx[2] - v * gx[0]) * ri_safe, gvy = (gy[2] - v * gy[0]) * ri_safe;
    const T ksq = T(0.5) * (u * u + v * v);
    const T gpx = (gamma - T(1)) * (gx[3] - ksq * gx[0] - rho * (u * gux + v * gvx));
    const T gpy = (gamma - T(1)) * (gy[3] - ksq * gy[0] - rho * (u * guy + v * gvy));
    const T irho2 = ri * ri;
    const T gTx = (rho * gpx - p * gx[0]) * irho2;
    const T gTy = (rho * gpy - p * gy[0]) * irho2;
    const T div = gux + gvy;
    const T lam = T(-2.0 / 3.0) * mu;
    const T txx = T(2) * mu * gux + lam * div;
    const T tyy = T(2) * mu * gvy + lam * div;
    const T txy = mu * (guy + gvx);
    Fv[0] = T(0);
    Fv[1] = txx;
    Fv[2] = txy;
    Fv[3] = u * txx + v * txy - kappa * gTx;
    Gv[0] = T(0);
    Gv[1] = txy;
    Gv[2] = tyy;
    Gv[3] = u * txy + v * tyy - kappa * gTy;
}

template <typename T>
__device__ __forceinline__ void p2c(const T W[4], T gamma, T U[4]) {
    U[0] = W[0];
    U[1] = W[0] * W[1];
    U[2] = W[0] * W[2];
    U[3] = W[3] / (gamma - T(1)) + T(0.5) * W[0] * (W[1] * W[1] + W[2] * W[2]);
}

template <int P, typename T, bool VISC>
__global__ void __launch_bounds__(TILE) element_kernel(const __grid_constant__ KArgs<P, T, VISC> ka) {
    constexpr int NP = n_basis(P), NQ = n_quad(P), NFQ = P + 1, NB = NP * NV, STR = NB + 1;
    const StepArgs& s = ka.s;
    const Ops<P, T>& o = ka.o;
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
        const T gamma = (T)s.gamma;
        const ElemGeom& G = s.geom[e];
        const T A00 = (T)G.A[0], A01 = (T)G.A[1], A10 = (T)G.A[2], A11 = (T)G.A[3];
        const T detJ = (T)G.detJ;
        const T* Ue = sU + tl * STR;
        T mu = T(0), kappa = T(0);
        if (VISC) {
            mu = (T)s.mu;
            kappa = (T)(s.mu * s.gamma / (s.prandtl * (s.gamma - 1.0)));
        }

        // ---------------- volume: EulerWeakFormulation::volume_residual (:72-115)
        //                  + NavierStokesWeakFormulation::viscous_volume_residual (:100-140)
#pragma unroll 1
        for (int q = 0; q < NQ; ++q) {
            T U[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
            for (int i = 0; i < NP; ++i)
#pragma unroll
                for (int v = 0; v < NV; ++v) U[v] += o.phi[q][i] * Ue[i * NV + v];
            T F[4], Gf[4], u, vv, pp, ri;
            euler_flux<T>(U, gamma - T(1), F, Gf, u, vv, pp, ri);
            if (VISC) {
                T gr[4] = {T(0), T(0), T(0), T(0)}, gs[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
                for (int i = 0; i < NP; ++i)
#pragma unroll
                    for (int v = 0; v < NV; ++v) {
                        gr[v] += o.dr[q][i] * Ue[i * NV + v];
                        gs[v] += o.ds[q][i] * Ue[i * NV + v];
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
            const T w = o.wq[q] * detJ;
            T Fr[4], Fs[4];
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                Fr[v] = w * (A00 * F[v] + A10 * Gf[v]);
                Fs[v] = w * (A01 * F[v] + A11 * Gf[v]);
            }
#pragma unroll
            for (int i = 0; i < NP; ++i)
#pragma unroll
                for (int v = 0; v < NV; ++v) R[i][v] += o.dr[q][i] * Fr[v] + o.ds[q][i] * Fs[v];
        }

        // ---------------- faces: interior_face_residual (:117-175), boundary_face_residual
        //                  (:177-250) and their viscous counterparts (NS :142-273)
        const ElemConn C = s.conn[e];
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
            const double* Un_g = nullptr;
            T B00 = T(0), B01 = T(0), B10 = T(0), B11 = T(0);
            BCSlot bc;
            bc.type = -1;
            if (nb >= 0) {
                if (nb >= e0 && nb < e0 + nloc) Un_s = sU + (nb - e0) * STR;
                else Un_g = s.u + (size_t)nb * NB;
                if (VISC) {
                    const ElemGeom& GN = s.geom[nb];
                    B00 = (T)GN.A[0]; B01 = (T)GN.A[1]; B10 = (T)GN.A[2]; B11 = (T)GN.A[3];
                }
            } else {
                bc = s.bc[-1 - nb];
            }
            // NavierStokesWeakFormulation::compute_penalty_parameter (:275-278)
            const T sigma = VISC ? (T)s.sigma0 * mu * T((P + 1) * (P + 1)) /
                                       (hF > T(1e-12) ? hF : T(1e-12))
                                 : T(0);
#pragma unroll 1
            for (int j = 0; j < NFQ; ++j) {
                T Uo[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
                for (int i = 0; i < NP; ++i)
#pragma unroll
                    for (int v = 0; v < NV; ++v) Uo[v] += o.phif[f][j][i] * Ue[i * NV + v];
                T Un[4] = {T(0), T(0), T(0), T(0)};
                const int k = rev ? NFQ - 1 - j : j;
                if (nb >= 0) {
                    if (Un_s) {
#pragma unroll
                        for (int i = 0; i < NP; ++i)
#pragma unroll
                            for (int v = 0; v < NV; ++v) Un[v] += o.phif[nf][k][i] * Un_s[i * NV + v];
                    } else {
#pragma unroll
                        for (int i = 0; i < NP; ++i) {
                            const double2 c0 = __ldg(reinterpret_cast<const double2*>(Un_g + i * NV));
                            const double2 c1 = __ldg(reinterpret_cast<const double2*>(Un_g + i * NV + 2));
                            const T ph = o.phif[nf][k][i];
                            Un[0] += ph * (T)c0.x;
                            Un[1] += ph * (T)c0.y;
                            Un[2] += ph * (T)c1.x;
                            Un[3] += ph * (T)c1.y;
                        }
                    }
                }
                T H[4];
                if (nb >= 0) {
                    rusanov<T>(Uo, Un, nx, ny, gamma, H);
                } else if (bc.type == 0 /*FAR_FIELD*/ || bc.type == 1 || bc.type == 2) {
                    T Ub[4];
                    if (bc.type == 0) {
#pragma unroll
                        for (int v = 0; v < 4; ++v) Ub[v] = (T)bc.value[v];
                    } else if (bc.type == 1) {  // slip wall: reflect the normal velocity
                        const T ri = rcp_<T>(Uo[0]);
                        const T u = Uo[1] * ri, vv = Uo[2] * ri;
                        const T p = (gamma - T(1)) * (Uo[3] - T(0.5) * Uo[0] * (u * u + vv * vv));
                        const T un = u * nx + vv * ny;
                        const T W[4] = {Uo[0], (u - un * nx) - un * nx, (vv - un * ny) - un * ny, p};
                        p2c<T>(W, gamma, Ub);
                    } else {  // no-slip: primitive wall state
                        const T W[4] = {(T)bc.value[0], (T)bc.value[1], (T)bc.value[2], (T)bc.value[3]};
                        p2c<T>(W, gamma, Ub);
                    }
                    rusanov<T>(Uo, Ub, nx, ny, gamma, H);
                } else {
#pragma unroll
                    for (int v = 0; v < 4; ++v) H[v] = T(0);
                }
                if (VISC) {
                    // own-side gradient
                    T gr[4] = {T(0), T(0), T(0), T(0)}, gs[4] = {T(0), T(0), T(0), T(0)};
#pragma unroll
                    for (int i = 0; i < NP; ++i)
#pragma unroll
                        for (int v = 0; v < NV; ++v) {
                            gr[v] += o.drf[f][j][i] * Ue[i * NV + v];
                            gs[v] += o.dsf[f][j][i] * Ue[i * NV + v];
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
                            if (Un_s) {
#pragma unroll
                                for (int v = 0; v < NV; ++v) c[v] = Un_s[i * NV + v];
                            } else {
                                const double2 d0 = __ldg(reinterpret_cast<const double2*>(Un_g + i * NV));
                                const double2 d1 = __ldg(reinterpret_cast<const double2*>(Un_g + i * NV + 2));
                                c[0] = (T)d0.x; c[1] = (T)d0.y; c[2] = (T)d1.x; c[3] = (T)d1.y;
                            }
#pragma unroll
                            for (int v = 0; v < NV; ++v) {
                                nr[v] += o.drf[nf][k][i] * c[v];
                                ns[v] += o.dsf[nf][k][i] * c[v];
                            }
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
                        T Ub[4] = {Uo[0], Uo[1], Uo[2], Uo[3]};
                        if (bc.type == 2) {
                            const T W[4] = {(T)bc.value[0], (T)bc.value[1], (T)bc.value[2], (T)bc.value[3]};
                            p2c<T>(W, gamma, Ub);
                        } else {
#pragma unroll
                            for (int v = 0; v < 4; ++v) Ub[v] = (T)bc.value[v];
                        }
#pragma unroll
                        for (int v = 0; v < NV; ++v)
                            H[v] += (Fv[v] * nx + Gv[v] * ny) - sigma * (Ub[v] - Uo[v]);
                    }
                }
                const T w = o.wf[j] * hF * T(0.5);
#pragma unroll
                for (int i = 0; i < NP; ++i) {
                    const T sc = w * o.phif[f][j][i];
#pragma unroll
                    for (int v = 0; v < NV; ++v) R[i][v] -= sc * H[v];
                }
            }
        }
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
                for (int v = 0; v < NV; ++v) sD[tl * STR + i * NV + v] = (double)R[i][v];
        } else {
            const double ij = 1.0 / s.geom[e].detJ;
#pragma unroll
            for (int v = 0; v < NV; ++v) {
                double col[NP];
#pragma unroll
                for (int i = 0; i < NP; ++i) {
                    double acc = 0.0;
#pragma unroll
                    for (int k = 0; k < NP; ++k) acc += ka.minv64[i][k] * (double)R[k][v];
                    col[i] = acc * ij;
                }
#pragma unroll
                for (int i = 0; i < NP; ++i) sD[tl * STR + i * NV + v] = col[i];
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
    return cudaFuncSetAttribute(element_kernel<P, T, VISC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)element_smem_bytes<P, T, VISC>()) == cudaSuccess ? 0 : -1;
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
    return cudaGetLastError() == cudaSuccess ? 0 : -1;
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
