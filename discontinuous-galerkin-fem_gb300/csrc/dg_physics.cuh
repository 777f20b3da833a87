// Pointwise physics of the DG path on the device: conserved/primitive conversion,
// Euler fluxes, the Rusanov numerical flux and the laminar viscous flux, templated on
// the arithmetic type (double for the FP64 path, float for the mixed path).
#pragma once

#include "../../include/dgx.h"
#include "dgx_internal.h"
#include "fp_bits.cuh"

namespace dgx {

// Reciprocal and square root.  FP64: correctly rounded (the oracle's arithmetic).  FP32 (the
// mixed path): the hardware approximations rcp.approx.f32 / sqrt.approx.f32 (about one ulp,
// bounded in tests/cpp/test_fast_math.cu) instead of the correctly rounded sequences, whose
// extra refinement steps and slow-path branches cost 6 % of the stage; the 500-step error of
// the mixed path against FP64 stays 4.68e-7 either way (512x512x2 vortex, p=3).
template <typename T>
__device__ __forceinline__ T rcp_(T x);
template <>
__device__ __forceinline__ double rcp_<double>(double x) { return 1.0 / x; }
template <>
__device__ __forceinline__ float rcp_<float>(float x) {
    float r;
    asm("rcp.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
template <typename T>
__device__ __forceinline__ T sqrt_(T x);
template <>
__device__ __forceinline__ double sqrt_<double>(double x) { return sqrt(x); }
template <>
__device__ __forceinline__ float sqrt_<float>(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// acc + a*b (one FMA for float / double); settle(x): x with its representation normalised.
// Types with their own fused form (double-float) provide overloads.
template <typename C, typename A, typename B>
__device__ __forceinline__ C mac(C acc, A a, B b) { return acc + a * b; }
template <typename C>
__device__ __forceinline__ C settle(C x) { return x; }

// the value as FP64: exact; from FP32 on the integer pipe (fp_bits.cuh)
__device__ __forceinline__ double to_f64(double x) { return x; }
__device__ __forceinline__ double to_f64(float x) { return f32_to_f64_bits(x); }
template <typename T>
__device__ __forceinline__ double to_f64(T x) { return (double)x; }

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

// Exterior state of a boundary face for the inviscid flux (EulerWeakFormulation::
// boundary_face_residual, src/weak_forms/euler_weak_formulation.cpp:177-250): the far-field
// state, the interior state with its normal velocity reflected (slip wall), or the no-slip
// wall's primitive state.  False when the condition contributes no inviscid flux.
template <typename T>
__device__ __forceinline__ bool inviscid_ghost(const BCSlot& bc, const T Uo[4], T nx, T ny, T gamma, T Ub[4]) {
    if (bc.type == DGX_BC_FAR_FIELD) {
#pragma unroll
        for (int v = 0; v < 4; ++v) Ub[v] = (T)bc.value[v];
        return true;
    }
    if (bc.type == DGX_BC_SLIP_WALL) {
        const T rr = rcp_<T>(Uo[0]);
        const T u = Uo[1] * rr, vv = Uo[2] * rr;
        const T p = (gamma - T(1)) * (Uo[3] - T(0.5) * Uo[0] * (u * u + vv * vv));
        const T un = u * nx + vv * ny;
        const T W[4] = {Uo[0], (u - un * nx) - un * nx, (vv - un * ny) - un * ny, p};
        p2c<T>(W, gamma, Ub);
        return true;
    }
    if (bc.type == DGX_BC_NO_SLIP_WALL) {
        const T W[4] = {(T)bc.value[0], (T)bc.value[1], (T)bc.value[2], (T)bc.value[3]};
        p2c<T>(W, gamma, Ub);
        return true;
    }
    return false;
}

// Boundary state of the viscous penalty term (NavierStokesWeakFormulation::
// viscous_boundary_face_residual, src/weak_forms/navier_stokes_weak_formulation.cpp:209-273):
// the no-slip wall's primitive state in conserved form, else the condition's value as given.
template <typename T>
__device__ __forceinline__ void viscous_ghost(const BCSlot& bc, T gamma, T Ub[4]) {
    if (bc.type == DGX_BC_NO_SLIP_WALL) {
        const T W[4] = {(T)bc.value[0], (T)bc.value[1], (T)bc.value[2], (T)bc.value[3]};
        p2c<T>(W, gamma, Ub);
    } else {
#pragma unroll
        for (int v = 0; v < 4; ++v) Ub[v] = (T)bc.value[v];
    }
}

}  // namespace dgx
