// Quadrilateral kernels: the FP64 element kernel (dg_quad.cuh) and the standalone inverse
// mass matrix, L2 projection and CFL / density monitor for bilinear quadrilaterals.
#include "dg_quad.cuh"

namespace dgx {

int configure_quad_element(int p, bool viscous, int precision) {
    if (precision == DGX_DF64) return configure_quad_element_df64(p, viscous);
    if (precision == DGX_MIXED) { DGX_QUAD_DISPATCH(configure_quad_t, float, ()) }
    DGX_QUAD_DISPATCH(configure_quad_t, double, ())
}

int launch_quad_element(int p, bool viscous, int precision, const StepArgs& a, const QuadGeom* geom,
                        const QuadConn* conn, const OpsHost& ops, cudaStream_t s) {
    if (precision == DGX_DF64) return launch_quad_element_df64(p, viscous, a, geom, conn, ops, s);
    if (precision == DGX_MIXED) { DGX_QUAD_DISPATCH(launch_quad_t, float, (a, geom, conn, ops, s)) }
    DGX_QUAD_DISPATCH(launch_quad_t, double, (a, geom, conn, ops, s))
}

#define DGX_QUAD_STAGE_DISPATCH(FN, ARGS)        \
    switch (p * 2 + (viscous ? 1 : 0)) {         \
    case 2: return FN<1, false> ARGS;            \
    case 3: return FN<1, true> ARGS;             \
    case 4: return FN<2, false> ARGS;            \
    case 5: return FN<2, true> ARGS;             \
    case 6: return FN<3, false> ARGS;            \
    case 7: return FN<3, true> ARGS;             \
    case 8: return FN<4, false> ARGS;            \
    case 9: return FN<4, true> ARGS;             \
    default: return -1;                          \
    }

int configure_quad_stage(int p, bool viscous) { DGX_QUAD_STAGE_DISPATCH(configure_quad_stage_t, ()) }

int launch_quad_stage(int p, bool viscous, const StageArgs& a, const OpsHost& ops, cudaStream_t s) {
    DGX_QUAD_STAGE_DISPATCH(launch_quad_stage_t, (a, ops, s))
}

// CompressibleDGSolverBase::apply_mass_inv (src/solver/compressible_solver_base.cpp:54-61)
template <int P>
__global__ void quad_mass_inv_kernel(const __grid_constant__ QuadOps<P, double> o, int ne, const QuadGeom* geom,
                                     const double* in, double* out) {
    constexpr int NP = n_basis_quad(P);
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double r[NP * NV], acc[NP][NV];
    const double* a = in + (size_t)e * NP * NV;
#pragma unroll
    for (int k = 0; k < NP * NV; ++k) r[k] = a[k];
    quad_mass_inv_row<P, double, double, double>(o.phi, o.wq, o.xq, o.dinv, geom[e], r, acc);
    double* b = out + (size_t)e * NP * NV;
#pragma unroll
    for (int k = 0; k < NP * NV; ++k) b[k] = r[k];
}

// CompressibleDGSolverBase::project_initial_condition (compressible_solver_base.cpp:63-104):
// F = sum_q w_q |J_q| phi_q U_q, then M_K^-1 F.
template <int P>
__global__ void quad_project_kernel(const __grid_constant__ QuadOps<P, double> o, int ne, const QuadGeom* geom,
                                    const double* uq, double* u) {
    constexpr int NP = n_basis_quad(P), NQ = NP;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const QuadGeom& G = geom[e];
    double F[NP * NV], acc[NP][NV];
#pragma unroll
    for (int k = 0; k < NP * NV; ++k) F[k] = 0.0;
    const double* U = uq + (size_t)e * NQ * NV;
    for (int q = 0; q < NQ; ++q) {
        double J00, J01, J10, J11;
        quad_jacobian<double>(G, o.xq[q][0], o.xq[q][1], J00, J01, J10, J11);
        const double w = o.wq[q] * fabs(J00 * J11 - J10 * J01);
#pragma unroll
        for (int i = 0; i < NP; ++i) {
            const double s = w * o.phi[q][i];
#pragma unroll
            for (int v = 0; v < NV; ++v) F[i * NV + v] += s * U[q * NV + v];
        }
    }
    quad_mass_inv_row<P, double, double, double>(o.phi, o.wq, o.xq, o.dinv, G, F, acc);
    double* b = u + (size_t)e * NP * NV;
#pragma unroll
    for (int k = 0; k < NP * NV; ++k) b[k] = F[k];
}

__device__ __forceinline__ void quad_atomic_max(double* addr, double v) {
    unsigned long long* a = reinterpret_cast<unsigned long long*>(addr);
    unsigned long long old = *a;
    while (__longlong_as_double(old) < v) {
        const unsigned long long prev = atomicCAS(a, old, __double_as_longlong(v));
        if (prev == old) break;
        old = prev;
    }
}
__device__ __forceinline__ void quad_atomic_min(double* addr, double v) {
    unsigned long long* a = reinterpret_cast<unsigned long long*>(addr);
    unsigned long long old = *a;
    while (__longlong_as_double(old) > v) {
        const unsigned long long prev = atomicCAS(a, old, __double_as_longlong(v));
        if (prev == old) break;
        old = prev;
    }
}

// compute_max_cfl + compute_density_range (compressible_solver_base.cpp:114-199), the
// output layout of the triangle monitor: out = {max CFL, rho min, rho max, bad point}.
template <int P>
__global__ void quad_monitor_kernel(const __grid_constant__ QuadOps<P, double> o, int ne, const QuadGeom* geom,
                                    const double* u, double dt, double gamma, double* out) {
    constexpr int NP = n_basis_quad(P), NQ = NP;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    double cfl = 0.0, lo = INFINITY, hi = -INFINITY, bad = 0.0;
    if (e < ne) {
        const double* ue = u + (size_t)e * NP * NV;
        double mws = 0.0;
        for (int q = 0; q < NQ; ++q) {
            double U[4] = {0, 0, 0, 0};
#pragma unroll
            for (int i = 0; i < NP; ++i)
#pragma unroll
                for (int v = 0; v < NV; ++v) U[v] += o.phi[q][i] * ue[i * NV + v];
            const double rho = U[0];
            if (isfinite(rho)) {
                lo = fmin(lo, rho);
                hi = fmax(hi, rho);
            }
            if (rho <= 0.0 || !isfinite(rho)) { bad = 1.0; continue; }
            const double uu = U[1] / rho, vv = U[2] / rho;
            const double p = (gamma - 1.0) * (U[3] - rho * (0.5 * (uu * uu + vv * vv)));
            if (p <= 0.0 || !isfinite(p)) { bad = 1.0; continue; }
            const double c = sqrt(fmax(gamma * p / rho, 0.0));
            mws = fmax(mws, sqrt(uu * uu + vv * vv) + c);
        }
        cfl = dt * mws / geom[e].hmin;
    }
    for (int off = 16; off > 0; off >>= 1) {
        cfl = fmax(cfl, __shfl_down_sync(0xffffffffu, cfl, off));
        lo = fmin(lo, __shfl_down_sync(0xffffffffu, lo, off));
        hi = fmax(hi, __shfl_down_sync(0xffffffffu, hi, off));
        bad = fmax(bad, __shfl_down_sync(0xffffffffu, bad, off));
    }
    if ((threadIdx.x & 31) == 0) {
        quad_atomic_max(out + 0, cfl);
        quad_atomic_min(out + 1, lo);
        quad_atomic_max(out + 2, hi);
        if (bad > 0.0) quad_atomic_max(out + 3, 1.0);
    }
}

#define DGX_QUAD_P(p, ...)                             \
    switch (p) {                                       \
    case 1: { constexpr int P = 1; __VA_ARGS__; break; } \
    case 2: { constexpr int P = 2; __VA_ARGS__; break; } \
    case 3: { constexpr int P = 3; __VA_ARGS__; break; } \
    case 4: { constexpr int P = 4; __VA_ARGS__; break; } \
    default: return -1;                                \
    }

int launch_quad_mass_inv(int ne, int p, const OpsHost& ops, const QuadGeom* geom, const double* in, double* out,
                         cudaStream_t s) {
    if (ne == 0) return 0;
    const int grid = (ne + 127) / 128;
    DGX_QUAD_P(p, QuadOps<P, double> o; fill_quad_ops<P, double>(ops, o);
               quad_mass_inv_kernel<P><<<grid, 128, 0, s>>>(o, ne, geom, in, out))
    return launch_status();
}

int launch_quad_project(int ne, int p, const OpsHost& ops, const QuadGeom* geom, const double* uq, double* u,
                        cudaStream_t s) {
    if (ne == 0) return 0;
    const int grid = (ne + 127) / 128;
    DGX_QUAD_P(p, QuadOps<P, double> o; fill_quad_ops<P, double>(ops, o);
               quad_project_kernel<P><<<grid, 128, 0, s>>>(o, ne, geom, uq, u))
    return launch_status();
}

int launch_quad_monitor(int ne, int p, const OpsHost& ops, const QuadGeom* geom, const double* u, double dt,
                        double gamma, double* d_out, cudaStream_t s) {
    const double init[4] = {0.0, INFINITY, -INFINITY, 0.0};
    if (cudaMemcpyAsync(d_out, init, sizeof(init), cudaMemcpyHostToDevice, s) != cudaSuccess) return -1;
    if (ne == 0) return 0;
    const int grid = (ne + 127) / 128;
    DGX_QUAD_P(p, QuadOps<P, double> o; fill_quad_ops<P, double>(ops, o);
               quad_monitor_kernel<P><<<grid, 128, 0, s>>>(o, ne, geom, u, dt, gamma, d_out))
    return launch_status();
}

}  // namespace dgx
