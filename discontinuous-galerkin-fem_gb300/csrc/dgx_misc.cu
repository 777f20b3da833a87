// FP64 utility kernels around the hot path: standalone inverse mass matrix, L2
// projection of an initial condition, CFL / density monitors and the NaN scan.
#include "dgx_internal.h"
#include "fp_bits.cuh"

namespace dgx {

struct MinvArgs {
    double minv[15][15];
    double phi[16][15];
    double wq[16];
};

static void fill_minv(const OpsHost& o, MinvArgs& m) {
    for (int i = 0; i < o.np; ++i)
        for (int j = 0; j < o.np; ++j) m.minv[i][j] = o.minv[i][j];
    for (int q = 0; q < o.nq; ++q) {
        m.wq[q] = o.wq[q];
        for (int i = 0; i < o.np; ++i) m.phi[q][i] = o.phi[q][i];
    }
}

// CompressibleDGSolverBase::apply_mass_inv, src/solver/compressible_solver_base.cpp:54-61,
// with M_K^-1 = M_ref^-1 / |J| for affine triangles.
template <int NP>
__global__ void mass_inv_kernel(const __grid_constant__ MinvArgs m, int ne, const ElemGeom* geom,
                                const double* in, double* out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const double ij = 1.0 / geom[e].detJ;
    double r[NP][NV];
    const double* a = in + (size_t)e * NP * NV;
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
        for (int v = 0; v < NV; ++v) r[i][v] = a[i * NV + v];
    double* o = out + (size_t)e * NP * NV;
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            double acc = 0.0;
#pragma unroll
            for (int k = 0; k < NP; ++k) acc += m.minv[i][k] * r[k][v];
            o[i * NV + v] = acc * ij;
        }
}

// CompressibleDGSolverBase::project_initial_condition, src/solver/compressible_solver_base.cpp:63-104
template <int NP, int NQ>
__global__ void project_kernel(const __grid_constant__ MinvArgs m, int ne, const ElemGeom* geom,
                               const double* uq, double* u) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const double dj = geom[e].detJ;
    double F[NP][NV];
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
        for (int v = 0; v < NV; ++v) F[i][v] = 0.0;
    const double* U = uq + (size_t)e * NQ * NV;
    for (int q = 0; q < NQ; ++q) {
        const double w = m.wq[q] * dj;
#pragma unroll
        for (int i = 0; i < NP; ++i) {
            const double s = w * m.phi[q][i];
#pragma unroll
            for (int v = 0; v < NV; ++v) F[i][v] += s * U[q * NV + v];
        }
    }
    double* o = u + (size_t)e * NP * NV;
    const double ij = 1.0 / dj;
#pragma unroll
    for (int i = 0; i < NP; ++i)
#pragma unroll
        for (int v = 0; v < NV; ++v) {
            double acc = 0.0;
#pragma unroll
            for (int k = 0; k < NP; ++k) acc += m.minv[i][k] * F[k][v];
            o[i * NV + v] = acc * ij;
        }
}

__device__ __forceinline__ void atomic_max_d(double* addr, double v) {
    unsigned long long* a = reinterpret_cast<unsigned long long*>(addr);
    unsigned long long old = *a;
    while (__longlong_as_double(old) < v) {
        const unsigned long long prev = atomicCAS(a, old, __double_as_longlong(v));
        if (prev == old) break;
        old = prev;
    }
}
__device__ __forceinline__ void atomic_min_d(double* addr, double v) {
    unsigned long long* a = reinterpret_cast<unsigned long long*>(addr);
    unsigned long long old = *a;
    while (__longlong_as_double(old) > v) {
        const unsigned long long prev = atomicCAS(a, old, __double_as_longlong(v));
        if (prev == old) break;
        old = prev;
    }
}

// compute_max_cfl + compute_density_range, src/solver/compressible_solver_base.cpp:114-199.
// out[0] = max CFL over elements, out[1] = rho min, out[2] = rho max (finite values only),
// out[3] = 1 when some point has rho <= 0, p <= 0 or a non-finite value (CFL = +inf).
template <int NP, int NQ>
__global__ void monitor_kernel(const __grid_constant__ MinvArgs m, int ne, const ElemGeom* geom,
                               const double* u, double dt, double gamma, double* out) {
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
                for (int v = 0; v < NV; ++v) U[v] += m.phi[q][i] * ue[i * NV + v];
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
        cfl = dt * mws / geom[e].pad[0];
    }
    for (int off = 16; off > 0; off >>= 1) {
        cfl = fmax(cfl, __shfl_down_sync(0xffffffffu, cfl, off));
        lo = fmin(lo, __shfl_down_sync(0xffffffffu, lo, off));
        hi = fmax(hi, __shfl_down_sync(0xffffffffu, hi, off));
        bad = fmax(bad, __shfl_down_sync(0xffffffffu, bad, off));
    }
    if ((threadIdx.x & 31) == 0) {
        atomic_max_d(out + 0, cfl);
        atomic_min_d(out + 1, lo);
        atomic_max_d(out + 2, hi);
        if (bad > 0.0) atomic_max_d(out + 3, 1.0);
    }
}

__global__ void has_nan_kernel(size_t n, const double* u, int* flag) {
    bool nan = false;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        nan |= isnan(u[i]);
    if (__any_sync(0xffffffffu, nan) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

__global__ void f64_to_f32_kernel(size_t n, const double* in, float* out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = f64_to_f32_bits(in[i]);  // on the integer pipe (fp_bits.cuh)
}

#define DGX_DISPATCH_P(p, ...)                                      \
    switch (p) {                                                    \
    case 1: { constexpr int NP = 3, NQ = 3; __VA_ARGS__; break; }   \
    case 2: { constexpr int NP = 6, NQ = 6; __VA_ARGS__; break; }   \
    case 3: { constexpr int NP = 10, NQ = 12; __VA_ARGS__; break; } \
    case 4: { constexpr int NP = 15, NQ = 16; __VA_ARGS__; break; } \
    default: return -1;                                             \
    }

int launch_mass_inv(int ne, int p, const OpsHost& ops, const ElemGeom* geom, const double* in,
                    double* out, cudaStream_t s) {
    if (ne == 0) return 0;
    MinvArgs m;
    fill_minv(ops, m);
    const int grid = (ne + 127) / 128;
    DGX_DISPATCH_P(p, (void)NQ; mass_inv_kernel<NP><<<grid, 128, 0, s>>>(m, ne, geom, in, out))
    return launch_status();
}

int launch_project(int ne, int p, const OpsHost& ops, const ElemGeom* geom, const double* uq,
                   double* u, cudaStream_t s) {
    if (ne == 0) return 0;
    MinvArgs m;
    fill_minv(ops, m);
    const int grid = (ne + 127) / 128;
    DGX_DISPATCH_P(p, (project_kernel<NP, NQ><<<grid, 128, 0, s>>>(m, ne, geom, uq, u)))
    return launch_status();
}

int launch_monitor(int ne, int p, const OpsHost& ops, const ElemGeom* geom, const double* u,
                   double dt, double gamma, double* d_out, cudaStream_t s) {
    MinvArgs m;
    fill_minv(ops, m);
    const double init[4] = {0.0, INFINITY, -INFINITY, 0.0};
    if (cudaMemcpyAsync(d_out, init, sizeof(init), cudaMemcpyHostToDevice, s) != cudaSuccess) return -1;
    if (ne == 0) return 0;
    const int grid = (ne + 127) / 128;
    DGX_DISPATCH_P(p, (monitor_kernel<NP, NQ><<<grid, 128, 0, s>>>(m, ne, geom, u, dt, gamma, d_out)))
    return launch_status();
}

int launch_has_nan(size_t n, const double* u, int* d_flag, cudaStream_t s) {
    if (cudaMemsetAsync(d_flag, 0, sizeof(int), s) != cudaSuccess) return -1;
    if (n == 0) return 0;
    size_t blocks = (n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    has_nan_kernel<<<(unsigned)blocks, 256, 0, s>>>(n, u, d_flag);
    return launch_status();
}

int prepare_f64_to_f32() {
    cudaFuncAttributes fa;
    return cudaFuncGetAttributes(&fa, f64_to_f32_kernel) == cudaSuccess ? 0 : -1;
}

int launch_f64_to_f32(size_t n, const double* in, float* out, cudaStream_t s) {
    if (n == 0) return 0;
    size_t blocks = (n + 255) / 256;
    if (blocks > 152 * 32) blocks = 152 * 32;
    f64_to_f32_kernel<<<(unsigned)blocks, 256, 0, s>>>(n, in, out);
    return launch_status();
}


// Point evaluation: out[(e * npts + k) * 4 + v] = sum_i phi[k][i] * u[(e * np + i) * 4 + v],
// one thread per (element, point).  phi holds the basis at reference points (host-built).
struct EvalArgs {
    int npts, np;
    double phi[EVAL_MAX_POINTS][OPS_MAX_NP];  // up to 25 modes (p=4 quadrilaterals)
};

__global__ void eval_points_kernel(const __grid_constant__ EvalArgs a, int ne, const double* u, double* out) {
    const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= (size_t)ne * a.npts) return;
    const int e = (int)(g / a.npts), k = (int)(g - (size_t)e * a.npts);
    const double* ue = u + (size_t)e * a.np * NV;
    double r[4] = {0.0, 0.0, 0.0, 0.0};
    for (int i = 0; i < a.np; ++i) {
        const double ph = a.phi[k][i];
#pragma unroll
        for (int v = 0; v < NV; ++v) r[v] = fma(ph, ue[i * NV + v], r[v]);
    }
#pragma unroll
    for (int v = 0; v < NV; ++v) out[g * NV + v] = r[v];
}

int launch_eval_points(int ne, int np, int npts, const double* phi, const double* u, double* out, cudaStream_t s) {
    if (ne == 0 || npts == 0) return 0;
    if (npts > EVAL_MAX_POINTS || np > OPS_MAX_NP) return -1;
    EvalArgs a;
    a.npts = npts;
    a.np = np;
    for (int k = 0; k < npts; ++k)
        for (int i = 0; i < np; ++i) a.phi[k][i] = phi[k * np + i];
    const size_t n = (size_t)ne * npts;
    eval_points_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, ne, u, out);
    return launch_status();
}

}  // namespace dgx
