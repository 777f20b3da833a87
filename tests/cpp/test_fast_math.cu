// The FP32 reciprocal and square root of the mixed path (rcp_<float>, sqrt_<float> in
// csrc/dg_physics.cuh, the hardware approximations) against the exact values computed in
// FP64: the largest error in units in the last place of the FP32 result over random inputs
// whose results are normal FP32 numbers, and the special values (zeros, infinities, NaN,
// negative square-root arguments).  Prints both maxima; exits 0 when each is at most 2 ulp
// and every special value is right.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "dg_physics.cuh"

__device__ __forceinline__ uint64_t mix(uint64_t x) {  // splitmix64
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// |r - t| in ulps of the FP32 number nearest t (t normal in FP32)
__device__ double ulp_err(float r, double t) {
    const double ulp = ldexp(1.0, ilogb(t) - 23);
    return fabs((double)r - t) / ulp;
}

__device__ void atomic_max_d(double* a, double v) {
    unsigned long long* p = reinterpret_cast<unsigned long long*>(a);
    unsigned long long old = *p;
    while (__longlong_as_double((long long)old) < v) {
        const unsigned long long prev = atomicCAS(p, old, (unsigned long long)__double_as_longlong(v));
        if (prev == old) break;
        old = prev;
    }
}

__global__ void check(uint64_t n, double* worst) {
    double wr = 0.0, ws = 0.0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = mix(i);
        // positive and negative normals with reciprocals in the normal range: exponents -125 .. 125
        const int e = (int)((r >> 32) % 251) - 125;
        const uint32_t bits = ((uint32_t)(e + 127) << 23) | ((uint32_t)r & 0x7FFFFFu) | ((uint32_t)(r >> 63) << 31);
        const float x = __uint_as_float(bits);
        wr = fmax(wr, ulp_err(dgx::rcp_<float>(x), 1.0 / (double)x));
        const float ax = fabsf(x);
        ws = fmax(ws, ulp_err(dgx::sqrt_<float>(ax), sqrt((double)ax)));
        // subnormal square-root arguments (results are normal)
        const float sub = __uint_as_float(((uint32_t)r & 0x7FFFFFu) | 1u);
        ws = fmax(ws, ulp_err(dgx::sqrt_<float>(sub), sqrt((double)sub)));
    }
    atomic_max_d(&worst[0], wr);
    atomic_max_d(&worst[1], ws);
}

__global__ void specials(int* bad) {
    const float inf = __int_as_float(0x7F800000), nan = __int_as_float(0x7FC00000);
    int b = 0;
    b += !(dgx::rcp_<float>(0.0f) == inf);
    b += !(dgx::rcp_<float>(-0.0f) == -inf);
    b += !(dgx::rcp_<float>(inf) == 0.0f);
    b += !(dgx::rcp_<float>(-inf) == -0.0f);
    b += !isnan(dgx::rcp_<float>(nan));
    b += !(dgx::sqrt_<float>(0.0f) == 0.0f);
    b += !(dgx::sqrt_<float>(inf) == inf);
    b += !isnan(dgx::sqrt_<float>(-1.0f));
    b += !isnan(dgx::sqrt_<float>(nan));
    b += !(dgx::sqrt_<float>(4.0f) == 2.0f);
    b += !(dgx::rcp_<float>(2.0f) == 0.5f);
    *bad = b;
}

int main() {
    double* worst;
    int* bad;
    if (cudaMallocManaged(&worst, 2 * sizeof(double)) != cudaSuccess ||
        cudaMallocManaged(&bad, sizeof(int)) != cudaSuccess) {
        std::printf("allocation failed\n");
        return 2;
    }
    worst[0] = worst[1] = 0.0;
    *bad = -1;
    check<<<1024, 256>>>(1ull << 26, worst);
    specials<<<1, 1>>>(bad);
    if (cudaDeviceSynchronize() != cudaSuccess) {
        std::printf("kernel failed: %s\n", cudaGetErrorString(cudaGetLastError()));
        return 2;
    }
    std::printf("rcp max ulp %.4f, sqrt max ulp %.4f, special values wrong %d\n", worst[0], worst[1], *bad);
    const bool ok = worst[0] <= 2.0 && worst[1] <= 2.0 && *bad == 0;
    cudaFree(worst);
    cudaFree(bad);
    return ok ? 0 : 1;
}
