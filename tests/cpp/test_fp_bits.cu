// The integer-pipe FP32 <-> FP64 conversions of csrc/fp_bits.cuh against the hardware
// conversions, value by value: random bit patterns of every class, signed zeros,
// subnormals, infinities, NaNs, the largest finite values and rounding ties of the
// binary64 -> binary32 direction across the normal, subnormal and overflow ranges.
// Prints the mismatch counts; exits 0 when both are zero.
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>

#include "fp_bits.cuh"

__device__ __forceinline__ uint64_t mix(uint64_t x) {  // splitmix64
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__global__ void check(uint64_t n, unsigned long long* bad) {
    unsigned long long b32 = 0, b64 = 0;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r = mix(i);
        // binary32 -> binary64: random patterns, every 16th a subnormal or a special value
        uint32_t fb = (uint32_t)r;
        if ((i & 15) == 0) fb &= 0x807FFFFFu;                       // subnormals and zeros
        if ((i & 15) == 1) fb |= 0x7F800000u;                       // infinities and NaNs
        const float f = __uint_as_float(fb);
        const double hw = (double)f, sw = dgx::f32_to_f64_bits(f);
        if (isnan(hw) ? !isnan(sw) : __double_as_longlong(hw) != __double_as_longlong(sw)) ++b32;
        // binary64 -> binary32: random patterns steered into the interesting exponent range
        uint64_t db = mix(r);
        const int sel = (int)(i & 7);
        const uint64_t sign = db & 0x8000000000000000ull;
        uint64_t mant = db & 0xFFFFFFFFFFFFFull;
        int e;
        if (sel <= 2) e = 896 + (int)((db >> 52) % 260) - 30;            // subnormal .. overflow
        else if (sel == 3) e = 1023 + 127 + (int)((db >> 52) % 3) - 1;   // around the largest binary32
        else if (sel == 4) e = (int)((db >> 52) & 0x7FF);                // any exponent
        else e = 1023 + (int)((db >> 52) % 40) - 20;                     // ordinary magnitudes
        if (e < 0) e = 0;
        if (e > 0x7FF) e = 0x7FF;
        if (sel == 5 || sel == 6) mant = (mant & ~0x1FFFFFFFull) | 0x10000000ull;  // exact ties (normal range)
        if (sel == 2) {  // ties in the subnormal range: the dropped bits are exactly one half
            const int shift = 926 - e;
            if (shift >= 30 && shift <= 53) {
                const uint64_t M = mant | (1ull << 52);
                const uint64_t keep = M & ~((1ull << shift) - 1ull);
                mant = (keep | (1ull << (shift - 1))) & 0xFFFFFFFFFFFFFull;
            }
        }
        const double d = __longlong_as_double((long long)(sign | ((uint64_t)e << 52) | mant));
        const float hf = (float)d, sf = dgx::f64_to_f32_bits(d);
        if (isnan(hf) ? !isnan(sf) : __float_as_uint(hf) != __float_as_uint(sf)) ++b64;
        if (dgx::finite_bits(d) != (bool)isfinite(d)) ++b64;
    }
    atomicAdd(bad, b32);
    atomicAdd(bad + 1, b64);
}

int main() {
    unsigned long long* bad;
    if (cudaMalloc(&bad, 2 * sizeof(unsigned long long)) != cudaSuccess) return 2;
    cudaMemset(bad, 0, 2 * sizeof(unsigned long long));
    const uint64_t n = 1ull << 28;
    check<<<1216, 256>>>(n, bad);
    unsigned long long h[2] = {1, 1};
    if (cudaMemcpy(h, bad, sizeof(h), cudaMemcpyDeviceToHost) != cudaSuccess) return 2;
    printf("values %llu: binary32->binary64 mismatches %llu, binary64->binary32 mismatches %llu\n",
           (unsigned long long)n, h[0], h[1]);
    return (h[0] || h[1]) ? 1 : 0;
}
