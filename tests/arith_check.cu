// Checks FastOps (joltphysics_gb300/csrc/kernels/common.cuh) against the IEEE routines on the GPU:
//   reciprocal: every significand of every binade in FastOps' range, both signs, against __frcp_rn;
//   division: four pseudo-random numerators in range per divisor above, against __fdiv_rn;
//   square root: every float in range, against __fsqrt_rn;
//   zero numerators and zero square-root arguments against jdiv / jsqrt.
// Prints one line per check with its mismatch count and exits non-zero on any mismatch.
// Built and run by tests/test_gpu_arith.py.
#include <cstdio>
#include <cstdint>

#include "../joltphysics_gb300/csrc/kernels/common.cuh"

using namespace jsb;

__global__ void check_div(unsigned long long *bad) {
    const uint32_t m = blockIdx.x * blockDim.x + threadIdx.x;  // significand
    if (m >= (1u << 23)) return;
    for (uint32_t e = 65; e <= 189; ++e)
        for (uint32_t sign = 0; sign < 2; ++sign) {
            const float b = __uint_as_float((sign << 31) | (e << 23) | m);
            FastOps f;
            const float y = f.recip(b);
            if (!f.ok() || __float_as_uint(y) != __float_as_uint(__frcp_rn(b))) atomicAdd(bad, 1ull);
            uint32_t h = (sign << 31) ^ (e << 23) ^ m ^ 0x9e3779b9u;
            for (int k = 0; k < 4; ++k) {
                h = h * 1664525u + 1013904223u;
                const float a = __uint_as_float((h & 0x807fffffu) | (((h >> 23) % 125u + 65u) << 23));
                const float q = f.div_y(a, b, y);
                if (!f.ok() || __float_as_uint(q) != __float_as_uint(__fdiv_rn(a, b))) atomicAdd(bad + 1, 1ull);
            }
            FastOps z;
            const float q0 = z.div(0.0f, b), q1 = z.div(-0.0f, b);
            if (__float_as_uint(q0) != __float_as_uint(jdiv(0.0f, b)) || __float_as_uint(q1) != __float_as_uint(jdiv(-0.0f, b)))
                atomicAdd(bad + 2, 1ull);
        }
}

__global__ void check_sqrt(uint32_t lo, uint32_t count, unsigned long long *bad) {
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
        const float a = __uint_as_float(lo + k);
        FastOps f;
        const float s = f.sqrt(a);
        if (!f.ok() || __float_as_uint(s) != __float_as_uint(__fsqrt_rn(a))) atomicAdd(bad, 1ull);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        FastOps f;
        if (__float_as_uint(f.sqrt(0.0f)) != 0u || __float_as_uint(f.sqrt(-0.0f)) != 0x80000000u) atomicAdd(bad + 1, 1ull);
    }
}

int main() {
    unsigned long long *d = nullptr, h[6] = {0, 0, 0, 0, 0, 0};
    if (cudaMalloc(&d, sizeof(h)) != cudaSuccess) return 2;
    cudaMemset(d, 0, sizeof(h));
    check_div<<<(1u << 23) / 256, 256>>>(d);
    const uint32_t lo = 65u << 23, hi = 190u << 23;
    check_sqrt<<<1216, 256>>>(lo, hi - lo, d + 3);
    const cudaError_t e = cudaDeviceSynchronize();
    cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    printf("reciprocal mismatches %llu\ndivision mismatches %llu\nzero numerator mismatches %llu\n", h[0], h[1], h[2]);
    printf("square root mismatches %llu (of %u)\nsquare root of zero mismatches %llu\ncuda %s\n", h[3], hi - lo, h[4],
           cudaGetErrorString(e));
    return (e != cudaSuccess || h[0] || h[1] || h[2] || h[3] || h[4]) ? 1 : 0;
}
