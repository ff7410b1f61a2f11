// Test helper: the engine's shared-reciprocal division (Recip<double>) against IEEE division,
// bit for bit, on pseudo-random operands generated on the device.
#include <cstdint>
#include "fv2d_kernels.cuh"

__device__ __forceinline__ uint64_t mix64(uint64_t z) {   // splitmix64 finaliser
    z += 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

// a double with a random 52-bit mantissa, random sign and exponent in [elo, ehi]
__device__ __forceinline__ double rand_double(uint64_t r, uint64_t s, int elo, int ehi, int mode) {
    uint64_t man = r & 0xFFFFFFFFFFFFFULL;
    if (mode == 1) man |= 0xFFFFFFFFFFF00ULL;          // mantissa near all ones
    if (mode == 2) man &= 0x00000000000FFULL;          // mantissa near zero (value near a power of two)
    // mode 3: a signed zero
    const int e = elo + (int)(s % (uint64_t)(ehi - elo + 1));
    const uint64_t sign = (s >> 40) & 1ULL;
    if (mode == 3) return __longlong_as_double((long long)(sign << 63));   // +0 or -0
    return __longlong_as_double((long long)((sign << 63) | ((uint64_t)(e + 1023) << 52) | man));
}

__global__ void k_div_check(uint64_t n, uint64_t seed, int elo, int ehi, int mode_a, int mode_b,
                            unsigned long long* bad, double* example) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t r1 = mix64(seed ^ (2 * i)), r2 = mix64(seed ^ (2 * i + 1));
        const double a = rand_double(r1, mix64(r1), elo, ehi, mode_a);
        const double b = rand_double(r2, mix64(r2), elo, ehi, mode_b);
        const double y = fv2d::Recip<double>::of(b);
        const double q = fv2d::Recip<double>::div(a, b, y);
        const double ref = a / b;
        if (__double_as_longlong(q) != __double_as_longlong(ref)) {
            if (atomicAdd(bad, 1ULL) == 0) { example[0] = a; example[1] = b; example[2] = q; example[3] = ref; }
        }
    }
}

extern "C" int div_check(unsigned long long n, unsigned long long seed, int elo, int ehi, int mode_a, int mode_b,
                         unsigned long long* bad_out, double* example_out) {
    unsigned long long* bad;
    double* ex;
    if (cudaMalloc(&bad, 8) != cudaSuccess || cudaMalloc(&ex, 32) != cudaSuccess) return 1;
    cudaMemset(bad, 0, 8);
    cudaMemset(ex, 0, 32);
    k_div_check<<<152 * 8, 256>>>(n, seed, elo, ehi, mode_a, mode_b, bad, ex);
    if (cudaDeviceSynchronize() != cudaSuccess) return 2;
    cudaMemcpy(bad_out, bad, 8, cudaMemcpyDeviceToHost);
    cudaMemcpy(example_out, ex, 32, cudaMemcpyDeviceToHost);
    cudaFree(bad);
    cudaFree(ex);
    return 0;
}
