// Test-only kernels: the library's division by a known divisor
// (mat::dvd_known) against IEEE division, and its small-argument exponential
// (mat::exp_small) against exp(), on random operands.  Built by
// tests/test_gpu_arith.py with nvcc into a temporary shared library.
#include <stdint.h>

#include "../../mpm-2d_gb300/csrc/mpmg_materials.cuh"

namespace {

__device__ uint64_t mix(uint64_t z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// A double with a random significand and an exponent in [e0, e0 + span).
__device__ double random_double(uint64_t r, int e0, int span)
{
    const uint64_t mant = r & 0xfffffffffffffull;
    const uint64_t e = (uint64_t)(1023 + e0 + (int)((r >> 52) % (uint64_t)span));
    const uint64_t sign = (r >> 63) << 63;
    return __longlong_as_double((long long)(sign | (e << 52) | mant));
}

__global__ void div_kernel(double b, double y, long long n, uint64_t seed, unsigned long long *bad,
                           double *example)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const double a = random_double(mix(seed ^ (uint64_t)i), -60, 120);
        const double want = __ddiv_rn(a, b);
        const double got = mat::dvd_known(a, b, y);
        if (__double_as_longlong(got) != __double_as_longlong(want)) {
            if (atomicAdd(bad, 1ull) == 0) {
                example[0] = a;
                example[1] = got;
                example[2] = want;
            }
        }
    }
}

// Largest |exp_small(x) - exp(x)| in units of exp(x)'s ulp, over |x| < 2^-9.
__global__ void exp_kernel(long long n, uint64_t seed, unsigned long long *max_ulp_bits)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const uint64_t r = mix(seed ^ (uint64_t)i);
        const double x = random_double(r, -40, 31);   // |x| in [2^-40, 2^-9)
        const double want = exp(x);
        const double got = mat::exp_small(x);
        const double ulps = fabs(got - want) / (nextafter(want, 2.0 * want) - want);
        atomicMax(max_ulp_bits, (unsigned long long)__double_as_longlong(ulps));
    }
}

}  // namespace

extern "C" int check_division(double b, long long n, unsigned long long seed, unsigned long long *mismatches,
                              double *example)
{
    unsigned long long *d_bad = nullptr;
    double *d_ex = nullptr;
    if (cudaMalloc(&d_bad, sizeof(*d_bad)) != cudaSuccess) return 1;
    if (cudaMalloc(&d_ex, 3 * sizeof(double)) != cudaSuccess) return 1;
    cudaMemset(d_bad, 0, sizeof(*d_bad));
    cudaMemset(d_ex, 0, 3 * sizeof(double));
    div_kernel<<<1216, 256>>>(b, 1.0 / b, n, seed, d_bad, d_ex);
    cudaError_t e = cudaMemcpy(mismatches, d_bad, sizeof(*d_bad), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(example, d_ex, 3 * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(d_bad);
    cudaFree(d_ex);
    return e == cudaSuccess ? 0 : 1;
}

extern "C" int check_exp(long long n, unsigned long long seed, double *max_ulps)
{
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, sizeof(*d)) != cudaSuccess) return 1;
    cudaMemset(d, 0, sizeof(*d));
    exp_kernel<<<1216, 256>>>(n, seed, d);
    unsigned long long bits = 0;
    cudaError_t e = cudaMemcpy(&bits, d, sizeof(bits), cudaMemcpyDeviceToHost);
    cudaFree(d);
    memcpy(max_ulps, &bits, sizeof(bits));
    return e == cudaSuccess ? 0 : 1;
}
