// Diagnostics (no counterpart in the reference).
//
// geo_selftest_bounded_wait: one block waits on an mbarrier that nothing
// ever arrives on, through the bounded-wait helper every pipeline wait of
// the library uses (tc::mbar_wait), with a limit of limit_ms.  The wait has
// to give up, record that in an error word and let the kernel end; the host
// reads the word, the way the 3D step and the tensor-core GEMM report a
// pipeline stage that never completed.  The context stays usable.
//
// geo_selftest_conversions: the integer-pipe float <-> double conversions
// (softcvt.cuh) against the hardware conversions, on the device: the
// widening over every binary32 bit pattern, the narrowing over random
// binary64 values from below the binary32 subnormal range to above its
// overflow threshold, exact ties of normal and subnormal results, and the
// binary64 images of random binary32 values.
#include "geo_internal.h"
#include "tc_util.cuh"
#include "softcvt.cuh"

namespace geo {

__global__ void k_wait_selftest(int *err, unsigned long long limit_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);   // one arrival expected, none will come
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0 && !tc::mbar_wait(&bar, 0, limit_ns)) atomicExch(err, 1);
}

__device__ __forceinline__ uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// One binary64 test value per index: category k % 4 of
//  0: random sign and significand, biased exponent 860..1160 (binary32
//     underflow to overflow);
//  1: an exact tie of a normal result (the 29 dropped bits 100..0);
//  2: an exact tie of a subnormal result (the dropped bits 100..0 at the
//     subnormal shift) or of the zero / smallest-subnormal boundary;
//  3: the binary64 image of a random finite binary32.
__device__ uint64_t cvt_case(uint64_t k, uint64_t seed) {
    const uint64_t h = mix64(seed ^ mix64(k)), h2 = mix64(h);
    const uint64_t sign = (h & 1ull) << 63, man = h2 & 0xfffffffffffffull;
    switch (k & 3) {
        case 0: return sign | ((uint64_t)(860 + (h >> 8) % 301) << 52) | man;
        case 1: {
            const uint64_t ex = 897 + (h >> 8) % 254;             // normal binary32 results
            return sign | (ex << 52) | (man & ~((1ull << 29) - 1)) | (1ull << 28);
        }
        case 2: {
            const uint64_t ex = 873 + (h >> 8) % 24;              // s = 926 - ex in 30..53
            const int s = 926 - (int)ex;
            const uint64_t sig = ((man | (1ull << 52)) & ~((1ull << s) - 1)) | (1ull << (s - 1));
            return sign | (ex << 52) | (sig & 0xfffffffffffffull);
        }
        default: {
            uint32_t u = (uint32_t)(h >> 16);
            if (((u >> 23) & 0xffu) == 0xffu) u &= 0xbfffffffu;   // finite
            return (uint64_t)__double_as_longlong((double)__uint_as_float(u));
        }
    }
}

__global__ void k_cvt_selftest(long long n, unsigned long long seed, unsigned long long *bad) {
    unsigned long long bf = 0, bd = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x, first = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    for (uint64_t i = first; i < (1ull << 32); i += stride) {
        const float f = __uint_as_float((uint32_t)i);
        bf += __double_as_longlong(f2d_exact(f)) != __double_as_longlong((double)f);
    }
    for (uint64_t k = first; k < (uint64_t)n; k += stride) {
        const double d = __longlong_as_double((long long)cvt_case(k, seed));
        bd += __float_as_uint(d2f_rn(d)) != __float_as_uint((float)d);
    }
    atomicAdd(&bad[0], bf);
    atomicAdd(&bad[1], bd);
}

}  // namespace geo

using namespace geo;

extern "C" int geo_selftest_conversions(long long n_random, unsigned long long seed, long long *f2d_bad,
                                        long long *d2f_bad, void *stream) {
    if (!f2d_bad || !d2f_bad || n_random < 0) return fail(GEO_ERR_ARG, "bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf bad;
    GEO_TRY(bad.alloc(16));
    GEO_TRY(bad.zero(s));
    k_cvt_selftest<<<152 * 8, 256, 0, s>>>(n_random, seed, bad.as<unsigned long long>());
    GEO_TRY(check_launch("cvt_selftest"));
    unsigned long long h[2] = {0, 0};
    GEO_CUDA(cudaMemcpyAsync(h, bad.p, 16, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    *f2d_bad = (long long)h[0];
    *d2f_bad = (long long)h[1];
    return GEO_OK;
}

extern "C" int geo_selftest_bounded_wait(int limit_ms, int *gave_up, void *stream) {
    if (!gave_up || limit_ms < 1 || limit_ms > 2000) return fail(GEO_ERR_ARG, "limit_ms must be 1..2000");
    cudaStream_t s = (cudaStream_t)stream;
    DevBuf err;
    GEO_TRY(err.alloc(4));
    GEO_TRY(err.zero(s));
    k_wait_selftest<<<1, 32, 0, s>>>(err.as<int>(), (unsigned long long)limit_ms * 1000000ull);
    GEO_TRY(check_launch("wait_selftest"));
    int h = 0;
    GEO_CUDA(cudaMemcpyAsync(&h, err.p, 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    *gave_up = h;
    return GEO_OK;
}
