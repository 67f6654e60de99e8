// Diagnostics (no counterpart in the reference).
//
// geo_selftest_bounded_wait: one block waits on an mbarrier that nothing
// ever arrives on, through the bounded-wait helper every pipeline wait of
// the library uses (tc::mbar_wait), with a limit of limit_ms.  The wait has
// to give up, record that in an error word and let the kernel end; the host
// reads the word, the way the 3D step and the tensor-core GEMM report a
// pipeline stage that never completed.  The context stays usable.
#include "geo_internal.h"
#include "tc_util.cuh"

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

}  // namespace geo

using namespace geo;

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
