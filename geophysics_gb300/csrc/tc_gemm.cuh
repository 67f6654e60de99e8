// BF16 tensor-core GEMM (tcgen05, TMEM accumulator, TMA-fed) used by the
// snapshot codec: C[M x N] = A[M x K] * B[N x K]^T with a fused epilogue.
#pragma once
#include <cuda_runtime.h>
#include <cuda_bf16.h>

namespace geo {

struct TcGemm {
    int M, N, K;                      // M % 128 == 0, N % 64 == 0, K % 64 == 0
    const __nv_bfloat16 *A;           // [M x K] row-major (K contiguous)
    const __nv_bfloat16 *B;           // [N x K] row-major
    const float *bias;                // [N] or null
    int act;                          // 1: leaky ReLU (slope kLeak) after the bias
    const __nv_bfloat16 *gate;        // [M x N] or null: multiply by the leaky-ReLU
                                      // derivative taken at gate's sign
    void *out;                        // [M x N] row-major
    int out_f32;                      // 1: fp32 output, 0: bf16 (round to nearest even)
    int *err;                         // device error word (wait timeouts)
};

constexpr float kLeak = 0.1f;

int tc_gemm(const TcGemm &g, cudaStream_t s);

}  // namespace geo
