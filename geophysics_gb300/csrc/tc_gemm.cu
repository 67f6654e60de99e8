// tcgen05 BF16 GEMM with FP32 accumulation in tensor memory.
//
// One CTA computes a 128 x BN tile of C = A * B^T.  Four warps:
//   warp 0 lane 0  TMA producer: per 64-wide K slice, one 128x64 tile of A
//                  and one BNx64 tile of B (128-byte swizzle) into a
//                  2- to 4-stage ring, one "full" mbarrier per stage;
//   warp 1 lane 0  MMA issuer: four tcgen05.mma (K = 16 each) per slice
//                  into a 128 x BN fp32 accumulator in TMEM; tcgen05.commit
//                  to the stage's "empty" mbarrier releases it to the
//                  producer, a final commit signals the epilogue;
//   all 4 warps    epilogue: warp w reads TMEM lanes 32w..32w+31 (rows) with
//                  tcgen05.ld, adds the bias, applies the activation or the
//                  activation-derivative gate, and stores fp32, or bf16
//                  staged in the freed ring and written back as whole rows.
// Every wait is bounded (2 s): on timeout the CTA sets the error word, lets
// its copies in flight land (bounded), frees its TMEM and returns.
#include "geo_internal.h"
#include "tc_util.cuh"
#include "tc_gemm.cuh"
#include <cudaTypedefs.h>

namespace geo {
using namespace tc;

constexpr int kGM = 128, kGK = 64;

// Stage ring sized so two CTAs fit on an SM (one's epilogue overlaps the
// other's main loop): 2 stages for BN 256, 3 for 128, 4 for 64.  A GEMM
// with fewer K slices than that gets as many stages as slices (ST), so that
// more CTAs share an SM and more tiles are in flight: the skinny codec
// levels (K = 64, 128) have one or two slices per tile.  The shared memory
// is then padded so that no more CTAs fit than tensor memory holds
// accumulators for (512 columns per SM), so no allocation ever waits.
constexpr int default_stages(int bn) { return bn >= 256 ? 2 : (bn >= 128 ? 3 : 4); }
constexpr size_t kSmSmem = 233472;      // shared memory per SM
constexpr size_t kCtaReserve = 1024;    // reserved per resident CTA

template <int BN, int ST = default_stages(BN)>
struct GemmShape {
    static constexpr int kA = kGM * kGK * 2;
    static constexpr int kB = BN * kGK * 2;
    static constexpr int kStage = kA + kB;
    static constexpr int kStages = ST;
    static constexpr uint32_t kCols = BN < 32 ? 32 : BN;
    // the ring, reused after the last MMA as the bf16 output tile
    static constexpr size_t kOut = (size_t)kGM * BN * 2;
    static constexpr size_t kData = (size_t)kStages * kStage > kOut ? (size_t)kStages * kStage : kOut;
    static constexpr size_t kRing = kData + 1024 + 256;
    // fewest bytes with which at most 512 / kCols CTAs fit on an SM
    static constexpr size_t kFloor = kSmSmem / (512 / kCols + 1) + 1 - kCtaReserve;
    static constexpr size_t kSmem = kRing > kFloor ? kRing : kFloor;
    static_assert(kA % 1024 == 0 && kB % 1024 == 0, "swizzle atoms stay 1024-byte aligned");
    static_assert(BN % 16 == 0 && BN >= 16 && BN <= 256, "UMMA N for M = 128");
    static_assert(ST >= 1 && ST <= default_stages(BN), "stage count");
    static_assert(2 * kSmem <= 232448, "two CTAs per SM");
    static_assert((kSmSmem / (kSmem + kCtaReserve)) * kCols <= 512, "resident CTAs' accumulators fit in TMEM");
};

// max(v, kLeak v) = (v > 0 ? v : kLeak v) for 0 < kLeak < 1, one instruction fewer
__device__ __forceinline__ float leaky(float v) { return fmaxf(v, kLeak * v); }

template <int BN, int ST>
__global__ void __launch_bounds__(128, 2)
    k_tc_gemm(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, const TcGemm g) {
    using S = GemmShape<BN, ST>;
    extern __shared__ unsigned char smem_raw[];
    uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    constexpr int kGStages = S::kStages;
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + S::kData);
    uint64_t *empty = full + kGStages;
    uint64_t *done = empty + kGStages;
    uint32_t *tslot = reinterpret_cast<uint32_t *>(done + 1);
    __shared__ int s_abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // consecutive CTAs share a row tile of A (its second and later reads hit L2)
    const int ntn = g.N / BN;
    const int m0 = (int)(blockIdx.x / ntn) * kGM, n0 = (int)(blockIdx.x % ntn) * BN;
    const int nk = g.K / kGK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < kGStages; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(done, 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (warp == 0) tmem_alloc(tslot, S::kCols);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0 && lane == 0) {
        // producer
        int issued = 0;
        for (int kb = 0; kb < nk; kb++) {
            const int s = kb % kGStages;
            if (kb >= kGStages && !mbar_wait(&empty[s], ((kb / kGStages) - 1) & 1)) {
                s_abort = 1;
                break;
            }
            uint8_t *st = sm + s * S::kStage;
            mbar_expect_tx(&full[s], S::kStage);
            tma2(st, &ta, kb * kGK, m0, &full[s]);
            tma2(st + S::kA, &tb, kb * kGK, n0, &full[s]);
            issued = kb + 1;
        }
        // after a failure, let the copies still in flight land (bounded)
        if (*(volatile int *)&s_abort)
            for (int kb = issued > kGStages ? issued - kGStages : 0; kb < issued; kb++)
                mbar_wait(&full[kb % kGStages], (kb / kGStages) & 1);
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        constexpr uint32_t idesc = idesc_bf16_f32(kGM, BN);
        for (int kb = 0; kb < nk; kb++) {
            const int s = kb % kGStages;
            if (!mbar_wait(&full[s], (kb / kGStages) & 1)) {
                s_abort = 1;
                break;
            }
            tc_fence_after();
            const uint32_t a0 = su32(sm + s * S::kStage), b0 = a0 + S::kA;
#pragma unroll
            for (int k = 0; k < kGK / 16; k++)
                mma_bf16(tmem, sdesc_k128(a0 + k * 32), sdesc_k128(b0 + k * 32), idesc, (kb | k) != 0);
            mma_commit(&empty[s]);
        }
        mma_commit(done);  // arrives once every MMA issued above has completed
    }
    __syncwarp();

    // epilogue.  bf16 output goes through shared memory (the ring is free
    // once every MMA has completed): each warp stages its 32 rows with the
    // 16-byte chunks of a row XOR-swizzled by the row (conflict-free in both
    // directions), then writes them back as whole rows, consecutive lanes on
    // consecutive 16-byte chunks.
    if (!mbar_wait(done, 0)) s_abort = 1;
    tc_fence_after();
    const int row = m0 + warp * 32 + lane;
    const bool ok = !*(volatile int *)&s_abort;
    uint4 *stg = reinterpret_cast<uint4 *>(sm + (size_t)warp * 32 * BN * 2);
    constexpr int CPR = BN / 8;   // 16-byte chunks per output row
#pragma unroll 1
    for (int c0 = 0; c0 < BN; c0 += 16) {
        uint32_t r[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
        if (!ok) continue;
        const int n = n0 + c0;
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
        if (g.bias) {
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] += g.bias[n + j];
        }
        if (g.act) {
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] = leaky(v[j]);
        }
        const long o = (long)row * g.N + n;
        if (g.gate) {
            const uint4 *gp = reinterpret_cast<const uint4 *>(g.gate + o);
            uint4 q[2] = {gp[0], gp[1]};
            const __nv_bfloat16 *gb = reinterpret_cast<const __nv_bfloat16 *>(q);
#pragma unroll
            for (int j = 0; j < 16; j++) v[j] = __bfloat162float(gb[j]) > 0.0f ? v[j] : kLeak * v[j];
        }
        if (g.out_f32) {
            float4 *op = reinterpret_cast<float4 *>(static_cast<float *>(g.out) + o);
#pragma unroll
            for (int j = 0; j < 4; j++) op[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        } else {
            uint4 q[2];
            __nv_bfloat162 *q2 = reinterpret_cast<__nv_bfloat162 *>(q);
#pragma unroll
            for (int j = 0; j < 8; j++) q2[j] = __floats2bfloat162_rn(v[2 * j], v[2 * j + 1]);
            const int q0 = c0 / 8;
            stg[lane * CPR + (q0 ^ (lane & 7))] = q[0];
            stg[lane * CPR + ((q0 + 1) ^ (lane & 7))] = q[1];
        }
    }
    if (ok && !g.out_f32) {
        __syncwarp();
        __nv_bfloat16 *out = static_cast<__nv_bfloat16 *>(g.out) + (long)(m0 + warp * 32) * g.N + n0;
#pragma unroll 4
        for (int it = 0; it < CPR; it++) {
            const int idx = it * 32 + lane, rl = idx / CPR, q = idx % CPR;
            reinterpret_cast<uint4 *>(out + (long)rl * g.N)[q] = stg[rl * CPR + (q ^ (rl & 7))];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (s_abort && threadIdx.x == 0) atomicExch(g.err, 2);
    if (warp == 0) tmem_dealloc(tmem, S::kCols);
}

static PFN_cuTensorMapEncodeTiled_v12000 g_enc2 = nullptr;

// 2D bf16 map over a row-major [rows x cols] matrix, box box_rows x 64
// columns (128 bytes), 128-byte swizzle.
static int encode_bf16_2d(CUtensorMap *map, const void *base, int rows, int cols, int box_rows) {
    if (!g_enc2) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        GEO_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
        if (!fn || q != cudaDriverEntryPointSuccess) return fail(GEO_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        g_enc2 = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * 2};
    cuuint32_t box[2] = {64, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = g_enc2(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(GEO_ERR_CUDA, "cuTensorMapEncodeTiled (bf16) failed (%d)", (int)r);
    return GEO_OK;
}

template <int BN, int ST>
static int launch_bn(const TcGemm &g, cudaStream_t s) {
    using S = GemmShape<BN, ST>;
    static bool attr = false;
    if (!attr) {
        GEO_CUDA(cudaFuncSetAttribute(k_tc_gemm<BN, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::kSmem));
        attr = true;
    }
    CUtensorMap ta, tb;
    GEO_TRY(encode_bf16_2d(&ta, g.A, g.M, g.K, kGM));
    GEO_TRY(encode_bf16_2d(&tb, g.B, g.N, g.K, BN));
    const dim3 grid((unsigned)(g.M / kGM) * (unsigned)(g.N / BN));
    k_tc_gemm<BN, ST><<<grid, 128, S::kSmem, s>>>(ta, tb, g);
    return check_launch("tc_gemm");
}

// stages = K slices, up to the tile width's default
template <int BN>
static int launch_bn_k(const TcGemm &g, cudaStream_t s) {
    const int nk = g.K / kGK;
    if constexpr (default_stages(BN) >= 4)
        if (nk >= 4) return launch_bn<BN, 4>(g, s);
    if constexpr (default_stages(BN) >= 3)
        if (nk >= 3) return launch_bn<BN, (default_stages(BN) >= 3 ? 3 : 1)>(g, s);
    if (nk >= 2) return launch_bn<BN, 2>(g, s);
    return launch_bn<BN, 1>(g, s);
}

int tc_gemm(const TcGemm &g, cudaStream_t s) {
    if (g.M <= 0 || g.N <= 0 || g.K <= 0 || g.M % kGM || g.N % 64 || g.K % kGK)
        return fail(GEO_ERR_ARG, "tc_gemm: M %% 128, N %% 64 and K %% 64 must be 0 (M=%d N=%d K=%d)", g.M, g.N, g.K);
    if (!g.A || !g.B || !g.out || !g.err) return fail(GEO_ERR_ARG, "tc_gemm: null pointer");
    const uintptr_t al = reinterpret_cast<uintptr_t>(g.A) | reinterpret_cast<uintptr_t>(g.B) |
                         reinterpret_cast<uintptr_t>(g.out) | reinterpret_cast<uintptr_t>(g.gate);
    if (al & 15) return fail(GEO_ERR_ARG, "tc_gemm: operands must be 16-byte aligned");
    if (g.N % 256 == 0) return launch_bn_k<256>(g, s);
    if (g.N % 128 == 0) return launch_bn_k<128>(g, s);
    return launch_bn_k<64>(g, s);
}

}  // namespace geo

// C-ABI entry for tests and callers with their own bf16 operands (device
// pointers): out[M x N] = A[M x K] * B[N x K]^T (+bias, leaky ReLU).
extern "C" int geo_tc_gemm_bf16(int M, int N, int K, const void *A, const void *B, const float *bias, int act,
                                void *out, int out_f32, void *stream) {
    using namespace geo;
    DevBuf err;
    GEO_TRY(err.alloc(16));
    cudaStream_t s = (cudaStream_t)stream;
    GEO_TRY(err.zero(s));
    TcGemm g{};
    g.M = M; g.N = N; g.K = K;
    g.A = static_cast<const __nv_bfloat16 *>(A);
    g.B = static_cast<const __nv_bfloat16 *>(B);
    g.bias = bias;
    g.act = act;
    g.out = out;
    g.out_f32 = out_f32;
    g.err = err.as<int>();
    GEO_TRY(tc_gemm(g, s));
    int e = 0;
    GEO_CUDA(cudaMemcpyAsync(&e, err.p, 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    if (e) return fail(GEO_ERR_CUDA, "tc_gemm: a pipeline wait timed out");
    return GEO_OK;
}
