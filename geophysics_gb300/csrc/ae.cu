// Learned snapshot codec: kernels, training and the geo_ae_* C ABI.
//
// Inference (snapshot encode in the forward pass of RTM, decode + imaging in
// the backward pass):
//   k_ae_e1_vol  gather one 16^3 block of the wavefield into Morton order,
//                scale by its max |value|, level E1 (8 -> 16) on CUDA cores;
//   tc_gemm x3   E2, E3, E4 on tcgen05 (the last one writes the bf16 code);
//   tc_gemm x3   D4, D3, D2 on tcgen05;
//   k_ae_d1_vol  level D1 (16 -> 8), unscale, scatter back to the field order
//                and either store the snapshot or add its product with the
//                receiver wavefield to the image (or, for the escape check,
//                compare it with the field).
// The snapshot kernels take E1's and D1's weights by value (a host copy kept
// per weight version), so every weight is an operand of its multiply-add.
// Training (one CUDA graph per iteration): the same forward on blocks drawn
// from a store of solver snapshots (k_ae_e1, weights read from the device
// copy that Adam updates inside the graph), the loss and the D1 backward in
// k_ae_d1, per level the weight gradient (k_ae_wgrad, CUDA cores, fp32), the
// bias gradient (k_ae_colsum) and the input gradient (tc_gemm against the
// transposed weights, the activation derivative fused as a gate), E1's
// weight gradient (k_ae_e1_bwd), then Adam and the bf16 repack.
#include "ae.cuh"
#include "tc_gemm.cuh"
#include "fd3d.cuh"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

using namespace geo;

namespace geo {

__host__ __device__ inline int morton_of(int z, int x, int y) {
    int m = 0;
#pragma unroll
    for (int l = 0; l < 4; l++)
        m |= (((z >> l) & 1) << (3 * l)) | (((x >> l) & 1) << (3 * l + 1)) | (((y >> l) & 1) << (3 * l + 2));
    return m;
}

__host__ __device__ inline unsigned long long splitmix(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ float bf16r(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }
// leaky ReLU as max(v, kLeak v): the same value as v > 0 ? v : kLeak v for
// 0 < kLeak < 1 (signed zeros, infinities and NaN included), one
// instruction fewer
__device__ __forceinline__ float leaky_d(float v) { return fmaxf(v, kLeak * v); }

// ---------------------------------------------------------------- layout
struct AeOffsets {
    long w[kAeLayers], b[kAeLayers], total;   // fp32 parameters: W [N x K] then b [N]
    long wb[kAeLayers], nbf;                  // bf16 copies of the GEMM layers (1..6)
};

static AeOffsets ae_offsets() {
    AeOffsets o{};
    long p = 0, q = 0;
    for (int l = 0; l < kAeLayers; l++) {
        o.w[l] = p;
        p += (long)kAeNet[l].N * kAeNet[l].K;
        o.b[l] = p;
        p += kAeNet[l].N;
        if (l >= 1 && l <= 6) {
            o.wb[l] = q;
            q += (long)kAeNet[l].N * kAeNet[l].K;
        } else {
            o.wb[l] = -1;
        }
    }
    o.total = p;
    o.nbf = q;
    return o;
}

// Weights of the two CUDA-core levels, passed by value to the snapshot
// kernels (the host keeps a copy of the current ones).
struct AeSmallW {
    float w1[128], b1[16];   // E1: W [16 x 8] (bf16 values), b [16]
    float v1[128], c1[8];    // D1: W [8 x 16] (bf16 values), b [8]
};

// E1 of one level-1 node: h = leaky(W1 x + b1) as 16 bf16 (32 bytes).
__device__ __forceinline__ void e1_node(const float *w1, const float *b1, const float *x8, __nv_bfloat16 *out) {
    uint4 q[2];
    __nv_bfloat16 *qb = reinterpret_cast<__nv_bfloat16 *>(q);
    float h[16];
#pragma unroll
    for (int c = 0; c < 16; c++) {
        float acc = 0.0f;
#pragma unroll
        for (int j = 0; j < 8; j++) acc = __fmaf_rn(w1[c * 8 + j], x8[j], acc);
        h[c] = leaky_d(acc + b1[c]);
    }
    // two channels per conversion (low half = even channel)
    __nv_bfloat162 *q2 = reinterpret_cast<__nv_bfloat162 *>(qb);
#pragma unroll
    for (int c = 0; c < 8; c++) q2[c] = __floats2bfloat162_rn(h[2 * c], h[2 * c + 1]);
    uint4 *dst = reinterpret_cast<uint4 *>(out);
    dst[0] = q[0];
    dst[1] = q[1];
}

// D1 of one level-1 node: y = V1 g + c1 from its 16 bf16 inputs.
__device__ __forceinline__ void d1_node(const float *v1, const float *c1, const __nv_bfloat16 *in, float *g,
                                        float *y) {
    const uint4 *src = reinterpret_cast<const uint4 *>(in);
    uint4 q[2] = {src[0], src[1]};
    const __nv_bfloat16 *qb = reinterpret_cast<const __nv_bfloat16 *>(q);
#pragma unroll
    for (int j = 0; j < 16; j++) g[j] = __bfloat162float(qb[j]);
#pragma unroll
    for (int c = 0; c < 8; c++) {
        float acc = 0.0f;
#pragma unroll
        for (int j = 0; j < 16; j++) acc = __fmaf_rn(v1[c * 16 + j], g[j], acc);
        y[c] = acc + c1[c];
    }
}

// ---------------------------------------------------------------- kernels
struct E1Args {
    const float *direct;          // given blocks (Morton, nb x 4096), or null
    const float *store;           // training store (Morton), sampled by hash
    long nstore;
    unsigned long long seed;
    const int *step;
    int nb;                       // real blocks (grid covers the padded count)
    const float *w1, *b1;         // E1: W [16 x 8] (bf16 values), b [16]
    __nv_bfloat16 *h1;            // [nbp*512 x 16]
    float *scale;                 // [nbp]
    float *xn;                    // [nbp x 4096] normalized input (training), or null
    const float *wstore;          // training: per-block weights of the store
    float *wrow;                  // training: weight of each row's block
    float *wsum;                  // training: batch weight sums, slot *step - step0
    int step0;
};

// Blocks whose max |value| is below this are coded as zero (their inverse
// scale would overflow).
constexpr float kAeTiny = 1e-30f;

__device__ __forceinline__ float block_max(float v, float *red) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float m = red[0];
#pragma unroll
    for (int w = 1; w < 8; w++) m = fmaxf(m, red[w]);
    return m;
}

// E1 on blocks given in Morton order (evaluation) or drawn from the training
// store: scale by the block max, W1 x + b1, leaky ReLU, bf16 out.
__global__ void __launch_bounds__(256) k_ae_e1(const E1Args a) {
    __shared__ float xs[kAePts];
    __shared__ float red[8];
    const int b = blockIdx.x, t = threadIdx.x;
    float mx = 0.0f;
    if (b < a.nb) {
        const float *src;
        if (a.direct) {
            src = a.direct + (long)b * kAePts;
        } else {
            const unsigned long long h = splitmix(a.seed ^ splitmix(((unsigned long long)*a.step << 24) + b));
            const long pick = (long)(h % (unsigned long long)a.nstore);
            src = a.store + pick * kAePts;
            if (t == 0 && a.wrow) {
                const float w = a.wstore ? a.wstore[pick] : 1.0f;
                a.wrow[b] = w;
                atomicAdd(a.wsum + (*a.step - a.step0), w);
            }
        }
#pragma unroll 4
        for (int p = 0; p < 16; p++) {
            const float val = src[p * 256 + t];
            xs[p * 256 + t] = val;
            mx = fmaxf(mx, fabsf(val));
        }
    } else {
        for (int p = 0; p < 16; p++) xs[p * 256 + t] = 0.0f;
    }
    const float s = block_max(mx, red);   // includes the barrier after the fills
    const float inv = s >= kAeTiny ? 1.0f / s : 0.0f;
    if (t == 0) a.scale[b] = s >= kAeTiny ? s : 0.0f;
#pragma unroll 1
    for (int r = 0; r < 2; r++) {
        const int p = t + 256 * r;
        float x8[8];
#pragma unroll
        for (int j = 0; j < 8; j++) {
            const float xv = xs[p * 8 + j] * inv;
            if (a.xn) a.xn[(long)b * kAePts + p * 8 + j] = xv;
            x8[j] = bf16r(xv);
        }
        e1_node(a.w1, a.b1, x8, a.h1 + ((long)b * 512 + p) * 16);
    }
}

// Interior-box gather of a snapshot, E1 with the weights passed by value
// (each weight a constant-bank operand of its multiply-add, no load).
// Thread t owns depth z = t & 15 of row x = t >> 4 of the block on all
// sixteen planes y, so its Morton slot is fixed up to the y bits.
struct E1Vol {
    AeVolume vol;
    int nb;
    __nv_bfloat16 *h1;            // [nbp*512 x 16]
    float *scale;                 // [nbp]
    AeSmallW w;
};

__global__ void __launch_bounds__(256) k_ae_e1_vol(const E1Vol a) {
    __shared__ float xs[kAePts];
    __shared__ float red[8];
    const int b = blockIdx.x, t = threadIdx.x;
    float mx = 0.0f;
    if (b < a.nb) {
        const AeVolume &v = a.vol;
        const int bz = b % v.nbz, bx = (b / v.nbz) % v.nbx, by = b / (v.nbz * v.nbx);
        const int z = t & 15, x = t >> 4, iz = bz * 16 + z, ix = bx * 16 + x, iy0 = by * 16;
        const bool zx = iz < v.nz && ix < v.nx;
        const float *col = v.src + (long)(v.oz + iz) + v.ldz * (v.ox + ix) + v.sxy * (v.oy + iy0);
        // all sixteen loads in flight before the first use
        float vals[16];
#pragma unroll
        for (int y = 0; y < 16; y++) vals[y] = zx && iy0 + y < v.ny ? __ldg(col + v.sxy * y) : 0.0f;
        const int m = morton_of(z, x, 0);
#pragma unroll
        for (int y = 0; y < 16; y++) {
            xs[m + morton_of(0, 0, y)] = vals[y];
            mx = fmaxf(mx, fabsf(vals[y]));
        }
    } else {
        for (int p = 0; p < 16; p++) xs[p * 256 + t] = 0.0f;
    }
    const float s = block_max(mx, red);
    const float inv = s >= kAeTiny ? 1.0f / s : 0.0f;
    if (t == 0) a.scale[b] = s >= kAeTiny ? s : 0.0f;
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const int p = t + 256 * r;
        float x8[8];
#pragma unroll
        for (int j = 0; j < 8; j++) x8[j] = bf16r(xs[p * 8 + j] * inv);
        e1_node(a.w.w1, a.w.b1, x8, a.h1 + ((long)b * 512 + p) * 16);
    }
}

struct D1Args {
    int nb;
    const __nv_bfloat16 *g1;      // [nbp*512 x 16]
    const float *v1, *c1;         // D1: W [8 x 16] (bf16 values), b [8]
    const float *xn;              // normalized target
    float *recon;                 // normalized reconstruction, or null
    __nv_bfloat16 *dg1;           // gradient at D2's output (gated)
    float *gd1;                   // D1 gradient (W then b, 136 floats)
    double *loss;                 // sum of squared errors, slot *step - step0
    const int *step;
    int step0;
    const float *wrow;            // block weights (null: all 1)
    const float *wsum;            // batch weight sum slot base (null: block count)
};

// D1 in training / evaluation: reconstruction, weighted loss, D1's weight
// and bias gradients and the gated gradient at D2's output.
// loss = sum_b w_b |e_b|^2 / (W * 4096), W = sum_b w_b.
__global__ void __launch_bounds__(256) k_ae_d1(const D1Args a) {
    __shared__ float sg[136];
    __shared__ float red[8];
    const int b = blockIdx.x, t = threadIdx.x;
    if (b >= a.nb) return;
    for (int i = t; i < 136; i += 256) sg[i] = 0.0f;
    __syncthreads();
    float lsum = 0.0f;
    const float W = a.wsum ? a.wsum[*a.step - a.step0] : (float)gridDim.x;
    const float wb = a.wrow ? a.wrow[b] : 1.0f;
    const float gsc = wb / (W * (float)kAePts);
#pragma unroll 1
    for (int r = 0; r < 2; r++) {
        const int p = t + 256 * r;
        float g[16], y[8];
        d1_node(a.v1, a.c1, a.g1 + ((long)b * 512 + p) * 16, g, y);
        float dy[8];
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const long o = (long)b * kAePts + p * 8 + c;
            const float d = y[c] - a.xn[o];
            lsum += d * d;
            dy[c] = 2.0f * d * gsc;
            if (a.recon) a.recon[o] = y[c];
        }
#pragma unroll
        for (int c = 0; c < 8; c++) {
#pragma unroll
            for (int j = 0; j < 16; j++) atomicAdd(&sg[c * 16 + j], dy[c] * g[j]);
            atomicAdd(&sg[128 + c], dy[c]);
        }
        uint4 o4[2];
        __nv_bfloat16 *ob = reinterpret_cast<__nv_bfloat16 *>(o4);
#pragma unroll
        for (int j = 0; j < 16; j++) {
            float acc = 0.0f;
#pragma unroll
            for (int c = 0; c < 8; c++) acc += a.v1[c * 16 + j] * dy[c];
            ob[j] = __float2bfloat16_rn(g[j] > 0.0f ? acc : kLeak * acc);
        }
        uint4 *dst = reinterpret_cast<uint4 *>(a.dg1 + ((long)b * 512 + p) * 16);
        dst[0] = o4[0];
        dst[1] = o4[1];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((t & 31) == 0) red[t >> 5] = lsum;
    __syncthreads();
    if (t == 0) {
        double tot = 0.0;
        for (int w = 0; w < 8; w++) tot += red[w];
        const double Wd = a.wsum ? (double)a.wsum[*a.step - a.step0] : (double)gridDim.x;
        atomicAdd(a.loss + (*a.step - a.step0), tot * wb / Wd);
    }
    for (int i = t; i < 136; i += 256) atomicAdd(&a.gd1[i], sg[i]);
}

// D1 of a snapshot's blocks with the weights passed by value, unscaled and
// scattered to the interior box: mode 0 stores the snapshot (dst, the box's
// strides), mode 1 adds wimg * snapshot * gP to the image, mode 3 compares
// with the field vol.src and keeps every block's residual (bf16, natural
// order) and its squared error and norm (the escape check).  Escaped blocks
// (esc) add their residual in modes 0 and 1.  Thread t owns depth
// z = t & 15 of row x = t >> 4 on all sixteen planes, as in k_ae_e1_vol.
struct D1Vol {
    AeVolume vol;
    int nb, mode;
    const __nv_bfloat16 *g1;      // [nbp*512 x 16]
    const float *scale;           // [nbp]
    float *dst;                   // mode 0
    const float *gP;              // mode 1: receiver field (vol's strides)
    float *mig;                   // mode 1: image, iz + nz*(ix + nx*iy)
    float wimg;                   // mode 1: weight of this snapshot
    const int *esc;               // modes 0/1: escaped-block slot per row (-1: none), or null
    const __nv_bfloat16 *res;     // modes 0/1: residual pool (4096 per slot, natural order)
    __nv_bfloat16 *resall;        // mode 3: residual of every row (natural order)
    float *err2, *norm2;          // mode 3: per-row squared error and squared norm
    AeSmallW w;
};

__global__ void __launch_bounds__(256) k_ae_d1_vol(const D1Vol a) {
    __shared__ float ys[kAePts];
    __shared__ float red2[2][8];
    const int b = blockIdx.x, t = threadIdx.x;
    if (b >= a.nb) return;
    const float s = a.scale[b];
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const int p = t + 256 * r;
        float g[16], y[8];
        d1_node(a.w.v1, a.w.c1, a.g1 + ((long)b * 512 + p) * 16, g, y);
#pragma unroll
        for (int c = 0; c < 8; c++) ys[p * 8 + c] = y[c] * s;
    }
    __syncthreads();
    const AeVolume &v = a.vol;
    const int bz = b % v.nbz, bx = (b / v.nbz) % v.nbx, by = b / (v.nbz * v.nbx);
    const int z = t & 15, x = t >> 4, iz = bz * 16 + z, ix = bx * 16 + x, iy0 = by * 16;
    const bool zx = iz < v.nz && ix < v.nx;
    const long col = (long)(v.oz + iz) + v.ldz * (v.ox + ix) + v.sxy * (v.oy + iy0);
    const int m = morton_of(z, x, 0);
    if (a.mode == 3) {
        float e2 = 0.0f, x2 = 0.0f;
        __nv_bfloat16 *rb = a.resall + (long)b * kAePts;
        float vals[16];
#pragma unroll
        for (int y = 0; y < 16; y++) vals[y] = zx && iy0 + y < v.ny ? __ldg(v.src + col + v.sxy * y) : 0.0f;
#pragma unroll
        for (int y = 0; y < 16; y++) {
            const float d = vals[y] - ys[m + morton_of(0, 0, y)];
            rb[y * 256 + t] = __float2bfloat16_rn(d);
            e2 += d * d;
            x2 += vals[y] * vals[y];
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) {
            e2 += __shfl_xor_sync(0xffffffffu, e2, o);
            x2 += __shfl_xor_sync(0xffffffffu, x2, o);
        }
        if ((t & 31) == 0) {
            red2[0][t >> 5] = e2;
            red2[1][t >> 5] = x2;
        }
        __syncthreads();
        if (t == 0) {
            float E = 0.0f, X = 0.0f;
            for (int w = 0; w < 8; w++) {
                E += red2[0][w];
                X += red2[1][w];
            }
            a.err2[b] = E;
            a.norm2[b] = X;
        }
        return;
    }
    if (!zx) return;
    const int slot = a.esc ? a.esc[b] : -1;
    const __nv_bfloat16 *res = slot >= 0 ? a.res + (long)slot * kAePts : nullptr;
    if (a.mode == 0) {
#pragma unroll
        for (int y = 0; y < 16; y++) {
            if (iy0 + y >= v.ny) break;
            float val = ys[m + morton_of(0, 0, y)];
            if (res) val += __bfloat162float(res[y * 256 + t]);   // escaped block: decoded + residual
            a.dst[col + v.sxy * y] = val;
        }
        return;
    }
    // mode 1: all image and receiver-field loads in flight first
    const long o0 = iz + (long)v.nz * (ix + (long)v.nx * iy0), so = (long)v.nz * v.nx;
    float gp[16], mg[16];
#pragma unroll
    for (int y = 0; y < 16; y++) {
        const bool in = iy0 + y < v.ny;
        gp[y] = in ? __ldg(a.gP + col + v.sxy * y) : 0.0f;
        mg[y] = in ? a.mig[o0 + so * y] : 0.0f;
    }
#pragma unroll
    for (int y = 0; y < 16; y++) {
        if (iy0 + y >= v.ny) break;
        float val = ys[m + morton_of(0, 0, y)];
        if (res) val += __bfloat162float(res[y * 256 + t]);
        a.mig[o0 + so * y] = mg[y] + a.wimg * val * gp[y];
    }
}

// Escape pass 1 is k_ae_d1_vol in mode 3: decode, compare with the field, keep
// every block's residual (bf16, natural order) and its squared error and norm.

// Escape pass 2 (one block of 1024 threads): the cap blocks with the
// largest squared error, among those with err2 > tau2 * norm2, get residual
// slots: a binary search on the float bits of err2 finds the threshold.
__global__ void __launch_bounds__(1024) k_ae_select(const float *err2, const float *norm2, int nb, float tau2, int cap,
                                                    int *esc, int *count) {
    __shared__ int cnt;
    __shared__ int next;
    auto eligible = [&](int b) { return err2[b] > 0.0f && err2[b] > tau2 * norm2[b]; };
    // smallest threshold bits T with #{eligible, bits(err2) > T} <= cap
    unsigned lo = 0u, hi = 0x7f800000u;   // error bits of non-negative floats
    while (lo < hi) {
        const unsigned mid = lo + (hi - lo) / 2;
        if (threadIdx.x == 0) cnt = 0;
        __syncthreads();
        int c = 0;
        for (int b = threadIdx.x; b < nb; b += blockDim.x) c += eligible(b) && __float_as_uint(err2[b]) > mid;
        atomicAdd(&cnt, c);
        __syncthreads();
        const int total = cnt;
        __syncthreads();
        if (total <= cap) hi = mid;
        else lo = mid + 1;
    }
    if (threadIdx.x == 0) next = 0;
    __syncthreads();
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        int sl = -1;
        if (eligible(b) && __float_as_uint(err2[b]) > lo) sl = atomicAdd(&next, 1);
        esc[b] = sl < cap ? sl : -1;
    }
    __syncthreads();
    if (threadIdx.x == 0) *count = min(next, cap);
}

// Escape pass 3: copy the selected residuals into their slots.
__global__ void __launch_bounds__(256) k_ae_escape_copy(const int *esc, const __nv_bfloat16 *resall,
                                                        __nv_bfloat16 *res, int nb) {
    const int b = blockIdx.x;
    if (b >= nb) return;
    const int sl = esc[b];
    if (sl < 0) return;
    const uint4 *src = reinterpret_cast<const uint4 *>(resall + (long)b * kAePts);
    uint4 *dst = reinterpret_cast<uint4 *>(res + (long)sl * kAePts);
    for (int i = threadIdx.x; i < kAePts / 8; i += 256) dst[i] = src[i];
}

// E1 weight and bias gradients from the normalized input and the gated
// gradient at E1's output.
__global__ void __launch_bounds__(256) k_ae_e1_bwd(const float *xn, const __nv_bfloat16 *dh1, float *ge1, int nb) {
    __shared__ float sg[144];
    const int b = blockIdx.x, t = threadIdx.x;
    if (b >= nb) return;
    for (int i = t; i < 144; i += 256) sg[i] = 0.0f;
    __syncthreads();
#pragma unroll 1
    for (int r = 0; r < 2; r++) {
        const int p = t + 256 * r;
        float x8[8];
#pragma unroll
        for (int j = 0; j < 8; j++) x8[j] = bf16r(xn[(long)b * kAePts + p * 8 + j]);
        const uint4 *src = reinterpret_cast<const uint4 *>(dh1 + ((long)b * 512 + p) * 16);
        uint4 q[2] = {src[0], src[1]};
        const __nv_bfloat16 *qb = reinterpret_cast<const __nv_bfloat16 *>(q);
#pragma unroll
        for (int c = 0; c < 16; c++) {
            const float d = __bfloat162float(qb[c]);
#pragma unroll
            for (int j = 0; j < 8; j++) atomicAdd(&sg[c * 8 + j], d * x8[j]);
            atomicAdd(&sg[128 + c], d);
        }
    }
    __syncthreads();
    for (int i = t; i < 144; i += 256) atomicAdd(&ge1[i], sg[i]);
}

// grad[n*K + k] += sum_m dy[m*N + n] * x[m*K + k] over this split's rows.
__global__ void __launch_bounds__(256) k_ae_wgrad(const __nv_bfloat16 *dy, const __nv_bfloat16 *x, float *grad, int M,
                                                  int N, int K, int rows) {
    __shared__ float ys[32][64];
    __shared__ float xs[32][65];
    const int k0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
    const int mb = blockIdx.z * rows, me = min(M, mb + rows);
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = 0.0f;
    for (int m0 = mb; m0 < me; m0 += 32) {
        for (int i = threadIdx.x; i < 32 * 64; i += 256) {
            const int r = i >> 6, c = i & 63, m = m0 + r;
            ys[r][c] = m < me ? __bfloat162float(dy[(long)m * N + n0 + c]) : 0.0f;
            xs[r][c] = m < me ? __bfloat162float(x[(long)m * K + k0 + c]) : 0.0f;
        }
        __syncthreads();
#pragma unroll 8
        for (int r = 0; r < 32; r++) {
            float av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                av[i] = ys[r][ty * 4 + i];
                bv[i] = xs[r][tx * 4 + i];
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] += av[i] * bv[j];
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) atomicAdd(&grad[(long)(n0 + ty * 4 + i) * K + k0 + tx * 4 + j], acc[i][j]);
}

// gb[n] += sum_m dy[m*N + n] over this split's rows.
__global__ void __launch_bounds__(256) k_ae_colsum(const __nv_bfloat16 *dy, float *gb, int M, int N, int rows) {
    const int n = blockIdx.x * 256 + threadIdx.x;
    if (n >= N) return;
    const int mb = blockIdx.y * rows, me = min(M, mb + rows);
    float s = 0.0f;
    for (int m = mb; m < me; m++) s += __bfloat162float(dy[(long)m * N + n]);
    atomicAdd(&gb[n], s);
}

// Adam (bias-corrected) with the step's learning rate from lrs[*step - step0].
__global__ void k_ae_adam(float *p, const float *g, float *m1, float *m2, long n, const int *step, int step0,
                          const float *lrs) {
    const int t = *step + 1;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float bc1 = 1.0f - powf(b1, (float)t), bc2 = 1.0f - powf(b2, (float)t);
    const float lr = lrs[*step - step0];
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float a = b1 * m1[i] + (1.0f - b1) * gi;
        const float v = b2 * m2[i] + (1.0f - b2) * gi * gi;
        m1[i] = a;
        m2[i] = v;
        p[i] -= lr * (a / bc1) / (sqrtf(v / bc2) + eps);
    }
}

// bf16 copies of the GEMM weights ([N x K] and transposed [K x N]) and the
// bf16-valued fp32 copies of E1 and D1; then step += inc.
struct PackArgs {
    const float *params;
    __nv_bfloat16 *wb, *wtb;
    float *small;                 // E1 W (128) then D1 W (128)
    long w[kAeLayers], wb_off[kAeLayers];
    int N[kAeLayers], K[kAeLayers];
    int *step, inc;
};

__global__ void k_ae_pack(const PackArgs a) {
    const long tid = blockIdx.x * (long)blockDim.x + threadIdx.x, nth = (long)gridDim.x * blockDim.x;
    for (int l = 1; l <= 6; l++) {
        const int N = a.N[l], K = a.K[l];
        const long n = (long)N * K;
        for (long i = tid; i < n; i += nth) {
            const int r = (int)(i / K), c = (int)(i % K);
            const __nv_bfloat16 v = __float2bfloat16_rn(a.params[a.w[l] + i]);
            a.wb[a.wb_off[l] + i] = v;
            a.wtb[a.wb_off[l] + (long)c * N + r] = v;
        }
    }
    for (long i = tid; i < 128; i += nth) {
        a.small[i] = bf16r(a.params[a.w[0] + i]);
        a.small[128 + i] = bf16r(a.params[a.w[7] + i]);
    }
    if (tid == 0 && a.inc) *a.step += a.inc;
}

// Per-snapshot max |value| of an interior box (as ordered int bits).
__global__ void k_ae_absmax(const AeVolume v, unsigned *out) {
    float mx = 0.0f;
    const long n = (long)v.nz * v.nx * v.ny;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(k % v.nz), ix = (int)((k / v.nz) % v.nx), iy = (int)(k / ((long)v.nz * v.nx));
        mx = fmaxf(mx, fabsf(v.src[(long)(v.oz + iz) + v.ldz * (v.ox + ix) + v.sxy * (v.oy + iy)]));
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(mx));
}

// Append the full blocks of a snapshot whose max |value| exceeds
// rel * (snapshot max) to the training store (Morton order).
__global__ void __launch_bounds__(256) k_ae_collect(const AeVolume v, const unsigned *snapmax, float rel, float *store,
                                                    float *wstore, long cap, unsigned long long *count) {
    __shared__ float xs[kAePts];
    __shared__ float red[8];
    __shared__ long slot;
    const int b = blockIdx.x, t = threadIdx.x;
    const int bz = b % v.nbz, bx = (b / v.nbz) % v.nbx, by = b / (v.nbz * v.nbx);
    if ((bz + 1) * 16 > v.nz || (bx + 1) * 16 > v.nx || (by + 1) * 16 > v.ny) return;  // full blocks only
    float mx = 0.0f;
    for (int p = 0; p < 16; p++) {
        const int idx = p * 256 + t, z = idx & 15, x = (idx >> 4) & 15, y = idx >> 8;
        const float val = v.src[(long)(v.oz + bz * 16 + z) + v.ldz * (v.ox + bx * 16 + x) + v.sxy * (v.oy + by * 16 + y)];
        xs[morton_of(z, x, y)] = val;
        mx = fmaxf(mx, fabsf(val));
    }
    const float s = block_max(mx, red);
    if (!(s > rel * __uint_as_float(*snapmax))) return;
    if (t == 0) slot = (long)atomicAdd(count, 1ull);
    __syncthreads();
    if (slot >= cap) return;
    if (t == 0) {
        const float r = s / __uint_as_float(*snapmax);
        wstore[slot] = r * r;   // the block's share of its snapshot's energy scale
    }
    for (int p = 0; p < 16; p++) store[slot * kAePts + p * 256 + t] = xs[p * 256 + t];
}

}  // namespace geo

// ---------------------------------------------------------------- host state
struct geo_ae {
    AeOffsets off;
    unsigned long long seed = 0;
    DevBuf params, grad, m1, m2, wb, wtb, small, step, err;
    int h_step = 0;
    // block store for training
    DevBuf store, wstore, count, snapmax;
    long cap = 0;
    // forward scratch (rows = padded blocks)
    int rows = 0;
    DevBuf h1, h2, h3, z, g3, g2, g1, scale;
    // training scratch
    int trows = 0;
    DevBuf xn, dg1, dg2, dg3, dz, dh3, dh2, dh1, wrow;
    // escape settings
    float tau = 0.05f, frac = 0.03f;
    DevBuf resall, err2, norm2;
    int erows = 0;
    long long st_blocks = 0, st_escaped = 0;   // totals over RTM shots
    // host copy of the CUDA-core levels' weights for the snapshot kernels:
    // wver counts weight updates (packs), hver the version copied
    geo::AeSmallW hw{};
    long wver = 1, hver = 0;
};

namespace geo {

static int pad128(long n) { return (int)((n + 127) / 128 * 128); }

static int ae_pack(geo_ae *ae, int inc, cudaStream_t s) {
    PackArgs a{};
    a.params = ae->params.as<float>();
    a.wb = ae->wb.as<__nv_bfloat16>();
    a.wtb = ae->wtb.as<__nv_bfloat16>();
    a.small = ae->small.as<float>();
    for (int l = 0; l < kAeLayers; l++) {
        a.w[l] = ae->off.w[l];
        a.wb_off[l] = ae->off.wb[l];
        a.N[l] = kAeNet[l].N;
        a.K[l] = kAeNet[l].K;
    }
    a.step = ae->step.as<int>();
    a.inc = inc;
    ae->wver++;
    k_ae_pack<<<152 * 4, 256, 0, s>>>(a);
    return check_launch("ae_pack");
}

static int ensure_rows(geo_ae *ae, int rows) {
    if (rows <= ae->rows) return GEO_OK;
    const size_t r = (size_t)rows;
    GEO_TRY(ae->h1.alloc(r * 512 * 16 * 2));
    GEO_TRY(ae->h2.alloc(r * 64 * 64 * 2));
    GEO_TRY(ae->h3.alloc(r * 8 * 256 * 2));
    GEO_TRY(ae->z.alloc(r * 512 * 2));
    GEO_TRY(ae->g3.alloc(r * 2048 * 2));
    GEO_TRY(ae->g2.alloc(r * 8 * 512 * 2));
    GEO_TRY(ae->g1.alloc(r * 64 * 128 * 2));
    GEO_TRY(ae->scale.alloc(r * 4));
    ae->rows = rows;
    return GEO_OK;
}

static int ensure_train(geo_ae *ae, int rows) {
    GEO_TRY(ensure_rows(ae, rows));
    if (rows <= ae->trows) return GEO_OK;
    const size_t r = (size_t)rows;
    GEO_TRY(ae->xn.alloc(r * kAePts * 4));
    GEO_TRY(ae->dg1.alloc(r * 8192 * 2));
    GEO_TRY(ae->dg2.alloc(r * 4096 * 2));
    GEO_TRY(ae->dg3.alloc(r * 2048 * 2));
    GEO_TRY(ae->dz.alloc(r * 512 * 2));
    GEO_TRY(ae->dh3.alloc(r * 2048 * 2));
    GEO_TRY(ae->dh2.alloc(r * 4096 * 2));
    GEO_TRY(ae->dh1.alloc(r * 8192 * 2));
    GEO_TRY(ae->wrow.alloc(r * 4));
    ae->trows = rows;
    return GEO_OK;
}

static __nv_bfloat16 *bf(const DevBuf &b) { return b.as<__nv_bfloat16>(); }

// One GEMM level: out = act(in * W^T + b) for `rows` blocks.
static int level(geo_ae *ae, int l, int rows, const __nv_bfloat16 *in, __nv_bfloat16 *out, cudaStream_t s) {
    const AeLayer &L = kAeNet[l];
    TcGemm g{};
    g.M = rows * L.rows;
    g.N = L.N;
    g.K = L.K;
    g.A = in;
    g.B = bf(ae->wb) + ae->off.wb[l];
    g.bias = ae->params.as<float>() + ae->off.b[l];
    g.act = L.act;
    g.out = out;
    g.err = ae->err.as<int>();
    return tc_gemm(g, s);
}

// Backward through GEMM level l: weight and bias gradients, and (if din)
// the input gradient gated by the input activation (null gate: linear).
static int level_bwd(geo_ae *ae, int l, int rows, const __nv_bfloat16 *dout, const __nv_bfloat16 *in,
                     __nv_bfloat16 *din, const __nv_bfloat16 *gate, cudaStream_t s) {
    const AeLayer &L = kAeNet[l];
    const int M = rows * L.rows;
    float *gw = ae->grad.as<float>() + ae->off.w[l], *gbias = ae->grad.as<float>() + ae->off.b[l];
    {
        const int tiles = (L.K / 64) * (L.N / 64);
        int splits = (2 * 152 * 2 + tiles - 1) / tiles;
        splits = std::max(1, std::min(splits, M / 32));
        const int rws = ((M + splits - 1) / splits + 31) / 32 * 32;
        splits = (M + rws - 1) / rws;
        k_ae_wgrad<<<dim3(L.K / 64, L.N / 64, splits), 256, 0, s>>>(dout, in, gw, M, L.N, L.K, rws);
        GEO_TRY(check_launch("ae_wgrad"));
    }
    {
        const int cb = (L.N + 255) / 256;
        int splits = std::max(1, std::min(M / 64, (152 * 8) / cb));
        const int rws = (M + splits - 1) / splits;
        splits = (M + rws - 1) / rws;
        k_ae_colsum<<<dim3(cb, splits), 256, 0, s>>>(dout, gbias, M, L.N, rws);
        GEO_TRY(check_launch("ae_colsum"));
    }
    if (din) {
        TcGemm g{};
        g.M = M;
        g.N = L.K;
        g.K = L.N;
        g.A = dout;
        g.B = bf(ae->wtb) + ae->off.wb[l];
        g.gate = gate;
        g.out = din;
        g.err = ae->err.as<int>();
        GEO_TRY(tc_gemm(g, s));
    }
    return GEO_OK;
}

// Encoder levels E2..E4 from h1 into `code` (rows x 512 bf16).
static int encode_rows(geo_ae *ae, int rows, __nv_bfloat16 *code, cudaStream_t s) {
    GEO_TRY(level(ae, 1, rows, bf(ae->h1), bf(ae->h2), s));
    GEO_TRY(level(ae, 2, rows, bf(ae->h2), bf(ae->h3), s));
    return level(ae, 3, rows, bf(ae->h3), code, s);
}

// Decoder levels D4..D2 from `code` into g1.
static int decode_rows(geo_ae *ae, int rows, const __nv_bfloat16 *code, cudaStream_t s) {
    GEO_TRY(level(ae, 4, rows, code, bf(ae->g3), s));
    GEO_TRY(level(ae, 5, rows, bf(ae->g3), bf(ae->g2), s));
    return level(ae, 6, rows, bf(ae->g2), bf(ae->g1), s);
}

static E1Args e1_args(geo_ae *ae, int nb) {
    E1Args a{};
    a.nb = nb;
    a.w1 = ae->small.as<float>();
    a.b1 = ae->params.as<float>() + ae->off.b[0];
    a.h1 = bf(ae->h1);
    a.scale = ae->scale.as<float>();
    a.step = ae->step.as<int>();
    a.seed = ae->seed;
    return a;
}

static D1Args d1_args(geo_ae *ae, int nb) {
    D1Args a{};
    a.nb = nb;
    a.g1 = bf(ae->g1);
    a.v1 = ae->small.as<float>() + 128;
    a.c1 = ae->params.as<float>() + ae->off.b[7];
    a.step = ae->step.as<int>();
    return a;
}

// The host copy of the E1/D1 weights, refreshed when a pack changed them
// (a 1 KB read and a wait on the stream, once per weight version).
static int ae_mirror(geo_ae *ae, cudaStream_t s) {
    if (ae->hver == ae->wver) return GEO_OK;
    AeSmallW &h = ae->hw;
    const float *sm = ae->small.as<float>(), *pr = ae->params.as<float>();
    GEO_CUDA(cudaMemcpyAsync(h.w1, sm, sizeof h.w1, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaMemcpyAsync(h.v1, sm + 128, sizeof h.v1, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaMemcpyAsync(h.b1, pr + ae->off.b[0], sizeof h.b1, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaMemcpyAsync(h.c1, pr + ae->off.b[7], sizeof h.c1, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    ae->hver = ae->wver;
    return GEO_OK;
}

int ae_check_err(geo_ae *ae, cudaStream_t s) {
    int e = 0;
    GEO_CUDA(cudaMemcpyAsync(&e, ae->err.p, 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    if (e) return fail(GEO_ERR_CUDA, "snapshot codec: a tensor-core pipeline wait timed out");
    return GEO_OK;
}

static int blocks_of(const AeVolume &v) { return v.nbz * v.nbx * v.nby; }

AeVolume ae_volume(const float *src, long ldz, long sxy, int oz, int ox, int oy, int nz, int nx, int ny) {
    AeVolume v{};
    v.src = src;
    v.ldz = ldz;
    v.sxy = sxy;
    v.oz = oz; v.ox = ox; v.oy = oy;
    v.nz = nz; v.nx = nx; v.ny = ny;
    v.nbz = (nz + 15) / 16;
    v.nbx = (nx + 15) / 16;
    v.nby = (ny + 15) / 16;
    return v;
}

int ae_code_rows(const AeVolume &v) { return pad128(blocks_of(v)); }

int ae_escape_cap(geo_ae *ae, const AeVolume &v) {
    const int nb = blocks_of(v);
    return std::min(nb, (int)std::ceil(ae->frac * nb));
}

// Encode the interior box v into code[rows x 512] (bf16) and scale[rows];
// with esc != null also decode, and keep the residuals of the blocks the
// code misses (esc[rows], res[cap x 4096] bf16, *count escaped blocks).
int ae_encode_volume(geo_ae *ae, const AeVolume &v, void *code, float *scale, int *esc, void *res, int *count,
                     cudaStream_t s) {
    const int nb = blocks_of(v), rows = pad128(nb);
    GEO_TRY(ensure_rows(ae, rows));
    GEO_TRY(ae_mirror(ae, s));
    E1Vol a{};
    a.vol = v;
    a.nb = nb;
    a.h1 = bf(ae->h1);
    a.scale = scale;
    a.w = ae->hw;
    k_ae_e1_vol<<<rows, 256, 0, s>>>(a);
    GEO_TRY(check_launch("ae_e1"));
    GEO_TRY(encode_rows(ae, rows, static_cast<__nv_bfloat16 *>(code), s));
    if (!esc) return GEO_OK;
    if (ae_escape_cap(ae, v) == 0) {   // no escape budget: no re-decode
        GEO_CUDA(cudaMemsetAsync(esc, 0xff, (size_t)rows * 4, s));
        if (count) GEO_CUDA(cudaMemsetAsync(count, 0, 4, s));
        return GEO_OK;
    }
    if (rows > ae->erows) {
        GEO_TRY(ae->resall.alloc((size_t)rows * kAePts * 2));
        GEO_TRY(ae->err2.alloc((size_t)rows * 4));
        GEO_TRY(ae->norm2.alloc((size_t)rows * 4));
        ae->erows = rows;
    }
    GEO_TRY(decode_rows(ae, rows, static_cast<const __nv_bfloat16 *>(code), s));
    D1Vol c{};
    c.vol = v;
    c.nb = nb;
    c.mode = 3;
    c.g1 = bf(ae->g1);
    c.scale = scale;
    c.resall = bf(ae->resall);
    c.err2 = ae->err2.as<float>();
    c.norm2 = ae->norm2.as<float>();
    c.w = ae->hw;
    k_ae_d1_vol<<<rows, 256, 0, s>>>(c);
    GEO_TRY(check_launch("ae_check"));
    k_ae_select<<<1, 1024, 0, s>>>(ae->err2.as<float>(), ae->norm2.as<float>(), nb, ae->tau * ae->tau,
                                   ae_escape_cap(ae, v), esc, count);
    GEO_TRY(check_launch("ae_select"));
    k_ae_escape_copy<<<nb, 256, 0, s>>>(esc, bf(ae->resall), static_cast<__nv_bfloat16 *>(res), nb);
    return check_launch("ae_escape_copy");
}

// Decode code/scale (and escaped residuals) of box geometry v: mode 0
// writes the snapshot into dst (v's strides), mode 1 adds w * snapshot * gP
// to mig.
int ae_decode_volume(geo_ae *ae, const AeVolume &v, const void *code, const float *scale, const int *esc,
                     const void *res, int mode, float *dst, const float *gP, float *mig, float w, cudaStream_t s) {
    const int nb = blocks_of(v), rows = pad128(nb);
    GEO_TRY(ensure_rows(ae, rows));
    GEO_TRY(decode_rows(ae, rows, static_cast<const __nv_bfloat16 *>(code), s));
    GEO_TRY(ae_mirror(ae, s));
    D1Vol a{};
    a.vol = v;
    a.nb = nb;
    a.mode = mode;
    a.g1 = bf(ae->g1);
    a.scale = scale;
    a.dst = dst;
    a.gP = gP;
    a.mig = mig;
    a.wimg = w;
    a.esc = esc;
    a.res = static_cast<const __nv_bfloat16 *>(res);
    a.w = ae->hw;
    k_ae_d1_vol<<<rows, 256, 0, s>>>(a);
    return check_launch("ae_d1");
}

// Forward (+ backward when grads are wanted) over `rows` blocks already
// loaded by k_ae_e1 (xn filled); loss slot from the step counter.
static int train_pass(geo_ae *ae, int rows, double *loss, const float *wsum, int step0, float *recon, bool backward,
                      cudaStream_t s) {
    GEO_TRY(encode_rows(ae, rows, bf(ae->z), s));
    GEO_TRY(decode_rows(ae, rows, bf(ae->z), s));
    D1Args a = d1_args(ae, rows);
    a.xn = ae->xn.as<float>();
    a.recon = recon;
    a.dg1 = bf(ae->dg1);
    a.gd1 = ae->grad.as<float>() + ae->off.w[7];
    a.loss = loss;
    a.step0 = step0;
    a.wrow = wsum ? ae->wrow.as<float>() : nullptr;
    a.wsum = wsum;
    k_ae_d1<<<rows, 256, 0, s>>>(a);
    GEO_TRY(check_launch("ae_d1_train"));
    if (!backward) return GEO_OK;
    GEO_TRY(level_bwd(ae, 6, rows, bf(ae->dg1), bf(ae->g2), bf(ae->dg2), bf(ae->g2), s));   // D2
    GEO_TRY(level_bwd(ae, 5, rows, bf(ae->dg2), bf(ae->g3), bf(ae->dg3), bf(ae->g3), s));   // D3
    GEO_TRY(level_bwd(ae, 4, rows, bf(ae->dg3), bf(ae->z), bf(ae->dz), nullptr, s));        // D4
    GEO_TRY(level_bwd(ae, 3, rows, bf(ae->dz), bf(ae->h3), bf(ae->dh3), bf(ae->h3), s));    // E4
    GEO_TRY(level_bwd(ae, 2, rows, bf(ae->dh3), bf(ae->h2), bf(ae->dh2), bf(ae->h2), s));   // E3
    GEO_TRY(level_bwd(ae, 1, rows, bf(ae->dh2), bf(ae->h1), bf(ae->dh1), bf(ae->h1), s));   // E2
    k_ae_e1_bwd<<<rows, 256, 0, s>>>(ae->xn.as<float>(), bf(ae->dh1), ae->grad.as<float>() + ae->off.w[0], rows);
    return check_launch("ae_e1_bwd");
}

// He-normal initial weights (own generator, identical on every host), zero biases.
static void init_params(const AeOffsets &o, unsigned long long seed, std::vector<float> &p) {
    p.assign(o.total, 0.0f);
    unsigned long long st = seed;
    auto uni = [&]() {
        st = splitmix(st);
        return ((st >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < kAeLayers; l++) {
        const double sd = std::sqrt((kAeNet[l].act || l == 3 ? 2.0 : 1.0) / kAeNet[l].K);
        const long n = (long)kAeNet[l].N * kAeNet[l].K;
        for (long i = 0; i < n; i += 2) {
            const double u1 = uni(), u2 = uni(), r = std::sqrt(-2.0 * std::log(u1));
            p[o.w[l] + i] = (float)(sd * r * std::cos(6.283185307179586 * u2));
            if (i + 1 < n) p[o.w[l] + i + 1] = (float)(sd * r * std::sin(6.283185307179586 * u2));
        }
    }
}

}  // namespace geo

// ---------------------------------------------------------------- C ABI
extern "C" size_t geo_ae_num_params(void) { return (size_t)ae_offsets().total; }

extern "C" int geo_ae_create(geo_ae **out, unsigned long long seed) {
    if (!out) return fail(GEO_ERR_ARG, "null argument");
    geo_ae *ae = new geo_ae();
    ae->off = ae_offsets();
    ae->seed = seed;
    const size_t P = ae->off.total;
    int st = GEO_OK;
    DevBuf *f32[4] = {&ae->params, &ae->grad, &ae->m1, &ae->m2};
    for (DevBuf *b : f32)
        if (st == GEO_OK) st = b->alloc(P * 4);
    if (st == GEO_OK) st = ae->wb.alloc(ae->off.nbf * 2);
    if (st == GEO_OK) st = ae->wtb.alloc(ae->off.nbf * 2);
    if (st == GEO_OK) st = ae->small.alloc(256 * 4);
    if (st == GEO_OK) st = ae->step.alloc(16);
    if (st == GEO_OK) st = ae->err.alloc(16);
    if (st == GEO_OK) st = ae->count.alloc(16);
    if (st == GEO_OK) st = ae->snapmax.alloc(16);
    if (st != GEO_OK) {
        delete ae;
        return st;
    }
    std::vector<float> p;
    init_params(ae->off, seed, p);
    int e = GEO_OK;
    if (cudaMemcpy(ae->params.p, p.data(), P * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(ae->m1.p, 0, P * 4) != cudaSuccess || cudaMemset(ae->m2.p, 0, P * 4) != cudaSuccess ||
        cudaMemset(ae->step.p, 0, 16) != cudaSuccess || cudaMemset(ae->err.p, 0, 16) != cudaSuccess ||
        cudaMemset(ae->count.p, 0, 16) != cudaSuccess)
        e = fail(GEO_ERR_CUDA, "codec initialisation copy failed");
    if (e == GEO_OK) e = ae_pack(ae, 0, nullptr);
    if (e == GEO_OK && cudaDeviceSynchronize() != cudaSuccess) e = fail(GEO_ERR_CUDA, "codec initialisation failed");
    if (e != GEO_OK) {
        delete ae;
        return e;
    }
    *out = ae;
    return GEO_OK;
}

extern "C" int geo_ae_destroy(geo_ae *ae) {
    delete ae;
    return GEO_OK;
}

extern "C" int geo_ae_get_params(geo_ae *ae, float *host) {
    if (!ae || !host) return fail(GEO_ERR_ARG, "null argument");
    GEO_CUDA(cudaMemcpy(host, ae->params.p, ae->off.total * 4, cudaMemcpyDeviceToHost));
    return GEO_OK;
}

extern "C" int geo_ae_set_params(geo_ae *ae, const float *host) {
    if (!ae || !host) return fail(GEO_ERR_ARG, "null argument");
    GEO_CUDA(cudaMemcpy(ae->params.p, host, ae->off.total * 4, cudaMemcpyHostToDevice));
    GEO_TRY(ae_pack(ae, 0, nullptr));
    GEO_CUDA(cudaDeviceSynchronize());
    return GEO_OK;
}

extern "C" long long geo_ae_num_blocks(geo_ae *ae) {
    if (!ae || !ae->cap) return 0;
    unsigned long long n = 0;
    if (cudaMemcpy(&n, ae->count.p, 8, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    return (long long)std::min<unsigned long long>(n, (unsigned long long)ae->cap);
}

extern "C" int geo_ae_reserve(geo_ae *ae, long long max_blocks) {
    if (!ae || max_blocks < 1) return fail(GEO_ERR_ARG, "bad argument");
    GEO_TRY(ae->store.alloc((size_t)max_blocks * kAePts * 4));
    GEO_TRY(ae->wstore.alloc((size_t)max_blocks * 4));
    ae->cap = max_blocks;
    GEO_CUDA(cudaMemset(ae->count.p, 0, 16));
    return GEO_OK;
}

extern "C" int geo_ae_add_blocks(geo_ae *ae, const float *blocks, long long n, int mem) {
    if (!ae || !blocks || n < 0) return fail(GEO_ERR_ARG, "bad argument");
    const long long have = geo_ae_num_blocks(ae);
    if (have < 0 || have + n > ae->cap) return fail(GEO_ERR_ARG, "block store full (reserve more)");
    GEO_CUDA(cudaMemcpy(ae->store.as<float>() + have * kAePts, blocks, (size_t)n * kAePts * 4,
                        mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice));
    std::vector<float> ones((size_t)n, 1.0f);
    GEO_CUDA(cudaMemcpy(ae->wstore.as<float>() + have, ones.data(), (size_t)n * 4, cudaMemcpyHostToDevice));
    const unsigned long long c = (unsigned long long)(have + n);
    GEO_CUDA(cudaMemcpy(ae->count.p, &c, 8, cudaMemcpyHostToDevice));
    return GEO_OK;
}

struct CollectCtx {
    geo_ae *ae;
    geo_fd3d_plan *plan;
    int snap_every, t_first;
    float rel;
    cudaStream_t s;
};

static int collect_step(void *ctx, int it) {
    CollectCtx *c = static_cast<CollectCtx *>(ctx);
    if (it < c->t_first || (it - c->t_first) % c->snap_every) return GEO_OK;
    const Grid3D g = make_grid(c->plan);
    const AeVolume v = ae_volume(g.P, g.ldz, g.sxy, g.npd, g.npd, g.npd, g.nz, g.nx, g.ny);
    GEO_CUDA(cudaMemsetAsync(c->ae->snapmax.p, 0, 4, c->s));
    k_ae_absmax<<<152 * 8, 256, 0, c->s>>>(v, c->ae->snapmax.as<unsigned>());
    GEO_TRY(check_launch("ae_absmax"));
    k_ae_collect<<<v.nbz * v.nbx * v.nby, 256, 0, c->s>>>(v, c->ae->snapmax.as<unsigned>(), c->rel,
                                                          c->ae->store.as<float>(), c->ae->wstore.as<float>(),
                                                          c->ae->cap,
                                                          c->ae->count.as<unsigned long long>());
    return check_launch("ae_collect");
}

extern "C" int geo_ae_add_shot(geo_ae *ae, geo_fd3d_plan *plan, int is, int snap_every, int t_first, float rel,
                               void *stream) {
    if (!ae || !plan || snap_every < 1 || t_first < 0) return fail(GEO_ERR_ARG, "bad argument");
    if (!ae->cap) return fail(GEO_ERR_ARG, "reserve the block store first");
    CollectCtx c{ae, plan, snap_every, t_first, rel, (cudaStream_t)stream};
    GEO_TRY(run_shot_3d(plan, is, c.s, collect_step, &c));
    GEO_CUDA(cudaStreamSynchronize(c.s));
    return GEO_OK;
}

// Forward (and backward) of the network on given blocks (Morton order, raw
// amplitudes): recon = normalized reconstruction, loss = mean squared error
// in normalized units, grad = d loss / d params (flat, like the params).
extern "C" int geo_ae_eval(geo_ae *ae, const float *blocks, int nb, float *recon, double *loss, float *grad,
                           int mem, void *stream) {
    if (!ae || !blocks || nb < 1) return fail(GEO_ERR_ARG, "bad argument");
    if (nb % 128) return fail(GEO_ERR_ARG, "block count must be a multiple of 128");
    cudaStream_t s = (cudaStream_t)stream;
    GEO_TRY(ensure_train(ae, nb));
    DevBuf in, rec, dl;
    const float *src = blocks;
    if (mem != GEO_MEM_DEVICE) {
        GEO_TRY(in.alloc((size_t)nb * kAePts * 4));
        GEO_CUDA(cudaMemcpyAsync(in.p, blocks, (size_t)nb * kAePts * 4, cudaMemcpyHostToDevice, s));
        src = in.as<float>();
    }
    GEO_TRY(rec.alloc((size_t)nb * kAePts * 4));
    GEO_TRY(dl.alloc(16));
    GEO_TRY(dl.zero(s));
    GEO_CUDA(cudaMemsetAsync(ae->grad.p, 0, ae->off.total * 4, s));
    GEO_CUDA(cudaMemsetAsync(ae->err.p, 0, 4, s));
    E1Args a = e1_args(ae, nb);
    a.direct = src;
    a.xn = ae->xn.as<float>();
    k_ae_e1<<<nb, 256, 0, s>>>(a);
    GEO_TRY(check_launch("ae_e1"));
    int h_step = 0;
    GEO_CUDA(cudaMemcpyAsync(&h_step, ae->step.p, 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    GEO_TRY(train_pass(ae, nb, dl.as<double>(), nullptr, h_step, rec.as<float>(), grad != nullptr, s));
    GEO_TRY(ae_check_err(ae, s));
    const cudaMemcpyKind k = mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (recon) GEO_CUDA(cudaMemcpyAsync(recon, rec.p, (size_t)nb * kAePts * 4, k, s));
    if (grad) GEO_CUDA(cudaMemcpyAsync(grad, ae->grad.p, ae->off.total * 4, k, s));
    double l = 0;
    GEO_CUDA(cudaMemcpyAsync(&l, dl.p, 8, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    if (loss) *loss = l / kAePts;
    return GEO_OK;
}

// iters Adam steps on batches of `batch` blocks drawn from the store;
// learning rate lr with a cosine decay to lr/20; loss[i] = the batch's mean
// squared error with each block weighted by (its max / its snapshot's max)^2.
extern "C" int geo_ae_train(geo_ae *ae, int iters, int batch, float lr, float *loss, void *stream) {
    if (!ae || iters < 1 || batch < 128 || batch % 128) return fail(GEO_ERR_ARG, "bad argument (batch %% 128)");
    const long long nstore = geo_ae_num_blocks(ae);
    if (nstore < 1) return fail(GEO_ERR_ARG, "the block store is empty");
    cudaStream_t s = nullptr;
    GEO_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct SG {
        cudaStream_t s;
        ~SG() { cudaStreamDestroy(s); }
    } sg{s};
    (void)stream;
    GEO_CUDA(cudaDeviceSynchronize());
    GEO_TRY(ensure_train(ae, batch));
    int step0 = 0;
    GEO_CUDA(cudaMemcpy(&step0, ae->step.p, 4, cudaMemcpyDeviceToHost));
    std::vector<float> lrs(iters);
    for (int i = 0; i < iters; i++)
        lrs[i] = (float)(lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(3.141592653589793 * i / iters))));
    DevBuf dlr, dloss, dwsum;
    GEO_TRY(dlr.alloc((size_t)iters * 4));
    GEO_TRY(dloss.alloc((size_t)iters * 8));
    GEO_TRY(dwsum.alloc((size_t)iters * 4));
    GEO_TRY(dwsum.zero(s));
    GEO_CUDA(cudaMemcpyAsync(dlr.p, lrs.data(), (size_t)iters * 4, cudaMemcpyHostToDevice, s));
    GEO_TRY(dloss.zero(s));
    GEO_CUDA(cudaMemsetAsync(ae->err.p, 0, 4, s));
    auto iteration = [&]() -> int {
        GEO_CUDA(cudaMemsetAsync(ae->grad.p, 0, ae->off.total * 4, s));
        E1Args a = e1_args(ae, batch);
        a.store = ae->store.as<float>();
        a.nstore = nstore;
        a.xn = ae->xn.as<float>();
        a.wstore = ae->wstore.as<float>();
        a.wrow = ae->wrow.as<float>();
        a.wsum = dwsum.as<float>();
        a.step0 = step0;
        k_ae_e1<<<batch, 256, 0, s>>>(a);
        GEO_TRY(check_launch("ae_e1"));
        GEO_TRY(train_pass(ae, batch, dloss.as<double>(), dwsum.as<float>(), step0, nullptr, true, s));
        k_ae_adam<<<152 * 4, 256, 0, s>>>(ae->params.as<float>(), ae->grad.as<float>(), ae->m1.as<float>(),
                                          ae->m2.as<float>(), ae->off.total, ae->step.as<int>(), step0,
                                          dlr.as<float>());
        GEO_TRY(check_launch("ae_adam"));
        return ae_pack(ae, 1, s);
    };
    // first iteration eagerly (sets kernel attributes), the rest from a graph
    GEO_TRY(iteration());
    if (iters > 1) {
        const long long before = launches_so_far();
        cudaGraph_t graph = nullptr;
        GEO_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const int st = iteration();
        cudaError_t ce = cudaStreamEndCapture(s, &graph);
        if (st != GEO_OK) {
            if (graph) cudaGraphDestroy(graph);
            return st;
        }
        if (ce != cudaSuccess) return fail(GEO_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
        const long long per = launches_so_far() - before;
        count_launch(-per);
        cudaGraphExec_t exec = nullptr;
        ce = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) return fail(GEO_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ce));
        for (int i = 1; i < iters && ce == cudaSuccess; i++) {
            ce = cudaGraphLaunch(exec, s);
            count_launch(per);
        }
        cudaGraphExecDestroy(exec);
        if (ce != cudaSuccess) return fail(GEO_ERR_CUDA, "graph launch: %s", cudaGetErrorString(ce));
    }
    ae->wver++;   // the graph's packs changed the weights
    GEO_TRY(ae_check_err(ae, s));
    std::vector<double> l(iters);
    GEO_CUDA(cudaMemcpyAsync(l.data(), dloss.p, (size_t)iters * 8, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    if (loss)
        for (int i = 0; i < iters; i++) loss[i] = (float)(l[i] / kAePts);
    return GEO_OK;
}

void geo::ae_note_run(geo_ae *ae, long long blocks, long long escaped) {
    ae->st_blocks += blocks;
    ae->st_escaped += escaped;
}

// Coded and escaped blocks over the RTM shots run with this codec.
extern "C" int geo_ae_stats(geo_ae *ae, long long *blocks, long long *escaped) {
    if (!ae) return fail(GEO_ERR_ARG, "null codec");
    if (blocks) *blocks = ae->st_blocks;
    if (escaped) *escaped = ae->st_escaped;
    return GEO_OK;
}

// Escape settings: per snapshot, the (at most frac of all) blocks with the
// largest squared decoding error, among those whose error exceeds tau times
// their norm, keep their residual.
extern "C" int geo_ae_set_escape(geo_ae *ae, float tau, float frac) {
    if (!ae || !(tau >= 0) || !(frac >= 0) || frac > 1) return fail(GEO_ERR_ARG, "bad argument");
    ae->tau = tau;
    ae->frac = frac;
    return GEO_OK;
}

// Encode + decode a dense nz-fastest volume (nx*ny*nz, layout
// iz + nz*(ix + nx*iy), device pointers): out = the codec's reconstruction
// (with escapes when `escape`); *nesc (optional) = escaped blocks.
extern "C" int geo_ae_roundtrip(geo_ae *ae, int nx, int ny, int nz, const float *vol, float *out, int escape,
                                int *nesc, void *stream) {
    if (!ae || !vol || !out || nx < 1 || ny < 1 || nz < 1) return fail(GEO_ERR_ARG, "bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    const AeVolume v = ae_volume(vol, nz, (long)nz * nx, 0, 0, 0, nz, nx, ny);
    const int rows = ae_code_rows(v), cap = ae_escape_cap(ae, v);
    DevBuf code, scale, esc, res, cnt;
    GEO_TRY(code.alloc((size_t)rows * kAeLat * 2));
    GEO_TRY(scale.alloc((size_t)rows * 4));
    if (escape) {
        GEO_TRY(esc.alloc((size_t)rows * 4));
        GEO_TRY(res.alloc((size_t)std::max(cap, 1) * kAePts * 2));
        GEO_TRY(cnt.alloc(16));
        GEO_TRY(cnt.zero(s));
    }
    GEO_CUDA(cudaMemsetAsync(ae->err.p, 0, 4, s));
    GEO_TRY(ae_encode_volume(ae, v, code.p, scale.as<float>(), esc.as<int>(), res.p, cnt.as<int>(), s));
    GEO_TRY(ae_decode_volume(ae, v, code.p, scale.as<float>(), esc.as<int>(), res.p, 0, out, nullptr, nullptr, 0.0f,
                             s));
    if (nesc) {
        *nesc = 0;
        if (escape) GEO_CUDA(cudaMemcpyAsync(nesc, cnt.p, 4, cudaMemcpyDeviceToHost, s));
    }
    return ae_check_err(ae, s);
}
