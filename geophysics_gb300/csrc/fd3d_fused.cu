// Fused 3D VTI time step: one kernel per step, marching along y.
//
// A block owns a 32(z) x 16(x) column of the grid and a chunk of y planes.
// Per plane it rebuilds the velocities it needs from P,Q (u with a 4-cell
// x halo, w with a 4-cell z halo, v from a register queue along y) and then
// updates the stresses, so u,v,w never make a round trip through HBM between
// the two half-steps of the reference (GPU_vti3dfd_kernels.cu:90-201).
//
// Data movement: the old level's P, Q, u, w, v arrive by TMA
// (cp.async.bulk.tensor) into shared memory, paced by one mbarrier per
// stage of a 4-deep plane pipeline; P planes stay resident in a ring (the 8
// y taps of dv/dt plus the planes in flight).  The model and the split
// sponge stresses, read only at their own point, come as coalesced loads
// issued at the top of each plane.  Writes are plain coalesced stores to the
// next level (u,v,w,P,Q ping-pong between steps; split stresses in place).
//
// Arithmetic: GEO_MODE_EXACT keeps the reference's operation chain (no
// contraction) and is bit-identical to it; GEO_MODE_FAST uses fused
// multiply-adds at fixed places and the premultiplied model (A,B,C), the
// same operations as the oracle's fast mode.
#include "geo_internal.h"
#include "fd3d.cuh"
#include "fd3d_fused.cuh"
#include <cudaTypedefs.h>

namespace geo {

__constant__ float cf_fd[4] = {1.196289f, -0.0797526f, 0.009570313f, -0.0006975447f};

// stage layout (floats)
constexpr int OFF_Q = 0;
constexpr int OFF_U = OFF_Q + kQB;
constexpr int OFF_W = OFF_U + kUB;
constexpr int OFF_V = OFF_W + kQB;
static_assert(OFF_V + kOB == kStageFloats, "stage layout");
static_assert((OFF_U * 4) % 128 == 0 && (OFF_W * 4) % 128 == 0 && (OFF_V * 4) % 128 == 0 &&
                  (kStageFloats * 4) % 128 == 0 && (kPB * 4) % 128 == 0,
              "TMA destinations must stay 128-byte aligned");
static_assert(kRing >= 9, "the new plane must not land on a tap of the current plane");

__device__ __forceinline__ uint32_t su32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(su32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t gtimer() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for a stage with a 2 s limit; false on timeout.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = gtimer();
    while (!mbar_try_wait(bar, parity))
        if (gtimer() - t0 > 2000000000ull) return false;
    return true;
}

__device__ __forceinline__ void tma3(float *dst, const CUtensorMap *map, int c0, int c1, int c2, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(su32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(su32(bar))
        : "memory");
}

// 8-tap staggered derivative sum_m c_m (a_m - b_m).  EXACT: the reference's
// accumulation from 0; FAST: first product, then three fused multiply-adds.
template <int MODE>
__device__ __forceinline__ float deriv(float a0, float b0, float a1, float b1, float a2, float b2, float a3,
                                       float b3) {
    if (MODE == GEO_MODE_FAST) {
        float d = cf_fd[0] * (a0 - b0);
        d = __fmaf_rn(cf_fd[1], a1 - b1, d);
        d = __fmaf_rn(cf_fd[2], a2 - b2, d);
        return __fmaf_rn(cf_fd[3], a3 - b3, d);
    }
    float d = 0.0f;
    d += cf_fd[0] * (a0 - b0);
    d += cf_fd[1] * (a1 - b1);
    d += cf_fd[2] * (a2 - b2);
    d += cf_fd[3] * (a3 - b3);
    return d;
}

// Velocity update: c2*old - k1*d with k1 = c1*dt.
template <int MODE>
__device__ __forceinline__ float vel_update(float c2, float old, float k1, float d) {
    if (MODE == GEO_MODE_FAST) return __fmaf_rn(-k1, d, c2 * old);
    return c2 * old - k1 * d;
}

// Derivative along a shared-memory line: taps p[(m+1)*s] - p[-m*s].
template <int MODE>
__device__ __forceinline__ float dline_fwd(const float *p, int s) {
    return deriv<MODE>(p[s], p[0], p[2 * s], p[-s], p[3 * s], p[-2 * s], p[4 * s], p[-3 * s]);
}
// Taps p[m*s] - p[-(m+1)*s].
template <int MODE>
__device__ __forceinline__ float dline_bwd(const float *p, int s) {
    return deriv<MODE>(p[0], p[-s], p[s], p[-2 * s], p[2 * s], p[-3 * s], p[3 * s], p[-4 * s]);
}

template <int MODE>
__global__ void __launch_bounds__(kTZ *kTXF, 2)
    k_fused3d(const __grid_constant__ StepMaps tm, const Fused3D g, const StepArgs3D st) {
    extern __shared__ unsigned char smem_raw[];
    float *base = reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    float *ring = base;
    float *stages = ring + kRing * kPB;
    float *utile = stages + kStages * kStageFloats;
    float *wtile = utile + kUTile;
    uint64_t *bar = reinterpret_cast<uint64_t *>(wtile + kWTile);
    __shared__ int s_abort;

    const int lane = threadIdx.x, wx = threadIdx.y, tid = wx * 32 + lane;
    const int tile = blockIdx.x % g.ntiles, chunk = blockIdx.x / g.ntiles;
    const int z0 = (tile % g.ntz) * kTZ, x0 = (tile / g.ntz) * kTXF;
    const int ylo = 4 + chunk * g.chunk;
    const int yhi = min(ylo + g.chunk, g.nny - 4);
    const int NJ = (yhi - ylo) + 7;
    const int ybase = ylo - 7;  // plane of iteration j is ybase + j
    const bool xz_inside = x0 >= g.npd && x0 + kTXF <= g.npd + g.nx && z0 >= g.npd && z0 + kTZ <= g.npd + g.nz;

    if (tid == 0) {
        for (int s = 0; s < kStages; s++) mbar_init(&bar[s], 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // Loads of iteration j into stage j % kStages and ring slot (j+7) % kRing.
    auto issue = [&](int j) {
        const int s = j % kStages;
        const int y = ybase + j;
        float *sp = stages + s * kStageFloats;
        uint32_t bytes = (kPB + kOB) * 4;
        if (j >= 7) bytes += (kQB + kUB + kQB) * 4;
        if (j == 0) bytes += 7 * kPB * 4;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_expect_tx(&bar[s], bytes);
        if (j == 0)
            for (int k = 0; k < 7; k++) tma3(ring + k * kPB, &tm.m[0], z0, x0 - 7, ybase + k, &bar[s]);
        tma3(ring + ((j + 7) % kRing) * kPB, &tm.m[0], z0, x0 - 7, y + 7, &bar[s]);
        tma3(sp + OFF_V, &tm.m[4], z0, x0, y + 3, &bar[s]);
        if (j >= 7) {
            tma3(sp + OFF_Q, &tm.m[1], z0 - 8, x0, y, &bar[s]);
            tma3(sp + OFF_U, &tm.m[2], z0, x0 - 4, y, &bar[s]);
            tma3(sp + OFF_W, &tm.m[3], z0 - 8, x0, y, &bar[s]);
        }
    };
    if (tid == 0)
        for (int j = 0; j < kStages && j < NJ; j++) issue(j);

    // ---- per-thread constants
    const int xo = x0 + wx, zo = z0 + lane;
    const bool x_upd = xo >= 4 && xo < g.nnx - 4, z_upd = zo >= 4 && zo < g.nnz - 4;
    const bool xz_upd = x_upd && z_upd;
    const int xc = min(max(xo, 0), g.nnx - 1), zc = min(max(zo, 0), g.nnz - 1);
    const float kx = g.cx1[xc] * g.dtx, cx2 = g.cx2[xc], ax1 = g.ax1[xc], ax2 = g.ax2[xc];
    const float kz = g.cz1[zc] * g.dtz, cz2 = g.cz2[zc], az1 = g.az1[zc], az2 = g.az2[zc];
    // halo velocities: warps 0-6 take u on the 7 halo columns (4 left, 3
    // right of the tile), threads 224-335 take w on the 7 halo depths of each
    // column (4 above, 3 below)
    int h_col = 0, h_q = 0;
    bool h_upd = false;
    float hk = 0.0f, hc2 = 0.0f;
    if (wx < 7) {
        h_col = wx < 4 ? wx : kTXF + wx;  // utile / u-box column
        const int x = x0 - 4 + h_col;
        h_upd = x >= 4 && x < g.nnx - 4 && z_upd;
        const int xcl = min(max(x, 0), g.nnx - 1);
        hk = g.cx1[xcl] * g.dtx;
        hc2 = g.cx2[xcl];
    } else if (tid < 224 + 7 * kTXF) {
        const int t = tid - 224;
        h_col = t / 7;
        const int h = t % 7;
        h_q = h < 4 ? h : kTZ + h;  // wtile index (z0-4 origin)
        const int z = z0 - 4 + h_q, x = x0 + h_col;
        h_upd = z >= 4 && z < g.nnz - 4 && x >= 4 && x < g.nnx - 4;
        const int zcl = min(max(z, 0), g.nnz - 1);
        hk = g.cz1[zcl] * g.dtz;
        hc2 = g.cz2[zcl];
    }
    const long ldz = g.ldz, sxy = g.sxy;
    const long col_off = zo + ldz * xo;  // own column at y = 0
    float q[8];
#pragma unroll
    for (int k = 0; k < 8; k++) q[k] = 0.0f;
    uint32_t phase = 0;
    int sj = 0;  // ring slot of plane ybase + j

    for (int j = 0; j < NJ; j++) {
        const int s = j % kStages;
        const int y = ybase + j;
        if (tid == 0 && !mbar_wait(&bar[s], (phase >> s) & 1u)) s_abort = 1;
        phase ^= 1u << s;
        __syncthreads();
        if (s_abort) {
            // a stage never completed: report, let copies in flight land
            // (bounded), and leave
            if (tid == 0) {
                atomicExch(g.err, 1);
                for (int k = 1; k < kStages; k++) {
                    const int s2 = (s + k) % kStages;
                    mbar_wait(&bar[s2], (phase >> s2) & 1u);
                }
            }
            return;
        }
        // stage (j-1) % kStages and ring slot of plane ybase+j-1 are free now
        if (tid == 0 && j >= 1 && j - 1 + kStages < NJ) issue(j - 1 + kStages);
        float *sp = stages + s * kStageFloats;
        const long yoff = sxy * y;

        // model and split stresses of this plane, consumed after the velocities
        const bool stress_plane = j >= 7;
        const bool need_split = MODE == GEO_MODE_EXACT || !xz_inside || y < g.npd || y >= g.npd + g.ny;
        float m0 = 0, m1 = 0, m2 = 0, s0 = 0, s1 = 0, s2 = 0, s3 = 0, s4 = 0, s5 = 0;
        if (stress_plane && xz_upd) {
            const long id = col_off + yoff;
            m0 = __ldg(g.m0 + id); m1 = __ldg(g.m1 + id); m2 = __ldg(g.m2 + id);
            if (need_split) {
                s0 = g.px[id]; s1 = g.py[id]; s2 = g.pz[id];
                s3 = g.qx[id]; s4 = g.qy[id]; s5 = g.qz[id];
            }
        }

        // point source, P,Q += amp before the velocity update
        // (GPU_vti3dfd_kernels.cu:135): patch the shared copies that hold the
        // source cell; the own-point stress update reads P,Q from global.
        if (st.src_on) {
            const int plo = (j == 0) ? ybase : y + 7;
            const bool pP = st.iys >= plo && st.iys <= y + 7 && st.izs >= z0 && st.izs < z0 + kTZ &&
                            st.ixs >= x0 - 7 && st.ixs < x0 + kTXF + 7;
            const bool pQ = stress_plane && st.iys == y && st.ixs >= x0 && st.ixs < x0 + kTXF &&
                            st.izs >= z0 - 8 && st.izs < z0 + 40;
            if (pP || pQ) {
                if (tid == 0) {
                    if (pP) ring[((st.iys - ybase) % kRing) * kPB + (st.ixs - (x0 - 7)) * 32 + (st.izs - z0)] += st.amp;
                    if (pQ) sp[OFF_Q + (st.ixs - x0) * 48 + (st.izs - (z0 - 8))] += st.amp;
                }
                __syncthreads();
            }
        }

        // slot of plane ybase + j + k
        auto slot = [&](int k) { const int t = sj + k; return t >= kRing ? t - kRing : t; };

        // v at plane y+3 from the ring (planes y .. y+7), into the queue
        {
            const int yv = y + 3;
            const float vold = sp[OFF_V + wx * 32 + lane];
            float vn = vold;
            if (xz_upd && yv >= 4 && yv < g.nny - 4) {
                const int col = (wx + 7) * 32 + lane;
                const float yy = deriv<MODE>(ring[slot(4) * kPB + col], ring[slot(3) * kPB + col],
                                             ring[slot(5) * kPB + col], ring[slot(2) * kPB + col],
                                             ring[slot(6) * kPB + col], ring[slot(1) * kPB + col],
                                             ring[slot(7) * kPB + col], ring[slot(0) * kPB + col]);
                vn = vel_update<MODE>(g.cy2[yv], vold, g.cy1[yv] * g.dty, yy);
                g.v1[col_off + sxy * yv] = vn;
            }
#pragma unroll
            for (int k = 0; k < 7; k++) q[k] = q[k + 1];
            q[7] = vn;
        }

        if (stress_plane) {
            const float *ry = ring + sj * kPB;
            // own u (column wx+4 of the u tile) and own w (depth lane+4)
            {
                const int c = wx + 4;
                const float uo = sp[OFF_U + c * 32 + lane];
                float un = uo;
                if (xz_upd) {
                    un = vel_update<MODE>(cx2, uo, kx, dline_fwd<MODE>(ry + (c + 3) * 32 + lane, 32));
                    g.u1[col_off + yoff] = un;
                }
                utile[c * 32 + lane] = un;
                const float wo = sp[OFF_W + wx * 48 + lane + 8];
                float wn = wo;
                if (xz_upd) {
                    wn = vel_update<MODE>(cz2, wo, kz, dline_fwd<MODE>(sp + OFF_Q + wx * 48 + lane + 8, 1));
                    g.w1[col_off + yoff] = wn;
                }
                wtile[wx * 40 + lane + 4] = wn;
            }
            // halo u and w
            if (wx < 7) {
                const float uo = sp[OFF_U + h_col * 32 + lane];
                float un = uo;
                if (h_upd) un = vel_update<MODE>(hc2, uo, hk, dline_fwd<MODE>(ry + (h_col + 3) * 32 + lane, 32));
                utile[h_col * 32 + lane] = un;
            } else if (tid < 224 + 7 * kTXF) {
                const float wo = sp[OFF_W + h_col * 48 + h_q + 4];
                float wn = wo;
                if (h_upd) wn = vel_update<MODE>(hc2, wo, hk, dline_fwd<MODE>(sp + OFF_Q + h_col * 48 + h_q + 4, 1));
                wtile[h_col * 40 + h_q] = wn;
            }
            __syncthreads();

            if (xz_upd) {
                const float yy = deriv<MODE>(q[4], q[3], q[5], q[2], q[6], q[1], q[7], q[0]);
                const float xx = dline_bwd<MODE>(utile + (wx + 4) * 32 + lane, 32);
                const float zz = dline_bwd<MODE>(wtile + wx * 40 + lane + 4, 1);
                const long id = col_off + yoff;
                const bool inside = MODE == GEO_MODE_FAST && xo >= g.npd && xo < g.npd + g.nx && y >= g.npd &&
                                    y < g.npd + g.ny && zo >= g.npd && zo < g.npd + g.nz;
                float P, Q;
                if (MODE == GEO_MODE_FAST) {
                    // m0,m1,m2 = A,B,C
                    const float Ax = m0 * g.dtx, Ay = m0 * g.dty, Bz = m1 * g.dtz;
                    const float Bx = m1 * g.dtx, By = m1 * g.dty, Cz = m2 * g.dtz;
                    if (inside) {
                        float p0 = ry[(wx + 7) * 32 + lane], q0 = sp[OFF_Q + wx * 48 + lane + 8];
                        if (st.src_on && id == st.src) {
                            p0 = g.P0[id];
                            q0 = g.Q0[id];
                        }
                        P = __fmaf_rn(-Bz, zz, __fmaf_rn(-Ay, yy, __fmaf_rn(-Ax, xx, p0)));
                        Q = __fmaf_rn(-Cz, zz, __fmaf_rn(-By, yy, __fmaf_rn(-Bx, xx, q0)));
                    } else {
                        const float ay1 = g.ay1[y], ay2 = g.ay2[y];
                        const float px = __fmaf_rn(-(ax1 * Ax), xx, ax2 * s0);
                        const float py = __fmaf_rn(-(ay1 * Ay), yy, ay2 * s1);
                        const float pz = __fmaf_rn(-(az1 * Bz), zz, az2 * s2);
                        const float qx = __fmaf_rn(-(ax1 * Bx), xx, ax2 * s3);
                        const float qy = __fmaf_rn(-(ay1 * By), yy, ay2 * s4);
                        const float qz = __fmaf_rn(-(az1 * Cz), zz, az2 * s5);
                        g.px[id] = px; g.py[id] = py; g.pz[id] = pz;
                        g.qx[id] = qx; g.qy[id] = qy; g.qz[id] = qz;
                        P = px + py + pz;
                        Q = qx + qy + qz;
                    }
                } else {
                    // m0,m1,m2 = vp, 1+2eps, sqrtf(1+2del); the reference's chain
                    const float vp = m0, e2 = m1, d2 = m2, ay1 = g.ay1[y], ay2 = g.ay2[y];
                    const float px = ax2 * s0 - ax1 * vp * vp * e2 * g.dtx * xx;
                    const float py = ay2 * s1 - ay1 * vp * vp * e2 * g.dty * yy;
                    const float pz = az2 * s2 - az1 * vp * vp * d2 * g.dtz * zz;
                    const float qx = ax2 * s3 - ax1 * vp * vp * d2 * g.dtx * xx;
                    const float qy = ay2 * s4 - ay1 * vp * vp * d2 * g.dty * yy;
                    const float qz = az2 * s5 - az1 * vp * vp * g.dtz * zz;
                    g.px[id] = px; g.py[id] = py; g.pz[id] = pz;
                    g.qx[id] = qx; g.qy[id] = qy; g.qz[id] = qz;
                    P = px + py + pz;
                    Q = qx + qy + qz;
                }
                g.P1[id] = P;
                g.Q1[id] = Q;
                if (st.rec && zo == st.rec_iz) {
                    const int rx = xo - g.npd - st.rx0, rr = y - g.npd - st.ry0;
                    if (rx >= 0 && rr >= 0 && rx % st.drx == 0 && rr % st.dry == 0) {
                        const int irx = rx / st.drx, iry = rr / st.dry;
                        if (irx < st.nrx && iry < st.nry)
                            st.rec[(long)st.it * st.nrx * st.nry + irx + (long)st.nrx * iry] = P;
                    }
                }
            }
        }
        sj = sj + 1 == kRing ? 0 : sj + 1;
    }
}

// ------------------------------------------------------------------ host
static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

int encode_map(CUtensorMap *map, const float *base, int nnz, int ldz, int nnx, int nny, int boxz, int boxx) {
    if (!g_encode) {
        void *fn = nullptr;
        cudaDriverEntryPointQueryResult q;
        GEO_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
        if (!fn || q != cudaDriverEntryPointSuccess) return fail(GEO_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
        g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
    }
    if ((ldz * 4) % 16 != 0 || (reinterpret_cast<uintptr_t>(base) & 15) != 0)
        return fail(GEO_ERR_ARG, "tensor map needs 16-byte aligned base and z stride");
    cuuint64_t dims[3] = {(cuuint64_t)nnz, (cuuint64_t)nnx, (cuuint64_t)nny};
    cuuint64_t strides[2] = {(cuuint64_t)ldz * 4, (cuuint64_t)ldz * nnx * 4};
    cuuint32_t box[3] = {(cuuint32_t)boxz, (cuuint32_t)boxx, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = g_encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box, estr,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(GEO_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return GEO_OK;
}

int launch_fused3d(const StepMaps &maps, const Fused3D &g, int mode, int it, int src_on, float amp, int ixs, int iys,
                   int izs, float *rec, int rec_iz, int rx0, int drx, int nrx, int ry0, int dry, int nry,
                   cudaStream_t s) {
    static bool attr_set[2] = {false, false};
    StepArgs3D st{};
    st.it = it; st.src_on = src_on; st.amp = amp;
    st.ixs = ixs; st.iys = iys; st.izs = izs;
    st.src = izs + (long)g.ldz * (ixs + (long)g.nnx * iys);
    st.rec = rec; st.rec_iz = rec_iz; st.rx0 = rx0; st.drx = drx; st.nrx = nrx; st.ry0 = ry0; st.dry = dry; st.nry = nry;
    dim3 block(kTZ, kTXF), grid(g.nitems);
    if (mode == GEO_MODE_FAST) {
        if (!attr_set[0]) {
            GEO_CUDA(cudaFuncSetAttribute(k_fused3d<GEO_MODE_FAST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFusedSmem));
            attr_set[0] = true;
        }
        k_fused3d<GEO_MODE_FAST><<<grid, block, kFusedSmem, s>>>(maps, g, st);
    } else {
        if (!attr_set[1]) {
            GEO_CUDA(cudaFuncSetAttribute(k_fused3d<GEO_MODE_EXACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFusedSmem));
            attr_set[1] = true;
        }
        k_fused3d<GEO_MODE_EXACT><<<grid, block, kFusedSmem, s>>>(maps, g, st);
    }
    return check_launch("fused3d");
}

}  // namespace geo
