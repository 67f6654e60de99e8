// 3D TTI time step: tilt t (from the vertical) and azimuth f of the symmetry
// axis per grid point.  No reference program has a 3D TTI scheme; this one
// extends the 2D TTI GPU programs' rotated-derivative scheme
// (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:81-183) to a tilted
// and rotated axis.  With the rotated frame
//   x' = (cos t cos f, cos t sin f, -sin t), y' = (-sin f, cos f, 0),
//   z' = (sin t cos f, sin t sin f, cos t):
//   u <- k2 u - k1 dP/dx',  v <- k2 v - k1 dP/dy',  w <- k2 w - k1 dQ/dz'
//   P <- k2 P - k1 (A a + B b),  Q <- k2 Q - k1 (B a + C b)
// a = du/dx' + dv/dy', b = dw/dz', A = vp^2(1+2eps), B = vp^2 sqrtf(1+2del),
// C = vp^2 (the plan's premultiplied model), k the 2D programs' product
// sponge (half-grid profiles for the velocities, integer-grid for the
// stresses).  Each axis derivative has the 2D programs' stagger (forward for
// the velocities, backward for the stresses).  With t = f = 0 the
// derivatives are the VTI step's; with f = 0 and no y the 2D programs'.
// The operation order per point is the oracle's (orc_tti3d), so FP32
// results are bit-identical to it.
//
// Two kernels per step, each marching along y over a 32(z) x 16(x) column
// and a chunk of planes, two x columns per thread, every read through a
// 3-stage TMA ring (one mbarrier per stage, waits bounded at 2 s like the
// VTI step's), writes as plain coalesced stores:
//
//   velocity: x and z taps of P and Q from a halo box of the output plane
//     (z 40 from z0-4, x 24 from x0-4); y taps from 8-deep register queues
//     of the thread's own columns, fed by own boxes four planes ahead; old
//     u,v,w and cos/sin of tilt and azimuth as own boxes;
//   stress: x and z taps of the new u, v, w from halo boxes of the output
//     plane, y taps from queues fed three planes ahead; P, Q of the old
//     level, the model and the trig as own boxes; receivers and the RTM
//     imaging epilogue.
//
// The point source is added to P,Q of the old level before the velocity
// kernel (the cell's old values kept in `save` for the stress update), so
// it reaches the velocities only, as in the VTI step.
#include "geo_internal.h"
#include "fd3d.cuh"
#include "fd3d_fused.cuh"
#include "tc_util.cuh"
#include <cudaTypedefs.h>
#include <map>
#include <mutex>
#include <tuple>

namespace geo {

__constant__ float c_tti3d[4] = {1.196289f, -0.0797526f, 0.009570313f, -0.0006975447f};

using tc::mbar_expect_tx;
using tc::mbar_init;
using tc::mbar_wait;
using tc::su32;

namespace {

constexpr int TZ = kTZ, TX = kTXF, NW = kTXF / 2, NST = 3;
constexpr int OB = TZ * TX;           // own box: z 32, x 16
constexpr int HB = 40 * (TX + 8);     // halo box: z 40 from z0-4, x 24 from x0-4
constexpr int VB = 32 * (TX + 8);     // x-halo box: z 32, x 24 from x0-4

// velocity stage: P own (queue plane), Q own, P halo, Q halo, u, v, w, ct, st, cp, sp
constexpr int V_PO = 0, V_QO = OB, V_PH = 2 * OB, V_QH = 2 * OB + HB, V_U = 2 * OB + 2 * HB, V_T = V_U + 3 * OB;
constexpr int VSTAGE = V_T + 4 * OB;
// stress stage: u,v,w own (queue plane), u halo, v halo, w halo, P own, Q own, A B C, ct st cp sp
constexpr int S_UO = 0, S_UH = 3 * OB, S_VH = S_UH + HB, S_WH = S_VH + VB, S_PQ = S_WH + HB, S_M = S_PQ + 2 * OB,
              S_T = S_M + 3 * OB;
constexpr int SSTAGE = S_T + 4 * OB;
static_assert((OB * 4) % 128 == 0 && (HB * 4) % 128 == 0 && (VB * 4) % 128 == 0, "TMA boxes stay 128-byte aligned");
constexpr size_t VEL_SMEM = (size_t)NST * VSTAGE * 4 + 256;
constexpr size_t STR_SMEM = (size_t)NST * SSTAGE * 4 + 256;
static_assert(2 * STR_SMEM + 2048 <= 233472 && 2 * VEL_SMEM + 2048 <= 233472, "two blocks per SM");

// Tensor maps of one step's reads (box shapes in the comments).
struct VelMaps {
    CUtensorMap ph, qh;        // P, Q of the old level: halo box
    CUtensorMap po, qo;        // P, Q of the old level: own box
    CUtensorMap u, v, w;       // old velocities: own box
    CUtensorMap t[4];          // cos/sin of tilt, cos/sin of azimuth: own box
};
struct StrMaps {
    CUtensorMap uo, vo, wo;    // new velocities: own box (queue feed)
    CUtensorMap uh, vh, wh;    // new velocities: halo boxes (v: x halo only)
    CUtensorMap po, qo;        // P, Q of the old level: own box
    CUtensorMap m[3];          // A, B, C: own box
    CUtensorMap t[4];
};

struct TtiGeom {
    int nnx, nny, nnz, ldz, npd, nx, ny, nz;
    int sxy;
    float dtx, dty, dtz;
    const float *cx1, *cx2, *ax1, *ax2, *cy1, *cy2, *ay1, *ay2, *cz1, *cz2, *az1, *az2;
    int ntz, ntiles, chunk;
    int *err;
};

__device__ __forceinline__ void tma3(float *dst, const CUtensorMap *map, int c0, int c1, int c2, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
            "r"(su32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(su32(bar))
        : "memory");
}

__device__ __forceinline__ float *align128(unsigned char *p) {
    return reinterpret_cast<float *>((reinterpret_cast<uintptr_t>(p) + 127) & ~uintptr_t(127));
}

// Wait for stage s of iteration i; on a timeout report, let the copies in
// flight land (bounded) and tell the caller to return.
__device__ __forceinline__ bool stage_ready(uint64_t *bar, int s, uint32_t &phase, int *s_abort, int tid, int *err) {
    if (tid == 0 && !mbar_wait(&bar[s], (phase >> s) & 1u)) *s_abort = 1;
    phase ^= 1u << s;
    __syncthreads();
    if (*s_abort) {
        if (tid == 0) {
            atomicExch(err, 1);
            for (int k = 1; k < NST; k++) {
                const int s2 = (s + k) % NST;
                mbar_wait(&bar[s2], (phase >> s2) & 1u);
            }
        }
        return false;
    }
    return true;
}

__global__ void __launch_bounds__(TZ *NW, 2)
    k_tti3d_vel(const __grid_constant__ VelMaps M, const TtiGeom g, float *__restrict__ u1, float *__restrict__ v1,
                float *__restrict__ w1) {
    extern __shared__ unsigned char smem_raw[];
    float *stages = align128(smem_raw);
    uint64_t *bar = reinterpret_cast<uint64_t *>(stages + NST * VSTAGE);
    __shared__ int s_abort;
    const int lane = threadIdx.x, wy = threadIdx.y, tid = wy * 32 + lane;
    const int tile = blockIdx.x % g.ntiles, chunk = blockIdx.x / g.ntiles;
    const int z0 = (tile % g.ntz) * TZ, x0 = (tile / g.ntz) * TX;
    const int ylo = 4 + chunk * g.chunk, yhi = min(ylo + g.chunk, g.nny - 4);
    // iteration i brings P,Q of plane ylo-3+i into the queues and, for
    // i >= 7, updates plane ylo+i-7 (its taps ylo+i-10 .. ylo+i-3)
    const int NI = (yhi - ylo) + 7;
    if (tid == 0) {
        for (int s = 0; s < NST; s++) mbar_init(&bar[s], 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int i) {
        const int s = i % NST, q = ylo - 3 + i, y = ylo + i - 7;
        const bool out = i >= 7;
        float *sp = stages + s * VSTAGE;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (wy == 0) {
            uint32_t bytes = 2 * OB * 4;
            if (out) bytes += (2 * HB + 7 * OB) * 4;
            mbar_expect_tx(&bar[s], bytes);
            tma3(sp + V_PO, &M.po, z0, x0, q, &bar[s]);
            tma3(sp + V_QO, &M.qo, z0, x0, q, &bar[s]);
        } else if (wy == 1) {
            if (out) {
                tma3(sp + V_PH, &M.ph, z0 - 4, x0 - 4, y, &bar[s]);
                tma3(sp + V_QH, &M.qh, z0 - 4, x0 - 4, y, &bar[s]);
            }
        } else if (wy == 2) {
            if (out) {
                tma3(sp + V_U, &M.u, z0, x0, y, &bar[s]);
                tma3(sp + V_U + OB, &M.v, z0, x0, y, &bar[s]);
                tma3(sp + V_U + 2 * OB, &M.w, z0, x0, y, &bar[s]);
            }
        } else {
            if (out)
                for (int r = 0; r < 4; r++) tma3(sp + V_T + r * OB, &M.t[r], z0, x0, y, &bar[s]);
        }
    };
    if (lane == 0 && wy < 4)
        for (int i = 0; i < NST && i < NI; i++) issue(i);

    const int ca = 2 * wy, xa = x0 + ca, zo = z0 + lane;
    const bool z_upd = zo >= 4 && zo < g.nnz - 4;
    const bool upd_a = z_upd && xa >= 4 && xa < g.nnx - 4, upd_b = z_upd && xa + 1 >= 4 && xa + 1 < g.nnx - 4;
    const int xca = min(max(xa, 0), g.nnx - 1), xcb = min(max(xa + 1, 0), g.nnx - 1), zc = min(max(zo, 0), g.nnz - 1);
    const float c1a = g.cx1[xca], c2a = g.cx2[xca], c1b = g.cx1[xcb], c2b = g.cx2[xcb];
    const float c1z = g.cz1[zc], c2z = g.cz2[zc];
    const int oa = ca * 32 + lane;          // own box index of column a (b: +32)
    const int col_a = zo + g.ldz * xa;      // global index of column a at y = 0 (b: + ldz)
    float pa[8], pb[8], qa[8], qb[8];
#pragma unroll
    for (int k = 0; k < 8; k++) pa[k] = pb[k] = qa[k] = qb[k] = 0.0f;
    uint32_t phase = 0;
    for (int i = 0; i < NI; i++) {
        const int s = i % NST;
        if (!stage_ready(bar, s, phase, &s_abort, tid, g.err)) return;
        if (lane == 0 && wy < 4 && i >= 1 && i - 1 + NST < NI) issue(i - 1 + NST);
        const float *sp = stages + s * VSTAGE;
#pragma unroll
        for (int k = 0; k < 7; k++) {
            pa[k] = pa[k + 1]; pb[k] = pb[k + 1];
            qa[k] = qa[k + 1]; qb[k] = qb[k + 1];
        }
        pa[7] = sp[V_PO + oa]; pb[7] = sp[V_PO + oa + 32];
        qa[7] = sp[V_QO + oa]; qb[7] = sp[V_QO + oa + 32];
        if (i < 7) continue;
        const int y = ylo + i - 7;
        const float cy1 = __ldg(g.cy1 + y), cy2 = __ldg(g.cy2 + y);
#pragma unroll
        for (int cb = 0; cb < 2; cb++) {
            const float *pq = cb ? pb : pa, *qq = cb ? qb : qa;
            const float *PH = sp + V_PH + (ca + cb + 4) * 40 + lane + 4;   // the point in the P halo box
            const float *QH = sp + V_QH + (ca + cb + 4) * 40 + lane + 4;
            float Px = 0.0f, Py = 0.0f, Pz = 0.0f, Qx = 0.0f, Qy = 0.0f, Qz = 0.0f;
#pragma unroll
            for (int im = 0; im < 4; im++) {
                const float c = c_tti3d[im];
                Px += c * (PH[(im + 1) * 40] - PH[-im * 40]);
                Py += c * (pq[im + 4] - pq[3 - im]);
                Pz += c * (PH[im + 1] - PH[-im]);
                Qx += c * (QH[(im + 1) * 40] - QH[-im * 40]);
                Qy += c * (qq[im + 4] - qq[3 - im]);
                Qz += c * (QH[im + 1] - QH[-im]);
            }
            const int o = oa + 32 * cb;
            const float a = sp[V_T + o], b = sp[V_T + OB + o], cc = sp[V_T + 2 * OB + o], sn = sp[V_T + 3 * OB + o];
            const float k2 = (cb ? c2b : c2a) * cy2 * c2z;
            const float k1 = (cb ? c1b : c1a) * cy1 * c1z;
            const float gx = a * cc * g.dtx * Px + a * sn * g.dty * Py - b * g.dtz * Pz;
            const float gy = cc * g.dty * Py - sn * g.dtx * Px;
            const float gz = b * cc * g.dtx * Qx + b * sn * g.dty * Qy + a * g.dtz * Qz;
            const float un = k2 * sp[V_U + o] - k1 * gx;
            const float vn = k2 * sp[V_U + OB + o] - k1 * gy;
            const float wn = k2 * sp[V_U + 2 * OB + o] - k1 * gz;
            if (cb ? upd_b : upd_a) {
                const int id = col_a + cb * g.ldz + g.sxy * y;
                u1[id] = un;
                v1[id] = vn;
                w1[id] = wn;
            }
        }
    }
}

__global__ void __launch_bounds__(TZ *NW, 2)
    k_tti3d_stress(const __grid_constant__ StrMaps M, const TtiGeom g, float *__restrict__ P1, float *__restrict__ Q1,
                   const float *__restrict__ save, const StepArgs3D st) {
    extern __shared__ unsigned char smem_raw[];
    float *stages = align128(smem_raw);
    uint64_t *bar = reinterpret_cast<uint64_t *>(stages + NST * SSTAGE);
    __shared__ int s_abort;
    const int lane = threadIdx.x, wy = threadIdx.y, tid = wy * 32 + lane;
    const int tile = blockIdx.x % g.ntiles, chunk = blockIdx.x / g.ntiles;
    const int z0 = (tile % g.ntz) * TZ, x0 = (tile / g.ntz) * TX;
    const int ylo = 4 + chunk * g.chunk, yhi = min(ylo + g.chunk, g.nny - 4);
    // iteration i brings u,v,w of plane ylo-4+i into the queues and, for
    // i >= 7, updates plane ylo+i-7 (its taps ylo+i-11 .. ylo+i-4)
    const int NI = (yhi - ylo) + 7;
    if (tid == 0) {
        for (int s = 0; s < NST; s++) mbar_init(&bar[s], 1);
        s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int i) {
        const int s = i % NST, q = ylo - 4 + i, y = ylo + i - 7;
        const bool out = i >= 7;
        float *sp = stages + s * SSTAGE;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if (wy == 0) {
            uint32_t bytes = 3 * OB * 4;
            if (out) bytes += (2 * HB + VB + 9 * OB) * 4;
            mbar_expect_tx(&bar[s], bytes);
            tma3(sp + S_UO, &M.uo, z0, x0, q, &bar[s]);
            tma3(sp + S_UO + OB, &M.vo, z0, x0, q, &bar[s]);
            tma3(sp + S_UO + 2 * OB, &M.wo, z0, x0, q, &bar[s]);
        } else if (wy == 1) {
            if (out) {
                tma3(sp + S_UH, &M.uh, z0 - 4, x0 - 4, y, &bar[s]);
                tma3(sp + S_VH, &M.vh, z0, x0 - 4, y, &bar[s]);
                tma3(sp + S_WH, &M.wh, z0 - 4, x0 - 4, y, &bar[s]);
            }
        } else if (wy == 2) {
            if (out) {
                tma3(sp + S_PQ, &M.po, z0, x0, y, &bar[s]);
                tma3(sp + S_PQ + OB, &M.qo, z0, x0, y, &bar[s]);
                for (int r = 0; r < 3; r++) tma3(sp + S_M + r * OB, &M.m[r], z0, x0, y, &bar[s]);
            }
        } else {
            if (out)
                for (int r = 0; r < 4; r++) tma3(sp + S_T + r * OB, &M.t[r], z0, x0, y, &bar[s]);
        }
    };
    if (lane == 0 && wy < 4)
        for (int i = 0; i < NST && i < NI; i++) issue(i);

    const int ca = 2 * wy, xa = x0 + ca, zo = z0 + lane;
    const bool z_upd = zo >= 4 && zo < g.nnz - 4;
    const bool upd_a = z_upd && xa >= 4 && xa < g.nnx - 4, upd_b = z_upd && xa + 1 >= 4 && xa + 1 < g.nnx - 4;
    const int xca = min(max(xa, 0), g.nnx - 1), xcb = min(max(xa + 1, 0), g.nnx - 1), zc = min(max(zo, 0), g.nnz - 1);
    const float a1a = g.ax1[xca], a2a = g.ax2[xca], a1b = g.ax1[xcb], a2b = g.ax2[xcb];
    const float a1z = g.az1[zc], a2z = g.az2[zc];
    const bool z_in = zo >= g.npd && zo < g.npd + g.nz;
    const bool in_a = z_in && xa >= g.npd && xa < g.npd + g.nx, in_b = z_in && xa + 1 >= g.npd && xa + 1 < g.npd + g.nx;
    int rec_a = -1, rec_b = -1;
    if (st.rec && zo == st.rec_iz) {
        const int ra = xa - g.npd - st.rx0, rb = ra + 1;
        if (ra >= 0 && ra % st.drx == 0 && ra / st.drx < st.nrx) rec_a = ra / st.drx;
        if (rb >= 0 && rb % st.drx == 0 && rb / st.drx < st.nrx) rec_b = rb / st.drx;
    }
    const int oa = ca * 32 + lane;
    const int col_a = zo + g.ldz * xa;
    float ua[8], ub[8], va[8], vb[8], wa[8], wb[8];
#pragma unroll
    for (int k = 0; k < 8; k++) ua[k] = ub[k] = va[k] = vb[k] = wa[k] = wb[k] = 0.0f;
    uint32_t phase = 0;
    for (int i = 0; i < NI; i++) {
        const int s = i % NST;
        if (!stage_ready(bar, s, phase, &s_abort, tid, g.err)) return;
        if (lane == 0 && wy < 4 && i >= 1 && i - 1 + NST < NI) issue(i - 1 + NST);
        const float *sp = stages + s * SSTAGE;
#pragma unroll
        for (int k = 0; k < 7; k++) {
            ua[k] = ua[k + 1]; ub[k] = ub[k + 1];
            va[k] = va[k + 1]; vb[k] = vb[k + 1];
            wa[k] = wa[k + 1]; wb[k] = wb[k + 1];
        }
        ua[7] = sp[S_UO + oa]; ub[7] = sp[S_UO + oa + 32];
        va[7] = sp[S_UO + OB + oa]; vb[7] = sp[S_UO + OB + oa + 32];
        wa[7] = sp[S_UO + 2 * OB + oa]; wb[7] = sp[S_UO + 2 * OB + oa + 32];
        if (i < 7) continue;
        const int y = ylo + i - 7;
        const float ay1 = __ldg(g.ay1 + y), ay2 = __ldg(g.ay2 + y);
        const bool y_in = y >= g.npd && y < g.npd + g.ny;
        // RTM operands of this plane, loaded before the arithmetic
        float pre_ill[2] = {0.0f, 0.0f}, pre_mig[2] = {0.0f, 0.0f}, pre_oth[2] = {0.0f, 0.0f};
        if ((st.ill || st.mig) && y_in) {
#pragma unroll
            for (int cb = 0; cb < 2; cb++) {
                if (!(cb ? in_b : in_a)) continue;
                const long o = (long)(zo - g.npd) + (long)g.nz * ((xa + cb - g.npd) + (long)g.nx * (y - g.npd));
                if (st.ill) pre_ill[cb] = st.ill[o];
                if (st.mig) {
                    pre_mig[cb] = st.mig[o];
                    pre_oth[cb] = st.other_P[col_a + cb * g.ldz + g.sxy * y];
                }
            }
        }
#pragma unroll
        for (int cb = 0; cb < 2; cb++) {
            const float *uq = cb ? ub : ua, *vq = cb ? vb : va, *wq = cb ? wb : wa;
            const float *UH = sp + S_UH + (ca + cb + 4) * 40 + lane + 4;
            const float *VH = sp + S_VH + (ca + cb + 4) * 32 + lane;
            const float *WH = sp + S_WH + (ca + cb + 4) * 40 + lane + 4;
            float ux = 0.0f, uy = 0.0f, uz = 0.0f, vx = 0.0f, vy = 0.0f, wx = 0.0f, wy_ = 0.0f, wz = 0.0f;
#pragma unroll
            for (int im = 0; im < 4; im++) {
                const float c = c_tti3d[im];
                ux += c * (UH[im * 40] - UH[-(im + 1) * 40]);
                uy += c * (uq[im + 4] - uq[3 - im]);
                uz += c * (UH[im] - UH[-im - 1]);
                vx += c * (VH[im * 32] - VH[-(im + 1) * 32]);
                vy += c * (vq[im + 4] - vq[3 - im]);
                wx += c * (WH[im * 40] - WH[-(im + 1) * 40]);
                wy_ += c * (wq[im + 4] - wq[3 - im]);
                wz += c * (WH[im] - WH[-im - 1]);
            }
            const int o = oa + 32 * cb;
            const float a = sp[S_T + o], b = sp[S_T + OB + o], cc = sp[S_T + 2 * OB + o], sn = sp[S_T + 3 * OB + o];
            const float ha = (a * cc * g.dtx * ux + a * sn * g.dty * uy - b * g.dtz * uz) + (cc * g.dty * vy - sn * g.dtx * vx);
            const float hb = b * cc * g.dtx * wx + b * sn * g.dty * wy_ + a * g.dtz * wz;
            const float k2 = (cb ? a2b : a2a) * ay2 * a2z;
            const float k1 = (cb ? a1b : a1a) * ay1 * a1z;
            const long id = (long)col_a + cb * g.ldz + (long)g.sxy * y;
            float p0 = sp[S_PQ + o], q0 = sp[S_PQ + OB + o];
            if (st.src_on && id == st.src) {
                p0 = save[0];
                q0 = save[1];
            }
            const float mA = sp[S_M + o], mB = sp[S_M + OB + o], mC = sp[S_M + 2 * OB + o];
            const float P = k2 * p0 - k1 * (mA * ha + mB * hb);
            const float Q = k2 * q0 - k1 * (mB * ha + mC * hb);
            if (!(cb ? upd_b : upd_a)) continue;
            P1[id] = P;
            Q1[id] = Q;
            const int rix = cb ? rec_b : rec_a;
            if (rix >= 0) {
                const int ry = y - g.npd - st.ry0;
                if (ry >= 0 && ry % st.dry == 0 && ry / st.dry < st.nry)
                    st.rec[(long)st.it * st.nrx * st.nry + rix + (long)st.nrx * (ry / st.dry)] = st.rec_pq ? P + Q : P;
            }
            if ((st.ill || st.mig) && (cb ? in_b : in_a) && y_in) {
                const long o2 = (long)(zo - g.npd) + (long)g.nz * ((xa + cb - g.npd) + (long)g.nx * (y - g.npd));
                if (st.ill) st.ill[o2] = pre_ill[cb] + (P * P + Q * Q);
                if (st.mig) st.mig[o2] = pre_mig[cb] + pre_oth[cb] * P;
            }
        }
    }
}

// Source cell: keep P,Q of level c, then add the amplitude.
__global__ void k_tti3d_source(float *P, float *Q, long src, float amp, float *save) {
    save[0] = P[src];
    save[1] = Q[src];
    P[src] += amp;
    Q[src] += amp;
}

// Tensor maps per set of buffers and grid, encoded once and kept.
struct MapKey {
    const void *p[16];
    int nnz, ldz, nnx, nny;
    bool operator<(const MapKey &o) const {
        return std::tie(nnz, ldz, nnx, nny) < std::tie(o.nnz, o.ldz, o.nnx, o.nny) ||
               (std::tie(nnz, ldz, nnx, nny) == std::tie(o.nnz, o.ldz, o.nnx, o.nny) &&
                std::lexicographical_compare(p, p + 16, o.p, o.p + 16));
    }
};
struct MapPair {
    VelMaps v;
    StrMaps s;
};
std::map<MapKey, MapPair> g_maps;
std::mutex g_maps_mu;

int tti_maps(const Tti3DStep &t, const MapPair **out) {
    const Grid3D &g = t.g;
    MapKey key{};
    const void *ptrs[16] = {t.P0, t.Q0, t.u0, t.v0, t.w0, t.u1, t.v1, t.w1, t.ct, t.st, t.cp, t.sp, g.vp, g.e2, g.d2,
                            nullptr};
    for (int k = 0; k < 16; k++) key.p[k] = ptrs[k];
    key.nnz = g.nnz; key.ldz = g.ldz; key.nnx = g.nnx; key.nny = g.nny;
    std::lock_guard<std::mutex> lock(g_maps_mu);
    auto it = g_maps.find(key);
    if (it == g_maps.end()) {
        if (g_maps.size() > 64) g_maps.clear();   // plans come and go: keep the cache small
        MapPair m;
        const int nz = g.nnz, ld = g.ldz, nx = g.nnx, ny = g.nny;
        GEO_TRY(encode_map(&m.v.ph, t.P0, nz, ld, nx, ny, 40, TX + 8));
        GEO_TRY(encode_map(&m.v.qh, t.Q0, nz, ld, nx, ny, 40, TX + 8));
        GEO_TRY(encode_map(&m.v.po, t.P0, nz, ld, nx, ny, TZ, TX));
        GEO_TRY(encode_map(&m.v.qo, t.Q0, nz, ld, nx, ny, TZ, TX));
        GEO_TRY(encode_map(&m.v.u, t.u0, nz, ld, nx, ny, TZ, TX));
        GEO_TRY(encode_map(&m.v.v, t.v0, nz, ld, nx, ny, TZ, TX));
        GEO_TRY(encode_map(&m.v.w, t.w0, nz, ld, nx, ny, TZ, TX));
        const float *tr[4] = {t.ct, t.st, t.cp, t.sp};
        for (int r = 0; r < 4; r++) {
            GEO_TRY(encode_map(&m.v.t[r], tr[r], nz, ld, nx, ny, TZ, TX));
            m.s.t[r] = m.v.t[r];
        }
        GEO_TRY(encode_map(&m.s.uo, t.u1, nz, ld, nx, ny, TZ, TX));
        GEO_TRY(encode_map(&m.s.vo, t.v1, nz, ld, nx, ny, TZ, TX));
        GEO_TRY(encode_map(&m.s.wo, t.w1, nz, ld, nx, ny, TZ, TX));
        GEO_TRY(encode_map(&m.s.uh, t.u1, nz, ld, nx, ny, 40, TX + 8));
        GEO_TRY(encode_map(&m.s.vh, t.v1, nz, ld, nx, ny, TZ, TX + 8));
        GEO_TRY(encode_map(&m.s.wh, t.w1, nz, ld, nx, ny, 40, TX + 8));
        m.s.po = m.v.po;
        m.s.qo = m.v.qo;
        const float *md[3] = {g.vp, g.e2, g.d2};
        for (int r = 0; r < 3; r++) GEO_TRY(encode_map(&m.s.m[r], md[r], nz, ld, nx, ny, TZ, TX));
        it = g_maps.emplace(key, m).first;
    }
    *out = &it->second;
    return GEO_OK;
}

int tti_chunks() {
    const char *e = getenv("GEO_TTI3D_CHUNKS");
    return e ? std::max(1, atoi(e)) : 4;
}

}  // namespace

int launch_tti3d(const Tti3DStep &t, const StepArgs3D &args, cudaStream_t s) {
    static bool attr = false;
    StepArgs3D st = args;
    const Grid3D &g = t.g;
    st.src = st.izs + (long)g.ldz * (st.ixs + (long)g.nnx * st.iys);
    if (st.src_on) {
        k_tti3d_source<<<1, 1, 0, s>>>(const_cast<float *>(t.P0), const_cast<float *>(t.Q0), st.src, st.amp, t.save);
        GEO_TRY(check_launch("tti3d_source"));
    }
    const MapPair *m = nullptr;
    GEO_TRY(tti_maps(t, &m));
    if (!attr) {
        GEO_CUDA(cudaFuncSetAttribute(k_tti3d_vel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)VEL_SMEM));
        GEO_CUDA(cudaFuncSetAttribute(k_tti3d_stress, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)STR_SMEM));
        attr = true;
    }
    if ((long)g.sxy * g.nny >= (1L << 31)) return fail(GEO_ERR_ARG, "grid too large for 32-bit plane offsets");
    TtiGeom G;
    G.nnx = g.nnx; G.nny = g.nny; G.nnz = g.nnz; G.ldz = g.ldz; G.npd = g.npd;
    G.nx = g.nx; G.ny = g.ny; G.nz = g.nz; G.sxy = (int)g.sxy;
    G.dtx = g.dtx; G.dty = g.dty; G.dtz = g.dtz;
    G.cx1 = g.cx1; G.cx2 = g.cx2; G.ax1 = g.ax1; G.ax2 = g.ax2; G.cy1 = g.cy1; G.cy2 = g.cy2; G.ay1 = g.ay1;
    G.ay2 = g.ay2; G.cz1 = g.cz1; G.cz2 = g.cz2; G.az1 = g.az1; G.az2 = g.az2;
    G.ntz = (g.nnz + TZ - 1) / TZ;
    G.ntiles = G.ntz * ((g.nnx + TX - 1) / TX);
    const int planes = g.nny - 8;
    const int nch = std::max(1, std::min(tti_chunks(), planes / 8));
    G.chunk = (planes + nch - 1) / nch;
    const int nchunks = (planes + G.chunk - 1) / G.chunk;
    G.err = t.err;
    const dim3 block(TZ, NW), grid(G.ntiles * nchunks);
    k_tti3d_vel<<<grid, block, VEL_SMEM, s>>>(m->v, G, t.u1, t.v1, t.w1);
    GEO_TRY(check_launch("tti3d_vel"));
    k_tti3d_stress<<<grid, block, STR_SMEM, s>>>(m->s, G, t.P1, t.Q1, t.save, st);
    return check_launch("tti3d_stress");
}

}  // namespace geo
