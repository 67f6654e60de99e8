// 2D VTI staggered-grid kernels, batched over shots.
//
// One launch updates every shot of a batch: the grid is persistent (a
// multiple of the SM count) and walks the list of (shot, tile) work items,
// so uneven aperture windows share one launch.  A tile is 32 z-points (one
// warp, z contiguous in memory) by `blockDim.y` x-columns.
//
// Arithmetic keeps the reference's operation order exactly (the library is
// compiled with contraction off), so results are bit-identical to the
// reference CPU code and to the oracle:
//   velocity  CPU_vti2dfd_kernels.c:79-106 / GPU_vti2dfd_kernels.cu:209-238
//   stress    CPU_vti2dfd_kernels.c:108-177 / GPU_vti2dfd_kernels.cu:240-299
//             MPI program Toa_rtm_vti_adcig_cdp.c:1227-1327 (rho*vp^2 form,
//             pz/qx chains in double after pow(1+2del, 0.5))
#include "geo_internal.h"
#include "tc_util.cuh"
#include "gridsync.cuh"
#include "softcvt.cuh"
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <cstdlib>

namespace geo {

__constant__ float c_fd[4] = {1.196289f, -0.0797526f, 0.009570313f, -0.0006975447f};
// exp(-x^2-z^2) on the 7x7 source window, x,z in [-3,3] (ptsource,
// CPU_vti2dfd_kernels.c:72); filled from the host's exp() at load.
__constant__ double c_gauss[49];

static bool g_gauss_ready = false;
static int ensure_gauss() {
    if (g_gauss_ready) return GEO_OK;
    double g[49];
    for (int x = -3; x <= 3; x++)
        for (int z = -3; z <= 3; z++) g[(x + 3) * 7 + (z + 3)] = std::exp((double)(-z * z - x * x));
    GEO_CUDA(cudaMemcpyToSymbol(c_gauss, g, sizeof g));
    g_gauss_ready = true;
    return GEO_OK;
}

struct Tile2D {
    const Shot2D *sh;
    int ix, iz;
};

__device__ __forceinline__ bool locate(const Shot2D *shots, const int *item_shot, int item, Tile2D &t) {
    const int s = item_shot[item];
    const Shot2D *sh = shots + s;
    const int tile = item - sh->tile_base;
    const int tz = tile % sh->ntz, tx = tile / sh->ntz;
    t.sh = sh;
    t.iz = tz * 32 + threadIdx.x;
    t.ix = tx * blockDim.y + threadIdx.y;
    return t.ix >= 4 && t.ix < sh->nnx - 4 && t.iz >= 4 && t.iz < sh->nnz - 4;
}

// Reads of neighbours' values.  Kernels of one half-step read fields that
// no thread of the launch writes, through the read-only path (NC); the
// persistent shot kernel reads values other blocks wrote before a grid
// barrier, through L2 (the read-only path is not coherent with them).
template <bool NC>
__device__ __forceinline__ float ldf(const float *p) {
    return NC ? __ldg(p) : __ldcg(p);
}

// P/Q read for the velocity update.  The GPU-form source (P,Q += amp at one
// cell before the velocity update, GPU_vti2dfd_kernels.cu:423) is applied on
// the fly to the taps that touch the source cell.
template <bool PT_SRC, bool NC>
__device__ __forceinline__ float tap(const float *a, long idx, long src, float amp) {
    float v = NC ? a[idx] : __ldcg(a + idx);
    if (PT_SRC && idx == src) v = v + amp;
    return v;
}

// Poynting-vector angle gathers (RTM_corr_adcig, Toa_rtm_vti_adcig_cdp.c:1004-1068):
// per image point the angle bin ia of the opening angle between the source
// and receiver Poynting vectors, and adcig[ia] += gP*sP*cos(ia)^3.  The
// program bins with (int)(float)(0.5*acosf(a1)*180/pi); that bin is a
// non-increasing function of the float a1, so the host finds, with the same
// libm, the largest a1 of every bin count (c_adthr[k-1]: largest a1 whose
// bin is >= k) and the kernel counts thresholds instead of calling acosf.
__constant__ float c_adthr[kAdcigAngles];
__constant__ double c_adw[kAdcigAngles];

__device__ __forceinline__ int adcig_bin(float a1) {
    if (!(a1 >= -1.0f && a1 <= 1.0f)) return 0;
    int lo = 0, hi = kAdcigAngles;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a1 <= c_adthr[mid - 1]) lo = mid;
        else hi = mid - 1;
    }
    return lo == kAdcigAngles ? kAdcigAngles - 1 : lo;   // ia == 90 -> 89
}

// Velocity update of one updated point (ix, iz) of a shot, every field.
template <int VARIANT, bool NC>
__device__ __forceinline__ void vel_point(const Shot2D &sh, int ix, int iz, const Step2D &st) {
    const int nnz = sh.nnz;
    const long id = (long)ix * nnz + iz;
    const bool pt_src = VARIANT == V_GPU && st.src_on;
    const long src = (long)sh.ixs * nnz + sh.izs;
    const bool near = pt_src && ((iz == sh.izs && abs(ix - sh.ixs) <= 4) || (ix == sh.ixs && abs(iz - sh.izs) <= 4));
    for (int f = 0; f < st.nf; f++) {
        const float *P = sh.P[f], *Q = sh.Q[f];
        float xx = 0.0f, zz = 0.0f;
        if (near) {
#pragma unroll
            for (int im = 0; im < 4; im++) {
                xx += c_fd[im] * (tap<true, NC>(P, id + (im + 1) * nnz, src, st.amp) - tap<true, NC>(P, id - im * nnz, src, st.amp));
                zz += c_fd[im] * (tap<true, NC>(Q, id + im + 1, src, st.amp) - tap<true, NC>(Q, id - im, src, st.amp));
            }
        } else {
#pragma unroll
            for (int im = 0; im < 4; im++) {
                xx += c_fd[im] * (ldf<NC>(P + id + (im + 1) * nnz) - ldf<NC>(P + id - im * nnz));
                zz += c_fd[im] * (ldf<NC>(Q + id + im + 1) - ldf<NC>(Q + id - im));
            }
        }
        float *u = sh.u[f], *w = sh.w[f];
        // u1 = coffx2*u0 - coffx1*dtx*xx (the MPI copy's extra *rho is *1.0f)
        u[id] = sh.cx2[ix] * u[id] - sh.cx1[ix] * sh.dtx * xx;
        w[id] = sh.cz2[iz] * w[id] - sh.cz1[iz] * sh.dtz * zz;
    }
}

template <int VARIANT>
__global__ void __launch_bounds__(256) k_vel2d(const Shot2D *__restrict__ shots, const int *__restrict__ item_shot,
                                               int nitems, Step2D st) {
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        Tile2D t;
        if (!locate(shots, item_shot, item, t)) continue;
        vel_point<VARIANT, true>(*t.sh, t.ix, t.iz, st);
    }
}

// Stress update of one updated point (ix, iz) of a shot, every field, and
// the phase's epilogue (records and edge lines forward; image, illumination
// and gathers backward).
template <int VARIANT, int PHASE, bool NC, bool FAST = false>
__device__ __forceinline__ void stress_point(const Shot2D &sh, int ix, int iz, const Step2D &st) {
    const int nnz = sh.nnz;
    const long id = (long)ix * nnz + iz;
    const float vp = __ldg(sh.vp + id);
    // the MPI form's exact arithmetic carries its pz and qx chains in double
    // (their fixed factors kz, kx formed per shot on the host in the
    // program's order); its fast form (FAST, a separate instantiation so
    // that no double operation is issued) uses the FP32 sqrtf(1+2del) of
    // the others
    constexpr bool dpw = VARIANT == V_MPI && !FAST;
    float e2 = __ldg(sh.e2 + id), d2 = 0.0f;
    double kz = 0.0, kx = 0.0;
    if (dpw) {
        kz = __ldg(sh.kz + id);
        kx = __ldg(sh.kx + id);
    } else {
        d2 = __ldg(sh.d2 + id);
    }
    if (st.taper) {
        const int bx = ix - sh.tx0, bz = iz - sh.tz0;
        if (bx >= 0 && bx < kTB && bz >= 0 && bz < kTB) {
            e2 = sh.te2[bx * kTB + bz];
            if (dpw) {
                kz = sh.tkz[bx * kTB + bz];
                kx = sh.tkx[bx * kTB + bz];
            } else {
                d2 = sh.td2[bx * kTB + bz];
            }
        }
    }
    const float ax1 = sh.ax1[ix], ax2 = sh.ax2[ix], az1 = sh.az1[iz], az2 = sh.az2[iz];
    // Gaussian source window value (CPU/MPI forward), added after the split sum.
    float s = 0.0f;
    if ((VARIANT == V_CPU || VARIANT == V_MPI) && PHASE == PH_FWD && st.src_on) {
        const int rx = ix - sh.ixs, rz = iz - sh.izs;
        if (rx >= -3 && rx <= 3 && rz >= -3 && rz <= 3)
            s = (float)((double)st.amp * c_gauss[(rx + 3) * 7 + (rz + 3)]);
    }
    float Pn[2], Qn[2];
    for (int f = 0; f < st.nf; f++) {
        const float *u = sh.u[f], *w = sh.w[f];
        float xx = 0.0f, zz = 0.0f;
#pragma unroll
        for (int im = 0; im < 4; im++) {
            xx += c_fd[im] * (ldf<NC>(u + id + im * nnz) - ldf<NC>(u + id - (im + 1) * nnz));
            zz += c_fd[im] * (ldf<NC>(w + id + im) - ldf<NC>(w + id - im - 1));
        }
        float px = sh.px[f][id], pz = sh.pz[f][id], qx = sh.qx[f][id], qz = sh.qz[f][id];
        if (VARIANT == V_MPI) {
            px = ax2 * px - ax1 * vp * e2 * sh.dtx * xx;
            if (dpw) {
                // the conversions on the integer pipe (softcvt.cuh): same bits
                pz = d2f_rn(f2d_exact(az2 * pz) - kz * f2d_exact(zz));
                qx = d2f_rn(f2d_exact(ax2 * qx) - kx * f2d_exact(xx));
            } else {
                pz = az2 * pz - az1 * vp * d2 * sh.dtz * zz;
                qx = ax2 * qx - ax1 * vp * d2 * sh.dtx * xx;
            }
            qz = az2 * qz - az1 * vp * sh.dtz * zz;
        } else {
            px = ax2 * px - ax1 * vp * vp * e2 * sh.dtx * xx;
            pz = az2 * pz - az1 * vp * vp * d2 * sh.dtz * zz;
            qx = ax2 * qx - ax1 * vp * vp * d2 * sh.dtx * xx;
            qz = az2 * qz - az1 * vp * vp * sh.dtz * zz;
        }
        sh.px[f][id] = px; sh.pz[f][id] = pz; sh.qx[f][id] = qx; sh.qz[f][id] = qz;
        float P, Q;
        if ((VARIANT == V_CPU || VARIANT == V_MPI) && PHASE == PH_FWD) {
            P = px + pz + s;
            Q = qx + qz + s;
        } else {
            P = px + pz;
            Q = qx + qz;
        }
        sh.P[f][id] = P;
        sh.Q[f][id] = Q;
        Pn[f] = P; Qn[f] = Q;
    }
    const int gx = ix - sh.npd, gz = iz - sh.npd;
    if (PHASE == PH_FWD) {
        // receiver gather at rec_iz, time-major
        if (iz == sh.rec_iz && gx >= 0 && gx < sh.nx) {
            const float r = sh.rec_scale == 2.0f ? Pn[0] + Pn[0] : Pn[0] * sh.rec_scale;
            sh.rec_p[(long)st.it * sh.nx + gx] = r;
            if (sh.rec_q) sh.rec_q[(long)st.it * sh.nx + gx] = Qn[0];
        }
        // interior-edge lines for the boundary-driven reconstruction
        // (Toa_rtm_vti_adcig_cdp.c:668-683): top, bottom, left, right
        if (sh.edge_p && gx >= 0 && gx < sh.nx && gz >= 0 && gz < sh.nz) {
            const long L = 2L * sh.nx + 2L * sh.nz, b = (long)st.it * L;
            if (gz == 0) { sh.edge_p[b + gx] = Pn[0]; sh.edge_q[b + gx] = Qn[0]; }
            if (gz == sh.nz - 1) { sh.edge_p[b + sh.nx + gx] = Pn[0]; sh.edge_q[b + sh.nx + gx] = Qn[0]; }
            if (gx == 0) { sh.edge_p[b + 2 * sh.nx + gz] = Pn[0]; sh.edge_q[b + 2 * sh.nx + gz] = Qn[0]; }
            if (gx == sh.nx - 1) { sh.edge_p[b + 2 * sh.nx + sh.nz + gz] = Pn[0]; sh.edge_q[b + 2 * sh.nx + sh.nz + gz] = Qn[0]; }
        }
    } else if (st.nf == 2 && gx >= 0 && gx < sh.nx && gz >= 0 && gz < sh.nz) {
        // zero-lag cross-correlation image and source illumination
        // (Toa_rtm_vti_adcig_cdp.c:1067-1076): the illumination sum is
        // formed in double, as pow() returns it, and a zero becomes 1
        const long o = (long)gx * sh.nz + gz;
        const float sv = Pn[0];
        float ill;
        if (FAST) ill = sh.ill[o] + sv * sv;
        else {
            const double svd = f2d_exact(sv);
            ill = d2f_rn(f2d_exact(sh.ill[o]) + svd * svd);
        }
        if (ill == 0.0f) ill = 1.0f;
        sh.ill[o] = ill;
        sh.mig[o] = sh.mig[o] + Pn[1] * sv;
        if (sh.adcig) {
            // Poynting vectors from the new P,Q and u,w of both fields
            const float sx = -Pn[0] * sh.u[0][id], sz = -Qn[0] * sh.w[0][id];
            const float gx = Pn[1] * sh.u[1][id], gz = Qn[1] * sh.w[1][id];
            const float b1 = sx * sx + sz * sz, b2 = gx * gx + gz * gz, a = sx * gx + sz * gz;
            const float a1 = (float)((double)a / ((double)sqrtf(b1 * b2) + 0.0000000000001));
            const int ia = adcig_bin(a1);
            float *ag = sh.adcig + (long)ia * sh.nx * sh.nz + o;
            *ag = d2f_rn(f2d_exact(*ag) + f2d_exact(Pn[1] * sv) * c_adw[ia]);
        }
    }
}

template <int VARIANT, int PHASE, bool FAST = false>
__global__ void __launch_bounds__(256) k_stress2d(const Shot2D *__restrict__ shots, const int *__restrict__ item_shot,
                                                  int nitems, Step2D st) {
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        Tile2D t;
        if (!locate(shots, item_shot, item, t)) continue;
        stress_point<VARIANT, PHASE, true, FAST>(*t.sh, t.ix, t.iz, st);
    }
}

// ------------------------------------------------------ persistent shot
// A whole single-shot forward run in one cooperative launch: per step the
// velocity half-step over every tile, a grid barrier, the stress half-step
// (records, edge lines), a grid barrier.  Same per-point arithmetic as the
// per-half-step kernels; neighbours' values are read through L2.
template <int VARIANT>
__global__ void __launch_bounds__(512) k_fd2d_shot(const Shot2D *__restrict__ shots,
                                                   const int *__restrict__ item_shot, int nitems, Persist2D a) {
    unsigned k = 0;
    for (int it = 0; it < a.nt; it++) {
        Step2D st;
        st.it = it;
        st.amp = a.amp[it];
        st.src_on = a.on[it];
        st.taper = a.taper;
        st.nf = 1;
        st.fast = 0;  // the single-shot forms have no double chains
        for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
            Tile2D t;
            if (locate(shots, item_shot, item, t)) vel_point<VARIANT, false>(*t.sh, t.ix, t.iz, st);
        }
        if (!grid_barrier(a.bar, ++k * gridDim.x, a.err)) return;
        for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
            Tile2D t;
            if (locate(shots, item_shot, item, t)) stress_point<VARIANT, PH_FWD, false>(*t.sh, t.ix, t.iz, st);
        }
        if (!grid_barrier(a.bar, ++k * gridDim.x, a.err)) return;
    }
}

int launch_fd2d_shot(int variant, const Shot2D *d_shots, const int *d_item_shot, int nitems, int by, Persist2D a,
                     cudaStream_t s) {
    const void *fn = variant == V_CPU ? (const void *)k_fd2d_shot<V_CPU>
                   : variant == V_GPU ? (const void *)k_fd2d_shot<V_GPU>
                                      : (const void *)k_fd2d_shot<V_MPI>;
    GEO_TRY(ensure_gauss());
    int dev = 0, sms = 0, occ = 0, coop = 0;
    GEO_CUDA(cudaGetDevice(&dev));
    GEO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GEO_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    GEO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, 32 * by, 0));
    if (!coop || occ < 1) return fail(GEO_ERR_CUDA, "cooperative launch unavailable");
    // every block resident at once (the barrier needs it; the cooperative
    // launch checks it), blocks walking the tiles when there are more
    const int grid = std::min(nitems, occ * sms);
    if ((long long)grid * 2 * a.nt >= 4000000000LL) return fail(GEO_ERR_ARG, "too many steps for one launch");
    dim3 block(32, by);
    void *args[] = {(void *)&d_shots, (void *)&d_item_shot, (void *)&nitems, (void *)&a};
    GEO_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), block, args, 0, s));
    return check_launch("fd2d_shot");
}

// ------------------------------------------------------ tile-resident shot
// A single shot (CPU or GPU form) whose fields stay in shared memory for the
// whole run: block b owns a TZ(z) x TX(x) tile of every field and of the
// model.  Per step it loads only halos from the previous step's exchange
// copy of P, Q, u, w (x halos of P and u, z halos of Q and w), recomputes
// the velocities on its tile and on the 4-cell halos the stress update
// reads (the same arithmetic as the neighbour's own update), updates its
// stresses, writes its P, Q, u, w to the other exchange copy and meets the
// other blocks at one grid barrier.  The per-point arithmetic is
// vel_point's and stress_point's (CPU/GPU forms, forward phase, receivers);
// the GPU form's point source (P,Q += amp at one cell before the velocity
// update) is added to every copy of that cell's P,Q the step reads.
struct TileShot2D {
    Shot2D sh;                         // fields: state at the launch's start and end
    float *xP[2], *xQ[2], *xu[2], *xw[2];  // exchange copies, by step parity
    const float *amp;
    const unsigned char *on;
    int lz_shift, TX, ntz, taper;      // TZ = 1 << lz_shift
    int it0, it1;                      // steps of this launch
    unsigned *bar;
    int *err;
};

// Shared floats of one tile: P with its x halo (7 each side), Q with its z
// halo (7), u with x halo (4 left, 3 right), w with z halo (4 above, 3
// below), the four split stresses and the three model arrays.
__host__ __device__ constexpr long tile2d_floats(int TZ, int TX) {
    return 11L * TX * TZ + 21L * (TX + TZ);
}

template <int VARIANT>
__global__ void __launch_bounds__(512) k_fd2d_tile(const TileShot2D a) {
    extern __shared__ float sm[];
    if (ld_acquire_u32(reinterpret_cast<const unsigned *>(a.err))) return;   // an earlier run gave up
    const Shot2D &sh = a.sh;
    const int TZ = 1 << a.lz_shift, TX = a.TX, nnx = sh.nnx, nnz = sh.nnz;
    const int z0 = (blockIdx.x % a.ntz) * TZ, x0 = (blockIdx.x / a.ntz) * TX;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    float *PH = sm, *QH = PH + (TX + 14) * TZ, *UH = QH + TX * (TZ + 14), *WH = UH + (TX + 7) * TZ;
    float *PX = WH + TX * (TZ + 7), *PZ = PX + TX * TZ, *QX = PZ + TX * TZ, *QZ = QX + TX * TZ;
    float *VP = QZ + TX * TZ, *E2 = VP + TX * TZ, *D2 = E2 + TX * TZ;
    // tile-local views: cx, lz relative to (x0, z0)
    auto ph = [&](int cx, int lz) -> float & { return PH[(cx + 7) * TZ + lz]; };          // cx in [-7, TX+7)
    auto qh = [&](int cx, int lz) -> float & { return QH[cx * (TZ + 14) + lz + 7]; };    // lz in [-7, TZ+7)
    auto uh = [&](int cx, int lz) -> float & { return UH[(cx + 4) * TZ + lz]; };          // cx in [-4, TX+3)
    auto wh = [&](int cx, int lz) -> float & { return WH[cx * (TZ + 7) + lz + 4]; };     // lz in [-4, TZ+3)
    auto upd = [&](int ix, int iz) { return ix >= 4 && ix < nnx - 4 && iz >= 4 && iz < nnz - 4; };

    // own state and model (SV taper applied to 1+2eps, sqrtf(1+2del))
    for (int cx = warp; cx < TX; cx += nw)
        for (int lz = lane; lz < TZ; lz += 32) {
            const int ix = x0 + cx, iz = z0 + lz, o = cx * TZ + lz;
            const bool in = ix < nnx && iz < nnz;
            const long id = (long)ix * nnz + iz;
            ph(cx, lz) = in ? sh.P[0][id] : 0.0f;
            qh(cx, lz) = in ? sh.Q[0][id] : 0.0f;
            uh(cx, lz) = in ? sh.u[0][id] : 0.0f;
            wh(cx, lz) = in ? sh.w[0][id] : 0.0f;
            PX[o] = in ? sh.px[0][id] : 0.0f;
            PZ[o] = in ? sh.pz[0][id] : 0.0f;
            QX[o] = in ? sh.qx[0][id] : 0.0f;
            QZ[o] = in ? sh.qz[0][id] : 0.0f;
            float e2 = in ? sh.e2[id] : 0.0f, d2 = in ? sh.d2[id] : 0.0f;
            if (a.taper) {
                const int bx = ix - sh.tx0, bz = iz - sh.tz0;
                if (bx >= 0 && bx < kTB && bz >= 0 && bz < kTB) {
                    e2 = sh.te2[bx * kTB + bz];
                    d2 = sh.td2[bx * kTB + bz];
                }
            }
            VP[o] = in ? sh.vp[id] : 0.0f;
            E2[o] = e2;
            D2[o] = d2;
        }
    // the own tile is read by other threads from here on (the source cell's
    // update below, the first step's taps)
    __syncthreads();
    unsigned k = 0;
    for (int it = a.it0; it < a.it1; it++) {
        const int b = it & 1;
        const bool on = a.on[it] != 0;
        const float amp = a.amp[it];
        const bool pt_src = VARIANT == V_GPU && on;
        // halos of the previous step (another block's values: through L2)
        auto halo = [&](const float *x, int ix, int iz) {
            if (ix < 0 || ix >= nnx || iz < 0 || iz >= nnz) return 0.0f;
            float v = __ldcg(x + (long)ix * nnz + iz);
            if (pt_src && ix == sh.ixs && iz == sh.izs) v = v + amp;
            return v;
        };
        for (int c = warp; c < 14; c += nw) {
            const int cx = c < 7 ? c - 7 : TX + c - 7;
            for (int lz = lane; lz < TZ; lz += 32) ph(cx, lz) = halo(a.xP[b], x0 + cx, z0 + lz);
        }
        for (int c = warp; c < 7; c += nw) {
            const int cx = c < 4 ? c - 4 : TX + c - 4;
            for (int lz = lane; lz < TZ; lz += 32) {
                const int ix = x0 + cx, iz = z0 + lz;
                uh(cx, lz) = ix >= 0 && ix < nnx && iz < nnz ? __ldcg(a.xu[b] + (long)ix * nnz + iz) : 0.0f;
            }
        }
        for (int t = threadIdx.x; t < TX * 14; t += blockDim.x) {
            const int cx = t / 14, r = t % 14, lz = r < 7 ? r - 7 : TZ + r - 7;
            qh(cx, lz) = halo(a.xQ[b], x0 + cx, z0 + lz);
        }
        for (int t = threadIdx.x; t < TX * 7; t += blockDim.x) {
            const int cx = t / 7, r = t % 7, lz = r < 4 ? r - 4 : TZ + r - 4;
            const int ix = x0 + cx, iz = z0 + lz;
            wh(cx, lz) = ix < nnx && iz >= 0 && iz < nnz ? __ldcg(a.xw[b] + (long)ix * nnz + iz) : 0.0f;
        }
        // the source cell inside the tile (its own copy)
        if (pt_src && threadIdx.x == 0) {
            const int cx = sh.ixs - x0, lz = sh.izs - z0;
            if (cx >= 0 && cx < TX && lz >= 0 && lz < TZ) {
                ph(cx, lz) = ph(cx, lz) + amp;
                qh(cx, lz) = qh(cx, lz) + amp;
            }
        }
        __syncthreads();
        // velocities on the tile and its halos (vel_point)
        for (int cx = warp - 4; cx < TX + 3; cx += nw)
            for (int lz = lane; lz < TZ; lz += 32) {
                const int ix = x0 + cx, iz = z0 + lz;
                if (!upd(ix, iz)) continue;
                float xx = 0.0f;
#pragma unroll
                for (int im = 0; im < 4; im++) xx += c_fd[im] * (ph(cx + im + 1, lz) - ph(cx - im, lz));
                uh(cx, lz) = sh.cx2[ix] * uh(cx, lz) - sh.cx1[ix] * sh.dtx * xx;
            }
        for (int cx = warp; cx < TX; cx += nw)
            for (int lz = lane - 4; lz < TZ + 3; lz += 32) {
                const int ix = x0 + cx, iz = z0 + lz;
                if (!upd(ix, iz)) continue;
                float zz = 0.0f;
#pragma unroll
                for (int im = 0; im < 4; im++) zz += c_fd[im] * (qh(cx, lz + im + 1) - qh(cx, lz - im));
                wh(cx, lz) = sh.cz2[iz] * wh(cx, lz) - sh.cz1[iz] * sh.dtz * zz;
            }
        __syncthreads();
        // stresses of the tile (stress_point, forward), receivers, exchange
        float *yP = a.xP[b ^ 1], *yQ = a.xQ[b ^ 1], *yu = a.xu[b ^ 1], *yw = a.xw[b ^ 1];
        for (int cx = warp; cx < TX; cx += nw)
            for (int lz = lane; lz < TZ; lz += 32) {
                const int ix = x0 + cx, iz = z0 + lz;
                if (!upd(ix, iz)) continue;
                float xx = 0.0f, zz = 0.0f;
#pragma unroll
                for (int im = 0; im < 4; im++) {
                    xx += c_fd[im] * (uh(cx + im, lz) - uh(cx - im - 1, lz));
                    zz += c_fd[im] * (wh(cx, lz + im) - wh(cx, lz - im - 1));
                }
                const int o = cx * TZ + lz;
                const float vp = VP[o], e2 = E2[o], d2 = D2[o];
                const float ax1 = sh.ax1[ix], ax2 = sh.ax2[ix], az1 = sh.az1[iz], az2 = sh.az2[iz];
                const float px = ax2 * PX[o] - ax1 * vp * vp * e2 * sh.dtx * xx;
                const float pz = az2 * PZ[o] - az1 * vp * vp * d2 * sh.dtz * zz;
                const float qx = ax2 * QX[o] - ax1 * vp * vp * d2 * sh.dtx * xx;
                const float qz = az2 * QZ[o] - az1 * vp * vp * sh.dtz * zz;
                PX[o] = px; PZ[o] = pz; QX[o] = qx; QZ[o] = qz;
                float P, Q;
                if (VARIANT == V_CPU) {
                    // 7x7 Gaussian source window, added after the split sum
                    float s = 0.0f;
                    const int rx = ix - sh.ixs, rz = iz - sh.izs;
                    if (on && rx >= -3 && rx <= 3 && rz >= -3 && rz <= 3)
                        s = (float)((double)amp * c_gauss[(rx + 3) * 7 + (rz + 3)]);
                    P = px + pz + s;
                    Q = qx + qz + s;
                } else {
                    P = px + pz;
                    Q = qx + qz;
                }
                ph(cx, lz) = P;
                qh(cx, lz) = Q;
                const long id = (long)ix * nnz + iz;
                yP[id] = P;
                yQ[id] = Q;
                yu[id] = uh(cx, lz);
                yw[id] = wh(cx, lz);
                const int gx = ix - sh.npd;
                if (iz == sh.rec_iz && gx >= 0 && gx < sh.nx)
                    sh.rec_p[(long)it * sh.nx + gx] = sh.rec_scale == 2.0f ? P + P : P * sh.rec_scale;
            }
        if (it + 1 < a.it1 && !grid_barrier(a.bar, ++k * gridDim.x, a.err)) return;
    }
    __syncthreads();
    // state back to the shot's fields
    for (int cx = warp; cx < TX; cx += nw)
        for (int lz = lane; lz < TZ; lz += 32) {
            const int ix = x0 + cx, iz = z0 + lz, o = cx * TZ + lz;
            if (ix >= nnx || iz >= nnz) continue;
            const long id = (long)ix * nnz + iz;
            sh.P[0][id] = ph(cx, lz);
            sh.Q[0][id] = qh(cx, lz);
            sh.u[0][id] = uh(cx, lz);
            sh.w[0][id] = wh(cx, lz);
            sh.px[0][id] = PX[o];
            sh.pz[0][id] = PZ[o];
            sh.qx[0][id] = QX[o];
            sh.qz[0][id] = QZ[o];
        }
}

constexpr size_t kTileSmemMax = 220 * 1024;

// Tile shape of the tile-resident shot: every tile's block resident at once
// (cooperative launch).  The half-steps are bound by shared-memory and L2
// latency chains, so more resident warps per SM beat less halo work: at
// 401^2 + 50 (2000 steps) 64x16 tiles (two blocks per SM) take 17.7 ms,
// 128x16 and 64x32 (one per SM) 18.0 and 18.2 ms, 32x32 18.7 ms, 32x64
// 20.5 ms.  So: TZ 64 first (then 128, 32, 256), the narrowest TX that
// fits.  Returns false when the grid does not fit on the device this way.
static bool tile2d_shape(const void *fn, int nnx, int nnz, int sms, int &lz_shift, int &TX, size_t &smem) {
    static const int kLz[] = {6, 7, 5, 8};
    static const int kTX[] = {8, 12, 16, 24, 32, 48, 64};
    for (int ls : kLz) {
        const int TZ = 1 << ls;
        for (int tx : kTX) {
            const size_t bytes = (size_t)tile2d_floats(TZ, tx) * 4;
            if (bytes > kTileSmemMax) continue;
            int per_sm = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 512, bytes) != cudaSuccess) return false;
            const long tiles = (long)((nnz + TZ - 1) / TZ) * ((nnx + tx - 1) / tx);
            if (per_sm < 1 || tiles > (long)per_sm * sms) continue;
            lz_shift = ls;
            TX = tx;
            smem = bytes;
            return true;
        }
    }
    return false;
}

int launch_fd2d_tile(int variant, const Shot2D &sh, float *xch, const float *amp, const unsigned char *on,
                     int taper, int it0, int it1, unsigned *bar, int *err, bool *fits, cudaStream_t s) {
    *fits = false;
    if (variant != V_CPU && variant != V_GPU) return GEO_OK;
    int dev = 0, sms = 0, coop = 0;
    GEO_CUDA(cudaGetDevice(&dev));
    GEO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GEO_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    const void *fn = variant == V_CPU ? (const void *)k_fd2d_tile<V_CPU> : (const void *)k_fd2d_tile<V_GPU>;
    GEO_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTileSmemMax));
    int ls = 0, TX = 0;
    size_t smem = 0;
    if (!coop || !tile2d_shape(fn, sh.nnx, sh.nnz, sms, ls, TX, smem)) return GEO_OK;
    // GEO_FD2D_TILE=TZxTX fixes the tile instead (TZ a power of two 32..256)
    if (const char *e = getenv("GEO_FD2D_TILE")) {
        int tz = 0, tx = 0;
        if (sscanf(e, "%dx%d", &tz, &tx) == 2 && tx >= 4 && tx <= 128)
            for (int l = 5; l <= 8; l++)
                if (tz == (1 << l)) {
                    ls = l;
                    TX = tx;
                    smem = (size_t)tile2d_floats(tz, tx) * 4;
                }
        if (smem > kTileSmemMax) return fail(GEO_ERR_ARG, "GEO_FD2D_TILE %s: tile too large", e);
    }
    int occ = 0;
    GEO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, 512, smem));
    const int TZ = 1 << ls, ntz = (sh.nnz + TZ - 1) / TZ, ntx = (sh.nnx + TX - 1) / TX;
    if (occ < 1 || (long)ntz * ntx > (long)occ * sms) return GEO_OK;
    if ((long long)ntz * ntx * (it1 - it0) >= 4000000000LL) return GEO_OK;
    GEO_TRY(ensure_gauss());
    *fits = true;
    const size_t n = (size_t)sh.nnx * sh.nnz;
    TileShot2D a{};
    a.sh = sh;
    for (int p = 0; p < 2; p++) {
        a.xP[p] = xch + (size_t)(4 * p) * n;
        a.xQ[p] = xch + (size_t)(4 * p + 1) * n;
        a.xu[p] = xch + (size_t)(4 * p + 2) * n;
        a.xw[p] = xch + (size_t)(4 * p + 3) * n;
    }
    a.amp = amp;
    a.on = on;
    a.lz_shift = ls;
    a.TX = TX;
    a.ntz = ntz;
    a.taper = taper;
    a.it0 = it0;
    a.it1 = it1;
    a.bar = bar;
    a.err = err;
    GEO_CUDA(cudaMemsetAsync(bar, 0, 4, s));
    void *args[] = {(void *)&a};
    GEO_CUDA(cudaLaunchCooperativeKernel(fn, dim3(ntz * ntx), dim3(512), args, smem, s));
    return check_launch("fd2d_tile");
}

// Boundary-driven reconstruction and receiver injection before step it of
// the backward pass (Toa_rtm_vti_adcig_cdp.c:914-927 and 953-957): the saved
// interior-edge lines go into the source-side P,Q (corners end with the
// left/right values, as the reference's loop order leaves them) and the
// muted surface records into the receiver-side P,Q at the surface row.
__global__ void k_inject2d(const Shot2D *__restrict__ shots, int maxline, int it) {
    const Shot2D &sh = shots[blockIdx.y];
    const int nx = sh.nx, nz = sh.nz, npd = sh.npd, nnz = sh.nnz;
    const long L = 2L * nx + 2L * nz;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < L; k += gridDim.x * blockDim.x) {
        int ix, iz;
        if (k < nx) { ix = npd + k; iz = npd; if (k == 0 || k == nx - 1) goto rec; }
        else if (k < 2 * nx) { ix = npd + k - nx; iz = npd + nz - 1; if (k - nx == 0 || k - nx == nx - 1) goto rec; }
        else if (k < 2 * nx + nz) { ix = npd; iz = npd + k - 2 * nx; }
        else { ix = npd + nx - 1; iz = npd + k - 2 * nx - nz; }
        {
            const long id = (long)ix * nnz + iz;
            sh.P[0][id] = sh.edge_p[(long)it * L + k];
            sh.Q[0][id] = sh.edge_q[(long)it * L + k];
        }
    rec:
        if (k < nx) {
            const long id = (long)(npd + k) * nnz + npd;
            sh.P[1][id] = sh.rec_p[(long)it * nx + k];
            sh.Q[1][id] = sh.rec_q[(long)it * nx + k];
        }
    }
    (void)maxline;
}

template <int V>
static void vel_dispatch(const Shot2D *d_shots, const int *d_item_shot, int nitems, dim3 grid, dim3 block,
                         Step2D st, cudaStream_t s) {
    k_vel2d<V><<<grid, block, 0, s>>>(d_shots, d_item_shot, nitems, st);
}

// Wavefield watchdog over a batch: block row y scans shot y's P of sides
// 0..nf-1 and sets *flag to tag (first writer wins) on a NaN or +-Inf.
__global__ void k_watch_shots(const Shot2D *__restrict__ S, int nf, int *flag, int tag) {
    const Shot2D &sh = S[blockIdx.y];
    const size_t n = (size_t)sh.nnx * sh.nnz;
    bool bad = false;
    for (int f = 0; f < nf; f++) {
        const float *P = sh.P[f];
        for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
            bad |= !(fabsf(P[k]) <= FLT_MAX);
    }
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicCAS(flag, 0, tag);
}

int launch_watch_shots(const Shot2D *d_shots, int ns, int nf, int *flag, int tag, cudaStream_t s) {
    if (!flag || ns < 1) return GEO_OK;
    k_watch_shots<<<dim3(64, ns), 256, 0, s>>>(d_shots, nf, flag, tag);
    return check_launch("watch_shots");
}

int launch_vel2d(int variant, const Shot2D *d_shots, const int *d_item_shot, int nitems, int by, int grid,
                 Step2D st, cudaStream_t s) {
    dim3 block(32, by), g(grid);
    switch (variant) {
        case V_CPU: vel_dispatch<V_CPU>(d_shots, d_item_shot, nitems, g, block, st, s); break;
        case V_GPU: vel_dispatch<V_GPU>(d_shots, d_item_shot, nitems, g, block, st, s); break;
        default: vel_dispatch<V_MPI>(d_shots, d_item_shot, nitems, g, block, st, s); break;
    }
    return check_launch("vel2d");
}

int launch_stress2d(int variant, int phase, const Shot2D *d_shots, const int *d_item_shot, int nitems, int by,
                    int grid, Step2D st, cudaStream_t s) {
    GEO_TRY(ensure_gauss());
    dim3 block(32, by), g(grid);
#define GEO_STRESS(V, PH) k_stress2d<V, PH><<<g, block, 0, s>>>(d_shots, d_item_shot, nitems, st)
#define GEO_STRESS_MPI(PH) \
    (st.fast ? k_stress2d<V_MPI, PH, true><<<g, block, 0, s>>>(d_shots, d_item_shot, nitems, st) \
             : k_stress2d<V_MPI, PH, false><<<g, block, 0, s>>>(d_shots, d_item_shot, nitems, st))
    if (phase == PH_FWD) {
        switch (variant) {
            case V_CPU: GEO_STRESS(V_CPU, PH_FWD); break;
            case V_GPU: GEO_STRESS(V_GPU, PH_FWD); break;
            default: GEO_STRESS_MPI(PH_FWD); break;
        }
    } else {
        switch (variant) {
            case V_CPU: GEO_STRESS(V_CPU, PH_BWD); break;
            case V_GPU: GEO_STRESS(V_GPU, PH_BWD); break;
            default: GEO_STRESS_MPI(PH_BWD); break;
        }
    }
#undef GEO_STRESS_MPI
#undef GEO_STRESS
    return check_launch("stress2d");
}

int launch_inject2d(const Shot2D *d_shots, int nshots, int maxline, int it, cudaStream_t s) {
    dim3 g((maxline + 255) / 256, nshots);
    k_inject2d<<<g, 256, 0, s>>>(d_shots, maxline, it);
    return check_launch("inject2d");
}

// One launch that runs velocity tiles of some shots and stress tiles of
// others (the MPI form of the batched RTM).  Each item is (shot | kind << 30,
// tile): kind 0 a velocity tile at step st_v, kind 1 a stress tile at st_s.
// The caller keeps the two kinds on disjoint shots, so the read-only path
// stays valid for both.  The exact form's stress tiles are bound by the FP64
// pipe and the velocity tiles by memory, so a launch that holds both keeps
// both busy on every SM.
template <int PHASE, bool FAST>
__global__ void __launch_bounds__(256) k_mix2d(const Shot2D *__restrict__ shots, const int2 *__restrict__ items,
                                               int nitems, Step2D st_v, Step2D st_s) {
    for (int item = blockIdx.x; item < nitems; item += gridDim.x) {
        const int2 e = items[item];
        const int kind = e.x >> 30;
        const Shot2D &sh = shots[e.x & ((1 << 30) - 1)];
        const int tz = e.y % sh.ntz, tx = e.y / sh.ntz;
        const int iz = tz * 32 + threadIdx.x, ix = tx * blockDim.y + threadIdx.y;
        if (ix < 4 || ix >= sh.nnx - 4 || iz < 4 || iz >= sh.nnz - 4) continue;
        if (kind == 0) vel_point<V_MPI, true>(sh, ix, iz, st_v);
        else stress_point<V_MPI, PHASE, true, FAST>(sh, ix, iz, st_s);
    }
}

int launch_mix2d(int phase, int fast, const Shot2D *d_shots, const int2 *d_items, int nitems, int by, int grid,
                 Step2D st_v, Step2D st_s, cudaStream_t s) {
    if (nitems < 1) return GEO_OK;
    GEO_TRY(ensure_gauss());
    dim3 block(32, by), g(grid < nitems ? grid : nitems);
    if (phase == PH_FWD) {
        if (fast) k_mix2d<PH_FWD, true><<<g, block, 0, s>>>(d_shots, d_items, nitems, st_v, st_s);
        else k_mix2d<PH_FWD, false><<<g, block, 0, s>>>(d_shots, d_items, nitems, st_v, st_s);
    } else {
        if (fast) k_mix2d<PH_BWD, true><<<g, block, 0, s>>>(d_shots, d_items, nitems, st_v, st_s);
        else k_mix2d<PH_BWD, false><<<g, block, 0, s>>>(d_shots, d_items, nitems, st_v, st_s);
    }
    return check_launch("mix2d");
}

// The MPI program's bin of one cosine a1 (before its 90 -> 89 clamp).
static int ref_adcig_bin(float a1) {
    const float a2 = (float)(0.5 * std::acos(a1) * 180 / kPiMpi);
    return (int)(a2 / 1.0);
}

static uint32_t order_key(float f) {
    uint32_t b;
    memcpy(&b, &f, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

static float key_float(uint32_t k) {
    const uint32_t b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

int load_adcig_tables(cudaStream_t s) {
    static float thr[kAdcigAngles];
    static double w[kAdcigAngles];
    static bool built = false;
    if (!built) {
        const uint32_t lo = order_key(-1.0f), hi = order_key(1.0f);
        for (int k = 1; k <= kAdcigAngles; k++) {
            if (ref_adcig_bin(-1.0f) < k) {
                thr[k - 1] = -2.0f;   // no cosine reaches this bin
                continue;
            }
            uint32_t a = lo, b = hi;  // ref_adcig_bin(key_float(a)) >= k
            while (a < b) {
                const uint32_t m = a + (b - a + 1) / 2;
                if (ref_adcig_bin(key_float(m)) >= k) a = m;
                else b = m - 1;
            }
            thr[k - 1] = key_float(a);
        }
        for (int ia = 0; ia < kAdcigAngles; ia++) w[ia] = std::pow(std::cos(ia * kPiMpi / 180.0), 3);
        built = true;
    }
    GEO_CUDA(cudaMemcpyToSymbolAsync(c_adthr, thr, sizeof thr, 0, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemcpyToSymbolAsync(c_adw, w, sizeof w, 0, cudaMemcpyHostToDevice, s));
    return GEO_OK;
}

}  // namespace geo
