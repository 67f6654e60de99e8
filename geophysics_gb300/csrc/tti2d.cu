// 2D TTI (tilted VTI) staggered-grid FD with the semantics of the GPU TTI
// program (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu):
//   update_vel (:81-112)     u <- cx2 cz2 u - cx1 cz1 (cos t dtx dP/dx - sin t dtz dP/dz)
//                            w <- cx2 cz2 w - cx1 cz1 (sin t dtx dQ/dx + cos t dtz dQ/dz)
//   update_stress (:114-183) px,pz,qx,qz with the same rotated derivatives of
//                            u and w, P = px + pz, Q = qx + qz
// with the sponge applied as products of the x and z profiles, the point
// source added to P and Q before the velocity update (add_source :47-79),
// the record taken from P at the surface row after each step
// (shot_record :273-283) and padded-P snapshots every snap_every steps from
// snap_every on (:451-456).  The program swaps its old/new pointers without
// keeping two buffers (u0 = u1 after the first step), so every field is
// updated in place; this file does that directly.
// cos and sin of the tilt are formed once on the device (cosf/sinf of the
// angle in radians, theta * pi/180 as the program converts it).
// The program launches four kernels per step; here the steps between two
// host events (a snapshot, a watchdog scan) run as one cooperative launch
// with grid barriers between the half-steps, the source folded into the
// velocity taps that read its cell and the record written by the stress
// phase.
#include "geo_internal.h"
#include <algorithm>
#include "tti2d.cuh"
#include "gridsync.cuh"
#include <cmath>
#include <vector>

namespace geo {

// cos and sin of the tilt (radians, in place: th -> cos, sin into sn).  The
// 2D TTI programs evaluate cos(theta[id]) and sin(theta[id]) of their float
// tilt inside their kernels (Toa_gpu_2dtti_fd_1orderfunction.cu:106-107,
// :168-175; Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu:155-156, :216-222),
// i.e. the device's single-precision cosf and sinf; the tables are formed
// here with the same device functions, so they hold the programs' values.
__global__ void k_tilt_trig(float *th_cos, float *sn, size_t n) {
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const float t = th_cos[k];
        th_cos[k] = cosf(t);
        sn[k] = sinf(t);
    }
}

int launch_tilt_trig(float *th_cos, float *sn, size_t n, cudaStream_t s) {
    const int grid = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
    k_tilt_trig<<<grid, 256, 0, s>>>(th_cos, sn, n);
    return check_launch("tilt_trig");
}


__constant__ float c_tti[4] = {1.196289f, -0.0797526f, 0.009570313f, -0.0006975447f};

// A whole 2D TTI shot (or a run of its steps) in one cooperative launch:
// per step the velocity half-step over every updated point (the step's
// point source folded into the taps that read the source cell), a grid
// barrier, the stress half-step with the surface record of P, a grid
// barrier.  The per-point arithmetic is tti_vel_at / tti_stress_at's; field
// values other blocks wrote are read through L2.
struct TtiShot {
    TtiGrid g;
    TtiField f;
    const float *e2, *d2;
    const float *amp;            // pfac*w(t) of every step
    const unsigned char *on;     // source active at every step
    long src;                    // source cell
    int ixs, izs;
    float *rec;                  // nx*nt, trace-major
    int nx, npd, rec_iz, nt;
    int it0, it1;                // steps of this launch
    unsigned *bar;               // grid-barrier arrival counter, zeroed before the launch
    int *err;                    // set when a barrier wait gave up
};

__global__ void __launch_bounds__(256) k_tti_shot(const TtiShot a) {
    if (ld_acquire_u32(reinterpret_cast<const unsigned *>(a.err))) return;   // an earlier run gave up
    const TtiGrid &g = a.g;
    const long n = (long)g.nnx * g.nnz, stride = (long)gridDim.x * blockDim.x;
    const long first = blockIdx.x * (long)blockDim.x + threadIdx.x;
    unsigned k = 0;
    for (int it = a.it0; it < a.it1; it++) {
        const bool on = a.on[it] != 0;
        const float amp = a.amp[it];
        for (long id = first; id < n; id += stride) {
            const int ix = (int)(id / g.nnz), iz = (int)(id % g.nnz);
            if (ix < 4 || ix >= g.nnx - 4 || iz < 4 || iz >= g.nnz - 4) continue;
            const bool near = on && ((iz == a.izs && abs(ix - a.ixs) <= 4) || (ix == a.ixs && abs(iz - a.izs) <= 4));
            if (near) tti_vel_at<true, true>(g, a.f, c_tti, id, ix, iz, a.src, amp);
            else tti_vel_at<true, false>(g, a.f, c_tti, id, ix, iz);
        }
        if (!grid_barrier(a.bar, ++k * gridDim.x, a.err)) return;
        for (long id = first; id < n; id += stride) {
            const int ix = (int)(id / g.nnz), iz = (int)(id % g.nnz);
            if (ix < 4 || ix >= g.nnx - 4 || iz < 4 || iz >= g.nnz - 4) continue;
            const float P = tti_stress_at<true>(g, a.f, a.e2, a.d2, c_tti, id, ix, iz).x;
            // shot_record (:273-283): P at the receiver row, after the step
            if (iz == a.rec_iz && ix >= a.npd && ix < a.npd + a.nx) a.rec[it + (long)a.nt * (ix - a.npd)] = P;
        }
        if (it + 1 < a.it1 && !grid_barrier(a.bar, ++k * gridDim.x, a.err)) return;
    }
}

}  // namespace geo

using namespace geo;

extern "C" int geo_tti2d_shot(const geo_fd2d_desc *desc, const float *v, const float *e, const float *d,
                              const float *theta, float *shot, float *snap, int snap_every, int mem, void *stream) {
    if (!desc || !v || !e || !d || !theta || !shot) return fail(GEO_ERR_ARG, "null argument");
    const geo_fd2d_desc &D = *desc;
    if (D.nx < 2 || D.nz < 2 || D.npd < 5 || D.nt < 1) return fail(GEO_ERR_ARG, "grid too small (npd must be >= 5)");
    if (!(D.dt > 0) || !(D.dx > 0) || !(D.dz > 0) || !(D.favg > 0)) return fail(GEO_ERR_ARG, "bad spacing");
    if (mem != GEO_MEM_HOST && mem != GEO_MEM_DEVICE) return fail(GEO_ERR_ARG, "bad mem kind");
    if (snap && snap_every < 1) return fail(GEO_ERR_ARG, "snap_every must be >= 1");
    const int nx = D.nx, nz = D.nz, npd = D.npd, nt = D.nt;
    const int nnx = nx + 2 * npd, nnz = nz + 2 * npd;
    const size_t n0 = (size_t)nx * nz, n = (size_t)nnx * nnz;
    if (D.rec_iz < 0 || D.rec_iz >= nnz) return fail(GEO_ERR_ARG, "receiver row outside the grid");
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<float> hv(n0), he(n0), hd(n0), ht(n0);
    const float *src[4] = {v, e, d, theta};
    float *dst[4] = {hv.data(), he.data(), hd.data(), ht.data()};
    for (int k = 0; k < 4; k++) {
        if (mem == GEO_MEM_DEVICE) GEO_CUDA(cudaMemcpyAsync(dst[k], src[k], n0 * 4, cudaMemcpyDeviceToHost, s));
        else std::copy(src[k], src[k] + n0, dst[k]);
    }
    GEO_CUDA(cudaStreamSynchronize(s));
    GEO_TRY(check_model(hv.data(), he.data(), hd.data(), n0));
    for (size_t k = 0; k < n0; k++)
        if (!std::isfinite(ht[k])) return fail(GEO_ERR_MODEL, "theta[%zu] not finite", k);
    std::vector<float> pv(n), pe(n), pd(n), pt(n);
    pad_model_2d(nx, nz, npd, hv.data(), pv.data());
    pad_model_2d(nx, nz, npd, he.data(), pe.data());
    pad_model_2d(nx, nz, npd, hd.data(), pd.data());
    pad_model_2d(nx, nz, npd, ht.data(), pt.data());
    // source cell (add_source :71-72), shot is 1-based
    const float fsx = D.fs + (D.is - 1) * D.ds;
    const int ixs = (int)(fsx + 0.5f) + npd - 1, izs = (int)(D.zs + 0.5f) + npd - 1;
    if (ixs < 4 || ixs >= nnx - 4 || izs < 4 || izs >= nnz - 4) return fail(GEO_ERR_ARG, "source outside the grid");
    if (D.sv) {
        // centre (fs+(is-1)ds+npml, zs+npml) (:131-132): one cell right/down of the source cell
        Taper2D tp;
        sv_taper_2d(V_GPU, nnx, nnz, npd, ixs + 1, izs + 1, pe.data(), pd.data(), tp);
        for (int bx = 0; bx < tp.n; bx++)
            for (int bz = 0; bz < tp.n; bz++) {
                const int ix = tp.x0 + bx, iz = tp.z0 + bz;
                if (ix < 0 || ix >= nnx || iz < 0 || iz >= nnz) continue;
                pe[(size_t)ix * nnz + iz] = tp.e[bx * tp.n + bz];
                pd[(size_t)ix * nnz + iz] = tp.d[bx * tp.n + bz];
            }
    }
    // model arrays: vp, 1+2eps, sqrtf(1+2del), and the tilt in radians as
    // read_file converts it (:235), whose cos and sin are then formed on the
    // device (launch_tilt_trig) as the program's kernels form them
    std::vector<float> model(5 * n);
    for (size_t k = 0; k < n; k++) {
        model[k] = pv[k];
        model[n + k] = 1 + 2 * pe[k];
        model[2 * n + k] = sqrtf(1 + 2 * pd[k]);
        model[3 * n + k] = (float)((double)pt[k] * (kPiGui / 180.0));
    }
    {
        const auto mm = std::minmax_element(pv.begin(), pv.end());
        GEO_TRY(check_stability(V_GPU, 2, *mm.first, *mm.second, D.dt, D.dx, D.dx, D.dz, D.favg));
    }
    // sponge (get_d0 :186-189 from the padded centre velocity; initial_coffe :227-271)
    const float d0 = sponge_d0(V_GPU, 2, 0.0f, pv[n / 2], npd, D.dx, D.dx, D.dz);
    std::vector<float> prof(4 * (size_t)(nnx + nnz));
    float *q = prof.data();
    sponge_profiles(V_GPU, nx, npd, D.dt, d0, q, q + nnx, q + 2 * nnx, q + 3 * nnx);
    q += 4 * nnx;
    sponge_profiles(V_GPU, nz, npd, D.dt, d0, q, q + nnz, q + 2 * nnz, q + 3 * nnz);
    std::vector<float> amp;
    std::vector<uint8_t> on;
    source_amplitudes(V_GPU, nt, D.dt, D.favg, D.pfac, D.wtype, amp, on);

    DevBuf dm, dprof, df, drec;
    GEO_TRY(dm.alloc(5 * n * 4));
    GEO_TRY(dprof.alloc(prof.size() * 4));
    GEO_TRY(df.alloc(8 * n * 4));
    GEO_TRY(drec.alloc((size_t)nx * nt * 4));
    GEO_CUDA(cudaMemcpyAsync(dm.p, model.data(), 5 * n * 4, cudaMemcpyHostToDevice, s));
    GEO_TRY(launch_tilt_trig(dm.as<float>() + 3 * n, dm.as<float>() + 4 * n, n, s));
    GEO_CUDA(cudaMemcpyAsync(dprof.p, prof.data(), prof.size() * 4, cudaMemcpyHostToDevice, s));
    GEO_TRY(df.zero(s));
    GEO_TRY(drec.zero(s));
    TtiGrid g{};
    g.nnx = nnx;
    g.nnz = nnz;
    g.dtx = D.dt / D.dx;
    g.dtz = D.dt / D.dz;
    const float *pp = dprof.as<float>();
    g.cx1 = pp; g.cx2 = pp + nnx; g.ax1 = pp + 2 * nnx; g.ax2 = pp + 3 * nnx;
    pp += 4 * nnx;
    g.cz1 = pp; g.cz2 = pp + nnz; g.az1 = pp + 2 * nnz; g.az2 = pp + 3 * nnz;
    const float *m = dm.as<float>();
    g.vp = m; g.ct = m + 3 * n; g.st = m + 4 * n;
    const float *e2 = m + n, *d2 = m + 2 * n;
    float *fb = df.as<float>();
    TtiField f;
    f.u = fb; f.w = fb + n; f.px = fb + 2 * n; f.pz = fb + 3 * n; f.qx = fb + 4 * n; f.qz = fb + 5 * n;
    f.P = fb + 6 * n; f.Q = fb + 7 * n;
    const cudaMemcpyKind kout = mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    DevBuf d_amp, d_on, d_sync;
    GEO_TRY(d_amp.alloc((size_t)nt * 4));
    GEO_TRY(d_on.alloc((size_t)nt));
    GEO_TRY(d_sync.alloc(8));
    GEO_TRY(d_sync.zero(s));
    GEO_CUDA(cudaMemcpyAsync(d_amp.p, amp.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemcpyAsync(d_on.p, on.data(), (size_t)nt, cudaMemcpyHostToDevice, s));
    TtiShot a{};
    a.g = g;
    a.f = f;
    a.e2 = e2;
    a.d2 = d2;
    a.amp = d_amp.as<float>();
    a.on = d_on.as<unsigned char>();
    a.src = (long)ixs * nnz + izs;
    a.ixs = ixs;
    a.izs = izs;
    a.rec = drec.as<float>();
    a.nx = nx;
    a.npd = npd;
    a.rec_iz = D.rec_iz;
    a.nt = nt;
    a.bar = d_sync.as<unsigned>();
    a.err = d_sync.as<int>() + 1;
    // every block resident at once (the grid barrier needs it; the
    // cooperative launch checks it), threads striding over the points
    int dev = 0, sms = 0, occ = 0, coop = 0;
    GEO_CUDA(cudaGetDevice(&dev));
    GEO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GEO_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    GEO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_tti_shot, 256, 0));
    if (!coop || occ < 1) return fail(GEO_ERR_CUDA, "cooperative launch unavailable");
    const int grid = (int)std::min<size_t>((n + 255) / 256, (size_t)occ * sms);
    Watchdog wd;
    GEO_TRY(wd.open());
    // runs of steps between the host's work: a snapshot after step it
    // (it % snap_every == 0, it > 0) and the watchdog's scan end a run
    for (int it0 = 0; it0 < nt;) {
        int it1 = it0;
        while (true) {
            const int it = it1++;
            const bool snap_due = snap && it % snap_every == 0 && it != 0;
            const bool watch_due = wd.every > 0 && (it + 1) % wd.every == 0;
            if (snap_due || watch_due || it1 == nt) break;
        }
        if ((long long)grid * 2 * (it1 - it0) >= 4000000000LL) it1 = it0 + (int)(1900000000LL / grid);
        a.it0 = it0;
        a.it1 = it1;
        GEO_CUDA(cudaMemsetAsync(a.bar, 0, 4, s));
        void *args[] = {(void *)&a};
        GEO_CUDA(cudaLaunchCooperativeKernel((const void *)k_tti_shot, dim3(grid), dim3(256), args, 0, s));
        GEO_TRY(check_launch("tti_shot"));
        const int it = it1 - 1;
        if (snap && it % snap_every == 0 && it != 0)
            GEO_CUDA(cudaMemcpyAsync(snap + (size_t)(it / snap_every - 1) * n, f.P, n * 4, kout, s));
        const int w = wd.check(f.P, n, it, it == nt - 1, s);
        if (w == GEO_ERR_NAN) break;
        GEO_TRY(w);
        it0 = it1;
    }
    int err = 0;
    GEO_CUDA(cudaMemcpyAsync(&err, a.err, 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    if (err) return fail(GEO_ERR_CUDA, "2D TTI shot: a grid barrier wait timed out");
    GEO_TRY(wd.verdict(s, "2D TTI shot"));
    GEO_CUDA(cudaMemcpyAsync(shot, drec.p, (size_t)nx * nt * 4, kout, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}
