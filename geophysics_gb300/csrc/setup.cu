// Host-side set-up shared by every path: padding, sponge profiles, source
// amplitudes, SV taper, mute windows, error plumbing.  Formulas follow the
// reference programs named at each function; the double-precision
// intermediates and the float accumulation of time are kept as they are so
// the device arithmetic downstream can reproduce the reference bit for bit.
#include "geo_internal.h"
#include <cmath>
#include <cstdarg>
#include <cstdlib>
#include <cstring>
#include <atomic>

namespace geo {

thread_local char g_last_error[256] = "";
static std::atomic<long long> g_launches{0};

int fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof g_last_error, fmt, ap);
    va_end(ap);
    return code;
}

void count_launch(long long n) { g_launches += n; }
long long launches_so_far() { return g_launches.load(); }

int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(GEO_ERR_CUDA, "launch %s: %s", what, cudaGetErrorString(e));
    count_launch();
    return GEO_OK;
}

int DevBuf::alloc(size_t n) {
    release();
    if (n == 0) n = 4;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
        p = nullptr;
        return fail(GEO_ERR_NOMEM, "cudaMalloc(%zu): %s", n, cudaGetErrorString(e));
    }
    bytes = n;
    return GEO_OK;
}

int DevBuf::zero(cudaStream_t s) {
    if (!p) return GEO_OK;
    GEO_CUDA(cudaMemsetAsync(p, 0, bytes, s));
    return GEO_OK;
}

void DevBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

// ---------------------------------------------------------------- padding
// pad_vv: left/right columns first, then top/bottom rows over the full
// width, so corners take the corner value (CPU_vti2dfd_kernels.c:221-246).
void pad_model_2d(int nx, int nz, int npd, const float *in, float *out) {
    const int nnx = nx + 2 * npd, nnz = nz + 2 * npd;
    for (int ix = 0; ix < nnx; ix++) {
        int sx = ix < npd ? 0 : (ix >= npd + nx ? nx - 1 : ix - npd);
        for (int iz = 0; iz < nnz; iz++) {
            int sz = iz < npd ? 0 : (iz >= npd + nz ? nz - 1 : iz - npd);
            out[(size_t)ix * nnz + iz] = in[(size_t)sx * nz + sz];
        }
    }
}

// ---------------------------------------------------------------- sponge
// d0 (CPU_vti2dfd_kernels.c:192; Toa_rtm_vti_adcig_cdp.c:1346;
// GPU_vti2dfd_kernels.cu:105; GPU_vti3dfd_kernels.cu:205).
float sponge_d0(Variant v, int dims, float vpmax, float vcenter, int npd, float dx, float dy, float dz) {
    const double l = std::log(100000.0);
    if (v == V_CPU || v == V_MPI) return (float)(3.0 * vpmax * l / (2.0 * npd * dx));
    // 2D TTI GPU RTM program, get_d0 (Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu:230-233)
    if (v == V_TTIRTM) return (float)(3.0 * vcenter * l / (2.0 * npd * ((dx + dz) / 2.0)));
    if (dims == 2) return (float)(10.0 * vcenter * l / (2.0 * npd * ((dx + dz) / 2.0)));
    return (float)(10.0 * vcenter * l / (2.0 * npd * ((dx + dy + dz) / 3.0)));
}

// Damping factors of the split-PML sponge.  With q the normalised distance
// into the sponge, f = dt*d0*q^2/2: coff1 = 1/(1+f), coff2 = coff1*(1-f).
// Half-cell distance for velocities, integer-cell for stresses; the CPU
// program builds acoff2 from coff1 (CPU_vti2dfd_kernels.c:307-319), the MPI
// program from acoff1 (Toa_rtm_vti_adcig_cdp.c:1497-1512), and the GPU
// programs measure the far side from the interior edge itself
// (GPU_vti2dfd_kernels.cu:132-136).  The 2D TTI GPU RTM program uses the
// integer-cell distance for both pairs (initial_coffe,
// Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu:289-320).
void sponge_profiles(Variant v, int n, int npd, float dt, float d0, float *coff1, float *coff2,
                     float *acoff1, float *acoff2) {
    const int nn = n + 2 * npd;
    for (int i = 0; i < nn; i++) coff1[i] = coff2[i] = acoff1[i] = acoff2[i] = 1.0f;
    const float dtd0 = dt * d0;  // float product, as the reference forms it
    auto half = [&](double q) { return (dtd0 * std::pow(q, 2.0)) / 2.0; };
    for (int i = 0; i < nn; i++) {
        double qh, qi;
        if (i < npd) {
            qh = (npd - 0.5 - i) / npd;
            qi = ((npd - i) * 1.0) / npd;
            if (v == V_TTIRTM) qh = (npd - i) * 1.0 / npd;
        } else if (i >= npd + n) {
            qh = (0.5 + i - n - npd) / npd;
            qi = (v == V_GPU || v == V_TTIRTM) ? ((i - n - npd) * 1.0) / npd : ((1 + i - n - npd) * 1.0) / npd;
            if (v == V_TTIRTM) qh = (i - n - npd) * 1.0 / npd;
        } else {
            continue;
        }
        coff1[i] = (float)(1.0 / (1.0 + half(qh)));
        coff2[i] = (float)(coff1[i] * (1.0 - half(qh)));
        acoff1[i] = (float)(1.0 / (1.0 + half(qi)));
        const float lead = (v == V_CPU) ? coff1[i] : acoff1[i];
        acoff2[i] = (float)(lead * (1.0 - half(qi)));
    }
}

// ---------------------------------------------------------------- source
static float wavelet(float ts, float favg, int wtype, double pi) {
    if (wtype == 1) {
        float x = favg * ts, xx = x * x;
        return (float)((1 - 2 * pi * pi * (xx)) * std::exp(-(pi * pi * xx)));
    } else if (wtype == 2) {
        double y = (-4) * favg * favg * pi * pi / std::log(0.1);
        return (float)((-2) * pi * pi * ts * std::exp(-y * ts * ts));
    } else if (wtype == 3) {
        double y = (-1) * favg * favg * pi * pi / std::log(0.1);
        return (float)std::exp(-y * ts * ts);
    }
    return 0.0f;
}

// Ricker / Gaussian-derivative wavelet with delay 1/favg, switched off after
// t > 2/favg (CPU_vti2dfd_kernels.c:30-76, GPU_vti2dfd_kernels.cu:176-207).
// Time is a float advanced by repeated addition from dt (GUI programs) or 0
// (MPI program), as in the reference loops.
void source_amplitudes(Variant v, int nt, float dt, float favg, float pfac, int wtype,
                       std::vector<float> &amp, std::vector<uint8_t> &on) {
    const double pi = (v == V_MPI) ? kPiMpi : kPiGui;
    amp.assign(nt, 0.0f);
    on.assign(nt, 0);
    const float tdelay = (float)(1.0 / favg);
    float t = (v == V_MPI) ? 0.0f : dt;
    for (int it = 0; it < nt; it++, t += dt) {
        const float ts = t - tdelay;
        on[it] = (t <= 2 * tdelay);
        if (on[it]) amp[it] = pfac * wavelet(ts, favg, wtype, pi);
    }
}

// ---------------------------------------------------------------- taper
// SV-suppression circle around the source.  CPU/MPI form: radius CR=15,
// eps=del=0 inside CR*CR/16 (integer), cosine ramp outside
// (CPU_vti2dfd_kernels.c:136-156).  GPU form: R=15, r=4, ramp on sqrtf of
// the radius (GPU_vti2dfd_kernels.cu:260-278).  Only the kTB*kTB box around
// the centre can change.
void sv_taper_2d(Variant v, int nnx, int nnz, int npd, int cx, int cz, const float *e_pad,
                 const float *d_pad, Taper2D &out) {
    (void)npd;
    out.n = kTB;
    out.x0 = cx - kTB / 2;
    out.z0 = cz - kTB / 2;
    out.e.assign(kTB * kTB, 0.0f);
    out.d.assign(kTB * kTB, 0.0f);
    for (int bx = 0; bx < kTB; bx++)
        for (int bz = 0; bz < kTB; bz++) {
            const int ix = out.x0 + bx, iz = out.z0 + bz;
            if (ix < 0 || ix >= nnx || iz < 0 || iz >= nnz) continue;
            const size_t id = (size_t)ix * nnz + iz;
            const int rx = ix - cx, rz = iz - cz, r2 = rx * rx + rz * rz;
            float e = e_pad[id], d = d_pad[id];
            if (v == V_CPU || v == V_MPI) {
                const double pi = (v == V_MPI) ? kPiMpi : kPiGui;
                const int CR = 15;
                if (r2 <= CR * CR) {
                    if (r2 <= (CR * CR / 16)) {
                        e = 0.0f; d = 0.0f;
                    } else {
                        const double g = 0.5 * (1 - std::cos(pi * ((std::pow((double)r2, 0.5) - CR / 4.0) * 4.0 / (CR * 3.0 - 1))));
                        e = (float)(g * e); d = (float)(g * d);
                    }
                }
            } else {
                const int R = 15, r = 4;
                if (r2 <= R * R) {
                    if (r2 <= r * r) {
                        e = 0.0f; d = 0.0f;
                    } else {
                        const double g = 0.5 * (1 - std::cos(kPiGui * ((sqrtf((float)r2) - r) * 4.0 / (R * 3.0 - 1))));
                        e = (float)(g * e); d = (float)(g * d);
                    }
                }
            }
            out.e[bx * kTB + bz] = e;
            out.d[bx * kTB + bz] = d;
        }
}

// ---------------------------------------------------------------- mute
// GPU form, zero (t0/dt - tt, t0/dt + 2/(dt f) + tt) (GPU_vti2dfd_kernels.cu:151-174).
void mute_window_gpu2d(int nx, int nt, float dt, float favg, float dx, float dz, int fs, int ds,
                       int zs, int is, float mu_v, int tt, std::vector<int> &lo, std::vector<int> &hi) {
    lo.assign(nx, 0);
    hi.assign(nx, 0);
    for (int ix = 0; ix < nx; ix++) {
        const float mu_x = dx * std::abs(ix - fs - (is - 1) * ds), mu_z = dz * zs;
        const float mu_t0 = sqrtf((float)(std::pow(mu_x, 2) + std::pow(mu_z, 2))) / mu_v;
        const int mu_t = (int)(2.0 / (dt * favg));
        const int mu_nt = (int)(mu_t0 / dt) + mu_t + tt;
        int a = (int)(mu_t0 / dt) - tt + 1;  // it > (int)(t0/dt) - tt
        if (a < 0) a = 0;
        int b = mu_nt < nt ? mu_nt : nt;
        lo[ix] = a;
        hi[ix] = b > a ? b : a;
    }
}

// MPI form, zero [0, mu_nt) with dt in ms (Toa_rtm_vti_adcig_cdp.c:1587-1605).
// The reference writes past the trace when mu_nt > nt; here the window is
// clipped to the trace.
void mute_window_mpi(int nx, int nt, float dt_ms, float favg, float dx, float dz, int fs, int ds,
                     int zs, int is, float mu_v, int tt, std::vector<int> &lo, std::vector<int> &hi) {
    lo.assign(nx, 0);
    hi.assign(nx, 0);
    for (int ix = 0; ix < nx; ix++) {
        const float mu_x = dx * std::abs(ix - fs - (is - 1) * ds), mu_z = dz * zs;
        const float mu_t0 = sqrtf((float)(std::pow(mu_x, 2) + std::pow(mu_z, 2))) / mu_v;
        const int mu_t = (int)(2.0 / (dt_ms / 1000 * favg));
        const int mu_nt = (int)(mu_t0 / dt_ms * 1000) + mu_t + tt;
        hi[ix] = mu_nt < 0 ? 0 : (mu_nt < nt ? mu_nt : nt);
    }
}

// mute_directwave3d (GPU_vti3dfd_kernels.cu:342-369): zero it < mu_nt.
void mute_window_3d(int nx, int ny, int nt, float dt, float favg, float dx, float dy, float dz,
                    int fsx, int fsy, int dsx, int dsy, int fsz, int is, float vp1, float eps1, int tt,
                    std::vector<int> &hi) {
    hi.assign((size_t)nx * ny, 0);
    for (int iy = 0; iy < ny; iy++)
        for (int ix = 0; ix < nx; ix++) {
            const float mu_x = dx * std::abs(ix - fsx - is * dsx), mu_y = dy * std::abs(iy - fsy - is * dsy);
            const float mu_z = dz * fsz;
            const float mu_t0 = sqrtf((float)(std::pow(mu_x, 2) + std::pow(mu_y, 2) + std::pow(mu_z, 2))) /
                                (vp1 * sqrtf(1 + 2 * eps1));
            const int mu_t = (int)(2.0 / (dt * favg));
            const int mu_nt = (int)(mu_t0 / dt) + mu_t + tt;
            hi[(size_t)iy * nx + ix] = mu_nt < 0 ? 0 : (mu_nt < nt ? mu_nt : nt);
        }
}

// mute_directwave (3D-vti-fd+rtm-cuda/Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:352-390),
// window form: zero mu_t0/dt - tt < it < mu_nt, as [lo, hi) per receiver.
void mute_window_3d_band(int nx, int ny, int nt, float dt, float favg, float dx, float dy, float dz,
                         int fsx, int fsy, int dsx, int dsy, int fsz, int is, float vp1, float eps1, int tt,
                         std::vector<int> &lo, std::vector<int> &hi) {
    lo.assign((size_t)nx * ny, 0);
    hi.assign((size_t)nx * ny, 0);
    for (int iy = 0; iy < ny; iy++)
        for (int ix = 0; ix < nx; ix++) {
            const float mu_x = dx * std::abs(ix - fsx - is * dsx), mu_y = dy * std::abs(iy - fsy - is * dsy);
            const float mu_z = dz * fsz;
            const float mu_t0 = sqrtf((float)(std::pow(mu_x, 2) + std::pow(mu_y, 2) + std::pow(mu_z, 2))) /
                                (vp1 * sqrtf(1 + 2 * eps1));
            const int mu_t = (int)(2.0 / (dt * favg));
            const int mu_nt = (int)(mu_t0 / dt) + mu_t + tt;
            const int a = (int)(mu_t0 / dt) - tt + 1;
            lo[(size_t)iy * nx + ix] = a < 0 ? 0 : (a < nt ? a : nt);
            hi[(size_t)iy * nx + ix] = mu_nt < 0 ? 0 : (mu_nt < nt ? mu_nt : nt);
        }
}

int check_model(const float *v, const float *e, const float *d, size_t n) {
    for (size_t i = 0; i < n; i++) {
        if (!std::isfinite(v[i]) || !(v[i] > 0.0f)) return fail(GEO_ERR_MODEL, "velocity[%zu]=%g", i, v[i]);
        if (!std::isfinite(e[i]) || !std::isfinite(d[i])) return fail(GEO_ERR_MODEL, "eps/del[%zu] not finite", i);
        if (1 + 2 * d[i] < 0) return fail(GEO_ERR_MODEL, "1+2*delta[%zu] < 0", i);
    }
    return GEO_OK;
}

}  // namespace geo
