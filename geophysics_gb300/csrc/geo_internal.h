// Internal declarations of libgeofd: host-side setup helpers, device
// descriptors and kernel launchers shared by the translation units.
#pragma once
#include <cuda_runtime.h>
#include <cstdio>
#include <cstdint>
#include <vector>
#include <string>
#include "../../include/geofd.h"

namespace geo {

// ------------------------------------------------------------ error plumbing
extern thread_local char g_last_error[256];
int fail(int code, const char *fmt, ...);

#define GEO_CUDA(call)                                                            \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess)                                                    \
            return ::geo::fail(GEO_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__,  \
                               #call, cudaGetErrorString(e_));                    \
    } while (0)
#define GEO_TRY(expr)                  \
    do {                               \
        int s_ = (expr);               \
        if (s_ != GEO_OK) return s_;   \
    } while (0)

void count_launch(long long n = 1);
long long launches_so_far();
int check_launch(const char *what);

// RAII device buffer (cudaMalloc/cudaFree).
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { release(); }
    int alloc(size_t n);
    int zero(cudaStream_t s);
    void release();
    template <class T> T *as() const { return static_cast<T *>(p); }
};

// ------------------------------------------------------------ host setup
// Reference program whose arithmetic a run follows.
// V_TTIRTM (internal): the 2D TTI GPU RTM program's sponge, which differs
// from the other GPU programs' (sponge_d0, sponge_profiles).
enum Variant { V_CPU = GEO_VARIANT_CPU, V_GPU = GEO_VARIANT_GPU, V_MPI = GEO_VARIANT_MPI, V_TTIRTM = 100 };

// pi as each reference program spells it.
constexpr double kPiGui = 3.141592653;      // CPU_vti2dfd_kernels.c:27, GPU_vti*_kernels.cu:31
constexpr double kPiMpi = 3.1415926535898;  // Toa_rtm_vti_adcig_cdp.c:39

// ------------------------------------------------------------ failure detection (guard.cu)
// The Madagascar-derived stability limit of the 8th-order staggered operator
// (Toa_gpu2DvtiFdRtmAdcigsLaplace.cu:941-965, mm = 4).
constexpr double kStabilityC = 0.777;
double stability_number(int dims, float vmax, float dt, float dx, float dy, float dz);
// GEO_ERR_CFL when dt*vmax*sqrt(sum 1/d^2) >= kStabilityC; for the CPU
// program also its get_constant limits (dx, dz <= vmin/favg*0.2 and
// dt <= 0.5*min(dx,dz)/vmax).
int check_stability(Variant v, int dims, float vmin, float vmax, float dt, float dx, float dy, float dz,
                    float favg);
// min and max of n positive finite floats into out[0], out[1] (float bits;
// out is written, not accumulated)
int launch_minmax(const float *a, size_t n, unsigned *out, cudaStream_t s);
// Interval of the wavefield watchdog (GEO_WATCH_EVERY, default 100; 0 = off).
int watch_every();
// Non-finite detector: a word of mapped pinned memory that k_watch sets to
// the tag of the first scan that found NaN/Inf.  check() scans every
// `every` steps (and on the last) and returns GEO_ERR_NAN, without a
// message, once the word is seen set, so the caller stops queueing steps;
// verdict() drains the stream and turns a set word into the error.
struct Watchdog {
    int *h = nullptr, *d = nullptr;
    int every = 100;
    Watchdog() = default;
    Watchdog(const Watchdog &) = delete;
    Watchdog &operator=(const Watchdog &) = delete;
    ~Watchdog() { close(); }
    int open();
    void close();
    void arm();
    bool tripped() const;
    int check(const float *a, size_t n, int it, bool last, cudaStream_t s);
    int scan(const float *a, size_t n, int tag, cudaStream_t s);
    int verdict(cudaStream_t s, const char *what);
};

// Edge-replicate an nx*nz model into its padded (nx+2npd)*(nz+2npd) form.
void pad_model_2d(int nx, int nz, int npd, const float *in, float *out);
// Same for 3D, reference layout iz + nz*(ix + nx*iy).

float sponge_d0(Variant v, int dims, float vpmax, float vcenter, int npd, float dx, float dy, float dz);
// coff1/coff2 on half cells (velocities), acoff1/acoff2 on integer cells
// (stresses); arrays of n+2npd.
void sponge_profiles(Variant v, int n, int npd, float dt, float d0, float *coff1, float *coff2,
                     float *acoff1, float *acoff2);
// pfac*w(t_it) per step and whether the source is still on.
void source_amplitudes(Variant v, int nt, float dt, float favg, float pfac, int wtype,
                       std::vector<float> &amp, std::vector<uint8_t> &on);
// Tapered (eps, del) near the source for the SV-suppression circle.
struct Taper2D {
    int x0 = 0, z0 = 0, n = 0;            // box origin (padded) and size
    std::vector<float> e, d;              // tapered values on the box
};
void sv_taper_2d(Variant v, int nnx, int nnz, int npd, int ixs_center, int izs_center,
                 const float *e_pad, const float *d_pad, Taper2D &out);

// Per-trace direct-wave mute window [lo, hi) of samples to zero.
void mute_window_gpu2d(int nx, int nt, float dt, float favg, float dx, float dz, int fs, int ds,
                       int zs, int is, float mu_v, int tt, std::vector<int> &lo, std::vector<int> &hi);
void mute_window_mpi(int nx, int nt, float dt_ms, float favg, float dx, float dz, int fs, int ds,
                     int zs, int is, float mu_v, int tt, std::vector<int> &lo, std::vector<int> &hi);
void mute_window_3d(int nx, int ny, int nt, float dt, float favg, float dx, float dy, float dz,
                    int fsx, int fsy, int dsx, int dsy, int fsz, int is, float vp1, float eps1, int tt,
                    std::vector<int> &hi);
void mute_window_3d_band(int nx, int ny, int nt, float dt, float favg, float dx, float dy, float dz,
                         int fsx, int fsy, int dsx, int dsy, int fsz, int is, float vp1, float eps1, int tt,
                         std::vector<int> &lo, std::vector<int> &hi);

// Angle-gather tables of the GPU RTM programs' Poynting bin, built on the
// device into device arrays of 128 floats each: thresholds (largest cosine
// of bins >= k, -2 where none) and cosf(ia*pi/180), from the device's acosf
// and cosf.
int adcig_angle_tables(int nangle, int dangle, float *thr, float *cs, cudaStream_t s);

// Raw float32 files: read exactly n values; write n values at a byte offset.
int read_floats(const char *fn, size_t n, std::vector<float> &out);
int write_at(FILE *fp, size_t offset_bytes, const float *a, size_t n);

// Model sanity: finite, velocity > 0.
int check_model(const float *v, const float *e, const float *d, size_t n);

// ------------------------------------------------------------ 2D device side
constexpr int kTB = 31;  // taper box edge (circle radius 15)

// Per-shot descriptor read by the batched 2D kernels (device memory).
struct Shot2D {
    int nnx, nnz, npd, nx, nz;
    float dtx, dtz;
    const float *cx1, *cx2, *cz1, *cz2, *ax1, *ax2, *az1, *az2;
    const float *vp, *e2, *d2;      // vp (or rho*vp^2), 1+2eps, sqrtf(1+2del)
    // MPI form, exact arithmetic: the double factors of its pz and qx
    // chains, ((double)(az1*vp)*pow(1+2del,0.5))*(double)dtz and the same
    // with ax1, dtx, formed once per shot in the program's order
    const double *kz, *kx;
    int tx0, tz0;                   // taper box origin; te2/td2/tkz/tkx on kTB*kTB
    const float *te2, *td2;
    const double *tkz, *tkx;
    int ixs, izs;                   // source cell (padded)
    float *u[2], *w[2], *P[2], *Q[2], *px[2], *pz[2], *qx[2], *qz[2];
    int rec_iz;                     // receiver row
    float rec_scale;
    float *rec_p, *rec_q;           // time-major records nt x nx
    float *edge_p, *edge_q;         // time-major edge lines nt x (2nx+2nz)
    float *mig, *ill;               // image and source illumination nx*nz
    float *adcig;                   // Poynting angle gathers [90][nx][nz], or null
    int tile_base, ntz;             // first work item, tiles along z
};

struct Step2D {
    int it;
    float amp;        // pfac*w(t) this step (0 when off)
    int src_on;       // source active this step
    int taper;        // use the taper box for eps/del
    int nf;           // fields updated (1: s only, 2: s and g)
    int fast;         // MPI form: double-precision chains in FP32
};

enum Phase2D { PH_FWD = 0, PH_BWD = 1 };

// A whole single-shot forward run in one cooperative launch (launch_fd2d_shot).
struct Persist2D {
    int nt, taper;
    const float *amp;             // pfac*w(t) of every step
    const unsigned char *on;      // source active at every step
    unsigned *bar;                // grid-barrier arrival counter, zeroed
    int *err;                     // set when a barrier wait gave up
};
int launch_fd2d_shot(int variant, const Shot2D *d_shots, const int *d_item_shot, int nitems, int by, Persist2D a,
                     cudaStream_t s);
// The same shot with each block's tile of the fields resident in shared
// memory (CPU and GPU forms), steps it0..it1-1; *fits is false (and nothing
// runs) when the grid does not fit on the device that way.  xch: 8 exchange
// fields of nnx*nnz floats, zeroed before the first run.
int launch_fd2d_tile(int variant, const Shot2D &sh, float *xch, const float *amp, const unsigned char *on,
                     int taper, int it0, int it1, unsigned *bar, int *err, bool *fits, cudaStream_t s);

int launch_vel2d(int variant, const Shot2D *d_shots, const int *d_item_shot, int nitems, int by,
                 int grid, Step2D st, cudaStream_t s);
int launch_stress2d(int variant, int phase, const Shot2D *d_shots, const int *d_item_shot, int nitems,
                    int by, int grid, Step2D st, cudaStream_t s);
int launch_inject2d(const Shot2D *d_shots, int nshots, int maxline, int it, cudaStream_t s);
// Velocity tiles (kind 0, step st_v) and stress tiles (kind 1, step st_s)
// of disjoint shots in one launch, MPI form (fd2d.cu, k_mix2d).
int launch_mix2d(int phase, int fast, const Shot2D *d_shots, const int2 *d_items, int nitems, int by, int grid,
                 Step2D st_v, Step2D st_s, cudaStream_t s);
int launch_mute_records(float *rec, int nx, int nt, const int *lo, const int *hi, cudaStream_t s);
// cos and sin of n tilt angles in radians on the device, as the 2D TTI
// programs form them (in place: th_cos holds the angles, then the cosines).
int launch_tilt_trig(float *th_cos, float *sn, size_t n, cudaStream_t s);
// Watchdog scan of the P fields (sides 0..nf-1) of ns shots (fd2d.cu).
int launch_watch_shots(const Shot2D *d_shots, int ns, int nf, int *flag, int tag, cudaStream_t s);
int launch_transpose_records(const float *tm, float *out, int ntr, int nt, cudaStream_t s);
int launch_normalize_image(float *mig, const float *ill, size_t n, cudaStream_t s);
// a[p*n + k] /= ill[k] for p < planes.
int launch_normalize_planes(float *a, const float *ill, size_t n, int planes, cudaStream_t s);
// Angle-bin thresholds and cos^3 weights of the Poynting ADCIG into constant memory.
int load_adcig_tables(cudaStream_t s);
constexpr int kAdcigAngles = 90;
int launch_stack_image(float *full, int nz, const float *const *imgs, const int *offsets,
                       const int *widths, int nshots, int nx, cudaStream_t s);
int launch_laplace2d(int nx, int nz, const float *in, float *out, cudaStream_t s);
int launch_laplace3d(int nx, int ny, int nz, const float *in, float *out, cudaStream_t s);

}  // namespace geo
