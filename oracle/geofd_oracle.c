/*
 * geofd_oracle.c -- CPU restatement of the reference's FP32 staggered-grid
 * VTI finite-difference hot path.  TEST INFRASTRUCTURE ONLY: it is the
 * checker for the CUDA library (tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py load it); the product never links or calls it.
 *
 * Compiled twice by oracle/Makefile:
 *   liborc32.so  REAL=float   -- follows the reference's FP32 arithmetic op
 *                               by op (same operand order, no contraction,
 *                               the same double-precision intermediates), so
 *                               a GPU kernel that keeps the order is
 *                               bit-exact against it;
 *   liborc64.so  REAL=double  -- the same algorithm in FP64, used to state
 *                               every FP32 result's error against FP64.
 *
 * Parity pinning: the FP32 build is checked against the reference's own CPU
 * code compiled unmodified from the reference tree (oracle/_ref, see
 * oracle/Makefile and tests/test_oracle_pin.py):
 *   - 2D FD, CPU variant  == CPU_vti2dfd        (2D-3D-vti-fd-cuda-gtk-GUI/CPU_vti2dfd_kernels.c:366)
 *   - 2D RTM, MPI variant == model_vti_get_boundry + RTM_corr_adcig
 *                            (2D-vti-fd+rtm-mpi/Toa_rtm_vti_adcig_cdp.c:483,739)
 *   - Laplacian          == laplac2_lop(adj=1) (utils-Laplacian-filter/laplace.c:9)
 * The 3D VTI and 2D TTI paths have no CPU code in the reference; they follow
 * the reference's CUDA kernels (2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti3dfd_kernels.cu:53-201,
 * 2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:81-183) and are
 * "parity unpinned" against the reference itself.
 *
 * Layouts follow the reference: 2D id = ix*nnz + iz, 3D id = iz + nnz*(ix + nnx*iy)
 * (z fastest); shot records are trace-major, shot[it + nt*trace].
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef REAL
#define REAL float
#endif

#if defined(ORC_FP64)
#define RSQRT(x) sqrt(x)
#define RFMA(a, b, c) fma(a, b, c)
#else
#define RSQRT(x) sqrtf(x)
#define RFMA(a, b, c) fmaf(a, b, c)
#endif

/* variant codes (which reference program's semantics) */
#define ORC_V_CPU    0   /* CPU_vti2dfd            (GUI CPU, C)          */
#define ORC_V_GPU    1   /* GPU_vti2dfd/GPU_vti3dfd (GUI GPU, CUDA)       */
#define ORC_V_MPI    2   /* Toa_rtm_vti_adcig_cdp.c (MPI CPU RTM)         */
#define ORC_V_GPURTM 3   /* Toa_gpu2DvtiFdRtmAdcigsLaplace.cu (GPU RTM)   */

/* pi literals differ between reference programs */
#define PI_GUI 3.141592653        /* CPU_vti2dfd_kernels.c:27, GPU_vti2dfd_kernels.cu:31 */
#define PI_MPI 3.1415926535898    /* Toa_rtm_vti_adcig_cdp.c:39 */

static const float C8[4] = {1.196289f, -0.0797526f, 0.009570313f, -0.0006975447f};
/* The 8th-order staggered coefficients (CPU_vti2dfd_kernels.c:334-343). */

/* ---------------------------------------------------------------- setup */

/* Edge replication into the sponge (CPU_vti2dfd_kernels.c:221-246; the
 * 3D form GPU_vti3dfd_kernels.cu:208-255).  `a` is the padded array. */
void orc_pad2d(int nx, int nz, int npd, REAL *a)
{
    int nnx = nx + 2 * npd, nnz = nz + 2 * npd, ix, iz;
    for (ix = 0; ix < nnx; ix++)
        for (iz = 0; iz < nnz; iz++) {
            if (ix < npd) a[ix * nnz + iz] = a[npd * nnz + iz];
            else if (ix >= nnx - npd) a[ix * nnz + iz] = a[(nnx - npd - 1) * nnz + iz];
        }
    for (ix = 0; ix < nnx; ix++)
        for (iz = 0; iz < nnz; iz++) {
            if (iz < npd) a[ix * nnz + iz] = a[ix * nnz + npd];
            else if (iz >= nnz - npd) a[ix * nnz + iz] = a[ix * nnz + nnz - npd - 1];
        }
}

void orc_pad3d(int nx, int ny, int nz, int npd, REAL *a)
{
    long nnx = nx + 2 * npd, nny = ny + 2 * npd, nnz = nz + 2 * npd, ix, iy, iz;
    for (iy = 0; iy < nny; iy++) for (ix = 0; ix < nnx; ix++) for (iz = 0; iz < nnz; iz++) {
        long id = iz + ix * nnz + iy * nnz * nnx;
        if (ix < npd) a[id] = a[iz + npd * nnz + iy * nnz * nnx];
        else if (ix >= nnx - npd) a[id] = a[iz + (nnx - npd - 1) * nnz + iy * nnz * nnx];
    }
    for (iy = 0; iy < nny; iy++) for (ix = 0; ix < nnx; ix++) for (iz = 0; iz < nnz; iz++) {
        long id = iz + ix * nnz + iy * nnz * nnx;
        if (iy < npd) a[id] = a[iz + ix * nnz + npd * nnz * nnx];
        else if (iy >= nny - npd) a[id] = a[iz + ix * nnz + (nny - npd - 1) * nnz * nnx];
    }
    for (iy = 0; iy < nny; iy++) for (ix = 0; ix < nnx; ix++) for (iz = 0; iz < nnz; iz++) {
        long id = iz + ix * nnz + iy * nnz * nnx;
        if (iz < npd) a[id] = a[npd + ix * nnz + iy * nnz * nnx];
        else if (iz >= nnz - npd) a[id] = a[nnz - npd - 1 + ix * nnz + iy * nnz * nnx];
    }
}

/* Sponge damping constant d0.
 *  CPU/MPI: 3*vpmax*ln(1e5)/(2*npd*dx)            CPU_vti2dfd_kernels.c:192, Toa_rtm_vti_adcig_cdp.c:1346
 *  GPU 2D : 10*vp[nnx*nnz/2]*ln(1e5)/(2*npd*(dx+dz)/2)   GPU_vti2dfd_kernels.cu:105
 *  GPU 3D : 10*vp[n/2]*ln(1e5)/(2*npd*(dx+dy+dz)/3)      GPU_vti3dfd_kernels.cu:205
 * `vpmax` is the interior maximum (the CPU loop's scan over the padded
 * array sees only replicated edge values outside the interior). */
float orc_d0(int variant, int dims, float vpmax, float vcenter, int npd, float dx, float dy, float dz)
{
    if (variant == ORC_V_CPU || variant == ORC_V_MPI)
        return (float)(3.0 * vpmax * log(100000.0) / (2.0 * npd * dx));
    if (dims == 2)
        return (float)(10.0 * vcenter * log(100000.0) / (2.0 * npd * ((dx + dz) / 2.0)));
    return (float)(10.0 * vcenter * log(100000.0) / (2.0 * npd * ((dx + dy + dz) / 3.0)));
}

/* 1D sponge profiles along one axis with n interior cells (nn = n + 2*npd).
 *  CPU  : CPU_vti2dfd_kernels.c:271-332 (acoff2 is built from coff1, and the
 *         far side uses (1+i-n-npd)/npd)
 *  MPI  : Toa_rtm_vti_adcig_cdp.c:1455-1525 (acoff2 from acoff1)
 *  GPU  : GPU_vti2dfd_kernels.cu:108-139 (far side (i-n-npd)/npd) */
void orc_sponge(int variant, int n, int npd, float dt, float d0,
                float *coff1, float *coff2, float *acoff1, float *acoff2)
{
    int i, nn = n + 2 * npd;
    for (i = 0; i < nn; i++) { coff1[i] = coff2[i] = acoff1[i] = acoff2[i] = 1.0f; }
    if (variant == ORC_V_GPU || variant == ORC_V_GPURTM) {
        for (i = 0; i < nn; i++) {
            if (i < npd) {
                coff1[i] = (float)(1.0 / (1.0 + (dt * d0 * pow((npd - 0.5 - i) / npd, 2.0)) / 2.0));
                coff2[i] = (float)(coff1[i] * (1.0 - (dt * d0 * pow((npd - 0.5 - i) / npd, 2.0)) / 2.0));
                acoff1[i] = (float)(1.0 / (1.0 + (dt * d0 * pow(((npd - i) * 1.0) / npd, 2.0)) / 2.0));
                acoff2[i] = (float)(acoff1[i] * (1.0 - (dt * d0 * pow(((npd - i) * 1.0) / npd, 2.0)) / 2.0));
            } else if (i >= npd + n) {
                coff1[i] = (float)(1.0 / (1.0 + (dt * d0 * pow((0.5 + i - n - npd) / npd, 2.0)) / 2.0));
                coff2[i] = (float)(coff1[i] * (1.0 - (dt * d0 * pow((0.5 + i - n - npd) / npd, 2.0)) / 2.0));
                acoff1[i] = (float)(1.0 / (1.0 + (dt * d0 * pow(((i - n - npd) * 1.0) / npd, 2.0)) / 2.0));
                acoff2[i] = (float)(acoff1[i] * (1.0 - (dt * d0 * pow(((i - n - npd) * 1.0) / npd, 2.0)) / 2.0));
            }
        }
        return;
    }
    /* CPU and MPI: identical except where acoff2 takes its leading factor */
    for (i = 0; i < npd; i++) {
        coff1[i] = 1 / (1 + (dt * d0 * pow((npd - 0.5 - i) / npd, 2)) / 2);
        coff2[i] = coff1[i] * (1 - (dt * d0 * pow((npd - 0.5 - i) / npd, 2)) / 2);
    }
    for (i = npd + n; i < n + 2 * npd; i++) {
        coff1[i] = 1 / (1 + (dt * d0 * pow((0.5 + i - n - npd) / npd, 2)) / 2);
        coff2[i] = coff1[i] * (1 - (dt * d0 * pow((0.5 + i - n - npd) / npd, 2)) / 2);
    }
    for (i = 0; i < npd; i++) {
        acoff1[i] = 1 / (1 + (dt * d0 * pow(((npd - i) * 1.0) / npd, 2)) / 2);
        acoff2[i] = (variant == ORC_V_CPU ? coff1[i] : acoff1[i]) * (1 - (dt * d0 * pow(((npd - i) * 1.0) / npd, 2)) / 2);
    }
    for (i = npd + n; i < n + 2 * npd; i++) {
        acoff1[i] = 1 / (1 + (dt * d0 * pow(((1 + i - n - npd) * 1.0) / npd, 2)) / 2);
        acoff2[i] = (variant == ORC_V_CPU ? coff1[i] : acoff1[i]) * (1 - (dt * d0 * pow(((1 + i - n - npd) * 1.0) / npd, 2)) / 2);
    }
}

/* Wavelet (CPU_vti2dfd_kernels.c:30-48 get_wavelet; same formula inlined in
 * add_source2d GPU_vti2dfd_kernels.cu:176-207).  Returns the float the
 * reference stores: the expression is evaluated in double. */
static float orc_wavelet(float ts, float favg, int wtype, double pi_)
{
    float x, xx, source = 0.0f;
    if (wtype == 1) { x = favg * ts; xx = x * x; source = (float)((1 - 2 * pi_ * pi_ * (xx)) * exp(-(pi_ * pi_ * xx))); }
    else if (wtype == 2) { double y = (-4) * favg * favg * pi_ * pi_ / log(0.1); source = (float)((-2) * pi_ * pi_ * ts * exp(-y * ts * ts)); }
    else if (wtype == 3) { double y = (-1) * favg * favg * pi_ * pi_ / log(0.1); source = (float)exp(-y * ts * ts); }
    return source;
}

/* Per-step source amplitude pfac*w(t) (0 once t > 2/favg), with the
 * reference's float time accumulation: t starts at dt (CPU/GPU variants,
 * CPU_vti2dfd_kernels.c:478) or at 0 (MPI, Toa_rtm_vti_adcig_cdp.c:654) and
 * advances by repeated float addition.  amp[it] is what the GPU variant adds
 * at one cell; the CPU/MPI variants multiply it by exp(-x^2-z^2) on a 7x7
 * window (ptsource CPU_vti2dfd_kernels.c:50-76). */
void orc_source_amp(int variant, int nt, float dt, float favg, float pfac, int wtype, float *amp, unsigned char *active)
{
    double pi_ = (variant == ORC_V_MPI) ? PI_MPI : PI_GUI;
    float t = (variant == ORC_V_MPI) ? 0.0f : dt, tdelay = (float)(1.0 / favg), ts;
    int it;
    for (it = 0; it < nt; it++, t += dt) {
        ts = t - tdelay;
        active[it] = (t <= 2 * tdelay);
        amp[it] = active[it] ? pfac * orc_wavelet(ts, favg, wtype, pi_) : 0.0f;
    }
}

/* SV-suppression taper: returns the tapered epsilon/delta near the source.
 *  CPU: CPU_vti2dfd_kernels.c:136-156 (CR=15, inner CR*CR/16, centre at the
 *       source cell ixs,izs, double cos/pow)
 *  MPI: Toa_rtm_vti_adcig_cdp.c:1258-1274 (same form, its own pi, always on)
 *  GPU: GPU_vti2dfd_kernels.cu:260-278 (R=15,r=4; centre (fs+(is-1)ds+npd,
 *       zs+npd); sqrtf of the radius), GPU RTM R=18,r=7
 *       (Toa_gpu2DvtiFdRtmAdcigsLaplace.cu:342-382).
 * The taper is applied in place to padded e,d (2D). */
void orc_sv_taper2d(int variant, int nnx, int nnz, int npd, float fs, float ds, float zs, int is,
                    const float *e_in, const float *d_in, float *e_out, float *d_out)
{
    int ix, iz;
    if (variant == ORC_V_CPU || variant == ORC_V_MPI) {
        double pi_ = (variant == ORC_V_MPI) ? PI_MPI : PI_GUI;
        float f = fs + (is - 1) * ds;
        int ixs = (int)(f + 0.5) + npd - 1, izs = (int)(zs + 0.5) + npd - 1, CR = 15;
        for (ix = 0; ix < nnx; ix++) for (iz = 0; iz < nnz; iz++) {
            int id = ix * nnz + iz, rx = ix - ixs, rz = iz - izs;
            if ((rx * rx + rz * rz) <= CR * CR) {
                if ((rx * rx + rz * rz) <= (CR * CR / 16)) { e_out[id] = 0.0f; d_out[id] = 0.0f; }
                else {
                    double g = 0.5 * (1 - cos(pi_ * ((pow((rx * rx + rz * rz), 0.5) - CR / 4.0) * 4.0 / (CR * 3.0 - 1))));
                    e_out[id] = (float)(g * e_in[id]);
                    d_out[id] = (float)(g * d_in[id]);
                }
            } else { e_out[id] = e_in[id]; d_out[id] = d_in[id]; }
        }
    } else {
        int R = (variant == ORC_V_GPURTM) ? 18 : 15, r = (variant == ORC_V_GPURTM) ? 7 : 4;
        int cx = (int)fs + (is - 1) * (int)ds + npd, cz = (int)zs + npd;
        for (ix = 0; ix < nnx; ix++) for (iz = 0; iz < nnz; iz++) {
            int id = ix * nnz + iz, rx = ix - cx, rz = iz - cz;
            if ((rx * rx + rz * rz) <= R * R) {
                if ((rx * rx + rz * rz) <= r * r) { e_out[id] = 0.0f; d_out[id] = 0.0f; }
                else {
                    double g = 0.5 * (1 - cos(PI_GUI * ((sqrtf((float)(rx * rx + rz * rz)) - r) * 4.0 / (R * 3.0 - 1))));
                    e_out[id] = (float)(g * e_in[id]);
                    d_out[id] = (float)(g * d_in[id]);
                }
            } else { e_out[id] = e_in[id]; d_out[id] = d_in[id]; }
        }
    }
}

/* ------------------------------------------------------------- 2D state */

typedef struct {
    int nnx, nnz, npd, variant;
    REAL dtx, dtz;
    const float *cx1, *cx2, *cz1, *cz2, *ax1, *ax2, *az1, *az2;
    const REAL *vp;     /* vp (CPU/GPU) or rho*vp^2 (MPI) */
    const REAL *e2;     /* 1+2*eps after the SV taper */
    const REAL *d2;     /* sqrtf(1+2*del) (CPU/GPU) */
    const double *pw;   /* pow(1+2*del,0.5) in double (MPI) */
} orc_st2d;

/* Velocity update (CPU_vti2dfd_kernels.c:79-106; the MPI copy
 * Toa_rtm_vti_adcig_cdp.c:1200-1225 multiplies by rho == 1). */
static void vel2d(const orc_st2d *s, REAL *u, REAL *w, const REAL *P, const REAL *Q)
{
    int ix, iz, im, nnz = s->nnz;
    for (ix = 4; ix < s->nnx - 4; ix++)
        for (iz = 4; iz < nnz - 4; iz++) {
            int id = ix * nnz + iz;
            REAL xx = 0, zz = 0;
            for (im = 0; im < 4; im++) {
                xx += (REAL)C8[im] * (P[id + (im + 1) * nnz] - P[id - im * nnz]);
                zz += (REAL)C8[im] * (Q[id + im + 1] - Q[id - im]);
            }
            if (s->variant == ORC_V_MPI) {
                u[id] = s->cx2[ix] * u[id] - s->cx1[ix] * s->dtx * (REAL)1.0 * xx;
                w[id] = s->cz2[iz] * w[id] - s->cz1[iz] * s->dtz * (REAL)1.0 * zz;
            } else {
                u[id] = s->cx2[ix] * u[id] - s->cx1[ix] * s->dtx * xx;
                w[id] = s->cz2[iz] * w[id] - s->cz1[iz] * s->dtz * zz;
            }
        }
}

/* Stress update with split sponge fields (CPU_vti2dfd_kernels.c:108-177,
 * GPU_vti2dfd_kernels.cu:240-299, MPI Toa_rtm_vti_adcig_cdp.c:1227-1327).
 * src (may be NULL) is added into P and Q after the split sum (CPU/MPI). */
static void stress2d(const orc_st2d *s, const REAL *u, const REAL *w, REAL *P, REAL *Q,
                     REAL *px, REAL *pz, REAL *qx, REAL *qz, const REAL *src)
{
    int ix, iz, im, nnz = s->nnz;
    for (ix = 4; ix < s->nnx - 4; ix++)
        for (iz = 4; iz < nnz - 4; iz++) {
            int id = ix * nnz + iz;
            REAL xx = 0, zz = 0, vp = s->vp[id];
            for (im = 0; im < 4; im++) {
                xx += (REAL)C8[im] * (u[id + im * nnz] - u[id - (im + 1) * nnz]);
                zz += (REAL)C8[im] * (w[id + im] - w[id - im - 1]);
            }
            if (s->variant == ORC_V_MPI) {
                /* the pow() factor turns the pz/qx chains into double */
                px[id] = s->ax2[ix] * px[id] - s->ax1[ix] * vp * s->e2[id] * s->dtx * xx;
                pz[id] = (REAL)(s->az2[iz] * pz[id] - s->az1[iz] * vp * s->pw[id] * s->dtz * zz);
                qx[id] = (REAL)(s->ax2[ix] * qx[id] - s->ax1[ix] * vp * s->pw[id] * s->dtx * xx);
                qz[id] = s->az2[iz] * qz[id] - s->az1[iz] * vp * s->dtz * zz;
            } else {
                px[id] = s->ax2[ix] * px[id] - s->ax1[ix] * vp * vp * s->e2[id] * s->dtx * xx;
                pz[id] = s->az2[iz] * pz[id] - s->az1[iz] * vp * vp * s->d2[id] * s->dtz * zz;
                qx[id] = s->ax2[ix] * qx[id] - s->ax1[ix] * vp * vp * s->d2[id] * s->dtx * xx;
                qz[id] = s->az2[iz] * qz[id] - s->az1[iz] * vp * vp * s->dtz * zz;
            }
            if (src) { P[id] = px[id] + pz[id] + src[id]; Q[id] = qx[id] + qz[id] + src[id]; }
            else     { P[id] = px[id] + pz[id];           Q[id] = qx[id] + qz[id]; }
        }
}

/* Fill the 7x7 Gaussian source window (ptsource, CPU_vti2dfd_kernels.c:50-76;
 * Toa_rtm_vti_adcig_cdp.c:1141-1174): s = (pfac*w) * exp(-x^2-z^2). */
static void gauss_src2d(int nnz, int ixs, int izs, float amp, int active, REAL *s, int nnx)
{
    int i, j;
    memset(s, 0, sizeof(REAL) * (size_t)nnx * nnz);
    if (!active) return;
    for (j = izs - 3; j <= izs + 3; j++)
        for (i = ixs - 3; i <= ixs + 3; i++) {
            int x = i - ixs, z = j - izs;
            s[i * nnz + j] = (REAL)(amp * exp(-z * z - x * x));
        }
}

typedef struct {
    int nx, nz, npd, nt, variant, sv, wtype;
    float dx, dz, dt, favg, pfac, fs, ds, zs;
    int is;          /* shot number, 1-based as in the reference loops */
    int rec_iz;      /* receiver row (padded z index) */
    float rec_scale; /* 2 for CPU_vti2dfd's P+P record */
} orc_fd2d_desc;

/* Allocated working set for one 2D propagation. */
typedef struct {
    orc_st2d st;
    REAL *u, *w, *P, *Q, *px, *pz, *qx, *qz, *s, *vp, *e2, *d2; double *pw;
    float *cx1, *cx2, *cz1, *cz2, *ax1, *ax2, *az1, *az2;
    float *amp; unsigned char *active;
    int ixs, izs;
} orc_prop2d;

static void prop2d_free(orc_prop2d *p)
{
    free(p->u); free(p->w); free(p->P); free(p->Q); free(p->px); free(p->pz); free(p->qx); free(p->qz);
    free(p->s); free(p->vp); free(p->e2); free(p->d2); free(p->pw);
    free(p->cx1); free(p->cx2); free(p->cz1); free(p->cz2); free(p->ax1); free(p->ax2); free(p->az1); free(p->az2);
    free(p->amp); free(p->active);
}

static void prop2d_zero_state(orc_prop2d *p)
{
    size_t n = (size_t)p->st.nnx * p->st.nnz * sizeof(REAL);
    memset(p->u, 0, n); memset(p->w, 0, n); memset(p->P, 0, n); memset(p->Q, 0, n);
    memset(p->px, 0, n); memset(p->pz, 0, n); memset(p->qx, 0, n); memset(p->qz, 0, n);
}

/* Build the propagator from an unpadded (nx x nz, x-major) model.  `taper`
 * selects whether the SV taper is applied (the MPI backward passes use the
 * untapered model, inv_update_stress Toa_rtm_vti_adcig_cdp.c:1293-1327). */
static void prop2d_init(orc_prop2d *p, const orc_fd2d_desc *d, const float *v, const float *e,
                        const float *dl, int taper)
{
    int nx = d->nx, nz = d->nz, npd = d->npd, nnx = nx + 2 * npd, nnz = nz + 2 * npd, ix, iz;
    size_t n = (size_t)nnx * nnz;
    float *vv = calloc(n, 4), *ee = calloc(n, 4), *dd = calloc(n, 4), *e1 = calloc(n, 4), *d1 = calloc(n, 4);
    float vpmax, d0, dtf = d->dt;
    memset(p, 0, sizeof(*p));
    for (ix = 0; ix < nx; ix++) for (iz = 0; iz < nz; iz++) {
        size_t id = (size_t)(ix + npd) * nnz + iz + npd;
        vv[id] = v[ix * nz + iz]; ee[id] = e[ix * nz + iz]; dd[id] = dl[ix * nz + iz];
    }
    /* pad in float (the pad is a pure copy) */
    {
        REAL *tmp = malloc(n * sizeof(REAL)); size_t k;
        float *arrs[3] = {ee, dd, vv};
        int a;
        for (a = 0; a < 3; a++) {
            for (k = 0; k < n; k++) tmp[k] = arrs[a][k];
            orc_pad2d(nx, nz, npd, tmp);
            for (k = 0; k < n; k++) arrs[a][k] = (float)tmp[k];
        }
        free(tmp);
    }
    vpmax = vv[npd * nnz + npd];
    for (ix = npd; ix < npd + nx; ix++) for (iz = npd; iz < npd + nz; iz++)
        if (vpmax < vv[ix * nnz + iz]) vpmax = vv[ix * nnz + iz];
    d0 = orc_d0(d->variant, 2, vpmax, vv[nnx * nnz / 2], npd, d->dx, d->dx, d->dz);

    p->cx1 = malloc(nnx * 4); p->cx2 = malloc(nnx * 4); p->ax1 = malloc(nnx * 4); p->ax2 = malloc(nnx * 4);
    p->cz1 = malloc(nnz * 4); p->cz2 = malloc(nnz * 4); p->az1 = malloc(nnz * 4); p->az2 = malloc(nnz * 4);
    orc_sponge(d->variant, nx, npd, dtf, d0, p->cx1, p->cx2, p->ax1, p->ax2);
    orc_sponge(d->variant, nz, npd, dtf, d0, p->cz1, p->cz2, p->az1, p->az2);

    if (taper) orc_sv_taper2d(d->variant, nnx, nnz, npd, d->fs, d->ds, d->zs, d->is, ee, dd, e1, d1);
    else { memcpy(e1, ee, n * 4); memcpy(d1, dd, n * 4); }

    p->vp = malloc(n * sizeof(REAL)); p->e2 = malloc(n * sizeof(REAL)); p->d2 = malloc(n * sizeof(REAL));
    p->pw = malloc(n * sizeof(double));
    for (size_t k = 0; k < n; k++) {
        if (d->variant == ORC_V_MPI) p->vp[k] = (REAL)1 * ((REAL)vv[k] * (REAL)vv[k]);  /* rho*vp^2, rho==1 */
        else p->vp[k] = vv[k];
        p->e2[k] = (REAL)1 + (REAL)2 * (REAL)e1[k];
        p->d2[k] = RSQRT((REAL)1 + (REAL)2 * (REAL)d1[k]);
        p->pw[k] = pow((1 + 2 * d1[k]), 0.5);
    }
    p->u = calloc(n, sizeof(REAL)); p->w = calloc(n, sizeof(REAL)); p->P = calloc(n, sizeof(REAL)); p->Q = calloc(n, sizeof(REAL));
    p->px = calloc(n, sizeof(REAL)); p->pz = calloc(n, sizeof(REAL)); p->qx = calloc(n, sizeof(REAL)); p->qz = calloc(n, sizeof(REAL));
    p->s = calloc(n, sizeof(REAL));
    p->amp = malloc(d->nt * 4); p->active = malloc(d->nt);
    orc_source_amp(d->variant, d->nt, dtf, d->favg, d->pfac, d->wtype, p->amp, p->active);
    {
        float f = d->fs + (d->is - 1) * d->ds;
        p->ixs = (int)(f + 0.5) + npd - 1;
        p->izs = (int)(d->zs + 0.5) + npd - 1;
    }
    p->st.nnx = nnx; p->st.nnz = nnz; p->st.npd = npd; p->st.variant = d->variant;
    p->st.dtx = (REAL)(dtf / d->dx); p->st.dtz = (REAL)(dtf / d->dz);
    p->st.cx1 = p->cx1; p->st.cx2 = p->cx2; p->st.cz1 = p->cz1; p->st.cz2 = p->cz2;
    p->st.ax1 = p->ax1; p->st.ax2 = p->ax2; p->st.az1 = p->az1; p->st.az2 = p->az2;
    p->st.vp = p->vp; p->st.e2 = p->e2; p->st.d2 = p->d2; p->st.pw = p->pw;
    free(vv); free(ee); free(dd); free(e1); free(d1);
}

/* One forward time step it of the chosen variant.  CPU/MPI: Gaussian source
 * enters after the stress update (CPU_vti2dfd_kernels.c:483-486).  GPU:
 * point source added to P,Q before the velocity update
 * (GPU_vti2dfd_kernels.cu:423-427). */
static void prop2d_step(orc_prop2d *p, int it)
{
    if (p->st.variant == ORC_V_CPU || p->st.variant == ORC_V_MPI) {
        gauss_src2d(p->st.nnz, p->ixs, p->izs, p->amp[it], p->active[it], p->s, p->st.nnx);
        vel2d(&p->st, p->u, p->w, p->P, p->Q);
        stress2d(&p->st, p->u, p->w, p->P, p->Q, p->px, p->pz, p->qx, p->qz, p->s);
    } else {
        if (p->active[it]) {
            size_t id = (size_t)p->ixs * p->st.nnz + p->izs;
            p->P[id] += (REAL)p->amp[it];
            p->Q[id] += (REAL)p->amp[it];
        }
        vel2d(&p->st, p->u, p->w, p->P, p->Q);
        stress2d(&p->st, p->u, p->w, p->P, p->Q, p->px, p->pz, p->qx, p->qz, NULL);
    }
}

/* 2D forward modelling of one shot.  shot (nt*nx, trace-major) receives
 * rec_scale*P at row rec_iz; snap (optional) receives the padded P every
 * `snap_every` steps (CPU_vti2dfd_kernels.c:488-506).  Returns 0. */
int orc_fd2d(const orc_fd2d_desc *d, const float *v, const float *e, const float *dl,
             float *shot, float *snap, int snap_every)
{
    orc_prop2d p;
    int it, ix, nnz = d->nz + 2 * d->npd;
    size_t n = (size_t)(d->nx + 2 * d->npd) * nnz;
    prop2d_init(&p, d, v, e, dl, d->variant == ORC_V_MPI ? 1 : d->sv);
    for (it = 0; it < d->nt; it++) {
        prop2d_step(&p, it);
        for (ix = 0; ix < d->nx; ix++) {
            REAL val = p.P[(size_t)(ix + d->npd) * nnz + d->rec_iz];
            shot[it + (size_t)d->nt * ix] = (d->rec_scale == 2.0f) ? (float)(val + val) : (float)(val * d->rec_scale);
        }
        if (snap && snap_every > 0 && it % snap_every == 0) {
            size_t k; float *dst = snap + (size_t)(it / snap_every) * n;
            for (k = 0; k < n; k++) dst[k] = (float)p.P[k];
        }
    }
    prop2d_free(&p);
    return 0;
}

/* A 2D TTI propagator of the GPU TTI programs: model (padded vp, 1+2eps and
 * sqrtf(1+2del) with and without the SV taper, cosf/sinf of the tilt,
 * x*z-product sponge profiles, source amplitudes) and in-place fields.
 *   theta (degrees) -> theta * (pi/180.0) in double, stored float;
 *   sponge: the TTI forward program's (get_d0 with 10.0, half-cell velocity
 *   profiles; Toa_gpu_2dtti_fd_1orderfunction.cu:186-189, :227-271) or, with
 *   rtm_sponge, the TTI RTM program's (get_d0 with 3.0 and whole-cell
 *   distances for both pairs; Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu:230-233,
 *   :289-320). */
typedef struct { REAL *u, *w, *P, *Q, *px, *pz, *qx, *qz; } orc_ttif;
typedef struct {
    int nnx, nnz; long n, src;
    REAL *vp;
    float *ct, *st, *e2, *d2, *e2t, *d2t;
    float *cx1, *cx2, *ax1, *ax2, *cz1, *cz2, *az1, *az2;
    float dtx, dtz, *amp;
    unsigned char *act;
} orc_ttim;

static void ttif_alloc(orc_ttif *f, long n)
{
    f->u = calloc(n, sizeof(REAL)); f->w = calloc(n, sizeof(REAL)); f->P = calloc(n, sizeof(REAL)); f->Q = calloc(n, sizeof(REAL));
    f->px = calloc(n, sizeof(REAL)); f->pz = calloc(n, sizeof(REAL)); f->qx = calloc(n, sizeof(REAL)); f->qz = calloc(n, sizeof(REAL));
}

static void ttif_free(orc_ttif *f)
{
    free(f->u); free(f->w); free(f->P); free(f->Q); free(f->px); free(f->pz); free(f->qx); free(f->qz);
}

static void ttim_free(orc_ttim *m)
{
    free(m->vp); free(m->ct); free(m->st); free(m->e2); free(m->d2); free(m->e2t); free(m->d2t);
    free(m->cx1); free(m->cx2); free(m->ax1); free(m->ax2); free(m->cz1); free(m->cz2); free(m->az1); free(m->az2);
    free(m->amp); free(m->act);
}

/* cos and sin of the tilt.  The GPU TTI programs evaluate them inside their
 * kernels with the device's cosf/sinf; a CPU cannot reproduce those bit for
 * bit, so the caller may hand over the device's values for the model's
 * nx*nz angles (padded here like the angles); without them the oracle uses
 * the host's cosf/sinf. */
static const float *g_tilt_cos, *g_tilt_sin;

void orc_set_tilt_trig(const float *ct, const float *st)
{
    g_tilt_cos = ct;
    g_tilt_sin = st;
}

/* The GPU RTM programs' angle-gather weight cosf(ia*pi/180) (pi =
 * 3.141592653), which their Poynting_Adcigs kernels evaluate with the
 * device's cosf: for some bins it differs from the host's cosf in the last
 * place, so the caller may hand over the device's values (ia < 128);
 * without them the host's cosf. */
static const float *g_angle_cos;

void orc_set_angle_cos(const float *tab)
{
    g_angle_cos = tab;
}

static float gpu_angle_cos(int ia)
{
    return g_angle_cos ? g_angle_cos[ia] : cosf(ia * PI_GUI / 180.0);
}

/* Their angle bin (int)((float)(0.5*acosf(a)*180/pi) / (da*1.0)) of a
 * cosine a in [-1, 1], likewise with the device's acosf: the host's acosf
 * can put a cosine next to a bin edge in the neighbouring bin, so the
 * caller may hand over the device's bin edges for the call's da (thr[k] =
 * largest float whose device bin is >= k+1, -2 where none, k < 128); the
 * bin is then the number of edges at or above a. */
static const float *g_angle_thr;

void orc_set_angle_thresholds(const float *thr)
{
    g_angle_thr = thr;
}

static int gpu_angle_bin(float a, int da)
{
    if (g_angle_thr) {
        int c = 0;
        while (c < 128 && a <= g_angle_thr[c]) c++;
        return c;
    }
    a = 0.5 * acosf(a) * 180.0 / PI_GUI;
    return (int)(a / (da * 1.0));
}

/* taper_R, taper_r: SV taper of e2t/d2t centred (fs+(is-1)ds+npd, zs+npd) (0: none) */
static void ttim_init(orc_ttim *m, const orc_fd2d_desc *d, const float *v, const float *e, const float *dl,
                      const float *theta, int rtm_sponge, int taper_R, int taper_r)
{
    const int nx = d->nx, nz = d->nz, npd = d->npd, nt = d->nt;
    const int nnx = nx + 2 * npd, nnz = nz + 2 * npd;
    const long n = (long)nnx * nnz;
    long id, ix, iz;
    REAL *ee = calloc(n, sizeof(REAL)), *dd = calloc(n, sizeof(REAL)), *th = calloc(n, sizeof(REAL));
    m->nnx = nnx; m->nnz = nnz; m->n = n;
    m->vp = calloc(n, sizeof(REAL));
    m->ct = malloc(n * 4); m->st = malloc(n * 4); m->e2 = malloc(n * 4); m->d2 = malloc(n * 4);
    m->e2t = malloc(n * 4); m->d2t = malloc(n * 4);
    m->cx1 = malloc(nnx * 4); m->cx2 = malloc(nnx * 4); m->ax1 = malloc(nnx * 4); m->ax2 = malloc(nnx * 4);
    m->cz1 = malloc(nnz * 4); m->cz2 = malloc(nnz * 4); m->az1 = malloc(nnz * 4); m->az2 = malloc(nnz * 4);
    m->amp = malloc(nt * 4); m->act = malloc(nt);
    for (ix = 0; ix < nx; ix++)
        for (iz = 0; iz < nz; iz++) {
            id = (ix + npd) * nnz + iz + npd;
            m->vp[id] = v[ix * nz + iz]; ee[id] = e[ix * nz + iz]; dd[id] = dl[ix * nz + iz];
            th[id] = (float)((double)theta[ix * nz + iz] * (PI_GUI / 180.0));
        }
    orc_pad2d(nx, nz, npd, m->vp); orc_pad2d(nx, nz, npd, ee); orc_pad2d(nx, nz, npd, dd); orc_pad2d(nx, nz, npd, th);
    REAL *tc = NULL, *ts = NULL;
    if (g_tilt_cos && g_tilt_sin) {
        tc = calloc(n, sizeof(REAL));
        ts = calloc(n, sizeof(REAL));
        for (ix = 0; ix < nx; ix++)
            for (iz = 0; iz < nz; iz++) {
                id = (ix + npd) * nnz + iz + npd;
                tc[id] = g_tilt_cos[ix * nz + iz];
                ts[id] = g_tilt_sin[ix * nz + iz];
            }
        orc_pad2d(nx, nz, npd, tc);
        orc_pad2d(nx, nz, npd, ts);
    }
    {
        const float fsx = d->fs + (d->is - 1) * d->ds;
        const int ixs = (int)(fsx + 0.5f) + npd - 1, izs = (int)(d->zs + 0.5f) + npd - 1;
        const double k0 = rtm_sponge ? 3.0 : 10.0;
        const float d0 = (float)(k0 * (float)m->vp[n / 2] * log(100000.0) / (2.0 * npd * ((d->dx + d->dz) / 2.0)));
        const int cx = (int)d->fs + (d->is - 1) * (int)d->ds + npd, cz = (int)d->zs + npd;
        m->src = (long)ixs * nnz + izs;
        for (id = 0; id < n; id++) {
            float thf = (float)th[id], te = (float)ee[id], td = (float)dd[id];
            m->e2[id] = 1 + 2 * te;
            m->d2[id] = sqrtf(1 + 2 * td);
            m->ct[id] = tc ? (float)tc[id] : cosf(thf);
            m->st[id] = ts ? (float)ts[id] : sinf(thf);
            ix = id / nnz; iz = id % nnz;
            if (taper_R > 0) {
                int rx = (int)ix - cx, rz = (int)iz - cz;
                if ((rx * rx + rz * rz) <= taper_R * taper_R) {
                    if ((rx * rx + rz * rz) <= taper_r * taper_r) { te = 0.0f; td = 0.0f; }
                    else {
                        double g = 0.5 * (1 - cos(PI_GUI * ((sqrtf((float)(rx * rx + rz * rz)) - taper_r) * 4.0 / (taper_R * 3.0 - 1))));
                        te = (float)(g * te);
                        td = (float)(g * td);
                    }
                }
            }
            m->e2t[id] = 1 + 2 * te;
            m->d2t[id] = sqrtf(1 + 2 * td);
        }
        if (rtm_sponge) {
            /* integer-cell distance for both pairs, far side (i-n-npd)/npd */
            int i, k;
            for (k = 0; k < 2; k++) {
                int nn = k ? nz : nx, nnn = nn + 2 * npd;
                float *c1 = k ? m->cz1 : m->cx1, *c2 = k ? m->cz2 : m->cx2, *a1 = k ? m->az1 : m->ax1, *a2 = k ? m->az2 : m->ax2;
                for (i = 0; i < nnn; i++) {
                    double q;
                    if (i < npd) q = (npd - i) * 1.0 / npd;
                    else if (i >= npd + nn) q = (i - nn - npd) * 1.0 / npd;
                    else { c1[i] = c2[i] = a1[i] = a2[i] = 1.0f; continue; }
                    c1[i] = (float)(1.0 / (1.0 + (d->dt * d0 * pow(q, 2.0)) / 2.0));
                    c2[i] = (float)(c1[i] * (1.0 - (d->dt * d0 * pow(q, 2.0)) / 2.0));
                    a1[i] = c1[i];
                    a2[i] = c2[i];
                }
            }
        } else {
            orc_sponge(ORC_V_GPU, nx, npd, d->dt, d0, m->cx1, m->cx2, m->ax1, m->ax2);
            orc_sponge(ORC_V_GPU, nz, npd, d->dt, d0, m->cz1, m->cz2, m->az1, m->az2);
        }
        orc_source_amp(ORC_V_GPU, nt, d->dt, d->favg, d->pfac, d->wtype, m->amp, m->act);
        m->dtx = d->dt / d->dx;
        m->dtz = d->dt / d->dz;
    }
    free(ee); free(dd); free(th); free(tc); free(ts);
}

/* update_vel then update_stress, in place, with e2/d2 (tapered or not) */
static void tti_step(const orc_ttim *m, orc_ttif *f, const float *e2, const float *d2)
{
    const int nnx = m->nnx, nnz = m->nnz;
    const long s = nnz;
    const float dtx = m->dtx, dtz = m->dtz;
    REAL *u = f->u, *w = f->w, *P = f->P, *Q = f->Q;
    long id, ix, iz;
    int im;
    for (ix = 4; ix < nnx - 4; ix++)
        for (iz = 4; iz < nnz - 4; iz++) {
            REAL Px = 0, Pz = 0, Qz = 0, Qx = 0, k1, k2;
            id = ix * nnz + iz;
            for (im = 0; im < 4; im++) {
                Px += C8[im] * (P[id + (im + 1) * s] - P[id - im * s]);
                Pz += C8[im] * (P[id + im + 1] - P[id - im]);
                Qz += C8[im] * (Q[id + im + 1] - Q[id - im]);
                Qx += C8[im] * (Q[id + (im + 1) * s] - Q[id - im * s]);
            }
            k2 = (REAL)m->cx2[ix] * m->cz2[iz];
            k1 = (REAL)m->cx1[ix] * m->cz1[iz];
            u[id] = k2 * u[id] - k1 * ((REAL)m->ct[id] * dtx * Px - (REAL)m->st[id] * dtz * Pz);
            w[id] = k2 * w[id] - k1 * ((REAL)m->st[id] * dtx * Qx + (REAL)m->ct[id] * dtz * Qz);
        }
    for (ix = 4; ix < nnx - 4; ix++)
        for (iz = 4; iz < nnz - 4; iz++) {
            REAL ux = 0, uz = 0, wz = 0, wx = 0, A, B, k1, k2, a, b, c_, e_;
            const REAL *vp = m->vp;
            id = ix * nnz + iz;
            for (im = 0; im < 4; im++) {
                ux += C8[im] * (u[id + im * s] - u[id - (im + 1) * s]);
                uz += C8[im] * (u[id + im] - u[id - im - 1]);
                wz += C8[im] * (w[id + im] - w[id - im - 1]);
                wx += C8[im] * (w[id + im * s] - w[id - (im + 1) * s]);
            }
            A = (REAL)m->ct[id] * dtx * ux - (REAL)m->st[id] * dtz * uz;
            B = (REAL)m->st[id] * dtx * wx + (REAL)m->ct[id] * dtz * wz;
            k2 = (REAL)m->ax2[ix] * m->az2[iz];
            k1 = (REAL)m->ax1[ix] * m->az1[iz];
            a = k2 * f->px[id] - k1 * vp[id] * vp[id] * e2[id] * A;
            b = k2 * f->pz[id] - k1 * vp[id] * vp[id] * d2[id] * B;
            c_ = k2 * f->qx[id] - k1 * vp[id] * vp[id] * d2[id] * A;
            e_ = k2 * f->qz[id] - k1 * vp[id] * vp[id] * B;
            f->px[id] = a; f->pz[id] = b; f->qx[id] = c_; f->qz[id] = e_;
            P[id] = a + b;
            Q[id] = c_ + e_;
        }
}

/* 2D TTI forward modelling with the GPU TTI program's semantics
 * (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu):
 *   theta (degrees) -> theta * (pi/180.0) in double, stored float (:235);
 *   d0 from the padded centre velocity (get_d0 :186-189), GPU-form sponge
 *   profiles (initial_coffe :227-271) applied as x*z products;
 *   point source P,Q += pfac*w(t) before the velocity update (:47-79),
 *   t from dt by float accumulation;
 *   update_vel (:81-112) and update_stress (:114-183) in place (the program's
 *   u0 = u1 pointer assignment leaves one buffer per field);
 *   record P at row rec_iz after each step; padded-P snapshots at it =
 *   snap_every, 2 snap_every, ... (:451-456);
 *   optional SV taper of the GPU form (R=15, r=4, centre one cell
 *   right/down of the source cell).
 * cos/sin of the tilt: cosf/sinf of the float angle. */
int orc_tti2d(const orc_fd2d_desc *d, const float *v, const float *e, const float *dl, const float *theta,
              float *shot, float *snaps, int snap_every)
{
    const int nx = d->nx, npd = d->npd, nt = d->nt;
    orc_ttim m;
    orc_ttif f;
    long id;
    int it, ix;
    ttim_init(&m, d, v, e, dl, theta, 0, d->sv ? 15 : 0, 4);
    ttif_alloc(&f, m.n);
    for (it = 0; it < nt; it++) {
        if (m.act[it]) { f.P[m.src] += m.amp[it]; f.Q[m.src] += m.amp[it]; }
        tti_step(&m, &f, m.e2t, m.d2t);
        for (ix = 0; ix < nx; ix++) shot[it + (long)nt * ix] = (float)f.P[d->rec_iz + (long)m.nnz * (ix + npd)];
        if (snaps && snap_every > 0 && it % snap_every == 0 && it != 0)
            for (id = 0; id < m.n; id++) snaps[(long)(it / snap_every - 1) * m.n + id] = (float)f.P[id];
    }
    ttif_free(&f);
    ttim_free(&m);
    return 0;
}

/* Direct-wave mute of a (nx traces x nt) record.
 *  GPU form (GPU_vti2dfd_kernels.cu:151-174): zero (t0/dt - tt, t0/dt+2/(dt f)+tt)
 *    with t0 = offset/(vp[1]*sqrt(1+2 eps[1])) from the padded model;
 *  MPI form (Toa_rtm_vti_adcig_cdp.c:1587-1605): zero [0, mu_nt), dt in ms. */
void orc_mute2d(int form, int nx, int nt, float dt, float favg, float dx, float dz,
                int fs, int ds, int zs, int is, float mu_v, int tt, float *shot)
{
    int ix, it;
    for (ix = 0; ix < nx; ix++) {
        if (form == 0) { /* GPU */
            float mu_x = dx * abs(ix - fs - (is - 1) * ds), mu_z = dz * zs;
            float mu_t0 = sqrtf((float)(pow(mu_x, 2) + pow(mu_z, 2))) / mu_v;
            int mu_t = (int)(2.0 / (dt * favg));
            int mu_nt = (int)(mu_t0 / dt) + mu_t + tt;
            for (it = 0; it < nt; it++)
                if ((it > (int)(mu_t0 / dt) - tt) && it < mu_nt) shot[ix * nt + it] = 0.0f;
        } else {        /* MPI, dt in ms */
            float mu_x = dx * abs(ix - fs - (is - 1) * ds), mu_z = dz * zs;
            float mu_t0 = sqrtf((float)(pow(mu_x, 2) + pow(mu_z, 2))) / mu_v;
            int mu_t = (int)(2.0 / (dt / 1000 * favg));
            int mu_nt = (int)(mu_t0 / dt * 1000) + mu_t + tt;
            for (it = 0; it < mu_nt && it < nt; it++) shot[ix * nt + it] = 0.0f;
        }
    }
}

/* ------------------------------------------------------------ 2D RTM */

/* One shot of the MPI CPU RTM (model_vti_get_boundry + RTM_corr_adcig,
 * Toa_rtm_vti_adcig_cdp.c:483-737, 739-1139, driven as main() drives them
 * :295-392) on the shot's aperture window:
 *   nxs  odd window width; the window is centred on k = fs_sxd+(is-1)*ds_sxd
 *        (1-based), window column c <-> padded global column npd+c+k-nxs/2;
 *   forward with Gaussian source, SV taper always on (CR=15), receivers
 *        txx,tzz at row npd+hsx-1 (hsx=1) and the four interior-edge lines;
 *   mute both records (tt=285);
 *   backward from a zero state: inject saved edges into s_txx0/s_tzz0,
 *        vel + inv_update_stress; inject the muted records into g_*0 at
 *        row npd, vel + inv_update_stress; image mig += g_txx*s_txx and
 *        source_x = (float)((double)source_x + pow(s_txx,2)), 0 -> 1;
 *   mig /= source_x.
 * Output: mig_is (nxs*nz, x-major) and the stacking offset of column 0 in the
 * full image (the reference adds column c at c + k - nxs/2 - 1, :1102-1104).
 * The full model is nx*nz unpadded. */
int orc_rtm2d_mpi_shot(int nx, int nz, int npd, int nt, float dx, float dz, float dt_ms,
                       float favg, float pfac, int fs_sxd, int ds_sxd, int zs_sxd, int is, int nxs,
                       const float *v, const float *e, const float *dl,
                       float *mig_is, int *stack_offset, float *p_cal_x_out, float *adcig_is)
{
    int nnzs = nz + 2 * npd, nnxs = nxs + 2 * npd, k = fs_sxd + (is - 1) * ds_sxd;
    int c, iz, it, i, j;
    float *vs = malloc((size_t)nxs * nz * 4), *es = malloc((size_t)nxs * nz * 4), *ds_ = malloc((size_t)nxs * nz * 4);
    /* padded full model to read the window from (edge replicated) */
    int nnx = nx + 2 * npd;
    REAL *vfull = calloc((size_t)nnx * nnzs, sizeof(REAL)), *efull = calloc((size_t)nnx * nnzs, sizeof(REAL)),
         *dfull = calloc((size_t)nnx * nnzs, sizeof(REAL));
    for (i = 0; i < nx; i++) for (j = 0; j < nz; j++) {
        size_t id = (size_t)(i + npd) * nnzs + j + npd;
        vfull[id] = v[i * nz + j]; efull[id] = e[i * nz + j]; dfull[id] = dl[i * nz + j];
    }
    orc_pad2d(nx, nz, npd, vfull); orc_pad2d(nx, nz, npd, efull); orc_pad2d(nx, nz, npd, dfull);
    for (c = 0; c < nxs; c++) for (iz = 0; iz < nz; iz++) {
        size_t g = (size_t)(npd + c + k - nxs / 2) * nnzs + iz + npd;
        vs[c * nz + iz] = (float)vfull[g]; es[c * nz + iz] = (float)efull[g]; ds_[c * nz + iz] = (float)dfull[g];
    }
    free(vfull); free(efull); free(dfull);

    orc_fd2d_desc d;
    memset(&d, 0, sizeof d);
    d.nx = nxs; d.nz = nz; d.npd = npd; d.nt = nt; d.variant = ORC_V_MPI; d.sv = 1; d.wtype = 1;
    d.dx = dx; d.dz = dz; d.dt = dt_ms / 1000; d.favg = favg; d.pfac = pfac;
    d.fs = (float)(nxs / 2 + 1); d.ds = 0; d.zs = (float)zs_sxd; d.is = is;

    orc_prop2d fw, sr, rc;
    prop2d_init(&fw, &d, vs, es, ds_, 1);
    float mu_v = (float)(vs[1 * nz + 1] * sqrtf((1 + 2 * es[1 * nz + 1])));
    size_t ntx = (size_t)nt * nxs, ntz = (size_t)nt * nz;
    float *pcx = calloc(ntx, 4), *pcz = calloc(ntx, 4), *tx = calloc(ntx, 4), *bx = calloc(ntx, 4),
          *tz = calloc(ntx, 4), *bz = calloc(ntx, 4), *lx = calloc(ntz, 4), *rx = calloc(ntz, 4),
          *lz = calloc(ntz, 4), *rz = calloc(ntz, 4);
    for (it = 0; it < nt; it++) {
        prop2d_step(&fw, it);
        for (i = npd; i < npd + nxs; i++) {
            size_t col = (size_t)i * nnzs;
            pcx[(size_t)(i - npd) * nt + it] = (float)fw.P[col + npd];
            pcz[(size_t)(i - npd) * nt + it] = (float)fw.Q[col + npd];
            tx[(size_t)(i - npd) * nt + it] = (float)fw.P[col + npd];
            bx[(size_t)(i - npd) * nt + it] = (float)fw.P[col + npd + nz - 1];
            tz[(size_t)(i - npd) * nt + it] = (float)fw.Q[col + npd];
            bz[(size_t)(i - npd) * nt + it] = (float)fw.Q[col + npd + nz - 1];
        }
        for (j = npd; j < npd + nz; j++) {
            lx[(size_t)(j - npd) * nt + it] = (float)fw.P[(size_t)npd * nnzs + j];
            rx[(size_t)(j - npd) * nt + it] = (float)fw.P[(size_t)(npd + nxs - 1) * nnzs + j];
            lz[(size_t)(j - npd) * nt + it] = (float)fw.Q[(size_t)npd * nnzs + j];
            rz[(size_t)(j - npd) * nt + it] = (float)fw.Q[(size_t)(npd + nxs - 1) * nnzs + j];
        }
    }
    prop2d_free(&fw);
    orc_mute2d(1, nxs, nt, dt_ms, favg, dx, dz, nxs / 2 + 1, 0, zs_sxd, is, mu_v, 285, pcx);
    orc_mute2d(1, nxs, nt, dt_ms, favg, dx, dz, nxs / 2 + 1, 0, zs_sxd, is, mu_v, 285, pcz);
    if (p_cal_x_out) memcpy(p_cal_x_out, pcx, ntx * 4);

    /* backward: both passes use the untapered model (inv_update_stress) */
    prop2d_init(&sr, &d, vs, es, ds_, 0);
    prop2d_init(&rc, &d, vs, es, ds_, 0);
    float *srcx = calloc((size_t)nxs * nz, 4);
    memset(mig_is, 0, (size_t)nxs * nz * 4);
    if (adcig_is) memset(adcig_is, 0, (size_t)90 * nxs * nz * 4);
    for (it = nt - 1; it >= 0; it--) {
        for (i = 0; i < nxs; i++) {
            sr.P[(size_t)(npd + i) * nnzs + npd] = (REAL)tx[(size_t)i * nt + it];
            sr.P[(size_t)(npd + i) * nnzs + npd + nz - 1] = (REAL)bx[(size_t)i * nt + it];
            sr.Q[(size_t)(npd + i) * nnzs + npd] = (REAL)tz[(size_t)i * nt + it];
            sr.Q[(size_t)(npd + i) * nnzs + npd + nz - 1] = (REAL)bz[(size_t)i * nt + it];
        }
        for (j = 0; j < nz; j++) {
            sr.P[(size_t)npd * nnzs + npd + j] = (REAL)lx[(size_t)j * nt + it];
            sr.P[(size_t)(npd + nxs - 1) * nnzs + npd + j] = (REAL)rx[(size_t)j * nt + it];
            sr.Q[(size_t)npd * nnzs + npd + j] = (REAL)lz[(size_t)j * nt + it];
            sr.Q[(size_t)(npd + nxs - 1) * nnzs + npd + j] = (REAL)rz[(size_t)j * nt + it];
        }
        vel2d(&sr.st, sr.u, sr.w, sr.P, sr.Q);
        stress2d(&sr.st, sr.u, sr.w, sr.P, sr.Q, sr.px, sr.pz, sr.qx, sr.qz, NULL);
        for (i = 0; i < nxs; i++) {
            rc.P[(size_t)(npd + i) * nnzs + npd] = (REAL)pcx[(size_t)i * nt + it];
            rc.Q[(size_t)(npd + i) * nnzs + npd] = (REAL)pcz[(size_t)i * nt + it];
        }
        vel2d(&rc.st, rc.u, rc.w, rc.P, rc.Q);
        stress2d(&rc.st, rc.u, rc.w, rc.P, rc.Q, rc.px, rc.pz, rc.qx, rc.qz, NULL);
        for (i = npd; i < nxs + npd; i++)
            for (j = npd; j < nz + npd; j++) {
                size_t id = (size_t)i * nnzs + j, o = (size_t)(i - npd) * nz + (j - npd);
                REAL sv = sr.P[id];
                if (adcig_is) {
                    /* Poynting ADCIG (flag_adcig = 1, :1004-1068): opening
                     * angle of -sP*u_s, -sQ*w_s and gP*u_g, gQ*w_g */
                    float sx = -(float)sr.P[id] * (float)sr.u[id], sz = -(float)sr.Q[id] * (float)sr.w[id];
                    float gx = (float)rc.P[id] * (float)rc.u[id], gz = (float)rc.Q[id] * (float)rc.w[id];
                    float b1 = sx * sx + sz * sz, b2 = gx * gx + gz * gz, a = sx * gx + sz * gz;
                    float a1 = (float)(a / (sqrtf(b1 * b2) + 0.0000000000001)), a2;
                    int ia = 0;
                    if (a1 >= -1 && a1 <= 1) {
                        a2 = (float)(0.5 * acosf(a1) * 180 / PI_MPI);
                        ia = (int)(a2 / 1.0);
                        if (ia == 90) ia -= 1;
                    }
                    float *ag = adcig_is + (size_t)ia * nxs * nz + o;
                    *ag = (float)(*ag + (double)((float)rc.P[id] * (float)sv) * pow(cos(ia * PI_MPI / 180.0), 3));
                }
                srcx[o] = (float)((double)srcx[o] + pow((double)sv, 2));
                if (srcx[o] == 0) srcx[o] = 1.0f;
                mig_is[o] = (float)(mig_is[o] + (REAL)rc.P[id] * sv);
            }
    }
    for (size_t o = 0; o < (size_t)nxs * nz; o++) mig_is[o] = mig_is[o] / srcx[o];
    if (adcig_is)
        for (size_t q = 0; q < (size_t)90 * nxs * nz; q++) adcig_is[q] = adcig_is[q] / srcx[q % ((size_t)nxs * nz)];
    *stack_offset = k - nxs / 2 - 1;
    prop2d_free(&sr); prop2d_free(&rc);
    free(srcx); free(pcx); free(pcz); free(tx); free(bx); free(tz); free(bz); free(lx); free(rx); free(lz); free(rz);
    free(vs); free(es); free(ds_);
    return 0;
}

/* 2D RTM with the 2D GPU RTM program's semantics
 * (2D-vti-fd+rtm-cuda/Toa_gpu2DvtiFdRtmAdcigsLaplace.cu, RTM() :1184-1566):
 * per shot (is = 1..ns) forward with the GPU source and the R=18, r=7 SV
 * taper, record P at row npml, ring of P,Q (rows npml-1, npml+nz+1,
 * columns npml-1, npml+nx+1; wavefield_bndr :532-612), illumination
 * ill += P*P + Q*Q then <= 0 -> 1 (:654-677); mute (:614-652, tt, with the
 * surplus threads of its launch zeroing flat samples past nt); obs (optional)
 * replaces the record; backward: ring restore + untapered step of the source
 * field, record into P,Q of the receiver field at row npml + step, image
 * += sP*gP (:679-698) and Poynting gathers (:718-766, acosf, cosf^3).
 * After all shots mig /= ill and gathers /= ill; the caller filters.
 * mig, ill: nx*nz; adcigs (optional): nx*nangle*nz [ix][ia][iz];
 * shots (optional): the muted modelled records ns*nx*nt. */
int orc_rtm2d_gpu(int nx, int nz, int npml, int nt, float dx, float dz, float dt, float favg, float pfac,
                  int wtype, int ns, int fs, int ds, int zs, int mute_tt, int nangle, int dangle,
                  const float *v, const float *e, const float *dl, const float *obs,
                  float *mig, float *ill, float *adcigs, float *shots)
{
    const int nnx = nx + 2 * npml, nnz = nz + 2 * npml, L = 2 * nx + 2 * nz;
    const size_t n = (size_t)nnx * nnz, n0 = (size_t)nx * nz;
    int is, it, ix, iz, k;
    float *rec = calloc((size_t)nt * nx, 4), *bp = calloc((size_t)nt * L, 4), *bq = calloc((size_t)nt * L, 4);
    memset(mig, 0, n0 * 4);
    memset(ill, 0, n0 * 4);
    if (adcigs) memset(adcigs, 0, n0 * nangle * 4);
    for (is = 1; is <= ns; is++) {
        orc_fd2d_desc d;
        orc_prop2d fw, sb, rc;
        memset(&d, 0, sizeof d);
        d.nx = nx; d.nz = nz; d.npd = npml; d.nt = nt; d.variant = ORC_V_GPURTM; d.sv = 1; d.wtype = wtype;
        d.dx = dx; d.dz = dz; d.dt = dt; d.favg = favg; d.pfac = pfac;
        d.fs = (float)fs; d.ds = (float)ds; d.zs = (float)zs; d.is = is;
        prop2d_init(&fw, &d, v, e, dl, 1);
        for (it = 0; it < nt; it++) {
            prop2d_step(&fw, it);
            for (ix = 0; ix < nx; ix++) rec[(size_t)ix * nt + it] = (float)fw.P[npml + (size_t)nnz * (ix + npml)];
            for (k = 0; k < L; k++) {
                size_t id;
                if (k < nx) id = npml - 1 + (size_t)nnz * (k + npml);
                else if (k < 2 * nx) id = npml + nz + 1 + (size_t)nnz * (k - nx + npml);
                else if (k < 2 * nx + nz) id = k - 2 * nx + npml + (size_t)nnz * (npml - 1);
                else id = k - 2 * nx - nz + npml + (size_t)nnz * (npml + nx + 1);
                bp[(size_t)it * L + k] = (float)fw.P[id];
                bq[(size_t)it * L + k] = (float)fw.Q[id];
            }
            for (ix = 0; ix < nx; ix++)
                for (iz = 0; iz < nz; iz++) {
                    size_t id = iz + npml + (size_t)nnz * (ix + npml), o = (size_t)ix * nz + iz;
                    float pp = (float)fw.P[id], qq = (float)fw.Q[id];
                    ill[o] += pp * pp + qq * qq;
                    if (ill[o] <= 0.0f) ill[o] = 1.0f;
                }
        }
        {
            /* mute_directwave: one thread per sample it < roundup(nt, 512), all traces */
            const float mu_v = (float)fw.vp[1] * sqrtf((float)(1 + 2 * e[0]));
            const int nt512 = (nt + 511) / 512 * 512;
            for (ix = 0; ix < nx; ix++) {
                float mu_x = dx * abs(ix - fs - (is - 1) * ds), mu_z = dz * zs;
                float mu_t0 = sqrtf((float)(pow(mu_x, 2) + pow(mu_z, 2))) / mu_v;
                int mu_t = (int)(2.0 / (dt * favg));
                int mu_nt = (int)(mu_t0 / dt) + mu_t + mute_tt;
                for (it = 0; it < nt512; it++)
                    if ((it > (int)(mu_t0 / dt) - mute_tt) && (it < mu_nt)) {
                        long j = (long)ix * nt + it;
                        if (j < (long)nx * nt) rec[j] = 0.0f;
                    }
            }
        }
        if (shots) memcpy(shots + (size_t)(is - 1) * nx * nt, rec, (size_t)nx * nt * 4);
        if (obs) memcpy(rec, obs + (size_t)(is - 1) * nx * nt, (size_t)nx * nt * 4);
        prop2d_init(&sb, &d, v, e, dl, 0);
        prop2d_init(&rc, &d, v, e, dl, 0);
        memcpy(sb.u, fw.u, n * sizeof(REAL)); memcpy(sb.w, fw.w, n * sizeof(REAL));
        memcpy(sb.P, fw.P, n * sizeof(REAL)); memcpy(sb.Q, fw.Q, n * sizeof(REAL));
        memcpy(sb.px, fw.px, n * sizeof(REAL)); memcpy(sb.pz, fw.pz, n * sizeof(REAL));
        memcpy(sb.qx, fw.qx, n * sizeof(REAL)); memcpy(sb.qz, fw.qz, n * sizeof(REAL));
        prop2d_free(&fw);
        for (it = nt - 1; it >= 0; it--) {
            for (k = 0; k < L; k++) {
                size_t id;
                if (k < nx) id = npml - 1 + (size_t)nnz * (k + npml);
                else if (k < 2 * nx) id = npml + nz + 1 + (size_t)nnz * (k - nx + npml);
                else if (k < 2 * nx + nz) id = k - 2 * nx + npml + (size_t)nnz * (npml - 1);
                else id = k - 2 * nx - nz + npml + (size_t)nnz * (npml + nx + 1);
                sb.P[id] = (REAL)bp[(size_t)it * L + k];
                sb.Q[id] = (REAL)bq[(size_t)it * L + k];
            }
            vel2d(&sb.st, sb.u, sb.w, sb.P, sb.Q);
            stress2d(&sb.st, sb.u, sb.w, sb.P, sb.Q, sb.px, sb.pz, sb.qx, sb.qz, NULL);
            for (ix = 0; ix < nx; ix++) {
                size_t id = npml + (size_t)nnz * (ix + npml);
                rc.P[id] = rc.Q[id] = (REAL)rec[(size_t)ix * nt + it];
            }
            vel2d(&rc.st, rc.u, rc.w, rc.P, rc.Q);
            stress2d(&rc.st, rc.u, rc.w, rc.P, rc.Q, rc.px, rc.pz, rc.qx, rc.qz, NULL);
            for (ix = 0; ix < nx; ix++)
                for (iz = 0; iz < nz; iz++) {
                    size_t id = iz + npml + (size_t)nnz * (ix + npml), o = (size_t)ix * nz + iz;
                    float sP = (float)sb.P[id], gP = (float)rc.P[id];
                    mig[o] += sP * gP;
                    if (adcigs) {
                        float Ssx = -sP * (float)sb.u[id], Ssz = -(float)sb.Q[id] * (float)sb.w[id];
                        float Sgx = gP * (float)rc.u[id], Sgz = (float)rc.Q[id] * (float)rc.w[id];
                        float b1 = Ssx * Ssx + Ssz * Ssz, b2 = Sgx * Sgx + Sgz * Sgz;
                        float a = (Ssx * Sgx + Ssz * Sgz) / (sqrtf(b1 * b2) * (1 - 0.1));
                        if (a >= -1 && a <= 1) {
                            int ia;
                            ia = gpu_angle_bin(a, dangle);
                            if (ia < nangle) {
                                float c = gpu_angle_cos(ia);
                                adcigs[iz + (size_t)nz * ia + (size_t)nz * nangle * ix] += sP * gP * c * c * c;
                            }
                        }
                    }
                }
        }
        prop2d_free(&sb); prop2d_free(&rc);
    }
    for (size_t o = 0; o < n0; o++) mig[o] /= ill[o];
    if (adcigs)
        for (size_t q = 0; q < n0 * nangle; q++) {
            size_t ixq = q / ((size_t)nz * nangle), izq = q % nz;
            adcigs[q] /= ill[izq + (size_t)nz * ixq];
        }
    free(rec); free(bp); free(bq);
    return 0;
}

/* 2D TTI RTM with the 2D TTI GPU RTM program's semantics
 * (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu, main
 * :500-800), shots is = 1..ns at fs + (is-1)*ds:
 *   forward: point source, TTI step with the SV taper (R=15, r=4), record P
 *     at row npml, ring of P,Q (rows npml-1, npml+nz+1, columns npml-1,
 *     npml+nx+1; wavefield_bndr :360-416), illumination ill += P*P + Q*Q,
 *     == 0 -> 1 (:430-442);
 *   mute (:336-358): zero (t0/dt - tt, t0/dt + 2/(dt f) + tt) with
 *     t0 = offset / (vp[1]*(1+(sqrtf(1+2 eps[1])-1)*cos(theta[1])));
 *   obs (optional) replaces the record;
 *   backward: ring restore + untapered step of the source field, record
 *     into P and Q of the receiver field at row npml + step, image
 *     += sP*gP (:418-428), Poynting gathers at ix = 0, dcdp, 2 dcdp, ...
 *     (:454-486).
 * After the shots mig /= ill and gathers /= ill (:444-452, :488-498); the
 * caller filters.  The model uses the RTM program's sponge (ttim_init with
 * rtm_sponge).  mig, ill: nx*nz; adcigs (optional): (nx/dcdp)*nangle*nz;
 * shots (optional): the muted records ns*nx*nt. */
int orc_rtm2d_tti(int nx, int nz, int npml, int nt, float dx, float dz, float dt, float favg, float pfac,
                  int wtype, int ns, int fs, int ds, int zs, int mute_tt, int nangle, int dangle, int dcdp,
                  const float *v, const float *e, const float *dl, const float *theta, const float *obs,
                  float *mig, float *ill, float *adcigs, float *shots)
{
    const int nnz = nz + 2 * npml, L = 2 * nx + 2 * nz, nxa = nx / dcdp;
    const size_t n0 = (size_t)nx * nz;
    int is, it, ix, iz, k;
    float *rec = calloc((size_t)nt * nx, 4), *bp = calloc((size_t)nt * L, 4), *bq = calloc((size_t)nt * L, 4);
    memset(mig, 0, n0 * 4);
    memset(ill, 0, n0 * 4);
    if (adcigs) memset(adcigs, 0, (size_t)nxa * nangle * nz * 4);
    for (is = 1; is <= ns; is++) {
        orc_fd2d_desc d;
        orc_ttim m;
        orc_ttif S, R;
        memset(&d, 0, sizeof d);
        d.nx = nx; d.nz = nz; d.npd = npml; d.nt = nt; d.variant = ORC_V_GPU; d.sv = 1; d.wtype = wtype;
        d.dx = dx; d.dz = dz; d.dt = dt; d.favg = favg; d.pfac = pfac;
        d.fs = (float)fs; d.ds = (float)ds; d.zs = (float)zs; d.is = is;
        ttim_init(&m, &d, v, e, dl, theta, 1, 15, 4);
        ttif_alloc(&S, m.n);
        ttif_alloc(&R, m.n);
#define RING_ID(k) ((k) < nx ? npml - 1 + (size_t)nnz * ((k) + npml) \
                 : (k) < 2 * nx ? npml + nz + 1 + (size_t)nnz * ((k) - nx + npml) \
                 : (k) < 2 * nx + nz ? (k) - 2 * nx + npml + (size_t)nnz * (npml - 1) \
                 : (k) - 2 * nx - nz + npml + (size_t)nnz * (npml + nx + 1))
        memset(rec, 0, (size_t)nt * nx * 4);
        for (it = 0; it < nt; it++) {
            if (m.act[it]) { S.P[m.src] += m.amp[it]; S.Q[m.src] += m.amp[it]; }
            tti_step(&m, &S, m.e2t, m.d2t);
            for (ix = 0; ix < nx; ix++) rec[(size_t)ix * nt + it] = (float)S.P[npml + (size_t)nnz * (ix + npml)];
            for (k = 0; k < L; k++) {
                bp[(size_t)it * L + k] = (float)S.P[RING_ID(k)];
                bq[(size_t)it * L + k] = (float)S.Q[RING_ID(k)];
            }
            for (ix = 0; ix < nx; ix++)
                for (iz = 0; iz < nz; iz++) {
                    size_t id = iz + npml + (size_t)nnz * (ix + npml), o = (size_t)ix * nz + iz;
                    float pp = (float)S.P[id], qq = (float)S.Q[id];
                    ill[o] += pp * pp + qq * qq;
                    if (ill[o] == 0.0f) ill[o] = 1.0f;
                }
        }
        {
            const float mu_v = (float)m.vp[1] * (1 + (sqrtf(1 + 2 * e[0]) - 1) * m.ct[1]);
            for (ix = 0; ix < nx; ix++) {
                float mu_x = dx * abs(ix - fs - (is - 1) * ds), mu_z = dz * zs;
                float mu_t0 = sqrtf((float)(pow(mu_x, 2) + pow(mu_z, 2))) / mu_v;
                int mu_t = (int)(2.0 / (dt * favg));
                int mu_nt = (int)(mu_t0 / dt) + mu_t + mute_tt;
                for (it = 0; it < nt; it++)
                    if ((it > (int)(mu_t0 / dt) - mute_tt) && (it < mu_nt)) rec[(size_t)ix * nt + it] = 0.0f;
            }
        }
        if (shots) memcpy(shots + (size_t)(is - 1) * nx * nt, rec, (size_t)nx * nt * 4);
        if (obs) memcpy(rec, obs + (size_t)(is - 1) * nx * nt, (size_t)nx * nt * 4);
        for (it = nt - 1; it >= 0; it--) {
            for (k = 0; k < L; k++) {
                S.P[RING_ID(k)] = (REAL)bp[(size_t)it * L + k];
                S.Q[RING_ID(k)] = (REAL)bq[(size_t)it * L + k];
            }
            tti_step(&m, &S, m.e2, m.d2);
            for (ix = 0; ix < nx; ix++) {
                size_t id = npml + (size_t)nnz * (ix + npml);
                R.P[id] = R.Q[id] = (REAL)rec[(size_t)ix * nt + it];
            }
            tti_step(&m, &R, m.e2, m.d2);
            for (ix = 0; ix < nx; ix++)
                for (iz = 0; iz < nz; iz++) {
                    size_t id = iz + npml + (size_t)nnz * (ix + npml), o = (size_t)ix * nz + iz;
                    float sP = (float)S.P[id], gP = (float)R.P[id];
                    mig[o] += sP * gP;
                    if (adcigs && ix % dcdp == 0 && ix / dcdp < nxa) {
                        float Ssx = -sP * (float)S.u[id], Ssz = -(float)S.Q[id] * (float)S.w[id];
                        float Sgx = gP * (float)R.u[id], Sgz = (float)R.Q[id] * (float)R.w[id];
                        float b1 = Ssx * Ssx + Ssz * Ssz, b2 = Sgx * Sgx + Sgz * Sgz;
                        float a = (Ssx * Sgx + Ssz * Sgz) / (sqrtf(b1 * b2) * (1 - 0.1));
                        if (a >= -1 && a <= 1) {
                            int ia;
                            ia = gpu_angle_bin(a, dangle);
                            if (ia < nangle) {
                                float c = gpu_angle_cos(ia);
                                adcigs[iz + (size_t)nz * ia + (size_t)nz * nangle * (ix / dcdp)] += sP * gP * c * c * c;
                            }
                        }
                    }
                }
        }
#undef RING_ID
        ttif_free(&S); ttif_free(&R); ttim_free(&m);
    }
    for (size_t o = 0; o < n0; o++) mig[o] /= ill[o];
    if (adcigs)
        for (size_t q = 0; q < (size_t)nxa * nz * nangle; q++) {
            size_t ixq = q / ((size_t)nz * nangle) * dcdp, izq = q % nz;
            adcigs[q] /= ill[izq + (size_t)nz * ixq];
        }
    free(rec); free(bp); free(bq);
    return 0;
}

/* Stack per-shot images into the full image in shot order
 * (Toa_rtm_vti_adcig_cdp.c:1102-1104; single-rank MPI_Reduce is a copy). */
void orc_stack2d(int nz, int nxs, int offset, const float *mig_is, float *mig_full)
{
    int c, j;
    for (c = 0; c < nxs; c++)
        for (j = 0; j < nz; j++)
            mig_full[(size_t)(c + offset) * nz + j] += mig_is[(size_t)c * nz + j];
}

/* Adjoint Laplacian (laplac2_lop adj=1, utils-Laplacian-filter/laplace.c:9-53;
 * in-program copy Toa_gpu2DvtiFdRtmAdcigsLaplace.cu:150-202 zeroes `out`). */
void orc_laplace2d_adj(int nz, int nx, const float *in, float *out)
{
    int iz, ix, j;
    for (j = 0; j < nx * nz; j++) out[j] = 0.0f;
    for (ix = 0; ix < nx; ix++)
        for (iz = 0; iz < nz; iz++) {
            j = iz + ix * nz;
            if (iz > 0) { out[j - 1] -= in[j]; out[j] += in[j]; }
            if (iz < nz - 1) { out[j + 1] -= in[j]; out[j] += in[j]; }
            if (ix > 0) { out[j - nz] -= in[j]; out[j] += in[j]; }
            if (ix < nx - 1) { out[j + nz] -= in[j]; out[j] += in[j]; }
        }
}

/* 3D adjoint Laplacian, the same first-difference operator along z, x, y
 * (the 3D RTM's laplace_3d_filter, 3D-vti-fd+rtm-cuda/
 * Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:555-616), out zeroed first. */
void orc_laplace3d_adj(int nz, int nx, int ny, const float *in, float *out)
{
    long iz, ix, iy, j, nxz = (long)nx * nz, n = nxz * ny;
    for (j = 0; j < n; j++) out[j] = 0.0f;
    for (iy = 0; iy < ny; iy++)
        for (ix = 0; ix < nx; ix++)
            for (iz = 0; iz < nz; iz++) {
                j = iz + ix * nz + iy * nxz;
                if (iz > 0) { out[j - 1] -= in[j]; out[j] += in[j]; }
                if (iz < nz - 1) { out[j + 1] -= in[j]; out[j] += in[j]; }
                if (ix > 0) { out[j - nz] -= in[j]; out[j] += in[j]; }
                if (ix < nx - 1) { out[j + nz] -= in[j]; out[j] += in[j]; }
                if (iy > 0) { out[j - nxz] -= in[j]; out[j] += in[j]; }
                if (iy < ny - 1) { out[j + nxz] -= in[j]; out[j] += in[j]; }
            }
}

/* ------------------------------------------------------------------ 3D */

typedef struct {
    int nx, ny, nz, npd, nt, sv, wtype;
    int mode;          /* 0: split sponge fields everywhere, the reference's
                          arithmetic; 1: the production fast path -- P,Q
                          unsplit inside the physical box, fused multiply-adds
                          at fixed places and the premultiplied model
                          A=vp^2(1+2eps), B=vp^2 sqrtf(1+2del), C=vp^2 */
    float dx, dy, dz, dt, favg, pfac;
    int fsx, fsy, fsz, dsx, dsy, dsz, is;   /* is 0-based (GPU_vti3dfd_kernels.cu:113) */
    int rec_iz, rx0, drx, nrx, ry0, dry, nry;
} orc_fd3d_desc;

/* 3D working set: model, sponge profiles and one or more wavefield sets. */
typedef struct {
    long nnx, nny, nnz, nxz, n;
    int npd, nx, ny, nz, fast;
    REAL dtx, dty, dtz;
    float *cx1, *cx2, *ax1, *ax2, *cy1, *cy2, *ay1, *ay2, *cz1, *cz2, *az1, *az2;
    REAL *vp, *e2, *d2, *mA, *mB, *mC;
    REAL *tct, *tst, *tcp, *tsp;   /* 3D TTI: cos/sin of tilt and azimuth (NULL: VTI) */
    float *amp; unsigned char *act;
    long src;
} orc_g3d;

typedef struct {
    REAL *u, *v, *w, *P, *Q, *px, *py, *pz, *qx, *qy, *qz;
} orc_f3d;

static void f3d_alloc(orc_f3d *f, long n)
{
    f->u = calloc(n, sizeof(REAL)); f->v = calloc(n, sizeof(REAL)); f->w = calloc(n, sizeof(REAL));
    f->P = calloc(n, sizeof(REAL)); f->Q = calloc(n, sizeof(REAL));
    f->px = calloc(n, sizeof(REAL)); f->py = calloc(n, sizeof(REAL)); f->pz = calloc(n, sizeof(REAL));
    f->qx = calloc(n, sizeof(REAL)); f->qy = calloc(n, sizeof(REAL)); f->qz = calloc(n, sizeof(REAL));
}

static void f3d_free(orc_f3d *f)
{
    free(f->u); free(f->v); free(f->w); free(f->P); free(f->Q);
    free(f->px); free(f->py); free(f->pz); free(f->qx); free(f->qy); free(f->qz);
}

/* Model set-up with the GUI GPU program's semantics (GPU_vti3dfd_kernels.cu):
 * edge padding, optional SV taper (R=15, r=4, centre fs+is*ds+npml-1),
 * sponge profiles of the GPU form with d0 from the centre velocity. */
static void g3d_init(orc_g3d *G, const orc_fd3d_desc *d, const float *v, const float *e, const float *dl)
{
    const int npd = d->npd;
    const long nnx = d->nx + 2 * npd, nny = d->ny + 2 * npd, nnz = d->nz + 2 * npd, nxz = nnx * nnz;
    const long n = nxz * nny;
    long ix, iy, iz, k;
    memset(G, 0, sizeof *G);
    G->nnx = nnx; G->nny = nny; G->nnz = nnz; G->nxz = nxz; G->n = n;
    G->npd = npd; G->nx = d->nx; G->ny = d->ny; G->nz = d->nz; G->fast = d->mode == 1;
    float *vv = calloc(n, 4), *ee = calloc(n, 4), *dd = calloc(n, 4);
    REAL *tmp = malloc(n * sizeof(REAL));
    for (iy = 0; iy < d->ny; iy++) for (ix = 0; ix < d->nx; ix++) for (iz = 0; iz < d->nz; iz++) {
        long g = (iz + npd) + nnz * (ix + npd) + nxz * (iy + npd), s = iz + (long)d->nz * (ix + (long)d->nx * iy);
        vv[g] = v[s]; ee[g] = e[s]; dd[g] = dl[s];
    }
    {
        float *arrs[3] = {ee, dd, vv}; int a;
        for (a = 0; a < 3; a++) {
            for (k = 0; k < n; k++) tmp[k] = arrs[a][k];
            orc_pad3d(d->nx, d->ny, d->nz, npd, tmp);
            for (k = 0; k < n; k++) arrs[a][k] = (float)tmp[k];
        }
    }
    free(tmp);
    if (d->sv) {
        int R = 15, r = 4;
        long cx = d->fsx + d->is * d->dsx + npd - 1, cy = d->fsy + d->is * d->dsy + npd - 1, cz = d->fsz + d->is * d->dsz + npd - 1;
        for (iy = 0; iy < nny; iy++) for (ix = 0; ix < nnx; ix++) for (iz = 0; iz < nnz; iz++) {
            int rx = (int)(ix - cx), ry = (int)(iy - cy), rz = (int)(iz - cz);
            long id = iz + nnz * ix + nxz * iy;
            int r2 = rx * rx + ry * ry + rz * rz;
            if (r2 <= R * R) {
                if (r2 <= r * r) { ee[id] = 0.0f; dd[id] = 0.0f; }
                else {
                    double g = 0.5 * (1 - cos(PI_GUI * ((sqrtf((float)r2) - r) * 4.0 / (R * 3.0 - 1))));
                    ee[id] = (float)(g * ee[id]); dd[id] = (float)(g * dd[id]);
                }
            }
        }
    }
    float d0 = orc_d0(ORC_V_GPU, 3, 0.0f, vv[nny * nnx * nnz / 2], npd, d->dx, d->dy, d->dz);
    G->cx1 = malloc(nnx * 4); G->cx2 = malloc(nnx * 4); G->ax1 = malloc(nnx * 4); G->ax2 = malloc(nnx * 4);
    G->cy1 = malloc(nny * 4); G->cy2 = malloc(nny * 4); G->ay1 = malloc(nny * 4); G->ay2 = malloc(nny * 4);
    G->cz1 = malloc(nnz * 4); G->cz2 = malloc(nnz * 4); G->az1 = malloc(nnz * 4); G->az2 = malloc(nnz * 4);
    orc_sponge(ORC_V_GPU, d->nx, npd, d->dt, d0, G->cx1, G->cx2, G->ax1, G->ax2);
    orc_sponge(ORC_V_GPU, d->ny, npd, d->dt, d0, G->cy1, G->cy2, G->ay1, G->ay2);
    orc_sponge(ORC_V_GPU, d->nz, npd, d->dt, d0, G->cz1, G->cz2, G->az1, G->az2);
    G->vp = malloc(n * sizeof(REAL)); G->e2 = malloc(n * sizeof(REAL)); G->d2 = malloc(n * sizeof(REAL));
    if (G->fast) { G->mA = malloc(n * sizeof(REAL)); G->mB = malloc(n * sizeof(REAL)); G->mC = malloc(n * sizeof(REAL)); }
    for (k = 0; k < n; k++) {
        G->vp[k] = vv[k];
        G->e2[k] = (REAL)1 + (REAL)2 * (REAL)ee[k];
        G->d2[k] = RSQRT((REAL)1 + (REAL)2 * (REAL)dd[k]);
        if (G->fast) {
            const REAL c2 = G->vp[k] * G->vp[k];
            G->mA[k] = c2 * G->e2[k];
            G->mB[k] = c2 * G->d2[k];
            G->mC[k] = c2;
        }
    }
    free(vv); free(ee); free(dd);
    G->amp = malloc(d->nt * 4); G->act = malloc(d->nt);
    orc_source_amp(ORC_V_GPU, d->nt, d->dt, d->favg, d->pfac, d->wtype, G->amp, G->act);
    {
        const long ixs = d->fsx + d->is * d->dsx + npd - 1, iys = d->fsy + d->is * d->dsy + npd - 1,
                   izs = d->fsz + d->is * d->dsz + npd - 1;
        G->src = izs + ixs * nnz + iys * nxz;
    }
    G->dtx = (REAL)(d->dt / d->dx); G->dty = (REAL)(d->dt / d->dy); G->dtz = (REAL)(d->dt / d->dz);
}

static void g3d_free(orc_g3d *G)
{
    free(G->cx1); free(G->cx2); free(G->ax1); free(G->ax2); free(G->cy1); free(G->cy2); free(G->ay1); free(G->ay2);
    free(G->cz1); free(G->cz2); free(G->az1); free(G->az2);
    free(G->vp); free(G->e2); free(G->d2); free(G->mA); free(G->mB); free(G->mC); free(G->amp); free(G->act);
    free(G->tct); free(G->tst); free(G->tcp); free(G->tsp);
}

/* 3D TTI: tilt theta (from the vertical) and azimuth phi in degrees on the
 * interior, iz + nz*(ix + nx*iy); their cosines and sines on the padded grid
 * (edge-replicated like the model).  The FP32 build forms them as the
 * library does, cosf(deg * 0.017453292519943295f); the FP64 build in
 * double. */
static void g3d_tilt(orc_g3d *G, const float *theta, const float *phi)
{
    const long n = G->n, nnz = G->nnz, nxz = G->nxz;
    const int npd = G->npd;
    long ix, iy, iz, k;
    REAL *t[4];
    for (k = 0; k < 4; k++) t[k] = calloc(n, sizeof(REAL));
    for (iy = 0; iy < G->ny; iy++) for (ix = 0; ix < G->nx; ix++) for (iz = 0; iz < G->nz; iz++) {
        const long g = (iz + npd) + nnz * (ix + npd) + nxz * (iy + npd), q = iz + (long)G->nz * (ix + (long)G->nx * iy);
#if defined(ORC_FP64)
        const double a = (double)theta[q] * (3.14159265358979323846 / 180.0);
        const double b = (double)phi[q] * (3.14159265358979323846 / 180.0);
        t[0][g] = cos(a); t[1][g] = sin(a); t[2][g] = cos(b); t[3][g] = sin(b);
#else
        const float a = theta[q] * 0.017453292519943295f, b = phi[q] * 0.017453292519943295f;
        t[0][g] = cosf(a); t[1][g] = sinf(a); t[2][g] = cosf(b); t[3][g] = sinf(b);
#endif
    }
    for (k = 0; k < 4; k++) orc_pad3d(G->nx, G->ny, G->nz, npd, t[k]);
    G->tct = t[0]; G->tst = t[1]; G->tcp = t[2]; G->tsp = t[3];
}

/* One 3D TTI time step (no reference counterpart: the 2D TTI GPU programs'
 * rotated-derivative scheme, 2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:81-183,
 * extended to a symmetry axis with tilt t and azimuth f).  With the rotated
 * frame x' = (cos t cos f, cos t sin f, -sin t), y' = (-sin f, cos f, 0),
 * z' = (sin t cos f, sin t sin f, cos t):
 *   u <- k2 u - k1 d/dx' P,  v <- k2 v - k1 d/dy' P,  w <- k2 w - k1 d/dz' Q
 *   P <- k2 P - k1 (A a + B b),  Q <- k2 Q - k1 (B a + C b)
 * with a = du/dx' + dv/dy', b = dw/dz', A = vp^2(1+2eps),
 * B = vp^2 sqrtf(1+2del), C = vp^2, and the 2D programs' product sponge
 * (k = cx*cy*cz on the half grid for the velocities, ax*ay*az for the
 * stresses).  Every axis derivative has the 2D programs' stagger: forward
 * (+1/2) for the velocities, backward for the stresses.  P,Q are unsplit
 * (the 2D programs' split pairs share one damping factor, so their sum is
 * the same update).  The source is added to P,Q before the velocity update
 * and only reaches the velocities, as in the VTI step. */
static void g3d_step_tti(const orc_g3d *G, orc_f3d *F, int src_on, REAL amp)
{
    const long nnx = G->nnx, nny = G->nny, nnz = G->nnz, nxz = G->nxz, src = G->src;
    const REAL dtx = G->dtx, dty = G->dty, dtz = G->dtz;
    REAL *u = F->u, *vv_ = F->v, *w = F->w, *P = F->P, *Q = F->Q;
    const float *cx1 = G->cx1, *cx2 = G->cx2, *cy1 = G->cy1, *cy2 = G->cy2, *cz1 = G->cz1, *cz2 = G->cz2;
    const float *ax1 = G->ax1, *ax2 = G->ax2, *ay1 = G->ay1, *ay2 = G->ay2, *az1 = G->az1, *az2 = G->az2;
    const REAL *mA = G->mA, *mB = G->mB, *mC = G->mC;
    const REAL *tct = G->tct, *tst = G->tst, *tcp = G->tcp, *tsp = G->tsp;
    long ix, iy, iz;
    REAL P_src0 = P[src], Q_src0 = Q[src];
    if (src_on) { P[src] += amp; Q[src] += amp; }
#pragma omp parallel for schedule(static) private(ix, iz)
    for (iy = 4; iy < nny - 4; iy++)
        for (ix = 4; ix < nnx - 4; ix++)
            for (iz = 4; iz < nnz - 4; iz++) {
                const long id = iz + ix * nnz + iy * nxz; int im;
                REAL Px = 0, Py = 0, Pz = 0, Qx = 0, Qy = 0, Qz = 0;
                for (im = 0; im < 4; im++) {
                    Px += (REAL)C8[im] * (P[id + (im + 1) * nnz] - P[id - im * nnz]);
                    Py += (REAL)C8[im] * (P[id + (im + 1) * nxz] - P[id - im * nxz]);
                    Pz += (REAL)C8[im] * (P[id + im + 1] - P[id - im]);
                    Qx += (REAL)C8[im] * (Q[id + (im + 1) * nnz] - Q[id - im * nnz]);
                    Qy += (REAL)C8[im] * (Q[id + (im + 1) * nxz] - Q[id - im * nxz]);
                    Qz += (REAL)C8[im] * (Q[id + im + 1] - Q[id - im]);
                }
                const REAL a = tct[id], b = tst[id], c = tcp[id], sn = tsp[id];
                const REAL k2 = (REAL)cx2[ix] * (REAL)cy2[iy] * (REAL)cz2[iz];
                const REAL k1 = (REAL)cx1[ix] * (REAL)cy1[iy] * (REAL)cz1[iz];
                const REAL gx = a * c * dtx * Px + a * sn * dty * Py - b * dtz * Pz;
                const REAL gy = c * dty * Py - sn * dtx * Px;
                const REAL gz = b * c * dtx * Qx + b * sn * dty * Qy + a * dtz * Qz;
                u[id] = k2 * u[id] - k1 * gx;
                vv_[id] = k2 * vv_[id] - k1 * gy;
                w[id] = k2 * w[id] - k1 * gz;
            }
#pragma omp parallel for schedule(static) private(ix, iz)
    for (iy = 4; iy < nny - 4; iy++)
        for (ix = 4; ix < nnx - 4; ix++)
            for (iz = 4; iz < nnz - 4; iz++) {
                const long id = iz + ix * nnz + iy * nxz; int im;
                REAL ux = 0, uy = 0, uz = 0, vx = 0, vy = 0, wx = 0, wy = 0, wz = 0;
                for (im = 0; im < 4; im++) {
                    ux += (REAL)C8[im] * (u[id + im * nnz] - u[id - (im + 1) * nnz]);
                    uy += (REAL)C8[im] * (u[id + im * nxz] - u[id - (im + 1) * nxz]);
                    uz += (REAL)C8[im] * (u[id + im] - u[id - im - 1]);
                    vx += (REAL)C8[im] * (vv_[id + im * nnz] - vv_[id - (im + 1) * nnz]);
                    vy += (REAL)C8[im] * (vv_[id + im * nxz] - vv_[id - (im + 1) * nxz]);
                    wx += (REAL)C8[im] * (w[id + im * nnz] - w[id - (im + 1) * nnz]);
                    wy += (REAL)C8[im] * (w[id + im * nxz] - w[id - (im + 1) * nxz]);
                    wz += (REAL)C8[im] * (w[id + im] - w[id - im - 1]);
                }
                const REAL a = tct[id], b = tst[id], c = tcp[id], sn = tsp[id];
                const REAL ha = (a * c * dtx * ux + a * sn * dty * uy - b * dtz * uz) + (c * dty * vy - sn * dtx * vx);
                const REAL hb = b * c * dtx * wx + b * sn * dty * wy + a * dtz * wz;
                const REAL k2 = (REAL)ax2[ix] * (REAL)ay2[iy] * (REAL)az2[iz];
                const REAL k1 = (REAL)ax1[ix] * (REAL)ay1[iy] * (REAL)az1[iz];
                const REAL p0 = (id == src) ? P_src0 : P[id], q0 = (id == src) ? Q_src0 : Q[id];
                P[id] = k2 * p0 - k1 * (mA[id] * ha + mB[id] * hb);
                Q[id] = k2 * q0 - k1 * (mB[id] * ha + mC[id] * hb);
            }
}

/* One 3D time step of field set F; the point source (amp, when src_on) is
 * added to P,Q before the velocity update (GPU_vti3dfd_kernels.cu:135) and
 * only affects the velocities (the stress update overwrites P,Q). */
static void g3d_step(const orc_g3d *G, orc_f3d *F, int src_on, REAL amp)
{
    if (G->tct) { g3d_step_tti(G, F, src_on, amp); return; }
    const long nnx = G->nnx, nny = G->nny, nnz = G->nnz, nxz = G->nxz, src = G->src;
    const int npd = G->npd, fast = G->fast;
    const REAL dtx = G->dtx, dty = G->dty, dtz = G->dtz;
    REAL *u = F->u, *vv_ = F->v, *w = F->w, *P = F->P, *Q = F->Q;
    REAL *px = F->px, *py = F->py, *pz = F->pz, *qx = F->qx, *qy = F->qy, *qz = F->qz;
    const float *cx1 = G->cx1, *cx2 = G->cx2, *cy1 = G->cy1, *cy2 = G->cy2, *cz1 = G->cz1, *cz2 = G->cz2;
    const float *ax1 = G->ax1, *ax2 = G->ax2, *ay1 = G->ay1, *ay2 = G->ay2, *az1 = G->az1, *az2 = G->az2;
    const REAL *vp = G->vp, *e2 = G->e2, *d2 = G->d2, *mA = G->mA, *mB = G->mB, *mC = G->mC;
    long ix, iy, iz;
    REAL P_src0 = P[src], Q_src0 = Q[src];
    if (src_on) { P[src] += amp; Q[src] += amp; }
#pragma omp parallel for schedule(static) private(ix, iz)
    for (iy = 4; iy < nny - 4; iy++)
        for (ix = 4; ix < nnx - 4; ix++)
            for (iz = 4; iz < nnz - 4; iz++) {
                long id = iz + ix * nnz + iy * nxz; int im;
                REAL xx = 0, yy = 0, zz = 0;
                if (fast) {
                    yy = (REAL)C8[0] * (P[id + nxz] - P[id]);
                    xx = (REAL)C8[0] * (P[id + nnz] - P[id]);
                    zz = (REAL)C8[0] * (Q[id + 1] - Q[id]);
                    for (im = 1; im < 4; im++) {
                        yy = RFMA((REAL)C8[im], P[id + (im + 1) * nxz] - P[id - im * nxz], yy);
                        xx = RFMA((REAL)C8[im], P[id + (im + 1) * nnz] - P[id - im * nnz], xx);
                        zz = RFMA((REAL)C8[im], Q[id + im + 1] - Q[id - im], zz);
                    }
                    u[id] = RFMA(-(cx1[ix] * dtx), xx, cx2[ix] * u[id]);
                    vv_[id] = RFMA(-(cy1[iy] * dty), yy, cy2[iy] * vv_[id]);
                    w[id] = RFMA(-(cz1[iz] * dtz), zz, cz2[iz] * w[id]);
                    continue;
                }
                for (im = 0; im < 4; im++) {
                    yy += (REAL)C8[im] * (P[id + (im + 1) * nxz] - P[id - im * nxz]);
                    xx += (REAL)C8[im] * (P[id + (im + 1) * nnz] - P[id - im * nnz]);
                    zz += (REAL)C8[im] * (Q[id + im + 1] - Q[id - im]);
                }
                u[id] = cx2[ix] * u[id] - cx1[ix] * dtx * xx;
                vv_[id] = cy2[iy] * vv_[id] - cy1[iy] * dty * yy;
                w[id] = cz2[iz] * w[id] - cz1[iz] * dtz * zz;
            }
#pragma omp parallel for schedule(static) private(ix, iz)
    for (iy = 4; iy < nny - 4; iy++)
        for (ix = 4; ix < nnx - 4; ix++)
            for (iz = 4; iz < nnz - 4; iz++) {
                long id = iz + ix * nnz + iy * nxz; int im;
                REAL xx = 0, yy = 0, zz = 0, c = vp[id];
                if (fast) {
                    const REAL A = mA[id], B = mB[id], Cc = mC[id];
                    yy = (REAL)C8[0] * (vv_[id] - vv_[id - nxz]);
                    xx = (REAL)C8[0] * (u[id] - u[id - nnz]);
                    zz = (REAL)C8[0] * (w[id] - w[id - 1]);
                    for (im = 1; im < 4; im++) {
                        yy = RFMA((REAL)C8[im], vv_[id + im * nxz] - vv_[id - (im + 1) * nxz], yy);
                        xx = RFMA((REAL)C8[im], u[id + im * nnz] - u[id - (im + 1) * nnz], xx);
                        zz = RFMA((REAL)C8[im], w[id + im] - w[id - im - 1], zz);
                    }
                    const REAL Ax = A * dtx, Ay = A * dty, Bz = B * dtz, Bx = B * dtx, By = B * dty, Cz = Cc * dtz;
                    int inside = ix >= npd && ix < npd + G->nx && iy >= npd && iy < npd + G->ny
                                 && iz >= npd && iz < npd + G->nz;
                    if (inside) {
                        REAL p0 = (id == src) ? P_src0 : P[id], q0 = (id == src) ? Q_src0 : Q[id];
                        p0 = RFMA(-Ax, xx, p0); p0 = RFMA(-Ay, yy, p0); p0 = RFMA(-Bz, zz, p0);
                        q0 = RFMA(-Bx, xx, q0); q0 = RFMA(-By, yy, q0); q0 = RFMA(-Cz, zz, q0);
                        P[id] = p0; Q[id] = q0;
                    } else {
                        px[id] = RFMA(-(ax1[ix] * Ax), xx, ax2[ix] * px[id]);
                        py[id] = RFMA(-(ay1[iy] * Ay), yy, ay2[iy] * py[id]);
                        pz[id] = RFMA(-(az1[iz] * Bz), zz, az2[iz] * pz[id]);
                        qx[id] = RFMA(-(ax1[ix] * Bx), xx, ax2[ix] * qx[id]);
                        qy[id] = RFMA(-(ay1[iy] * By), yy, ay2[iy] * qy[id]);
                        qz[id] = RFMA(-(az1[iz] * Cz), zz, az2[iz] * qz[id]);
                        P[id] = px[id] + py[id] + pz[id];
                        Q[id] = qx[id] + qy[id] + qz[id];
                    }
                    continue;
                }
                for (im = 0; im < 4; im++) {
                    yy += (REAL)C8[im] * (vv_[id + im * nxz] - vv_[id - (im + 1) * nxz]);
                    xx += (REAL)C8[im] * (u[id + im * nnz] - u[id - (im + 1) * nnz]);
                    zz += (REAL)C8[im] * (w[id + im] - w[id - im - 1]);
                }
                px[id] = ax2[ix] * px[id] - ax1[ix] * c * c * e2[id] * dtx * xx;
                py[id] = ay2[iy] * py[id] - ay1[iy] * c * c * e2[id] * dty * yy;
                pz[id] = az2[iz] * pz[id] - az1[iz] * c * c * d2[id] * dtz * zz;
                qx[id] = ax2[ix] * qx[id] - ax1[ix] * c * c * d2[id] * dtx * xx;
                qy[id] = ay2[iy] * qy[id] - ay1[iy] * c * c * d2[id] * dty * yy;
                qz[id] = az2[iz] * qz[id] - az1[iz] * c * c * dtz * zz;
                P[id] = px[id] + py[id] + pz[id];
                Q[id] = qx[id] + qy[id] + qz[id];
            }
}

/* 3D VTI forward modelling of one shot with the GUI GPU program's semantics
 * (GPU_vti3dfd_kernels.cu): point Ricker source added to P,Q before the
 * velocity update (:53-88), velocity (:90-129) and split-sponge stress
 * (:131-201) updates on [4, nn-4) in every axis, optional SV taper (R=15,
 * r=4, centre fs+is*ds+npml-1), sponge profiles of the GPU form, d0 from the
 * centre velocity (:203-206).  shot is (nt x nrx*nry) trace-major,
 * shot[it + nt*(irx + nrx*iry)] = P[rec_iz, npd+rx0+irx*drx, npd+ry0+iry*dry].
 * final_P/final_Q (optional) receive the padded P, Q at the end. */
static int fd3d_run(const orc_fd3d_desc *d, const float *v, const float *e, const float *dl, const float *theta,
                    const float *phi, float *shot, float *final_P, float *final_Q)
{
    orc_g3d G; orc_f3d F;
    int it; long k;
    g3d_init(&G, d, v, e, dl);
    if (theta) g3d_tilt(&G, theta, phi);
    f3d_alloc(&F, G.n);
    for (it = 0; it < d->nt; it++) {
        g3d_step(&G, &F, G.act[it], (REAL)G.amp[it]);
        int irx, iry;
        for (iry = 0; iry < d->nry; iry++)
            for (irx = 0; irx < d->nrx; irx++) {
                long gx = d->npd + d->rx0 + (long)irx * d->drx, gy = d->npd + d->ry0 + (long)iry * d->dry;
                shot[it + (long)d->nt * (irx + (long)d->nrx * iry)] = (float)F.P[d->rec_iz + G.nnz * gx + G.nxz * gy];
            }
    }
    if (final_P) for (k = 0; k < G.n; k++) final_P[k] = (float)F.P[k];
    if (final_Q) for (k = 0; k < G.n; k++) final_Q[k] = (float)F.Q[k];
    f3d_free(&F); g3d_free(&G);
    return 0;
}

/* 3D RTM of one shot with the 3D GPU RTM program's semantics
 * (3D-vti-fd+rtm-cuda/Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:882-968):
 *   forward: source step (SV taper on), save one ring of P,Q just outside
 *     the interior (faces z=npml-1, z=npml+nz, x=npml-1, x=npml+nx,
 *     y=npml-1, y=npml+ny; wavefield_bndr :405-506), record P+Q at z=npml
 *     for every surface node (:319-334), illum += P^2+Q^2 (:523-537);
 *   mute the record (window form, tt; :352-390);
 *   backward it=nt-1..0: restore the ring into the source field and step it
 *     again (the program's boundary-driven reconstruction), write the record
 *     into P,Q of the receiver field at z=npml-1 and step it, illum +=
 *     gP^2+gQ^2, mig += sP*gP (:926-968).
 * mig and illum (nx*ny*nz interior, iz + nz*(ix + nx*iy)) accumulate over
 * calls; the caller divides (migration_illum :539-553) and filters.  The
 * wavefields start from zero for every shot (the program zeroes them once
 * before its shot loop).
 * adcigs (optional): after each backward step's image, the Poynting
 * angle gathers (Poynting_Adcigs :618-661) over iy < ny/dcdp, ix < nx/dcdp,
 * iz < nz at the padded point (iz, ix*dcdp, iy*dcdp) + npml:
 *   Ss = -(sP*su, sP*sv, sQ*sw), Sg = (gP*gu, gP*gv, gQ*gw),
 *   a = (Ss.Sg) / (sqrtf(|Ss|^2 |Sg|^2) * (1 - 0.1))  (double quotient, kept as float),
 *   if -1 <= a <= 1: ia = (int)((float)(0.5*acosf(a)*180/pi) / (da*1.0)), and if ia < na
 *   adcigs[iz + nz*(ia + na*(ix + nxa*iy))] += sP*gP*c*c*c, c = cosf(ia*pi/180)
 * (velocities of the new time level: the program's u0 = u1 pointer
 * assignment makes the update in place); the caller divides (adcigs_illum). */
static int rtm3d_shot_run(const orc_fd3d_desc *d, int mute_tt, const float *v, const float *e, const float *dl,
                          const float *theta, const float *phi, float *mig, float *illum, float *rec_out, int na,
                          int da, int dcdp, float *adcigs)
{
    orc_g3d G; orc_f3d S, R;
    const int nx = d->nx, ny = d->ny, nz = d->nz, npd = d->npd, nt = d->nt;
    /* receivers (record at z = npd, re-inject at npd - 1): the grid
     * (rx0 + jx drx, ry0 + jy dry); every surface node is the program's
     * (shot_record :319-334) */
    const int nrx = d->nrx, nry = d->nry;
    long it, ix, iy, iz, jx, jy;
#define RX(j) (d->rx0 + (long)(j) * d->drx)
#define RY(j) (d->ry0 + (long)(j) * d->dry)
    g3d_init(&G, d, v, e, dl);
    if (theta) g3d_tilt(&G, theta, phi);
    f3d_alloc(&S, G.n);
    f3d_alloc(&R, G.n);
    const long L = 2L * nx * ny + 2L * nz * ny + 2L * nx * nz;
    float *bp = calloc((size_t)nt * L, 4), *bq = calloc((size_t)nt * L, 4);
    float *rec = calloc((size_t)nt * nrx * nry, 4);
#define GID(z, x, y) ((long)(z) + G.nnz * (long)(x) + G.nxz * (long)(y))
    /* ring position of entry k (the program's face order) */
#define RING(k, gid) do { long k_ = (k); \
        if (k_ < (long)nx * ny) { gid = GID(npd - 1, npd + k_ % nx, npd + k_ / nx); } \
        else if (k_ < 2L * nx * ny) { k_ -= (long)nx * ny; gid = GID(npd + nz, npd + k_ % nx, npd + k_ / nx); } \
        else if (k_ < 2L * nx * ny + (long)nz * ny) { k_ -= 2L * nx * ny; gid = GID(npd + k_ % nz, npd - 1, npd + k_ / nz); } \
        else if (k_ < 2L * nx * ny + 2L * nz * ny) { k_ -= 2L * nx * ny + (long)nz * ny; gid = GID(npd + k_ % nz, npd + nx, npd + k_ / nz); } \
        else if (k_ < 2L * nx * ny + 2L * nz * ny + (long)nx * nz) { k_ -= 2L * nx * ny + 2L * nz * ny; gid = GID(npd + k_ % nz, npd + k_ / nz, npd - 1); } \
        else { k_ -= 2L * nx * ny + 2L * nz * ny + (long)nx * nz; gid = GID(npd + k_ % nz, npd + k_ / nz, npd + ny); } } while (0)
    for (it = 0; it < nt; it++) {
        long k;
        g3d_step(&G, &S, G.act[it], (REAL)G.amp[it]);
        for (k = 0; k < L; k++) {
            long gid; RING(k, gid);
            bp[it * L + k] = (float)S.P[gid]; bq[it * L + k] = (float)S.Q[gid];
        }
        for (jy = 0; jy < nry; jy++) for (jx = 0; jx < nrx; jx++) {
            long gid = GID(npd, npd + RX(jx), npd + RY(jy));
            rec[it + (long)nt * jx + (long)nt * nrx * jy] = (float)(S.P[gid] + S.Q[gid]);
        }
        for (iy = 0; iy < ny; iy++) for (ix = 0; ix < nx; ix++) for (iz = 0; iz < nz; iz++) {
            long gid = GID(npd + iz, npd + ix, npd + iy), o = iz + (long)nz * ix + (long)nz * nx * iy;
            REAL p = S.P[gid], q = S.Q[gid];
            illum[o] = (float)(illum[o] + (p * p + q * q));
        }
    }
    /* mute_directwave, window form (:352-390), source at (fsx+is*dsx, fsy+is*dsy) */
    {
        /* vp[1], eps[1] of the padded model = the model's first cell */
        const float eps1 = e[0], vp1 = v[0];
        for (jy = 0; jy < nry; jy++) for (jx = 0; jx < nrx; jx++) {
            ix = RX(jx); iy = RY(jy);
            float mu_x = d->dx * abs((int)ix - d->fsx - d->is * d->dsx), mu_y = d->dy * abs((int)iy - d->fsy - d->is * d->dsy);
            float mu_z = d->dz * d->fsz;
            float mu_t0 = sqrtf((float)(pow(mu_x, 2) + pow(mu_y, 2) + pow(mu_z, 2))) / (vp1 * sqrtf(1 + 2 * eps1));
            int mu_t = (int)(2.0 / (d->dt * d->favg));
            int mu_nt = (int)(mu_t0 / d->dt) + mu_t + mute_tt;
            for (it = 0; it < nt; it++)
                if ((it > (int)(mu_t0 / d->dt) - mute_tt) && (it < mu_nt)) rec[it + (long)nt * jx + (long)nt * nrx * jy] = 0.0f;
        }
    }
    if (rec_out) memcpy(rec_out, rec, (size_t)nt * nrx * nry * 4);
    for (it = nt - 1; it >= 0; it--) {
        long k;
        for (k = 0; k < L; k++) {
            long gid; RING(k, gid);
            S.P[gid] = (REAL)bp[it * L + k]; S.Q[gid] = (REAL)bq[it * L + k];
        }
        g3d_step(&G, &S, 0, 0);
        for (jy = 0; jy < nry; jy++) for (jx = 0; jx < nrx; jx++) {
            long gid = GID(npd - 1, npd + RX(jx), npd + RY(jy));
            R.P[gid] = R.Q[gid] = (REAL)rec[it + (long)nt * jx + (long)nt * nrx * jy];
        }
        g3d_step(&G, &R, 0, 0);
        for (iy = 0; iy < ny; iy++) for (ix = 0; ix < nx; ix++) for (iz = 0; iz < nz; iz++) {
            long gid = GID(npd + iz, npd + ix, npd + iy), o = iz + (long)nz * ix + (long)nz * nx * iy;
            REAL gp = R.P[gid], gq = R.Q[gid];
            illum[o] = (float)(illum[o] + (gp * gp + gq * gq));
            mig[o] = (float)(mig[o] + S.P[gid] * gp);
        }
        if (adcigs) {
            const int nxa = nx / dcdp, nya = ny / dcdp;
            for (iy = 0; iy < nya; iy++) for (ix = 0; ix < nxa; ix++) for (iz = 0; iz < nz; iz++) {
                long gid = GID(npd + iz, npd + ix * dcdp, npd + iy * dcdp);
                float sP = (float)S.P[gid], gP = (float)R.P[gid];
                float Ssx = -sP * (float)S.u[gid], Ssy = -sP * (float)S.v[gid], Ssz = -(float)S.Q[gid] * (float)S.w[gid];
                float Sgx = gP * (float)R.u[gid], Sgy = gP * (float)R.v[gid], Sgz = (float)R.Q[gid] * (float)R.w[gid];
                float b1 = Ssx * Ssx + Ssy * Ssy + Ssz * Ssz, b2 = Sgx * Sgx + Sgy * Sgy + Sgz * Sgz;
                float a = (Ssx * Sgx + Ssy * Sgy + Ssz * Sgz) / (sqrtf(b1 * b2) * (1 - 0.1));
                if (a >= -1 && a <= 1) {
                    int ia;
                    ia = gpu_angle_bin(a, da);
                    if (ia < na) {
                        float c = gpu_angle_cos(ia);
                        adcigs[iz + (long)nz * (ia + (long)na * (ix + (long)nxa * iy))] += sP * gP * c * c * c;
                    }
                }
            }
        }
    }
#undef RING
#undef GID
    free(bp); free(bq); free(rec);
    f3d_free(&S); f3d_free(&R); g3d_free(&G);
    return 0;
}

/* 3D RTM of one shot with stored source snapshots (the library's
 * GEO_RTM_SNAPSHOT method; no reference counterpart): the forward pass of
 * orc_rtm3d_shot (record, source illumination, window mute) keeping the
 * interior P of every step it with it % k == k-1; the backward pass
 * propagates only the receiver field (same injection and illumination) and
 * at those steps adds mig += (k * snap) * gP. */
static int rtm3d_snap_run(const orc_fd3d_desc *d, int mute_tt, int k, const float *v, const float *e,
                          const float *dl, const float *theta, const float *phi, float *mig, float *illum)
{
    orc_g3d G; orc_f3d S, R;
    const int nx = d->nx, ny = d->ny, nz = d->nz, npd = d->npd, nt = d->nt;
    const long nimg = (long)nx * ny * nz;
    const int nsnap = nt / k;
    const int nrx = d->nrx, nry = d->nry;   /* receiver grid, as in rtm3d_shot_run */
    long it, ix, iy, iz, jx, jy;
    g3d_init(&G, d, v, e, dl);
    if (theta) g3d_tilt(&G, theta, phi);
    f3d_alloc(&S, G.n);
    f3d_alloc(&R, G.n);
    float *snap = calloc((size_t)(nsnap > 0 ? nsnap : 1) * nimg, 4);
    float *rec = calloc((size_t)nt * nrx * nry, 4);
#define GID(z, x, y) ((long)(z) + G.nnz * (long)(x) + G.nxz * (long)(y))
    for (it = 0; it < nt; it++) {
        g3d_step(&G, &S, G.act[it], (REAL)G.amp[it]);
        for (jy = 0; jy < nry; jy++) for (jx = 0; jx < nrx; jx++) {
            long gid = GID(npd, npd + RX(jx), npd + RY(jy));
            rec[it + (long)nt * jx + (long)nt * nrx * jy] = (float)(S.P[gid] + S.Q[gid]);
        }
        for (iy = 0; iy < ny; iy++) for (ix = 0; ix < nx; ix++) for (iz = 0; iz < nz; iz++) {
            long gid = GID(npd + iz, npd + ix, npd + iy), o = iz + (long)nz * ix + (long)nz * nx * iy;
            REAL p = S.P[gid], q = S.Q[gid];
            illum[o] = (float)(illum[o] + (p * p + q * q));
            if (it % k == k - 1 && it / k < nsnap) snap[(it / k) * nimg + o] = (float)p;
        }
    }
    {
        const float eps1 = e[0], vp1 = v[0];
        for (jy = 0; jy < nry; jy++) for (jx = 0; jx < nrx; jx++) {
            ix = RX(jx); iy = RY(jy);
            float mu_x = d->dx * abs((int)ix - d->fsx - d->is * d->dsx), mu_y = d->dy * abs((int)iy - d->fsy - d->is * d->dsy);
            float mu_z = d->dz * d->fsz;
            float mu_t0 = sqrtf((float)(pow(mu_x, 2) + pow(mu_y, 2) + pow(mu_z, 2))) / (vp1 * sqrtf(1 + 2 * eps1));
            int mu_t = (int)(2.0 / (d->dt * d->favg));
            int mu_nt = (int)(mu_t0 / d->dt) + mu_t + mute_tt;
            for (it = 0; it < nt; it++)
                if ((it > (int)(mu_t0 / d->dt) - mute_tt) && (it < mu_nt)) rec[it + (long)nt * jx + (long)nt * nrx * jy] = 0.0f;
        }
    }
    for (it = nt - 1; it >= 0; it--) {
        for (jy = 0; jy < nry; jy++) for (jx = 0; jx < nrx; jx++) {
            long gid = GID(npd - 1, npd + RX(jx), npd + RY(jy));
            R.P[gid] = R.Q[gid] = (REAL)rec[it + (long)nt * jx + (long)nt * nrx * jy];
        }
        g3d_step(&G, &R, 0, 0);
        for (iy = 0; iy < ny; iy++) for (ix = 0; ix < nx; ix++) for (iz = 0; iz < nz; iz++) {
            long gid = GID(npd + iz, npd + ix, npd + iy), o = iz + (long)nz * ix + (long)nz * nx * iy;
            REAL gp = R.P[gid], gq = R.Q[gid];
            illum[o] = (float)(illum[o] + (gp * gp + gq * gq));
            if (it % k == k - 1 && it / k < nsnap) {
                float w = (float)k * snap[(it / k) * nimg + o];
                mig[o] = (float)(mig[o] + w * gp);
            }
        }
    }
#undef GID
#undef RX
#undef RY
    free(snap); free(rec);
    f3d_free(&S); f3d_free(&R); g3d_free(&G);
    return 0;
}

int orc_fd3d(const orc_fd3d_desc *d, const float *v, const float *e, const float *dl,
             float *shot, float *final_P, float *final_Q)
{
    return fd3d_run(d, v, e, dl, NULL, NULL, shot, final_P, final_Q);
}

int orc_rtm3d_shot(const orc_fd3d_desc *d, int mute_tt, const float *v, const float *e, const float *dl,
                   float *mig, float *illum, float *rec_out, int na, int da, int dcdp, float *adcigs)
{
    return rtm3d_shot_run(d, mute_tt, v, e, dl, NULL, NULL, mig, illum, rec_out, na, da, dcdp, adcigs);
}

int orc_rtm3d_snap_shot(const orc_fd3d_desc *d, int mute_tt, int k, const float *v, const float *e, const float *dl,
                        float *mig, float *illum)
{
    return rtm3d_snap_run(d, mute_tt, k, v, e, dl, NULL, NULL, mig, illum);
}

/* The same three runs on a 3D TTI medium (g3d_step_tti); theta and phi in
 * degrees on the interior.  The model takes the premultiplied form. */
static orc_fd3d_desc tti_desc(const orc_fd3d_desc *d)
{
    orc_fd3d_desc t = *d;
    t.mode = 1;
    return t;
}

int orc_tti3d(const orc_fd3d_desc *d, const float *v, const float *e, const float *dl, const float *theta,
              const float *phi, float *shot, float *final_P, float *final_Q)
{
    const orc_fd3d_desc t = tti_desc(d);
    return fd3d_run(&t, v, e, dl, theta, phi, shot, final_P, final_Q);
}

int orc_rtm3d_tti_shot(const orc_fd3d_desc *d, int mute_tt, const float *v, const float *e, const float *dl,
                       const float *theta, const float *phi, float *mig, float *illum, float *rec_out)
{
    const orc_fd3d_desc t = tti_desc(d);
    return rtm3d_shot_run(&t, mute_tt, v, e, dl, theta, phi, mig, illum, rec_out, 0, 1, 1, NULL);
}

int orc_rtm3d_tti_snap_shot(const orc_fd3d_desc *d, int mute_tt, int k, const float *v, const float *e,
                            const float *dl, const float *theta, const float *phi, float *mig, float *illum)
{
    const orc_fd3d_desc t = tti_desc(d);
    return rtm3d_snap_run(&t, mute_tt, k, v, e, dl, theta, phi, mig, illum);
}

/* migration_illum (:539-553): mig /= illum where illum != 0. */
void orc_image_illum(long n, float *mig, const float *illum)
{
    long k;
    for (k = 0; k < n; k++) if (illum[k] != 0) mig[k] = mig[k] / illum[k];
}

/* adcigs_illum (3D-vti-fd+rtm-cuda/Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:663-684):
 * gather element (iz, ia, ix, iy) /= illum at (iz, ix*dcdp, iy*dcdp) where that is non-zero. */
void orc_adcig3d_illum(int nx, int ny, int nz, int na, int dcdp, float *adcigs, const float *illum)
{
    const int nxa = nx / dcdp, nya = ny / dcdp;
    long iy, ix, ia, iz;
    for (iy = 0; iy < nya; iy++) for (ix = 0; ix < nxa; ix++) for (ia = 0; ia < na; ia++) for (iz = 0; iz < nz; iz++) {
        float w = illum[iz + (long)ix * dcdp * nz + (long)iy * dcdp * nx * nz];
        long o = iz + (long)nz * (ia + (long)na * (ix + (long)nxa * iy));
        if (w != 0) adcigs[o] /= w;
    }
}

/* Direct-wave mute of a 3D record (mute_directwave3d, GPU_vti3dfd_kernels.cu:342-369):
 * zero it < mu_nt with t0 = |offset|/(vp[1]*sqrtf(1+2 eps[1])) (padded index 1). */
void orc_mute3d(int nx, int ny, int nt, float dt, float favg, float dx, float dy, float dz,
                int fsx, int fsy, int dsx, int dsy, int fsz, int is, float vp1, float eps1, int tt, float *shot)
{
    int ix, iy, it;
    for (iy = 0; iy < ny; iy++) for (ix = 0; ix < nx; ix++) {
        float mu_x = dx * abs(ix - fsx - is * dsx), mu_y = dy * abs(iy - fsy - is * dsy), mu_z = dz * fsz;
        float mu_t0 = sqrtf((float)(pow(mu_x, 2) + pow(mu_y, 2) + pow(mu_z, 2))) / (vp1 * sqrtf(1 + 2 * eps1));
        int mu_t = (int)(2.0 / (dt * favg));
        int mu_nt = (int)(mu_t0 / dt) + mu_t + tt;
        for (it = 0; it < nt && it < mu_nt; it++) shot[it + (long)ix * nt + (long)iy * nx * nt] = 0.0f;
    }
}
