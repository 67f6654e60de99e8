/*
 * geofd.h -- C ABI of the GB300 finite-difference library (libgeofd.so).
 *
 * Everything here is plain C: ints, floats, pointers and sizes.  Arrays use
 * the reference's layouts:
 *   2D model / image   a[ix*nz + iz]                  (x-major, z fastest)
 *   3D model / image   a[iz + nz*(ix + nx*iy)]        (z fastest)
 *   shot records       shot[it + nt*trace]            (trace-major)
 *   3D traces          trace = irx + nrx*iry
 * Units follow the reference's drop-in entry points where noted (dx in m,
 * dt in microseconds, favg in Hz); the geo_* descriptors take SI floats.
 *
 * Memory: every geo_* call that takes a `mem` argument reads its inputs from
 * and writes its outputs to host memory (GEO_MEM_HOST) or device memory of
 * the current CUDA device (GEO_MEM_DEVICE).  Work buffers are allocated by the
 * library unless stated otherwise.  `stream` is a cudaStream_t (NULL = the
 * legacy default stream); calls are synchronous with respect to the host.
 */
#ifndef GEOFD_H
#define GEOFD_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GEO_OK            0
#define GEO_ERR_ARG       1   /* bad size, position or flag                   */
#define GEO_ERR_CUDA      2   /* a CUDA runtime call failed                   */
#define GEO_ERR_IO        3   /* a file could not be opened/read/written      */
#define GEO_ERR_MODEL     4   /* NaN/Inf or non-positive velocity in a model  */
#define GEO_ERR_CFL       5   /* stability check failed                       */
#define GEO_ERR_WINDOW    6   /* RTM aperture window leaves the model         */
#define GEO_ERR_NOMEM     7   /* device allocation failed                     */
#define GEO_ERR_NAN       8   /* wavefield watchdog saw NaN/Inf               */

#define GEO_MEM_HOST   0
#define GEO_MEM_DEVICE 1

/* Semantic variants: which reference program the arithmetic follows.     */
#define GEO_VARIANT_CPU    0  /* CPU_vti2dfd (GUI CPU, 7x7 Gaussian source
                                 after the stress update, acoff2 from coff1,
                                 2*P receivers)                              */
#define GEO_VARIANT_GPU    1  /* GPU_vti2dfd / GPU_vti3dfd (point source
                                 before the velocity update)                 */
#define GEO_VARIANT_MPI    2  /* the MPI CPU RTM program (rho*vp^2 form,
                                 t = it*dt, SV taper always on)              */

/* 3D stress formulation */
#define GEO_MODE_EXACT 0      /* split sponge fields everywhere (bit-exact
                                 with the reference's arithmetic)            */
#define GEO_MODE_FAST  1      /* P,Q unsplit inside the physical box         */

const char *geo_version(void);
const char *geo_strerror(int status);
/* Number of kernel launches the library issued since load (all kinds). */
long long geo_launch_count(void);

/* ======================================================================
 * Drop-in entry points: identical signatures and file formats to the
 * reference's C ABI.  They return void like the originals and report a
 * failure on stderr (the originals printf and exit(0)).
 * ====================================================================== */

/* 2D VTI FD with the GUI GPU program's semantics.
 * Replaces GPU_vti2dfd, 2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti2dfd_kernels.cu:301-304. */
void GPU_vti2dfd(int nx, int nz, int dx, int dz, int npd, int SV,
                 const char FNv[], const char FNe[], const char FNd[],
                 int favg, int ns, int fs, int ds, int zs,
                 const char FNshot[], const char FNsnap[], int nt, int dt, int run_count);

/* 2D VTI FD with the GUI CPU program's semantics, computed on the GPU.
 * Replaces CPU_vti2dfd, 2D-3D-vti-fd-cuda-gtk-GUI/CPU_vti2dfd_kernels.c:366-367. */
void CPU_vti2dfd(int nx, int nz, int dx, int dz, int npd, int SV,
                 const char FNv[], const char FNe[], const char FNd[],
                 int favg, int ns, int fs, int ds, int zs,
                 const char FNshot[], const char FNsnap[], int nt, int dt, int run_count);

/* 3D VTI FD with the GUI GPU program's semantics.
 * Replaces GPU_vti3dfd, 2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti3dfd_kernels.cu:371-374. */
void GPU_vti3dfd(int nx, int ny, int nz, int dx, int dy, int dz, int npml, int SV,
                 const char FNv[], const char FNe[], const char FNd[],
                 int favg, int ns, int fsx, int dsx, int fsy, int dsy, int fsz, int dsz,
                 const char FNshot[], const char FNsnap[], int nt, int dt, int run_count);

/* ======================================================================
 * Status-returning API
 * ====================================================================== */

/* 2D forward modelling of one shot.  Mirrors the reference's per-shot loop
 * (CPU_vti2dfd_kernels.c:465-510, GPU_vti2dfd_kernels.cu:404-444): zero the
 * state, nt steps of source + velocity + stress + receiver gather. */
typedef struct geo_fd2d_desc {
    int   nx, nz, npd, nt;
    float dx, dz, dt;        /* m, m, s                                      */
    float favg, pfac;        /* Hz, source gain                              */
    int   wtype;             /* 1 Ricker, 2/3 Gaussian derivatives           */
    float fs, ds, zs;        /* source x (1-based), shot step, source z      */
    int   is;                /* shot number, 1-based                         */
    int   variant;           /* GEO_VARIANT_*                                */
    int   sv;                /* SV-suppression taper around the source       */
    int   rec_iz;            /* receiver row, padded index (npd = surface)   */
    float rec_scale;         /* 1, or 2 for CPU_vti2dfd's P+P record         */
    int   mute_tt;           /* >0: apply the GPU-form direct-wave mute      */
} geo_fd2d_desc;

/* v,e,d: nx*nz model; shot: nt*nx record.  snap (optional, may be NULL):
 * receives the padded P every snap_every steps ((nt-1)/snap_every+1 frames
 * of (nx+2npd)*(nz+2npd)). */
int geo_fd2d_shot(const geo_fd2d_desc *desc, const float *v, const float *e, const float *d,
                  float *shot, float *snap, int snap_every, int mem, void *stream);

/* geo_fd2d_shot for callers that cannot allocate GPU memory (a program
 * whose device memory is all reserved by its own pool, a framework that
 * forbids allocation outside its allocator, a loop that must never block in
 * the allocator).  No counterpart in the reference: it is an addition.
 *   - v, e, d (nx*nz) and shot (nt*nx) are DEVICE pointers the caller owns;
 *   - nothing is allocated: the wavefields live in one static device array
 *     of geo_fd2d_noalloc_limit() bytes (32 MiB) that every GPU loading the
 *     library keeps until exit; larger shots fail with GEO_ERR_ARG;
 *   - CPU and GPU variants (SV taper and GPU-form mute included), no
 *     snapshots;
 *   - the first call on a device resolves the array's device address,
 *     which is kept for the life of the process: do not call this on a
 *     device after cudaDeviceReset;
 *   - the host-side set-up is one fixed set of static arrays guarded by a
 *     mutex: calls from several host threads (on one or several devices)
 *     take turns for it;
 *   - all calls on one device share the array: calls that overlap on the
 *     GPU (other streams, other host threads) race and corrupt each
 *     other's results. */
int geo_fd2d_shot_noalloc(const geo_fd2d_desc *desc, const float *v, const float *e, const float *d,
                          float *shot, void *stream);
size_t geo_fd2d_noalloc_limit(void);

/* 2D TTI forward modelling of one shot with the GPU TTI program's
 * semantics (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:81-183,
 * replacing its main() shot loop :421-461).  desc as for geo_fd2d_shot
 * (variant ignored, mute_tt and rec_scale unused); theta: nx*nz tilt in
 * degrees.  shot: nx*nt (shot[it + nt*ix]); snap (optional): padded P at
 * it = snap_every, 2*snap_every, ... ((nt-1)/snap_every frames). */
int geo_tti2d_shot(const geo_fd2d_desc *desc, const float *v, const float *e, const float *d, const float *theta,
                   float *shot, float *snap, int snap_every, int mem, void *stream);

/* 3D forward modelling of one shot (GPU_vti3dfd semantics).
 * Replaces the per-shot body of GPU_vti3dfd_kernels.cu:113-160. */
typedef struct geo_fd3d_desc {
    int   nx, ny, nz, npd, nt;
    float dx, dy, dz, dt;
    float favg, pfac;
    int   wtype, sv, mode;   /* mode: GEO_MODE_EXACT / GEO_MODE_FAST         */
    int   fsx, fsy, fsz, dsx, dsy, dsz;   /* source, 1-based grid cells      */
    int   rec_iz;            /* receiver depth, padded index                 */
    int   rx0, drx, nrx;     /* receiver x: npd+rx0+irx*drx                  */
    int   ry0, dry, nry;     /* receiver y: npd+ry0+iry*dry                  */
    int   mute_tt;           /* >0: mute_directwave3d with this tt           */
} geo_fd3d_desc;

typedef struct geo_fd3d_plan geo_fd3d_plan;

/* A plan owns the device state of one 3D grid (model, wavefields, sponge
 * profiles, record buffer) so repeated shots reuse it. */
int geo_fd3d_plan_create(geo_fd3d_plan **plan, const geo_fd3d_desc *desc);
int geo_fd3d_plan_destroy(geo_fd3d_plan *plan);
/* v,e,d: nx*ny*nz model in the reference layout. */
int geo_fd3d_set_model(geo_fd3d_plan *plan, const float *v, const float *e, const float *d,
                       int mem, void *stream);
/* 3D TTI medium (no reference counterpart: the 2D TTI GPU programs'
 * rotated-derivative scheme, 2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:81-183,
 * extended to a symmetry axis with tilt theta from the vertical and azimuth
 * phi, both in degrees on the nx*ny*nz model layout and smooth in space).
 * After this call the plan steps with the TTI scheme; the plan must use
 * GEO_MODE_FAST (the premultiplied model). */
int geo_fd3d_set_tilt(geo_fd3d_plan *plan, const float *theta, const float *phi, int mem, void *stream);
/* Shot number `is` (0-based, as the reference's loop): shot is nt*nrx*nry. */
int geo_fd3d_run_shot(geo_fd3d_plan *plan, int is, float *shot, int mem, void *stream);
/* Runs nsteps bare time steps (no source or receivers) on the current
 * state and returns their device time in ms -- used to time the stencil. */
int geo_fd3d_time_steps(geo_fd3d_plan *plan, int nsteps, float *ms, void *stream);
/* Copies the padded P (and Q) of the current state out. */
int geo_fd3d_get_fields(geo_fd3d_plan *plan, float *P, float *Q, int mem, void *stream);
/* One-call convenience: create, set model, run, destroy. */
int geo_fd3d_shot(const geo_fd3d_desc *desc, int is, const float *v, const float *e, const float *d,
                  float *shot, int mem, void *stream);

/* 3D boundary-saving RTM with the 3D GPU RTM program's semantics
 * (3D-vti-fd+rtm-cuda/Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:882-981):
 * per shot a forward run records P+Q at z = npml on every surface node and
 * saves one ring of P,Q just outside the model box per step; the record is
 * muted (window form, tt = mute_tt); the backward loop rebuilds the source
 * field from the ring and back-propagates the record; illumination sums
 * P^2+Q^2 of both fields, the image sums sP*gP.  Replaces that program's
 * shot loop and its migration_illum / laplace_3d_filter tail (:970-981).
 * fd.rec_* and fd.mute_tt are ignored (the receivers are the whole
 * surface); shots are is = 0..ns-1 at fs + is*ds. */
typedef struct geo_ae geo_ae;

enum {
    GEO_RTM_BOUNDARY = 0,    /* the program's boundary-saving recompute      */
    GEO_RTM_SNAPSHOT = 1,    /* source P stored every snap_every steps       */
    GEO_RTM_LEARNED  = 2,    /* same snapshots through the learned codec     */
    GEO_RTM_CHECKPOINT = 3   /* exact recompute: the full wavefield saved
                                every ckpt_every steps, each segment
                                re-propagated in the backward pass; image
                                bit-identical to GEO_RTM_SNAPSHOT's          */
};

typedef struct geo_rtm3d_desc {
    geo_fd3d_desc fd;
    int   ns;                /* number of shots                              */
    int   mute_tt;           /* window half-width of the direct-wave mute    */
    int   method;            /* GEO_RTM_*                                    */
    int   snap_every;        /* snapshot interval (methods 1, 2)             */
    geo_ae *ae;              /* trained codec (method 2)                     */
    int   na, da, dcdp;      /* angle gathers: bins, bin width in degrees,
                                CDP decimation (0 = the program's 65, 1, 1)   */
    const float *theta, *phi;/* 3D TTI medium (geo_fd3d_set_tilt; in `mem`
                                like the model) or NULL for VTI; no angle
                                gathers on a TTI medium                       */
    int   ckpt_every;        /* checkpoint interval in steps (method 3; a
                                multiple of snap_every; 0 = the interval that
                                minimises states plus segment snapshots)      */
    int   rec_grid;          /* 0: every surface node records P+Q at z = npml
                                and takes the record back at npml-1 (the
                                program's receivers, shot_record :319-334);
                                1: only the nodes of fd's grid rx0+k*drx
                                (k < nrx), ry0+j*dry (j < nry) do (an
                                addition: decimated receiver grids)          */
} geo_rtm3d_desc;

/* v,e,d: nx*ny*nz.  mig: nx*ny*nz image divided by the illumination where
 * it is non-zero.  mig_lap, illum (optional, may be NULL): the image after
 * laplace_3d_filter, and the illumination.
 * Methods 1 and 2 are additions without a reference counterpart: the
 * forward pass keeps the source P of every snap_every-th step (it %
 * snap_every == snap_every-1) -- as fp32 (SNAPSHOT) or as the codec's
 * 16x-smaller code (LEARNED) -- so the backward pass propagates only the
 * receiver field and images mig += snap_every * sP * gP at those steps.
 * Illumination is the same as method 0 (every step, both fields). */
int geo_rtm3d(const geo_rtm3d_desc *desc, const float *v, const float *e, const float *d,
              float *mig, float *mig_lap, float *illum, int mem, void *stream);

/* geo_rtm3d plus the Poynting angle-domain common-image gathers of the 3D
 * GPU RTM program (Poynting_Adcigs, 3D-vti-fd+rtm-cuda/
 * Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:618-661, after every backward
 * step; adcigs_illum :663-684 after the shots).  Method 0 only: the gathers
 * need the source particle velocities.  adcigs: nxa*nya*na*nz with
 * nxa = nx/dcdp, nya = ny/dcdp, element iz + nz*(ia + na*(ixa + nxa*iya)),
 * divided by the illumination at (iz, ixa*dcdp, iya*dcdp) where it is
 * non-zero; NULL gives geo_rtm3d. */
int geo_rtm3d_adcig(const geo_rtm3d_desc *desc, const float *v, const float *e, const float *d,
                    float *mig, float *mig_lap, float *illum, float *adcigs, int mem, void *stream);

/* 2D RTM with the MPI CPU program's semantics on per-shot aperture windows
 * (2D-vti-fd+rtm-mpi/Toa_rtm_vti_adcig_cdp.c:295-392 with
 * model_vti_get_boundry :483 and RTM_corr_adcig :739).  All shots run
 * together: each time step is one persistent launch over every shot's
 * tiles, and the time loop is replayed from a CUDA graph.  The stacked image
 * is formed in shot order and optionally passed through the adjoint
 * Laplacian (laplac2_lop adj=1). */
typedef struct geo_rtm2d_desc {
    int   nx, nz, npd, nt;   /* full model                                   */
    float dx, dz, dt_ms;     /* dt in milliseconds, as that program takes it */
    float favg, pfac;
    int   zs;                /* source depth (1-based, zs_sxd)               */
    int   ns;                /* number of shots                              */
    const int *shot_x;       /* ns source x positions k (1-based), host      */
    const int *shot_nxs;     /* ns odd window widths, host                   */
    int   laplace;           /* apply the adjoint Laplacian to the stack     */
    int   tile_z, tile_x;    /* 0 = autotuned                                */
    int   mode;              /* GEO_MODE_EXACT (0): the program's arithmetic,
                                bit for bit, with its double-precision chains;
                                GEO_MODE_FAST: those chains in FP32 (pz, qx
                                with sqrtf(1+2del), the illumination sum)     */
} geo_rtm2d_desc;

/* v,e,d: nx*nz; image: nx*nz stacked (Laplacian-filtered if asked).
 * per_shot (optional): ns images concatenated, shot s of size nxs_s*nz. */
int geo_rtm2d_batch(const geo_rtm2d_desc *desc, const float *v, const float *e, const float *d,
                    float *image, float *per_shot, int mem, void *stream);
/* The same run with the Poynting-vector angle gathers of the MPI program
 * (flag_adcig = 1, RTM_corr_adcig Toa_rtm_vti_adcig_cdp.c:1004-1068, stacked
 * as adcig_ns0 :1083-1096): adcig receives 90*nx*nz floats in the program's
 * array order adcig_ns[ia][ix][iz] (its output file stores ix, ia, iz). */
int geo_rtm2d_batch_adcig(const geo_rtm2d_desc *desc, const float *v, const float *e, const float *d,
                          float *image, float *per_shot, float *adcig, int mem, void *stream);

/* 2D RTM with the 2D GPU RTM program's semantics
 * (2D-vti-fd+rtm-cuda/Toa_gpu2DvtiFdRtmAdcigsLaplace.cu, RTM() :1184-1566):
 * full-model shots is = 1..ns at fs + (is-1)*ds, ring saving of P,Q,
 * forward-stepped reconstruction, receiver re-injection, image, forward
 * source illumination and Poynting angle gathers, summed over the shots and
 * divided by the illumination at the end.  obs (optional): observed shots
 * ns*nx*nt (trace-major, readShot) replacing the modelled records.
 * mig_lap: Laplacian of the image (the program's migration file); illum,
 * adcigs (nx*nangle*nz, [ix][ia][iz]), stk_lap (Laplacian of the angle
 * stack), shots (the muted modelled records ns*nx*nt): optional.  The
 * readFile checks (:930-965) return GEO_ERR_CFL. */
typedef struct geo_rtm2d_gpu_desc {
    int   nx, nz, npml, nt;
    float dx, dz, dt;        /* m, m, s                                      */
    float favg, pfac;
    int   wtype;
    int   ns, fs, ds, zs;    /* shots; source x (1-based), step, depth       */
    int   mute_tt;           /* 20 in the program                            */
    int   nangle, dangle;    /* 70 and 1 in the program                      */
    int   dcdp;              /* gathers at every dcdp-th CDP: TTI program
                                only (0 = 1); the VTI program takes 0 or 1  */
} geo_rtm2d_gpu_desc;

int geo_rtm2d_gpu(const geo_rtm2d_gpu_desc *desc, const float *v, const float *e, const float *d,
                  const float *obs, float *mig_lap, float *illum, float *adcigs, float *stk_lap, float *shots,
                  int mem, void *stream);

/* 2D TTI RTM with the 2D TTI GPU RTM program's semantics
 * (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu, main
 * :500-800): the shot structure of geo_rtm2d_gpu with the TTI stencil
 * (update_vel / update_stress :126-228) over theta (nx*nz tilt in degrees),
 * SV taper R=15, r=4 in the forward pass, direct-wave mute with velocity
 * vp*(1+(sqrtf(1+2 eps)-1)*cos(theta)) at the first model cell (:336-358;
 * tt = 30 in the program), forward illumination (:430-442), and Poynting
 * gathers at CDPs 0, dcdp, 2 dcdp, ... (:454-498): adcigs is
 * (nx/dcdp)*nangle*nz, [ixa][ia][iz].  The program's defaults: nangle 65,
 * dangle 1, dcdp 1.  No readFile checks, no angle stack.  mig_lap: the
 * Laplacian-filtered image; illum, adcigs, shots (muted records
 * ns*nx*nt): optional. */
int geo_rtm2d_tti(const geo_rtm2d_gpu_desc *desc, const float *v, const float *e, const float *d,
                  const float *theta, const float *obs, float *mig_lap, float *illum, float *adcigs,
                  float *shots, int mem, void *stream);

/* Adjoint first-difference Laplacian (laplac2_lop adj=1,
 * utils-Laplacian-filter/laplace.c:9-53; the in-program copy
 * Toa_gpu2DvtiFdRtmAdcigsLaplace.cu:150-202 clears `out` first, as this does). */
int geo_laplace2d(int nx, int nz, const float *in, float *out, int mem, void *stream);
/* 3D form (laplace_3d_filter, 3D-vti-fd+rtm-cuda/
 * Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:555-616). */
int geo_laplace3d(int nx, int ny, int nz, const float *in, float *out, int mem, void *stream);

/* ---- post-processing and model tools --------------------------------
 * geo_smooth_lines: `passes` Jacobi passes of 3-point averaging along
 *   nlines lines of n samples, sample k of line l at v[l*line_stride +
 *   k*elem_stride] -- smooth1float of the MPI RTM program
 *   (2D-vti-fd+rtm-mpi/Toa_rtm_vti_adcig_cdp.c:1642-1664): inside
 *   (v[k-1]+v[k]+v[k+1])/3, ends (v[0]+v[1])/2 and (v[n-1]+v[n-2])/2.
 *   n <= 24576.
 * geo_smooth2d: smooth2float (:1607-1639) on v[ix*nz + iz]: rx passes along
 *   x for every iz, then rz passes along z for every ix.
 * geo_adcig_smooth_stack: the program's smoothed gathers and angle stack
 *   (:416-437): adcig[ia][ix][iz] (na*nx*nz, the geo_rtm2d_batch_adcig
 *   order) smoothed in place along ia with `passes` passes (10 in the
 *   program); stack (optional, nx*nz) = sum over ia in order.
 * geo_mute_direct: the direct-wave mute utility
 *   (2D-vti-fd+rtm-cuda/functions/shot_muteDirect.c:11-33) on a trace-major
 *   record shot[ix*nt + it]: zero (t0/dt - tt, t0/dt + 2/(dt favg) + tt),
 *   t0 = sqrt(offset^2 + (dz zs)^2) / (vp sqrtf(1+2 epsilon)) in double,
 *   offset = dx |ix - fs - (is-1) ds|. */
int geo_smooth_lines(float *v, int n, long long nlines, long long line_stride, long long elem_stride, int passes,
                     int mem, void *stream);
int geo_smooth2d(int nx, int rx, int nz, int rz, float *v, int mem, void *stream);
int geo_adcig_smooth_stack(int nx, int nz, int na, int passes, float *adcig, float *stack, int mem, void *stream);
int geo_mute_direct(int nx, int nt, float dt, float favg, float dx, float dz, int fs, int ds, int zs, int is,
                    float vp, float epsilon, int tt, float *shot, int mem, void *stream);

/* In-place model smoothers.  Both sweep the model Gauss-Seidel fashion
 * (each update reads neighbours already updated in the same pass), so the
 * result depends on the visiting order; they run on the host in the
 * programs' order (device buffers are copied through the host).
 * geo_smooth_model3d: utils-3D-smooth-f95/Toa_smooth3D.c:50-161 on
 *   v[iz + nz*(ix + nx*iy)]: `passes` passes over z >= mmz (1 <= mmz <= nz-2)
 *   -- 27-point inner average, 18-point faces, 12-point edges, 8-point
 *   corners; reads past a z column follow the program's memory layout.
 * geo_smooth_model2d: utils-3D-smooth-f95/smooth.f95:44-70 on v[ix*nz + iz]:
 *   `passes` passes of the 3x3 (1 2 1) weighted average over rows iz >= z0
 *   (the program's nzs - 1), with its 9- and 12-point edge forms. */
int geo_smooth_model3d(int nx, int ny, int nz, int passes, int mmz, float *v, int mem, void *stream);
int geo_smooth_model2d(int nx, int nz, int z0, int passes, float *v, int mem, void *stream);

/* ---- SU / SEG-Y traces ------------------------------------------------
 * A trace = 240-byte header (the segy struct of hc/cjbsegy.h) + ns floats.
 * geo_su_read: ntr traces into data[ntr*ns] (samples byte-swapped when
 *   big_endian; the MPI RTM program's seismic==2 model reader,
 *   2D-vti-fd+rtm-mpi/Toa_rtm_vti_adcig_cdp.c:1415-1453); headers (optional)
 *   receives the raw 240-byte headers.
 * geo_su_write: headers copied from `headers` when given, else generated
 *   (tracl = tracr = trace number, trid = 1, ns, dt in microseconds), header
 *   and samples big-endian when big_endian (SEG-Y trace order).
 * geo_su_replace_data: the binary2segy utility (utils-binary2segy/
 *   binary2segy.c:47-85): headers of the template file, samples from a raw
 *   native float file, byte-swapped. */
int geo_su_read(const char *path, int ntr, int ns, int big_endian, float *data, void *headers);
int geo_su_write(const char *path, int ntr, int ns, float dt_us, int big_endian, const float *data,
                 const void *headers);
int geo_su_replace_data(const char *template_path, const char *raw_path, const char *out_path, int ntr, int ns);

/* ---- learned snapshot codec (no reference counterpart) -----------------
 * A 4-level convolutional autoencoder over 16^3 blocks (kernel = stride = 2
 * per level, leaky ReLU, bf16 weights and activations, fp32 accumulation on
 * the tensor cores): 4096 fp32 points -> 512 bf16 + one fp32 scale.  It is
 * trained on the GPU on snapshots the solver generates. */
int geo_ae_create(geo_ae **ae, unsigned long long seed);
int geo_ae_destroy(geo_ae *ae);
size_t geo_ae_num_params(void);
/* Flat fp32 parameters: per level E1 E2 E3 E4 D4 D3 D2 D1, W [N x K] then b [N]. */
int geo_ae_get_params(geo_ae *ae, float *host);
int geo_ae_set_params(geo_ae *ae, const float *host);
/* Training store: room for max_blocks blocks (16 KiB each, device). */
int geo_ae_reserve(geo_ae *ae, long long max_blocks);
long long geo_ae_num_blocks(geo_ae *ae);
/* Append n blocks (Morton order within the block, raw amplitudes). */
int geo_ae_add_blocks(geo_ae *ae, const float *blocks, long long n, int mem);
/* Run shot `is` on a 3D plan and append, every snap_every steps from
 * t_first, the full interior blocks of P whose max |P| exceeds rel times
 * the snapshot's. */
int geo_ae_add_shot(geo_ae *ae, geo_fd3d_plan *plan, int is, int snap_every, int t_first, float rel,
                    void *stream);
/* iters Adam steps on batches of `batch` (multiple of 128) blocks drawn from
 * the store; loss (host, optional) receives each step's mean squared error
 * in block-normalized units. */
int geo_ae_train(geo_ae *ae, int iters, int batch, float lr, float *loss, void *stream);
/* Forward (and backward when grad != NULL) on nb (multiple of 128) given
 * blocks: recon = normalized reconstruction, loss = mean squared error,
 * grad = d loss / d params. */
int geo_ae_eval(geo_ae *ae, const float *blocks, int nb, float *recon, double *loss, float *grad, int mem,
                void *stream);
/* Encode + decode a dense nx*ny*nz volume (iz + nz*(ix + nx*iy), device);
 * with `escape`, blocks the code misses keep a bf16 residual (*nesc of them). */
int geo_ae_roundtrip(geo_ae *ae, int nx, int ny, int nz, const float *vol, float *out, int escape, int *nesc,
                     void *stream);
/* Escaped blocks: per snapshot, the blocks with the largest squared
 * decoding error (at most frac of the snapshot's blocks, and only blocks
 * whose error exceeds tau times their norm) keep their residual x - x' in
 * bf16 (8 KiB each).  Defaults tau 0.05, frac 0.03. */
int geo_ae_set_escape(geo_ae *ae, float tau, float frac);
/* Blocks coded and blocks escaped over the learned RTM shots run so far. */
int geo_ae_stats(geo_ae *ae, long long *blocks, long long *escaped);
/* The codec's tensor-core GEMM (device pointers, bf16 row-major A [M x K],
 * B [N x K]): out[M x N] = A * B^T (+bias) (leaky ReLU if act), fp32 or bf16
 * out.  M % 128, N % 64, K % 64 must be 0. */
int geo_tc_gemm_bf16(int M, int N, int K, const void *A, const void *B, const float *bias, int act, void *out,
                     int out_f32, void *stream);

/* ---- par file -------------------------------------------------------- */
/* `key= value` lines (the reference's .par format, e.g.
 * 2D-ISO-tomography-inversion-c-0.0/tomo-1.par) with the reference's
 * parameter names.  geo_par_get* look a key up after geo_par_load. */
typedef struct geo_par geo_par;
int geo_par_load(const char *path, geo_par **par);
int geo_par_get_int(const geo_par *par, const char *key, int *out);
int geo_par_get_float(const geo_par *par, const char *key, float *out);
int geo_par_get_string(const geo_par *par, const char *key, char *out, int cap);
void geo_par_free(geo_par *par);

/* Runs driven by a loaded par file.  device >= 0 makes that GPU current for
 * the call (the caller's current device is restored); -1 uses the current
 * one.  The result goes to the par file's output files and, when the device
 * pointer is not NULL, into that caller-owned device buffer as well.
 *
 * geo_fd2d: the shots of GPU_vti2dfd / CPU_vti2dfd
 *   (2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti2dfd_kernels.cu:301-444,
 *   CPU_vti2dfd_kernels.c:366-510).  Keys, named after those functions'
 *   arguments: nx nz dx dz npd nt dt (microseconds) favg ns fs ds zs FNv FNe
 *   FNd; optional FNshot (ns records nx*nt, trace-major), FNsnap (padded P of
 *   shot 1 every snap_every = 50 steps), SV, variant (gpu | cpu | mpi, default
 *   gpu), pfac (10), wtype (1), rec_iz (npd), mute_tt (100 for gpu, else 0).
 *   d_shots: ns*nx*nt.
 * geo_fd3d: the shots of GPU_vti3dfd (GPU_vti3dfd_kernels.cu:371-573),
 *   shots 0..ns-1.  Keys: nx ny nz dx dy dz npml nt dt (microseconds) favg ns
 *   fsx fsy fsz FNv FNe FNd; optional dsx dsy dsz, FNshot, SV, mode (exact |
 *   fast, default exact), pfac, wtype, rec_iz, rx0 drx nrx ry0 dry nry (every
 *   surface node by default), mute_tt (100), FNtheta FNphi (a 3D TTI medium:
 *   tilt and azimuth files in degrees, with mode fast; geo_fd3d_set_tilt).
 *   d_shots: ns*nt*nrx*nry.
 * geo_rtm2d: the MPI RTM program (2D-vti-fd+rtm-mpi/Toa_rtm_vti_adcig_cdp.c:
 *   59-481), shot is at fs_sxd + (is-1)*ds_sxd with an nxs-wide window.
 *   Keys, its variable names: nx nz dx dz npd nt dt (ms) favg pfac ns_sxd
 *   fs_sxd ds_sxd zs_sxd nxs FN1 FN2 FN3 (vp, epsilon, delta); optional seismic
 *   (1 raw floats, 2 SU), laplace (0: the program's raw stack), FN6 (stacked
 *   image), FN7 (per-shot images), FN8 (angle gathers, x-major), FN9
 *   (smoothed gathers) and FN10 (their stack) as the program writes them.
 *   d_image: nx*nz. */
/* Diagnostic without a reference counterpart: a kernel waits on a barrier
 * that nothing arrives on, through the bounded wait every pipeline wait of
 * the library uses, with a limit of limit_ms (1..2000).  *gave_up = 1 when
 * the wait gave up and the kernel reported it; GEO_OK means the kernel ended
 * and the context is usable -- what a stuck pipeline stage looks like to a
 * caller of the 3D step or the codec (GEO_ERR_CUDA, "... timed out"). */
int geo_selftest_bounded_wait(int limit_ms, int *gave_up, void *stream);
/* Diagnostic without a reference counterpart: the library's integer-pipe
 * float <-> double conversions (used in the MPI program's double chains)
 * against the hardware conversions on the device -- the widening over all
 * 2^32 binary32 patterns, the narrowing (round to nearest even) over
 * n_random binary64 values spanning underflow to overflow, exact ties and
 * binary32 images.  Mismatch counts in *f2d_bad, *d2f_bad. */
int geo_selftest_conversions(long long n_random, unsigned long long seed, long long *f2d_bad, long long *d2f_bad,
                             void *stream);

int geo_fd2d(const geo_par *par, int device, float *d_shots, void *stream);
int geo_fd3d(const geo_par *par, int device, float *d_shots, void *stream);
int geo_rtm2d(const geo_par *par, int device, float *d_image, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* GEOFD_H */
