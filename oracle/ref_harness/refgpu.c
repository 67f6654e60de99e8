/* Runs the reference's own GPU kernels, compiled unmodified from
 * 2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti3dfd_kernels.cu, GPU_vti2dfd_kernels.cu and
 * 2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu into cubins by
 * oracle/Makefile, through the CUDA driver API.
 *
 * Test infrastructure only (the parity pin of the oracle and of the
 * library's 3D and 2D GPU-variant paths); nothing in the product links it.
 *
 * Each entry point repeats, step for step, the host side of the reference
 * program it names -- the same padding, the same launch sequence and grid
 * shapes, the same float time accumulation, the same pointer assignment
 * that makes every update after step 0 run in place, the same mute -- with
 * arrays instead of file names.  All arithmetic of the reference program
 * runs on the GPU in its kernels, so every number in the output comes from
 * the reference's own compiled code:
 *
 *   refgpu_vti3d  GPU_vti3dfd  (GPU_vti3dfd_kernels.cu:371-574)
 *   refgpu_vti2d  GPU_vti2dfd  (GPU_vti2dfd_kernels.cu:301-484)
 *   refgpu_tti2d  the 2D TTI forward program's main()
 *                 (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:312-470)
 *   refgpu_rtm2d  the 2D GPU RTM program's RTM()
 *                 (2D-vti-fd+rtm-cuda/Toa_gpu2DvtiFdRtmAdcigsLaplace.cu:1184-1566)
 *   refgpu_rtm2d_tti  the 2D TTI GPU RTM program's main()
 *                 (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu:500-800)
 *   refgpu_rtm3d  the 3D GPU RTM program's main()
 *                 (3D-vti-fd+rtm-cuda/Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:686-981)
 *
 * Kernels are looked up by their C++ names in the module (the mangled name
 * starts with "_Z<len><name>").  Every index the launched kernels form was
 * checked against the buffers allocated here (the kernels guard their
 * points; the 3D y-sponge arrays are allocated with nny elements, so the
 * reference's nnx-sized allocation for them, GPU_vti3dfd_kernels.cu:471,474,
 * cannot be overrun here; callers still keep ny <= nx as that program needs).
 */
#include <cuda.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define CK(x)                                                                      \
    do {                                                                           \
        CUresult r_ = (x);                                                         \
        if (r_ != CUDA_SUCCESS) {                                                  \
            const char *s_ = 0;                                                    \
            cuGetErrorString(r_, &s_);                                             \
            fprintf(stderr, "refgpu: %s failed: %s (line %d)\n", #x, s_ ? s_ : "?", \
                    __LINE__);                                                     \
            rc = 1;                                                                \
            goto done;                                                             \
        }                                                                          \
    } while (0)

typedef struct {
    CUcontext ctx;
    CUmodule mod;
    int pushed;
} Rt;

static int rt_open(Rt *rt, const char *cubin) {
    int rc = 0;
    CUdevice dev;
    memset(rt, 0, sizeof *rt);
    CK(cuInit(0));
    CK(cuDeviceGet(&dev, 0));
    CK(cuDevicePrimaryCtxRetain(&rt->ctx, dev));
    CK(cuCtxPushCurrent(rt->ctx));
    rt->pushed = 1;
    CK(cuModuleLoad(&rt->mod, cubin));
done:
    return rc;
}

static void rt_close(Rt *rt) {
    CUdevice dev;
    if (rt->mod) cuModuleUnload(rt->mod);
    if (rt->pushed) {
        CUcontext c;
        cuCtxPopCurrent(&c);
    }
    if (rt->ctx && cuDeviceGet(&dev, 0) == CUDA_SUCCESS) cuDevicePrimaryCtxRelease(dev);
}

/* The kernel whose mangled name is _Z<strlen(name)><name>... */
static int find_fn(CUmodule mod, const char *name, CUfunction *out) {
    unsigned n = 0, i;
    CUfunction fs[64];
    char want[128];
    snprintf(want, sizeof want, "_Z%d%s", (int)strlen(name), name);
    if (cuModuleGetFunctionCount(&n, mod) != CUDA_SUCCESS || n > 64) return 1;
    if (cuModuleEnumerateFunctions(fs, n, mod) != CUDA_SUCCESS) return 1;
    for (i = 0; i < n; i++) {
        const char *nm = 0;
        if (cuFuncGetName(&nm, fs[i]) == CUDA_SUCCESS && nm && !strncmp(nm, want, strlen(want))) {
            *out = fs[i];
            return 0;
        }
    }
    fprintf(stderr, "refgpu: kernel %s not found in the module\n", name);
    return 1;
}

static CUresult launch(CUfunction f, unsigned gx, unsigned gy, unsigned bx, unsigned by, void **args) {
    return cuLaunchKernel(f, gx, gy, 1, bx, by, 1, 0, 0, args, 0);
}

/* pad_vv3d (GPU_vti3dfd_kernels.cu:203-245): x faces, then y, then z. */
static void pad3(int nnx, int nny, int nnz, int npml, float *ee) {
    int ix, iy, iz;
    for (iy = 0; iy < nny; iy++)
        for (ix = 0; ix < nnx; ix++)
            for (iz = 0; iz < nnz; iz++) {
                size_t id = iz + (size_t)ix * nnz + (size_t)iy * nnz * nnx;
                if (ix < npml) ee[id] = ee[iz + (size_t)npml * nnz + (size_t)iy * nnz * nnx];
                else if (ix >= nnx - npml) ee[id] = ee[iz + (size_t)(nnx - npml - 1) * nnz + (size_t)iy * nnz * nnx];
            }
    for (iy = 0; iy < nny; iy++)
        for (ix = 0; ix < nnx; ix++)
            for (iz = 0; iz < nnz; iz++) {
                size_t id = iz + (size_t)ix * nnz + (size_t)iy * nnz * nnx;
                if (iy < npml) ee[id] = ee[iz + (size_t)ix * nnz + (size_t)npml * nnz * nnx];
                else if (iy >= nny - npml) ee[id] = ee[iz + (size_t)ix * nnz + (size_t)(nny - npml - 1) * nnz * nnx];
            }
    for (iy = 0; iy < nny; iy++)
        for (ix = 0; ix < nnx; ix++)
            for (iz = 0; iz < nnz; iz++) {
                size_t id = iz + (size_t)ix * nnz + (size_t)iy * nnz * nnx;
                if (iz < npml) ee[id] = ee[npml + (size_t)ix * nnz + (size_t)iy * nnz * nnx];
                else if (iz >= nnz - npml) ee[id] = ee[nnz - npml - 1 + (size_t)ix * nnz + (size_t)iy * nnz * nnx];
            }
}

/* GPU_vti3dfd with arrays: v, e, d hold nx*ny*nz floats in the model
 * files' order (z fastest, then x, then y); shot receives ns records of
 * nt*nx*ny floats (trace-major, shot[it + nt*ix + nt*nx*iy]); snap, when
 * not NULL, receives the interior window of P of shot 0 at it = 300, 600,
 * ... (nsnap = (nt-1)/300 windows of nx*ny*nz).  *ms_per_step receives the
 * device time of the time loops divided by ns*nt. */
int refgpu_vti3d(const char *cubin, int nx, int ny, int nz, int dx, int dy, int dz, int npml, int SV,
                 const float *v_in, const float *e_in, const float *d_in, int favg, int ns, int fsx, int dsx,
                 int fsy, int dsy, int fsz, int dsz, int nt, int dt, float *shot, float *snap,
                 float *ms_per_step) {
    int rc = 0, is, it, ix, iy, iz, wtype = 1, tt = 100;
    int nnx = nx + 2 * npml, nny = ny + 2 * npml, nnz = nz + 2 * npml;
    size_t nn = (size_t)nnx * nny * nnz, nb = nn * sizeof(float);
    float dx_ = (float)dx, dy_ = (float)dy, dz_ = (float)dz, favg_ = (float)favg;
    float dt_ = (float)(dt * 1.0 / 1000000), pfac = 10.0f, t;
    float *v = 0, *e = 0, *d = 0, *win = 0;
    Rt rt;
    CUfunction f_src, f_vel, f_str, f_d0, f_coff, f_rec, f_mute;
    CUdeviceptr vp = 0, eps = 0, del = 0, P = 0, Q = 0, shotd = 0;
    CUdeviceptr u[2] = {0, 0}, vv[2] = {0, 0}, w[2] = {0, 0};
    CUdeviceptr px[2] = {0, 0}, py[2] = {0, 0}, pz[2] = {0, 0}, qx[2] = {0, 0}, qy[2] = {0, 0}, qz[2] = {0, 0};
    CUdeviceptr cf[12] = {0};
    CUevent ev0 = 0, ev1 = 0;
    float tot_ms = 0.f;
    CUdeviceptr *all[] = {&vp, &eps, &del, &P, &Q, &u[0], &u[1], &vv[0], &vv[1], &w[0], &w[1], &px[0], &px[1],
                          &py[0], &py[1], &pz[0], &pz[1], &qx[0], &qx[1], &qy[0], &qy[1], &qz[0], &qz[1]};
    size_t nall = sizeof all / sizeof all[0], k;

    if (rt_open(&rt, cubin)) {
        rt_close(&rt);
        return 1;
    }
    if (find_fn(rt.mod, "add_source3d", &f_src) || find_fn(rt.mod, "update_vel3d", &f_vel) ||
        find_fn(rt.mod, "update_stress3d", &f_str) || find_fn(rt.mod, "get_d03d", &f_d0) ||
        find_fn(rt.mod, "initial_coffe3d", &f_coff) || find_fn(rt.mod, "shot_record3d", &f_rec) ||
        find_fn(rt.mod, "mute_directwave3d", &f_mute)) {
        rc = 1;
        goto done;
    }
    v = (float *)calloc(nn, sizeof(float));
    e = (float *)calloc(nn, sizeof(float));
    d = (float *)calloc(nn, sizeof(float));
    if (!v || !e || !d) {
        rc = 1;
        goto done;
    }
    /* read_file3d (GPU_vti3dfd_kernels.cu:247-279) */
    k = 0;
    for (iy = npml; iy < ny + npml; iy++)
        for (ix = npml; ix < nx + npml; ix++)
            for (iz = npml; iz < nz + npml; iz++, k++) {
                size_t id = iz + (size_t)ix * nnz + (size_t)iy * nnz * nnx;
                v[id] = v_in[k];
                e[id] = e_in[k];
                d[id] = d_in[k];
            }
    pad3(nnx, nny, nnz, npml, e);
    pad3(nnx, nny, nnz, npml, d);
    pad3(nnx, nny, nnz, npml, v);

    for (k = 0; k < nall; k++) CK(cuMemAlloc(all[k], nb));
    CK(cuMemAlloc(&cf[0], nnx * 4)); CK(cuMemAlloc(&cf[1], nnx * 4)); /* coffx1/2 */
    CK(cuMemAlloc(&cf[2], nny * 4)); CK(cuMemAlloc(&cf[3], nny * 4)); /* coffy1/2 */
    CK(cuMemAlloc(&cf[4], nnz * 4)); CK(cuMemAlloc(&cf[5], nnz * 4)); /* coffz1/2 */
    CK(cuMemAlloc(&cf[6], nnx * 4)); CK(cuMemAlloc(&cf[7], nnx * 4)); /* acoffx1/2 */
    CK(cuMemAlloc(&cf[8], nny * 4)); CK(cuMemAlloc(&cf[9], nny * 4)); /* acoffy1/2 */
    CK(cuMemAlloc(&cf[10], nnz * 4)); CK(cuMemAlloc(&cf[11], nnz * 4)); /* acoffz1/2 */
    CK(cuMemAlloc(&shotd, (size_t)nt * nx * ny * 4));
    CK(cuMemcpyHtoD(vp, v, nb));
    CK(cuMemcpyHtoD(eps, e, nb));
    CK(cuMemcpyHtoD(del, d, nb));
    CK(cuEventCreate(&ev0, CU_EVENT_DEFAULT));
    CK(cuEventCreate(&ev1, CU_EVENT_DEFAULT));
    {
        void *a[] = {&dx_, &dy_, &dz_, &nnx, &nny, &nnz, &npml, &vp};
        CK(launch(f_d0, 1, 1, 1, 1, a));
    }
    {
        void *ax[] = {&dt_, &nx, &cf[0], &cf[1], &cf[6], &cf[7], &npml};
        void *ay[] = {&dt_, &ny, &cf[2], &cf[3], &cf[8], &cf[9], &npml};
        void *az[] = {&dt_, &nz, &cf[4], &cf[5], &cf[10], &cf[11], &npml};
        CK(launch(f_coff, (nnx + 511) / 512, 1, 512, 1, ax));
        CK(launch(f_coff, (nny + 511) / 512, 1, 512, 1, ay));
        CK(launch(f_coff, (nnz + 511) / 512, 1, 512, 1, az));
    }
    {
        /* the program's buffers: index 0 = "...0" pointer, 1 = "...1";
         * after step 0 the program assigns s_u0 = s_u1 etc. (in place). */
        CUdeviceptr u0 = u[0], u1 = u[1], v0 = vv[0], v1 = vv[1], w0 = w[0], w1 = w[1];
        CUdeviceptr px0 = px[0], px1 = px[1], py0 = py[0], py1 = py[1], pz0 = pz[0], pz1 = pz[1];
        CUdeviceptr qx0 = qx[0], qx1 = qx[1], qy0 = qy[0], qy1 = qy[1], qz0 = qz[0], qz1 = qz[1];
        unsigned gzx = (nnz + 15) / 16, gxx = (nnx + 15) / 16, Xgx = (nnx + 15) / 16, Xgy = (nny + 15) / 16;
        if (snap) win = (float *)malloc(nb);
        for (is = 0; is < ns; is++) {
            for (k = 3; k < nall; k++) CK(cuMemsetD32(*all[k], 0, nn));
            CK(cuMemsetD32(u0, 0, nn)); CK(cuMemsetD32(u1, 0, nn));
            CK(cuMemsetD32(shotd, 0, (size_t)nt * nx * ny));
            CK(cuEventRecord(ev0, 0));
            for (it = 0, t = dt_; it < nt; it++, t += dt_) {
                void *as[] = {&pfac, &fsx, &fsy, &fsz, &nx, &ny, &nz, &nnx, &nny, &nnz, &dt_, &t, &favg_,
                              &wtype, &npml, &is, &dsx, &dsy, &dsz, &P, &Q};
                void *av[] = {&nx, &ny, &nz, &nnx, &nny, &nnz, &npml, &dt_, &dx_, &dy_, &dz_, &u0, &v0, &w0,
                              &u1, &v1, &w1, &P, &Q, &cf[0], &cf[1], &cf[2], &cf[3], &cf[4], &cf[5]};
                void *ap[] = {&nx, &ny, &nz, &nnx, &nny, &nnz, &dt_, &dx_, &dy_, &dz_, &u1, &v1, &w1, &P, &Q,
                              &vp, &npml, &px1, &px0, &py1, &py0, &pz1, &pz0, &qx1, &qx0, &qy1, &qy0, &qz1,
                              &qz0, &cf[6], &cf[7], &cf[8], &cf[9], &cf[10], &cf[11], &del, &eps, &fsx, &dsx,
                              &fsy, &dsy, &fsz, &dsz, &is, &SV};
                void *ar[] = {&nnx, &nny, &nnz, &nx, &ny, &nz, &npml, &it, &nt, &P, &shotd};
                CK(launch(f_src, 1, 1, 1, 1, as));
                CK(launch(f_vel, gzx, gxx, 16, 16, av));
                CK(launch(f_str, gzx, gxx, 16, 16, ap));
                u0 = u1; v0 = v1; w0 = w1; px0 = px1; py0 = py1; pz0 = pz1; qx0 = qx1; qy0 = qy1; qz0 = qz1;
                CK(launch(f_rec, (nx * ny + 511) / 512, 1, 512, 1, ar));
                if (snap && is == 0 && it != 0 && it % 300 == 0) {
                    float *dst = snap + (size_t)(it / 300 - 1) * nx * ny * nz;
                    CK(cuMemcpyDtoH(win, P, nb));
                    for (iy = 0; iy < ny; iy++)
                        for (ix = 0; ix < nx; ix++)
                            for (iz = 0; iz < nz; iz++)
                                dst[iz + (size_t)nz * ix + (size_t)nz * nx * iy] =
                                    win[(iz + npml) + (size_t)nnz * (ix + npml) + (size_t)nnz * nnx * (iy + npml)];
                }
            }
            CK(cuEventRecord(ev1, 0));
            CK(cuEventSynchronize(ev1));
            {
                float ms = 0.f;
                CK(cuEventElapsedTime(&ms, ev0, ev1));
                tot_ms += ms;
            }
            {
                void *am[] = {&nx, &ny, &nt, &dt_, &favg_, &dx_, &dy_, &dz_, &fsx, &fsy, &dsx, &dsy, &fsz, &is,
                              &vp, &eps, &shotd, &tt};
                CK(launch(f_mute, Xgx, Xgy, 16, 16, am));
            }
            CK(cuMemcpyDtoH(shot + (size_t)is * nt * nx * ny, shotd, (size_t)nt * nx * ny * 4));
        }
    }
    CK(cuCtxSynchronize());
    if (ms_per_step) *ms_per_step = tot_ms / (float)(ns * nt);
done:
    for (k = 0; k < nall; k++)
        if (*all[k]) cuMemFree(*all[k]);
    for (k = 0; k < 12; k++)
        if (cf[k]) cuMemFree(cf[k]);
    if (shotd) cuMemFree(shotd);
    if (ev0) cuEventDestroy(ev0);
    if (ev1) cuEventDestroy(ev1);
    rt_close(&rt);
    free(v); free(e); free(d); free(win);
    return rc;
}

/* pad_vv2d (GPU_vti2dfd_kernels.cu:48-73): x faces, then z. */
static void pad2(int nnx, int nnz, int npd, float *ee) {
    int id;
    for (id = 0; id < nnx * nnz; id++) {
        int ix = id / nnz, iz = id % nnz;
        if (ix < npd) ee[id] = ee[npd * nnz + iz];
        else if (ix >= nnx - npd) ee[id] = ee[(nnx - npd - 1) * nnz + iz];
    }
    for (id = 0; id < nnx * nnz; id++) {
        int ix = id / nnz, iz = id % nnz;
        if (iz < npd) ee[id] = ee[ix * nnz + npd];
        else if (iz >= nnz - npd) ee[id] = ee[ix * nnz + nnz - npd - 1];
    }
}

/* GPU_vti2dfd with arrays: v, e, d hold nx*nz floats in the model files'
 * order (z fastest); shot receives ns records of nt*nx floats
 * (shot[it + nt*ix], muted); snap, when not NULL, receives the padded P of
 * shot 1 at it = 0, 50, 100, ... ((nt-1)/50 + 1 fields of nnx*nnz). */
int refgpu_vti2d(const char *cubin, int nx, int nz, int dx, int dz, int npd, int SV, const float *v_in,
                 const float *e_in, const float *d_in, int favg, int ns, int fs, int ds, int zs, int nt, int dt,
                 float *shot, float *snap, float *ms_per_step) {
    int rc = 0, is, it, ix, iz, wtype = 1, tt = 100;
    int nnx = nx + 2 * npd, nnz = nz + 2 * npd;
    size_t nn = (size_t)nnx * nnz, nb = nn * sizeof(float);
    float dx_ = (float)dx, dz_ = (float)dz, favg_ = (float)favg, dt_ = (float)(dt * 1.0 / 1000000);
    float pfac = 10.0f, t, xsn = (float)fs, zsn = (float)zs;
    float *v = 0, *e = 0, *d = 0;
    Rt rt;
    CUfunction f_src, f_vel, f_str, f_d0, f_coff, f_rec, f_mute;
    CUdeviceptr vp = 0, eps = 0, del = 0, P = 0, Q = 0, shotd = 0;
    CUdeviceptr u[2] = {0, 0}, w[2] = {0, 0}, px[2] = {0, 0}, pz[2] = {0, 0}, qx[2] = {0, 0}, qz[2] = {0, 0};
    CUdeviceptr cf[8] = {0};
    CUevent ev0 = 0, ev1 = 0;
    float tot_ms = 0.f;
    CUdeviceptr *all[] = {&vp, &eps, &del, &P, &Q, &u[0], &u[1], &w[0], &w[1], &px[0], &px[1],
                          &pz[0], &pz[1], &qx[0], &qx[1], &qz[0], &qz[1]};
    size_t nall = sizeof all / sizeof all[0], k;

    if (rt_open(&rt, cubin)) {
        rt_close(&rt);
        return 1;
    }
    if (find_fn(rt.mod, "add_source2d", &f_src) || find_fn(rt.mod, "update_vel2d", &f_vel) ||
        find_fn(rt.mod, "update_stress2d", &f_str) || find_fn(rt.mod, "get_d02d", &f_d0) ||
        find_fn(rt.mod, "initial_coffe2d", &f_coff) || find_fn(rt.mod, "shot_record2d", &f_rec) ||
        find_fn(rt.mod, "mute_directwave2d", &f_mute)) {
        rc = 1;
        goto done;
    }
    v = (float *)calloc(nn, sizeof(float));
    e = (float *)calloc(nn, sizeof(float));
    d = (float *)calloc(nn, sizeof(float));
    if (!v || !e || !d) {
        rc = 1;
        goto done;
    }
    /* read_file2d (GPU_vti2dfd_kernels.cu:75-100) */
    k = 0;
    for (ix = npd; ix < nx + npd; ix++)
        for (iz = npd; iz < nz + npd; iz++, k++) {
            v[ix * nnz + iz] = v_in[k];
            e[ix * nnz + iz] = e_in[k];
            d[ix * nnz + iz] = d_in[k];
        }
    pad2(nnx, nnz, npd, e);
    pad2(nnx, nnz, npd, d);
    pad2(nnx, nnz, npd, v);

    for (k = 0; k < nall; k++) CK(cuMemAlloc(all[k], nb));
    CK(cuMemAlloc(&cf[0], nnx * 4)); CK(cuMemAlloc(&cf[1], nnx * 4)); /* coffx1/2 */
    CK(cuMemAlloc(&cf[2], nnz * 4)); CK(cuMemAlloc(&cf[3], nnz * 4)); /* coffz1/2 */
    CK(cuMemAlloc(&cf[4], nnx * 4)); CK(cuMemAlloc(&cf[5], nnx * 4)); /* acoffx1/2 */
    CK(cuMemAlloc(&cf[6], nnz * 4)); CK(cuMemAlloc(&cf[7], nnz * 4)); /* acoffz1/2 */
    CK(cuMemAlloc(&shotd, (size_t)nt * nx * 4));
    CK(cuMemcpyHtoD(vp, v, nb));
    CK(cuMemcpyHtoD(eps, e, nb));
    CK(cuMemcpyHtoD(del, d, nb));
    CK(cuEventCreate(&ev0, CU_EVENT_DEFAULT));
    CK(cuEventCreate(&ev1, CU_EVENT_DEFAULT));
    {
        void *a[] = {&dx_, &dz_, &nnx, &nnz, &npd, &vp};
        CK(launch(f_d0, 1, 1, 1, 1, a));
    }
    {
        void *ax[] = {&dt_, &nx, &cf[0], &cf[1], &cf[4], &cf[5], &npd};
        void *az[] = {&dt_, &nz, &cf[2], &cf[3], &cf[6], &cf[7], &npd};
        CK(launch(f_coff, (nnx + 511) / 512, 1, 512, 1, ax));
        CK(launch(f_coff, (nnz + 511) / 512, 1, 512, 1, az));
    }
    {
        CUdeviceptr u0 = u[0], u1 = u[1], w0 = w[0], w1 = w[1];
        CUdeviceptr px0 = px[0], px1 = px[1], pz0 = pz[0], pz1 = pz[1];
        CUdeviceptr qx0 = qx[0], qx1 = qx[1], qz0 = qz[0], qz1 = qz[1];
        unsigned g = (unsigned)((nn + 511) / 512);
        for (is = 1; is <= ns; is++) {
            for (k = 3; k < nall; k++) CK(cuMemsetD32(*all[k], 0, nn));
            CK(cuMemsetD32(shotd, 0, (size_t)nt * nx));
            CK(cuEventRecord(ev0, 0));
            for (it = 0, t = dt_; it < nt; it++, t += dt_) {
                void *as[] = {&pfac, &xsn, &zsn, &nx, &nz, &nnx, &nnz, &dt_, &t, &favg_, &wtype, &npd, &is, &ds,
                              &P, &Q};
                void *av[] = {&nx, &nz, &nnx, &nnz, &npd, &dt_, &dx_, &dz_, &u0, &w0, &u1, &w1, &P, &Q,
                              &cf[0], &cf[1], &cf[2], &cf[3]};
                void *ap[] = {&nx, &nz, &nnx, &nnz, &dt_, &dx_, &dz_, &u1, &w1, &P, &Q, &vp, &npd, &px1, &px0,
                              &pz1, &pz0, &qx1, &qx0, &qz1, &qz0, &cf[4], &cf[5], &cf[6], &cf[7], &del, &eps,
                              &fs, &ds, &zs, &is, &SV};
                void *ar[] = {&nnx, &nnz, &nx, &nz, &npd, &it, &nt, &P, &shotd};
                CK(launch(f_src, 1, 1, 1, 1, as));
                CK(launch(f_vel, g, 1, 512, 1, av));
                CK(launch(f_str, g, 1, 512, 1, ap));
                u0 = u1; w0 = w1; px0 = px1; pz0 = pz1; qx0 = qx1; qz0 = qz1;
                CK(launch(f_rec, (nx + 511) / 512, 1, 512, 1, ar));
                if (snap && is == 1 && it % 50 == 0) CK(cuMemcpyDtoH(snap + (size_t)(it / 50) * nn, P, nb));
            }
            CK(cuEventRecord(ev1, 0));
            CK(cuEventSynchronize(ev1));
            {
                float ms = 0.f;
                CK(cuEventElapsedTime(&ms, ev0, ev1));
                tot_ms += ms;
            }
            {
                void *am[] = {&nx, &nt, &dt_, &favg_, &dx_, &dz_, &fs, &ds, &zs, &is, &vp, &eps, &shotd, &tt};
                CK(launch(f_mute, (nx * nt + 511) / 512, 1, 512, 1, am));
            }
            CK(cuMemcpyDtoH(shot + (size_t)(is - 1) * nt * nx, shotd, (size_t)nt * nx * 4));
        }
    }
    CK(cuCtxSynchronize());
    if (ms_per_step) *ms_per_step = tot_ms / (float)(ns * nt);
done:
    for (k = 0; k < nall; k++)
        if (*all[k]) cuMemFree(*all[k]);
    for (k = 0; k < 8; k++)
        if (cf[k]) cuMemFree(cf[k]);
    if (shotd) cuMemFree(shotd);
    if (ev0) cuEventDestroy(ev0);
    if (ev1) cuEventDestroy(ev1);
    rt_close(&rt);
    free(v); free(e); free(d);
    return rc;
}

/* The 2D TTI GPU program (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:
 * main, :312-470) with arrays: v, e, d, theta (degrees, converted as its
 * read_file does, :235) hold nx*nz floats, z fastest; shot receives ns
 * records of nt*nx floats (not muted: the program's mute call is commented
 * out); snap, when not NULL, receives the padded P of shot 1 at it = 100,
 * 200, ... ((nt-1)/100 fields).  dx, dz, dt, favg, pfac are the program's
 * float parameters; SV is its update_stress flag (the program passes false). */
int refgpu_tti2d(const char *cubin, int nx, int nz, float dx, float dz, int npml, int SV, const float *v_in,
                 const float *e_in, const float *d_in, const float *th_in, float favg, float pfac, int ns, int fs,
                 int ds, int zs, int nt, float dt, float *shot, float *snap, float *ms_per_step) {
    int rc = 0, is, it, ix, iz, wtype = 1;
    int nnx = nx + 2 * npml, nnz = nz + 2 * npml;
    size_t nn = (size_t)nnx * nnz, nb = nn * sizeof(float);
    float t, xsn = (float)fs, zsn = (float)zs;
    unsigned char sv = SV ? 1 : 0;
    float *v = 0, *e = 0, *d = 0, *b = 0;
    Rt rt;
    CUfunction f_src, f_vel, f_str, f_d0, f_coff, f_rec;
    CUdeviceptr vp = 0, eps = 0, del = 0, th = 0, P = 0, Q = 0, shotd = 0;
    CUdeviceptr u[2] = {0, 0}, w[2] = {0, 0}, px[2] = {0, 0}, pz[2] = {0, 0}, qx[2] = {0, 0}, qz[2] = {0, 0};
    CUdeviceptr cf[8] = {0};
    CUevent ev0 = 0, ev1 = 0;
    float tot_ms = 0.f;
    CUdeviceptr *all[] = {&vp, &eps, &del, &th, &P, &Q, &u[0], &u[1], &w[0], &w[1], &px[0], &px[1],
                          &pz[0], &pz[1], &qx[0], &qx[1], &qz[0], &qz[1]};
    size_t nall = sizeof all / sizeof all[0], k;

    if (rt_open(&rt, cubin)) {
        rt_close(&rt);
        return 1;
    }
    if (find_fn(rt.mod, "add_source", &f_src) || find_fn(rt.mod, "update_vel", &f_vel) ||
        find_fn(rt.mod, "update_stress", &f_str) || find_fn(rt.mod, "get_d0", &f_d0) ||
        find_fn(rt.mod, "initial_coffe", &f_coff) || find_fn(rt.mod, "shot_record", &f_rec)) {
        rc = 1;
        goto done;
    }
    v = (float *)calloc(nn, sizeof(float));
    e = (float *)calloc(nn, sizeof(float));
    d = (float *)calloc(nn, sizeof(float));
    b = (float *)calloc(nn, sizeof(float));
    if (!v || !e || !d || !b) {
        rc = 1;
        goto done;
    }
    /* read_file (:206-236): theta in degrees *= pi/180 (pi = 3.141592653) */
    k = 0;
    for (ix = npml; ix < nx + npml; ix++)
        for (iz = npml; iz < nz + npml; iz++, k++) {
            v[ix * nnz + iz] = v_in[k];
            e[ix * nnz + iz] = e_in[k];
            d[ix * nnz + iz] = d_in[k];
            b[ix * nnz + iz] = (float)(th_in[k] * (3.141592653 / 180.0));
        }
    pad2(nnx, nnz, npml, e);
    pad2(nnx, nnz, npml, d);
    pad2(nnx, nnz, npml, v);
    pad2(nnx, nnz, npml, b);

    for (k = 0; k < nall; k++) CK(cuMemAlloc(all[k], nb));
    CK(cuMemAlloc(&cf[0], nnx * 4)); CK(cuMemAlloc(&cf[1], nnx * 4)); /* coffx1/2 */
    CK(cuMemAlloc(&cf[2], nnz * 4)); CK(cuMemAlloc(&cf[3], nnz * 4)); /* coffz1/2 */
    CK(cuMemAlloc(&cf[4], nnx * 4)); CK(cuMemAlloc(&cf[5], nnx * 4)); /* acoffx1/2 */
    CK(cuMemAlloc(&cf[6], nnz * 4)); CK(cuMemAlloc(&cf[7], nnz * 4)); /* acoffz1/2 */
    CK(cuMemAlloc(&shotd, (size_t)nt * nx * 4));
    CK(cuMemcpyHtoD(vp, v, nb));
    CK(cuMemcpyHtoD(eps, e, nb));
    CK(cuMemcpyHtoD(del, d, nb));
    CK(cuMemcpyHtoD(th, b, nb));
    CK(cuEventCreate(&ev0, CU_EVENT_DEFAULT));
    CK(cuEventCreate(&ev1, CU_EVENT_DEFAULT));
    {
        void *a[] = {&dx, &dz, &nnx, &nnz, &npml, &vp};
        CK(launch(f_d0, 1, 1, 1, 1, a));
    }
    {
        void *ax[] = {&dt, &nx, &cf[0], &cf[1], &cf[4], &cf[5], &npml};
        void *az[] = {&dt, &nz, &cf[2], &cf[3], &cf[6], &cf[7], &npml};
        CK(launch(f_coff, (nnx + 511) / 512, 1, 512, 1, ax));
        CK(launch(f_coff, (nnz + 511) / 512, 1, 512, 1, az));
    }
    {
        CUdeviceptr u0 = u[0], u1 = u[1], w0 = w[0], w1 = w[1];
        CUdeviceptr px0 = px[0], px1 = px[1], pz0 = pz[0], pz1 = pz[1];
        CUdeviceptr qx0 = qx[0], qx1 = qx[1], qz0 = qz[0], qz1 = qz[1];
        unsigned g = (unsigned)((nn + 511) / 512);
        for (is = 1; is <= ns; is++) {
            for (k = 4; k < nall; k++) CK(cuMemsetD32(*all[k], 0, nn));
            CK(cuMemsetD32(shotd, 0, (size_t)nt * nx));
            CK(cuEventRecord(ev0, 0));
            for (it = 0, t = dt; it < nt; it++, t += dt) {
                void *as[] = {&pfac, &xsn, &zsn, &nx, &nz, &nnx, &nnz, &dt, &t, &favg, &wtype, &npml, &is, &ds,
                              &P, &Q};
                void *av[] = {&nx, &nz, &nnx, &nnz, &npml, &dt, &dx, &dz, &u0, &w0, &u1, &w1, &P, &Q,
                              &cf[0], &cf[1], &cf[2], &cf[3], &th};
                void *ap[] = {&nx, &nz, &nnx, &nnz, &dt, &dx, &dz, &u1, &w1, &P, &Q, &vp, &npml, &px1, &px0,
                              &pz1, &pz0, &qx1, &qx0, &qz1, &qz0, &cf[4], &cf[5], &cf[6], &cf[7], &del, &eps,
                              &th, &fs, &ds, &zs, &is, &sv};
                void *ar[] = {&nnx, &nnz, &nx, &nz, &npml, &it, &nt, &P, &shotd};
                CK(launch(f_src, 1, 1, 1, 1, as));
                CK(launch(f_vel, g, 1, 512, 1, av));
                CK(launch(f_str, g, 1, 512, 1, ap));
                u0 = u1; w0 = w1; px0 = px1; pz0 = pz1; qx0 = qx1; qz0 = qz1;
                CK(launch(f_rec, (nx + 511) / 512, 1, 512, 1, ar));
                if (snap && is == 1 && it % 100 == 0 && it != 0)
                    CK(cuMemcpyDtoH(snap + (size_t)(it / 100 - 1) * nn, P, nb));
            }
            CK(cuEventRecord(ev1, 0));
            CK(cuEventSynchronize(ev1));
            {
                float ms = 0.f;
                CK(cuEventElapsedTime(&ms, ev0, ev1));
                tot_ms += ms;
            }
            CK(cuMemcpyDtoH(shot + (size_t)(is - 1) * nt * nx, shotd, (size_t)nt * nx * 4));
        }
    }
    CK(cuCtxSynchronize());
    if (ms_per_step) *ms_per_step = tot_ms / (float)(ns * nt);
done:
    for (k = 0; k < nall; k++)
        if (*all[k]) cuMemFree(*all[k]);
    for (k = 0; k < 8; k++)
        if (cf[k]) cuMemFree(cf[k]);
    if (shotd) cuMemFree(shotd);
    if (ev0) cuEventDestroy(ev0);
    if (ev1) cuEventDestroy(ev1);
    rt_close(&rt);
    free(v); free(e); free(d); free(b);
    return rc;
}


/* cos and sin of n angles (radians) by the device (k_ref_trig of
 * oracle/ref_harness/trig.cu, loaded from `cubin`). */
int refgpu_cuda_trig(const char *cubin, const float *th, float *c, float *s, long n) {
    int rc = 0;
    Rt rt;
    CUfunction f;
    CUdeviceptr dth = 0, dc = 0, ds = 0;
    size_t nb = (size_t)n * sizeof(float);
    if (rt_open(&rt, cubin)) {
        rt_close(&rt);
        return 1;
    }
    CK(cuModuleGetFunction(&f, rt.mod, "k_ref_trig"));
    CK(cuMemAlloc(&dth, nb));
    CK(cuMemAlloc(&dc, nb));
    CK(cuMemAlloc(&ds, nb));
    CK(cuMemcpyHtoD(dth, th, nb));
    {
        void *a[] = {&dth, &dc, &ds, &n};
        unsigned g = (unsigned)((n + 255) / 256);
        CK(launch(f, g > 1024 ? 1024 : g, 1, 256, 1, a));
    }
    CK(cuMemcpyDtoH(c, dc, nb));
    CK(cuMemcpyDtoH(s, ds, nb));
done:
    if (dth) cuMemFree(dth);
    if (dc) cuMemFree(dc);
    if (ds) cuMemFree(ds);
    rt_close(&rt);
    return rc;
}


/* The two 2D GPU RTM programs share their host side: per shot, zero every
 * field, step the source field forward (add_source, update_vel,
 * update_stress with the SV taper, then the record, the ring of P,Q just
 * outside the interior and the illumination), mute the record, then step
 * backward: restore the ring into the source field and step it again,
 * write the record into the receiver field's P and Q and step it, image
 * and angle gathers.  After the shots the image and the gathers are
 * divided by the illumination.  Differences, by `tti`:
 *   VTI (Toa_gpu2DvtiFdRtmAdcigsLaplace.cu RTM() :1184-1566): observed
 *     records may replace the modelled ones (readShot); mute tt = 20 over
 *     (nt+511)/512 blocks of samples, each looping over the traces;
 *     gathers at every trace;
 *   TTI (Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu main :500-800): the
 *     tilt field enters update_vel, update_stress and the mute; mute tt =
 *     30 over (nx*nt+511)/512 blocks; gathers at every dcdp-th trace.
 * The image and gather kernels form field indices from thread ids past the
 * image (cal_illumination / cal_migration test id < nnx*nnz on nx*nz
 * arrays; Poynting_Adcigs reads before its bounds test; the VTI mute has no
 * bound on the sample; the TTI adcigs_illum bounds by nx*nz/dcdp*na): every
 * such index is computed below for the launch shapes used and the buffers
 * are allocated to cover it, zero-filled, so no launch reads or writes
 * outside memory allocated here.  The values written there are outside
 * the outputs. */

static size_t umax(size_t a, size_t b) { return a > b ? a : b; }

static int rtm2d_prog(int tti, const char *cubin, int nx, int nz, int npml, int nt, float dx, float dz, float dt,
                      float favg, float pfac, int wtype, int ns, int fs, int ds, int zs, int na, int da, int dcdp,
                      const float *v_in, const float *e_in, const float *d_in, const float *th_in, const float *obs,
                      float *mig_out, float *ill_out, float *ag_out, float *shots, float *ms_per_step) {
    int rc = 0, is, it, ix, iz, tt = tti ? 30 : 20;
    const int nnx = nx + 2 * npml, nnz = nz + 2 * npml, L = 2 * nx + 2 * nz;
    const int nxa = tti ? nx / dcdp : nx;
    const size_t nn = (size_t)nnx * nnz;
    float t, xsn = (float)fs, zsn = (float)zs;
    unsigned char yes = 1, no = 0;
    float *v = 0, *e = 0, *d = 0, *b = 0, *rec = 0;
    Rt rt;
    CUfunction f_src, f_vel, f_str, f_d0, f_coff, f_rec, f_mute, f_bnd, f_ill, f_mig, f_migi, f_poy, f_agi;
    /* fields: 0..11 source (u0 u1 w0 w1 P Q px0 px1 pz0 pz1 qx0 qx1, qz0 qz1 below), receiver likewise */
    CUdeviceptr sf[14] = {0}, gf[14] = {0};
    CUdeviceptr vp = 0, eps = 0, del = 0, th = 0, shotd = 0, pb = 0, qb = 0, mig = 0, ill = 0, ag = 0;
    CUdeviceptr cf[8] = {0};
    CUevent ev0 = 0, ev1 = 0;
    float tot_ms = 0.f;
    size_t k, nfield, nimg, nag, nshot;
    const unsigned gimg = (unsigned)(((size_t)nx * nz + 511) / 512);
    const unsigned gpoy = (unsigned)(((size_t)nxa * nz + 511) / 512);
    const unsigned gagi = (unsigned)(((size_t)nxa * nz * na + 511) / 512);
    const unsigned gmute = tti ? (unsigned)(((size_t)nx * nt + 511) / 512) : (unsigned)((nt + 511) / 512);

    /* the largest index each launch forms (see above) */
    {
        size_t top_img = (size_t)gimg * 512 - 1, top_poy = (size_t)gpoy * 512 - 1;
        size_t ixi = top_img / nz, ixp = (top_poy / nz) * (tti ? dcdp : 1);
        size_t agi_lim = (size_t)gagi * 512, agi_bound = tti ? (size_t)nx * nz / dcdp * na : (size_t)nx * nz * na;
        size_t agi_top = (agi_lim < agi_bound ? agi_lim : agi_bound) - 1;
        size_t agi_ix = tti ? agi_top / ((size_t)nz * na) * dcdp : agi_top / ((size_t)nz * na);
        nfield = umax(nn, umax((size_t)nz - 1 + npml + (size_t)nnz * (ixi + npml),
                               (size_t)nz - 1 + npml + (size_t)nnz * (ixp + npml)) + 1);
        nimg = umax(top_img + 1, (size_t)nz - 1 + (size_t)nz * agi_ix + 1);
        nag = umax((size_t)nxa * nz * na, agi_top + 1);
        nshot = (size_t)nx * nt + (tti ? 0 : (size_t)gmute * 512);
    }

    if (rt_open(&rt, cubin)) {
        rt_close(&rt);
        return 1;
    }
    if (find_fn(rt.mod, "add_source", &f_src) || find_fn(rt.mod, "update_vel", &f_vel) ||
        find_fn(rt.mod, "update_stress", &f_str) || find_fn(rt.mod, "get_d0", &f_d0) ||
        find_fn(rt.mod, "initial_coffe", &f_coff) || find_fn(rt.mod, "shot_record", &f_rec) ||
        find_fn(rt.mod, "mute_directwave", &f_mute) || find_fn(rt.mod, "wavefield_bndr", &f_bnd) ||
        find_fn(rt.mod, "cal_illumination", &f_ill) || find_fn(rt.mod, "cal_migration", &f_mig) ||
        find_fn(rt.mod, "migration_illum", &f_migi) || find_fn(rt.mod, "Poynting_Adcigs", &f_poy) ||
        find_fn(rt.mod, "adcigs_illum", &f_agi)) {
        rc = 1;
        goto done;
    }
    v = (float *)calloc(nn, sizeof(float));
    e = (float *)calloc(nn, sizeof(float));
    d = (float *)calloc(nn, sizeof(float));
    b = (float *)calloc(nn, sizeof(float));
    rec = (float *)calloc((size_t)nt * nx, sizeof(float));
    if (!v || !e || !d || !b || !rec) {
        rc = 1;
        goto done;
    }
    /* readFile / read_file: the interior in file order, the TTI tilt in
     * degrees *= pi/180 (pi = 3.141592653), then edge padding */
    k = 0;
    for (ix = npml; ix < nx + npml; ix++)
        for (iz = npml; iz < nz + npml; iz++, k++) {
            v[ix * nnz + iz] = v_in[k];
            e[ix * nnz + iz] = e_in[k];
            d[ix * nnz + iz] = d_in[k];
            if (tti) b[ix * nnz + iz] = (float)(th_in[k] * (3.141592653 / 180.0));
        }
    pad2(nnx, nnz, npml, e);
    pad2(nnx, nnz, npml, d);
    pad2(nnx, nnz, npml, v);
    if (tti) pad2(nnx, nnz, npml, b);

    CK(cuMemAlloc(&vp, nn * 4)); CK(cuMemAlloc(&eps, nn * 4)); CK(cuMemAlloc(&del, nn * 4));
    CK(cuMemAlloc(&th, nn * 4));
    for (k = 0; k < 14; k++) {
        CK(cuMemAlloc(&sf[k], nfield * 4));
        CK(cuMemAlloc(&gf[k], nfield * 4));
    }
    CK(cuMemAlloc(&cf[0], nnx * 4)); CK(cuMemAlloc(&cf[1], nnx * 4)); /* coffx1/2 */
    CK(cuMemAlloc(&cf[2], nnz * 4)); CK(cuMemAlloc(&cf[3], nnz * 4)); /* coffz1/2 */
    CK(cuMemAlloc(&cf[4], nnx * 4)); CK(cuMemAlloc(&cf[5], nnx * 4)); /* acoffx1/2 */
    CK(cuMemAlloc(&cf[6], nnz * 4)); CK(cuMemAlloc(&cf[7], nnz * 4)); /* acoffz1/2 */
    CK(cuMemAlloc(&shotd, nshot * 4));
    CK(cuMemAlloc(&pb, (size_t)nt * L * 4)); CK(cuMemAlloc(&qb, (size_t)nt * L * 4));
    CK(cuMemAlloc(&mig, nimg * 4)); CK(cuMemAlloc(&ill, nimg * 4)); CK(cuMemAlloc(&ag, nag * 4));
    CK(cuMemcpyHtoD(vp, v, nn * 4));
    CK(cuMemcpyHtoD(eps, e, nn * 4));
    CK(cuMemcpyHtoD(del, d, nn * 4));
    CK(cuMemcpyHtoD(th, b, nn * 4));
    CK(cuMemsetD32(mig, 0, nimg)); CK(cuMemsetD32(ill, 0, nimg)); CK(cuMemsetD32(ag, 0, nag));
    CK(cuEventCreate(&ev0, CU_EVENT_DEFAULT));
    CK(cuEventCreate(&ev1, CU_EVENT_DEFAULT));
    {
        void *a[] = {&dx, &dz, (void *)&nnx, (void *)&nnz, &npml, &vp};
        CK(launch(f_d0, 1, 1, 1, 1, a));
    }
    {
        void *ax[] = {&dt, &nx, &cf[0], &cf[1], &cf[4], &cf[5], &npml};
        void *az[] = {&dt, &nz, &cf[2], &cf[3], &cf[6], &cf[7], &npml};
        CK(launch(f_coff, (nnx + 511) / 512, 1, 512, 1, ax));
        CK(launch(f_coff, (nnz + 511) / 512, 1, 512, 1, az));
    }
    for (is = 1; is <= ns; is++) {
        /* the program's pointer assignments (u0 = u1, ...): after the
         * first step every update runs in place */
        CUdeviceptr su0 = sf[0], su1 = sf[1], sw0 = sf[2], sw1 = sf[3], sP = sf[4], sQ = sf[5];
        CUdeviceptr spx0 = sf[6], spx1 = sf[7], spz0 = sf[8], spz1 = sf[9], sqx0 = sf[10], sqx1 = sf[11];
        CUdeviceptr sqz0 = sf[12], sqz1 = sf[13];
        CUdeviceptr gu0 = gf[0], gu1 = gf[1], gw0 = gf[2], gw1 = gf[3], gP = gf[4], gQ = gf[5];
        CUdeviceptr gpx0 = gf[6], gpx1 = gf[7], gpz0 = gf[8], gpz1 = gf[9], gqx0 = gf[10], gqx1 = gf[11];
        CUdeviceptr gqz0 = gf[12], gqz1 = gf[13];
        const unsigned g = (unsigned)((nn + 511) / 512);
        for (k = 0; k < 14; k++) {
            CK(cuMemsetD32(sf[k], 0, nfield));
            CK(cuMemsetD32(gf[k], 0, nfield));
        }
        CK(cuMemsetD32(shotd, 0, nshot));
        CK(cuMemsetD32(pb, 0, (size_t)nt * L));
        CK(cuMemsetD32(qb, 0, (size_t)nt * L));
        CK(cuEventRecord(ev0, 0));
        for (it = 0, t = dt; it < nt; it++, t += dt) {
            void *as[] = {&pfac, &xsn, &zsn, &nx, &nz, (void *)&nnx, (void *)&nnz, &dt, &t, &favg, &wtype, &npml,
                          &is, &ds, &sP, &sQ};
            void *av[] = {&nx, &nz, (void *)&nnx, (void *)&nnz, &npml, &dt, &dx, &dz, &su0, &sw0, &su1, &sw1, &sP,
                          &sQ, &cf[0], &cf[1], &cf[2], &cf[3], &th};
            void *ap_v[] = {&nx, &nz, (void *)&nnx, (void *)&nnz, &dt, &dx, &dz, &su1, &sw1, &sP, &sQ, &vp, &npml,
                            &spx1, &spx0, &spz1, &spz0, &sqx1, &sqx0, &sqz1, &sqz0, &cf[4], &cf[5], &cf[6],
                            &cf[7], &del, &eps, &fs, &ds, &zs, &is, &yes};
            void *ap_t[] = {&nx, &nz, (void *)&nnx, (void *)&nnz, &dt, &dx, &dz, &su1, &sw1, &sP, &sQ, &vp, &npml,
                            &spx1, &spx0, &spz1, &spz0, &sqx1, &sqx0, &sqz1, &sqz0, &cf[4], &cf[5], &cf[6],
                            &cf[7], &del, &eps, &th, &fs, &ds, &zs, &is, &yes};
            void *ar[] = {(void *)&nnx, (void *)&nnz, &nx, &nz, &npml, &it, &nt, &sP, &shotd, &yes};
            void *ab[] = {(void *)&nnx, (void *)&nnz, &nx, &nz, &npml, &it, &nt, &sP, &sQ, &pb, &qb, &yes};
            void *ai[] = {(void *)&nnx, (void *)&nnz, &nz, &npml, &ill, &sP, &sQ};
            CK(launch(f_src, 1, 1, 1, 1, as));
            CK(launch(f_vel, g, 1, 512, 1, av));   /* the VTI kernel ignores the trailing argument */
            CK(launch(f_str, g, 1, 512, 1, tti ? ap_t : ap_v));
            su0 = su1; sw0 = sw1; spx0 = spx1; spz0 = spz1; sqx0 = sqx1; sqz0 = sqz1;
            CK(launch(f_rec, (nx + 511) / 512, 1, 512, 1, ar));
            CK(launch(f_bnd, (L + 511) / 512, 1, 512, 1, ab));
            CK(launch(f_ill, gimg, 1, 512, 1, ai));
        }
        {
            void *am_v[] = {&nx, &nt, &dt, &favg, &dx, &dz, &fs, &ds, &zs, &is, &vp, &eps, &shotd, &tt};
            void *am_t[] = {&nx, &nt, &dt, &favg, &dx, &dz, &fs, &ds, &zs, &is, &vp, &eps, &th, &shotd, &tt};
            CK(launch(f_mute, gmute, 1, 512, 1, tti ? am_t : am_v));
        }
        CK(cuMemcpyDtoH(rec, shotd, (size_t)nt * nx * 4));
        if (shots) memcpy(shots + (size_t)(is - 1) * nt * nx, rec, (size_t)nt * nx * 4);
        if (!tti && obs) CK(cuMemcpyHtoD(shotd, obs + (size_t)(is - 1) * nt * nx, (size_t)nt * nx * 4));
        for (it = nt - 1; it >= 0; it--) {
            void *ab[] = {(void *)&nnx, (void *)&nnz, &nx, &nz, &npml, &it, &nt, &sP, &sQ, &pb, &qb, &no};
            void *av[] = {&nx, &nz, (void *)&nnx, (void *)&nnz, &npml, &dt, &dx, &dz, &su0, &sw0, &su1, &sw1, &sP,
                          &sQ, &cf[0], &cf[1], &cf[2], &cf[3], &th};
            void *ap_v[] = {&nx, &nz, (void *)&nnx, (void *)&nnz, &dt, &dx, &dz, &su1, &sw1, &sP, &sQ, &vp, &npml,
                            &spx1, &spx0, &spz1, &spz0, &sqx1, &sqx0, &sqz1, &sqz0, &cf[4], &cf[5], &cf[6],
                            &cf[7], &del, &eps, &fs, &ds, &zs, &is, &no};
            void *ap_t[] = {&nx, &nz, (void *)&nnx, (void *)&nnz, &dt, &dx, &dz, &su1, &sw1, &sP, &sQ, &vp, &npml,
                            &spx1, &spx0, &spz1, &spz0, &sqx1, &sqx0, &sqz1, &sqz0, &cf[4], &cf[5], &cf[6],
                            &cf[7], &del, &eps, &th, &fs, &ds, &zs, &is, &no};
            CK(launch(f_bnd, (L + 511) / 512, 1, 512, 1, ab));
            CK(launch(f_vel, g, 1, 512, 1, av));
            CK(launch(f_str, g, 1, 512, 1, tti ? ap_t : ap_v));
            su0 = su1; sw0 = sw1; spx0 = spx1; spz0 = spz1; sqx0 = sqx1; sqz0 = sqz1;
            {
                void *arP[] = {(void *)&nnx, (void *)&nnz, &nx, &nz, &npml, &it, &nt, &gP, &shotd, &no};
                void *arQ[] = {(void *)&nnx, (void *)&nnz, &nx, &nz, &npml, &it, &nt, &gQ, &shotd, &no};
                void *gv[] = {&nx, &nz, (void *)&nnx, (void *)&nnz, &npml, &dt, &dx, &dz, &gu0, &gw0, &gu1, &gw1, &gP,
                              &gQ, &cf[0], &cf[1], &cf[2], &cf[3], &th};
                void *gp_v[] = {&nx, &nz, (void *)&nnx, (void *)&nnz, &dt, &dx, &dz, &gu1, &gw1, &gP, &gQ, &vp,
                                &npml, &gpx1, &gpx0, &gpz1, &gpz0, &gqx1, &gqx0, &gqz1, &gqz0, &cf[4], &cf[5],
                                &cf[6], &cf[7], &del, &eps, &fs, &ds, &zs, &is, &no};
                void *gp_t[] = {&nx, &nz, (void *)&nnx, (void *)&nnz, &dt, &dx, &dz, &gu1, &gw1, &gP, &gQ, &vp,
                                &npml, &gpx1, &gpx0, &gpz1, &gpz0, &gqx1, &gqx0, &gqz1, &gqz0, &cf[4], &cf[5],
                                &cf[6], &cf[7], &del, &eps, &th, &fs, &ds, &zs, &is, &no};
                CK(launch(f_rec, (nx + 511) / 512, 1, 512, 1, arP));
                CK(launch(f_rec, (nx + 511) / 512, 1, 512, 1, arQ));
                CK(launch(f_vel, g, 1, 512, 1, gv));
                CK(launch(f_str, g, 1, 512, 1, tti ? gp_t : gp_v));
            }
            gu0 = gu1; gw0 = gw1; gpx0 = gpx1; gpz0 = gpz1; gqx0 = gqx1; gqz0 = gqz1;
            {
                void *am[] = {(void *)&nnx, (void *)&nnz, &nz, &npml, &mig, &sP, &gP};
                void *ag_v[] = {(void *)&nnz, &nx, &nz, &npml, &na, &da, &ag, &sP, &sQ, &su0, &sw0, &gP, &gQ,
                                &gu0, &gw0};
                void *ag_t[] = {(void *)&nnz, &nx, &nz, &npml, &na, &da, &dcdp, &ag, &sP, &sQ, &su0, &sw0, &gP,
                                &gQ, &gu0, &gw0};
                CK(launch(f_mig, gimg, 1, 512, 1, am));
                CK(launch(f_poy, gpoy, 1, 512, 1, tti ? ag_t : ag_v));
            }
        }
        CK(cuEventRecord(ev1, 0));
        CK(cuEventSynchronize(ev1));
        {
            float ms = 0.f;
            CK(cuEventElapsedTime(&ms, ev0, ev1));
            tot_ms += ms;
        }
    }
    {
        void *a1[] = {&nx, &nz, &npml, &mig, &ill};
        void *a2_v[] = {&nx, &nz, &na, &da, &ag, &ill};
        void *a2_t[] = {&nx, &nz, &na, &da, &dcdp, &ag, &ill};
        CK(launch(f_migi, gimg, 1, 512, 1, a1));
        CK(launch(f_agi, gagi, 1, 512, 1, tti ? a2_t : a2_v));
    }
    CK(cuCtxSynchronize());
    CK(cuMemcpyDtoH(mig_out, mig, (size_t)nx * nz * 4));
    CK(cuMemcpyDtoH(ill_out, ill, (size_t)nx * nz * 4));
    if (ag_out) CK(cuMemcpyDtoH(ag_out, ag, (size_t)nxa * nz * na * 4));
    if (ms_per_step) *ms_per_step = tot_ms / (float)(ns * nt);
done:
    if (vp) cuMemFree(vp);
    if (eps) cuMemFree(eps);
    if (del) cuMemFree(del);
    if (th) cuMemFree(th);
    for (k = 0; k < 14; k++) {
        if (sf[k]) cuMemFree(sf[k]);
        if (gf[k]) cuMemFree(gf[k]);
    }
    for (k = 0; k < 8; k++)
        if (cf[k]) cuMemFree(cf[k]);
    if (shotd) cuMemFree(shotd);
    if (pb) cuMemFree(pb);
    if (qb) cuMemFree(qb);
    if (mig) cuMemFree(mig);
    if (ill) cuMemFree(ill);
    if (ag) cuMemFree(ag);
    if (ev0) cuEventDestroy(ev0);
    if (ev1) cuEventDestroy(ev1);
    rt_close(&rt);
    free(v); free(e); free(d); free(b); free(rec);
    return rc;
}

/* The 2D GPU RTM program's RTM() with arrays: v, e, d hold nx*nz floats, z
 * fastest; obs (optional) holds ns observed records of nt*nx floats
 * (readShot); mig (the image divided by the illumination, before the
 * program's host Laplacian), ill: nx*nz; adcigs: nx*na*nz [ix][ia][iz]
 * divided by the illumination; shots: the muted modelled records, ns*nx*nt. */
int refgpu_rtm2d(const char *cubin, int nx, int nz, int npml, int nt, float dx, float dz, float dt, float favg,
                 float pfac, int wtype, int ns, int fs, int ds, int zs, int na, int da, const float *v,
                 const float *e, const float *d, const float *obs, float *mig, float *ill, float *adcigs,
                 float *shots, float *ms_per_step) {
    return rtm2d_prog(0, cubin, nx, nz, npml, nt, dx, dz, dt, favg, pfac, wtype, ns, fs, ds, zs, na, da, 1, v, e,
                      d, NULL, obs, mig, ill, adcigs, shots, ms_per_step);
}

/* The 2D TTI GPU RTM program's main() with arrays: theta in degrees; adcigs
 * (nx/dcdp)*na*nz; no observed records (the program images its own). */
int refgpu_rtm2d_tti(const char *cubin, int nx, int nz, int npml, int nt, float dx, float dz, float dt, float favg,
                     float pfac, int wtype, int ns, int fs, int ds, int zs, int na, int da, int dcdp,
                     const float *v, const float *e, const float *d, const float *theta, float *mig, float *ill,
                     float *adcigs, float *shots, float *ms_per_step) {
    return rtm2d_prog(1, cubin, nx, nz, npml, nt, dx, dz, dt, favg, pfac, wtype, ns, fs, ds, zs, na, da, dcdp, v,
                      e, d, theta, NULL, mig, ill, adcigs, shots, ms_per_step);
}

/* The 3D GPU RTM program's main()
 * (3D-vti-fd+rtm-cuda/Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:686-981)
 * with arrays: v, e, d hold nx*ny*nz floats, z fastest, then x, then y;
 * shots is = 0..ns-1 at (fsx + is*dsx, fsy + is*dsy, zs).  Per shot: zero
 * every field, step the source field forward with the SV taper (add_source,
 * update_vel, update_stress, then the ring of P,Q on the six faces just
 * outside the interior, the record P+Q at z = npml, the illumination), mute
 * the record (tt = 70), then step backward: restore the ring into the
 * source field and step it again, write the record into the receiver
 * field's P and Q at z = npml-1 and step it, illumination of the receiver
 * field, image and angle gathers.  After the shots the image and the
 * gathers are divided by the illumination where it is not zero.  The
 * launch shapes are the program's: 16x16 blocks over (nnz, nnx) marching
 * in y for the stencils and images, over (nnx, nny) for the mute and over
 * (nz, nx/dcdp) for the gathers; every kernel bounds its indices (the
 * stencils read the model at wrapped ids below nnx*nny*nnz - 4 only).  The
 * y sponge arrays get nny elements (the program allocates nnx,
 * :811-812,819-820; cases keep ny <= nx as it needs).
 * mig, ill: nx*ny*nz; adcigs: (ny/dcdp)*(nx/dcdp)*na*nz [iy][ix][ia][iz];
 * shots: the muted records, ns*ny*nx*nt. */
int refgpu_rtm3d(const char *cubin, int nx, int ny, int nz, int npml, int nt, float dx, float dy, float dz, float dt,
                 float favg, float pfac, int ns, int fsx, int dsx, int fsy, int dsy, int zs, int na, int da, int dcdp,
                 const float *v_in, const float *e_in, const float *d_in, float *mig_out, float *ill_out,
                 float *ag_out, float *shots, float *ms_per_step) {
    int rc = 0, is, it, ix, iy, iz, wtype = 1, tt = 70, nsx = 1;
    const int nnx = nx + 2 * npml, nny = ny + 2 * npml, nnz = nz + 2 * npml;
    const int nxa = nx / dcdp, nya = ny / dcdp;
    const size_t nn = (size_t)nnx * nny * nnz, n0 = (size_t)nx * ny * nz;
    const size_t L = 2 * (size_t)nx * ny + 2 * (size_t)nz * ny + 2 * (size_t)nx * nz;
    const size_t nag = (size_t)nya * nxa * na * nz;
    float t;
    unsigned char yes = 1, no = 0;
    float *v = 0, *e = 0, *d = 0;
    Rt rt;
    CUfunction f_src, f_vel, f_str, f_d0, f_coff, f_rec, f_mute, f_bnd, f_ill, f_mig, f_migi, f_poy, f_agi;
    /* fields: u0 u1 v0 v1 w0 w1 P Q px0 px1 py0 py1 pz0 pz1 qx0 qx1 qy0 qy1 qz0 qz1 */
    CUdeviceptr sf[20] = {0}, gf[20] = {0};
    CUdeviceptr vp = 0, eps = 0, del = 0, shotd = 0, pb = 0, qb = 0, mig = 0, ill = 0, ag = 0;
    CUdeviceptr cf[12] = {0};
    CUevent ev0 = 0, ev1 = 0;
    float tot_ms = 0.f;
    size_t k;
    const unsigned gz = (unsigned)((nnz + 15) / 16), gx = (unsigned)((nnx + 15) / 16);
    const unsigned mx = (unsigned)((nnx + 15) / 16), my = (unsigned)((nny + 15) / 16);
    const unsigned az_ = (unsigned)((nz + 15) / 16), ax_ = (unsigned)((nxa + 15) / 16);
    const unsigned gb = (unsigned)((L + 511) / 512), gr = (unsigned)(((size_t)nx * ny + 511) / 512);
    const int nyc = nny > nnx ? nny : nnx;

    if (rt_open(&rt, cubin)) {
        rt_close(&rt);
        return 1;
    }
    if (find_fn(rt.mod, "add_source", &f_src) || find_fn(rt.mod, "update_vel", &f_vel) ||
        find_fn(rt.mod, "update_stress", &f_str) || find_fn(rt.mod, "get_d0", &f_d0) ||
        find_fn(rt.mod, "initial_coffe", &f_coff) || find_fn(rt.mod, "shot_record", &f_rec) ||
        find_fn(rt.mod, "mute_directwave", &f_mute) || find_fn(rt.mod, "wavefield_bndr", &f_bnd) ||
        find_fn(rt.mod, "cal_illumination", &f_ill) || find_fn(rt.mod, "cal_migration", &f_mig) ||
        find_fn(rt.mod, "migration_illum", &f_migi) || find_fn(rt.mod, "Poynting_Adcigs", &f_poy) ||
        find_fn(rt.mod, "adcigs_illum", &f_agi)) {
        rc = 1;
        goto done;
    }
    v = (float *)calloc(nn, sizeof(float));
    e = (float *)calloc(nn, sizeof(float));
    d = (float *)calloc(nn, sizeof(float));
    if (!v || !e || !d) {
        rc = 1;
        goto done;
    }
    /* read_file (:261-284), then pad_vv (:212-259) */
    k = 0;
    for (iy = npml; iy < ny + npml; iy++)
        for (ix = npml; ix < nx + npml; ix++)
            for (iz = npml; iz < nz + npml; iz++, k++) {
                size_t id = iz + (size_t)ix * nnz + (size_t)iy * nnz * nnx;
                v[id] = v_in[k];
                e[id] = e_in[k];
                d[id] = d_in[k];
            }
    pad3(nnx, nny, nnz, npml, e);
    pad3(nnx, nny, nnz, npml, d);
    pad3(nnx, nny, nnz, npml, v);

    CK(cuMemAlloc(&vp, nn * 4)); CK(cuMemAlloc(&eps, nn * 4)); CK(cuMemAlloc(&del, nn * 4));
    for (k = 0; k < 20; k++) {
        CK(cuMemAlloc(&sf[k], nn * 4));
        CK(cuMemAlloc(&gf[k], nn * 4));
    }
    CK(cuMemAlloc(&cf[0], nnx * 4)); CK(cuMemAlloc(&cf[1], nnx * 4));   /* coffx1/2 */
    CK(cuMemAlloc(&cf[2], nyc * 4)); CK(cuMemAlloc(&cf[3], nyc * 4));   /* coffy1/2 */
    CK(cuMemAlloc(&cf[4], nnz * 4)); CK(cuMemAlloc(&cf[5], nnz * 4));   /* coffz1/2 */
    CK(cuMemAlloc(&cf[6], nnx * 4)); CK(cuMemAlloc(&cf[7], nnx * 4));   /* acoffx1/2 */
    CK(cuMemAlloc(&cf[8], nyc * 4)); CK(cuMemAlloc(&cf[9], nyc * 4));   /* acoffy1/2 */
    CK(cuMemAlloc(&cf[10], nnz * 4)); CK(cuMemAlloc(&cf[11], nnz * 4)); /* acoffz1/2 */
    CK(cuMemAlloc(&shotd, (size_t)nt * nx * ny * 4));
    CK(cuMemAlloc(&pb, (size_t)nt * L * 4)); CK(cuMemAlloc(&qb, (size_t)nt * L * 4));
    CK(cuMemAlloc(&mig, n0 * 4)); CK(cuMemAlloc(&ill, n0 * 4)); CK(cuMemAlloc(&ag, nag * 4));
    CK(cuMemcpyHtoD(vp, v, nn * 4));
    CK(cuMemcpyHtoD(eps, e, nn * 4));
    CK(cuMemcpyHtoD(del, d, nn * 4));
    CK(cuMemsetD32(mig, 0, n0)); CK(cuMemsetD32(ill, 0, n0)); CK(cuMemsetD32(ag, 0, nag));
    CK(cuEventCreate(&ev0, CU_EVENT_DEFAULT));
    CK(cuEventCreate(&ev1, CU_EVENT_DEFAULT));
    {
        void *a[] = {&dx, &dy, &dz, (void *)&nnx, (void *)&nny, (void *)&nnz, &npml, &vp};
        CK(launch(f_d0, 1, 1, 1, 1, a));
    }
    {
        void *ax[] = {&dt, &nx, &cf[0], &cf[1], &cf[6], &cf[7], &npml};
        void *ay[] = {&dt, &ny, &cf[2], &cf[3], &cf[8], &cf[9], &npml};
        void *az[] = {&dt, &nz, &cf[4], &cf[5], &cf[10], &cf[11], &npml};
        CK(launch(f_coff, (nnx + 511) / 512, 1, 512, 1, ax));
        CK(launch(f_coff, (nny + 511) / 512, 1, 512, 1, ay));
        CK(launch(f_coff, (nnz + 511) / 512, 1, 512, 1, az));
    }
    for (is = 0; is < ns; is++) {
        /* the program's pointer assignments (u0 = u1, ...): every update
         * after the first runs in place */
        CUdeviceptr s[20], g[20];
        for (k = 0; k < 20; k++) {
            s[k] = sf[k];
            g[k] = gf[k];
            CK(cuMemsetD32(sf[k], 0, nn));
            CK(cuMemsetD32(gf[k], 0, nn));
        }
        CK(cuMemsetD32(pb, 0, (size_t)nt * L));
        CK(cuMemsetD32(qb, 0, (size_t)nt * L));
        CK(cuMemsetD32(shotd, 0, (size_t)nt * nx * ny));
        CK(cuEventRecord(ev0, 0));
#define VEL3(f) void *av[] = {&nx, &ny, &nz, (void *)&nnx, (void *)&nny, (void *)&nnz, &npml, &dt, &dx, &dy, &dz, \
        &f[0], &f[2], &f[4], &f[1], &f[3], &f[5], &f[6], &f[7], &cf[0], &cf[1], &cf[2], &cf[3], &cf[4], &cf[5]}
#define STR3(f) void *ap[] = {&nx, &ny, &nz, (void *)&nnx, (void *)&nny, (void *)&nnz, &dt, &dx, &dy, &dz, \
        &f[1], &f[3], &f[5], &f[6], &f[7], &vp, &npml, &f[9], &f[8], &f[11], &f[10], &f[13], &f[12], \
        &f[15], &f[14], &f[17], &f[16], &f[19], &f[18], &cf[6], &cf[7], &cf[8], &cf[9], &cf[10], &cf[11], \
        &del, &eps, &fsx, &dsx, &fsy, &dsy, &zs, &is, &nsx, &yes}
#define SWAP3(f) do { f[0] = f[1]; f[2] = f[3]; f[4] = f[5]; f[8] = f[9]; f[10] = f[11]; f[12] = f[13]; \
        f[14] = f[15]; f[16] = f[17]; f[18] = f[19]; } while (0)
        for (it = 0, t = dt; it < nt; it++, t += dt) {
            void *as[] = {&pfac, &fsx, &fsy, &zs, &nx, &ny, &nz, (void *)&nnx, (void *)&nny, (void *)&nnz, &dt, &t,
                          &favg, &wtype, &npml, &is, &dsx, &dsy, &s[6], &s[7], &nsx};
            VEL3(s);
            STR3(s);
            CK(launch(f_src, 1, 1, 1, 1, as));
            CK(launch(f_vel, gz, gx, 16, 16, av));
            CK(launch(f_str, gz, gx, 16, 16, ap));
            SWAP3(s);
            {
                void *ab[] = {(void *)&nnx, (void *)&nny, (void *)&nnz, &nx, &ny, &nz, &npml, &it, &nt, &s[6], &s[7],
                              &pb, &qb, &yes};
                void *ar[] = {(void *)&nnx, (void *)&nny, (void *)&nnz, &nx, &ny, &nz, &npml, &it, &nt, &s[6], &s[7],
                              &shotd, &yes};
                void *ai[] = {(void *)&nnx, (void *)&nny, (void *)&nnz, &nx, &ny, &nz, &npml, &ill, &s[6], &s[7]};
                CK(launch(f_bnd, gb, 1, 512, 1, ab));
                CK(launch(f_rec, gr, 1, 512, 1, ar));
                CK(launch(f_ill, gz, gx, 16, 16, ai));
            }
        }
        {
            void *am[] = {&nx, &ny, &nt, &dt, &favg, &dx, &dy, &dz, &fsx, &fsy, &dsx, &dsy, &zs, &is, &vp, &eps,
                          &shotd, &tt, &nsx};
            CK(launch(f_mute, mx, my, 16, 16, am));
        }
        if (shots) CK(cuMemcpyDtoH(shots + (size_t)is * nt * nx * ny, shotd, (size_t)nt * nx * ny * 4));
        for (it = nt - 1; it >= 0; it--) {
            {
                void *ab[] = {(void *)&nnx, (void *)&nny, (void *)&nnz, &nx, &ny, &nz, &npml, &it, &nt, &s[6], &s[7],
                              &pb, &qb, &no};
                VEL3(s);
                STR3(s);
                CK(launch(f_bnd, gb, 1, 512, 1, ab));
                CK(launch(f_vel, gz, gx, 16, 16, av));
                CK(launch(f_str, gz, gx, 16, 16, ap));
                SWAP3(s);
            }
            {
                void *ar[] = {(void *)&nnx, (void *)&nny, (void *)&nnz, &nx, &ny, &nz, &npml, &it, &nt, &g[6], &g[7],
                              &shotd, &no};
                VEL3(g);
                STR3(g);
                CK(launch(f_rec, gr, 1, 512, 1, ar));
                CK(launch(f_vel, gz, gx, 16, 16, av));
                CK(launch(f_str, gz, gx, 16, 16, ap));
                SWAP3(g);
            }
            {
                void *ai[] = {(void *)&nnx, (void *)&nny, (void *)&nnz, &nx, &ny, &nz, &npml, &ill, &g[6], &g[7]};
                void *am[] = {(void *)&nnx, (void *)&nny, (void *)&nnz, &nx, &ny, &nz, &npml, &mig, &s[6], &g[6]};
                void *ap[] = {(void *)&nnx, (void *)&nny, (void *)&nnz, &nx, &ny, &nz, &npml, &na, &da, &ag, &dcdp,
                              &s[6], &s[7], &s[0], &s[2], &s[4], &g[6], &g[7], &g[0], &g[2], &g[4]};
                CK(launch(f_ill, gz, gx, 16, 16, ai));
                CK(launch(f_mig, gz, gx, 16, 16, am));
                CK(launch(f_poy, az_, ax_, 16, 16, ap));
            }
        }
#undef VEL3
#undef STR3
#undef SWAP3
        CK(cuEventRecord(ev1, 0));
        CK(cuEventSynchronize(ev1));
        {
            float ms = 0.f;
            CK(cuEventElapsedTime(&ms, ev0, ev1));
            tot_ms += ms;
        }
    }
    {
        void *a1[] = {(void *)&nnx, (void *)&nny, (void *)&nnz, &nx, &ny, &nz, &npml, &ill, &mig};
        void *a2[] = {(void *)&nnx, (void *)&nny, (void *)&nnz, &nx, &ny, &nz, &npml, &na, &ag, &dcdp, &ill};
        CK(launch(f_migi, gz, gx, 16, 16, a1));
        CK(launch(f_agi, az_, ax_, 16, 16, a2));
    }
    CK(cuCtxSynchronize());
    CK(cuMemcpyDtoH(mig_out, mig, n0 * 4));
    CK(cuMemcpyDtoH(ill_out, ill, n0 * 4));
    if (ag_out) CK(cuMemcpyDtoH(ag_out, ag, nag * 4));
    if (ms_per_step) *ms_per_step = tot_ms / (float)(ns * nt);
done:
    if (vp) cuMemFree(vp);
    if (eps) cuMemFree(eps);
    if (del) cuMemFree(del);
    for (k = 0; k < 20; k++) {
        if (sf[k]) cuMemFree(sf[k]);
        if (gf[k]) cuMemFree(gf[k]);
    }
    for (k = 0; k < 12; k++)
        if (cf[k]) cuMemFree(cf[k]);
    if (shotd) cuMemFree(shotd);
    if (pb) cuMemFree(pb);
    if (qb) cuMemFree(qb);
    if (mig) cuMemFree(mig);
    if (ill) cuMemFree(ill);
    if (ag) cuMemFree(ag);
    if (ev0) cuEventDestroy(ev0);
    if (ev1) cuEventDestroy(ev1);
    rt_close(&rt);
    free(v); free(e); free(d);
    return rc;
}


/* Counts the floats a in [-1, 1] whose Poynting bin by the device's acosf
 * differs from the count of thresholds thr[0..na) at or above a
 * (k_ref_bin_check of oracle/ref_harness/trig.cu, loaded from `cubin`). */
int refgpu_bin_check(const char *cubin, const float *thr, int na, int da, unsigned long long *bad) {
    int rc = 0;
    Rt rt;
    CUfunction f;
    CUdeviceptr dthr = 0, dbad = 0;
    if (rt_open(&rt, cubin)) {
        rt_close(&rt);
        return 1;
    }
    CK(cuModuleGetFunction(&f, rt.mod, "k_ref_bin_check"));
    CK(cuMemAlloc(&dthr, (size_t)(na > 0 ? na : 1) * 4));
    CK(cuMemAlloc(&dbad, 8));
    if (na > 0) CK(cuMemcpyHtoD(dthr, thr, (size_t)na * 4));
    CK(cuMemsetD32(dbad, 0, 2));
    {
        void *a[] = {&dthr, &na, &da, &dbad};
        CK(launch(f, 152 * 16, 1, 256, 1, a));
    }
    CK(cuMemcpyDtoH(bad, dbad, 8));
done:
    if (dthr) cuMemFree(dthr);
    if (dbad) cuMemFree(dbad);
    rt_close(&rt);
    return rc;
}

/* The device's Poynting bin thresholds thr[0..na) for angle step da
 * (k_ref_bin_thresholds of oracle/ref_harness/trig.cu). */
int refgpu_bin_thresholds(const char *cubin, float *thr, int na, int da) {
    int rc = 0;
    Rt rt;
    CUfunction f;
    CUdeviceptr dthr = 0;
    if (na <= 0) return 1;
    if (rt_open(&rt, cubin)) {
        rt_close(&rt);
        return 1;
    }
    CK(cuModuleGetFunction(&f, rt.mod, "k_ref_bin_thresholds"));
    CK(cuMemAlloc(&dthr, (size_t)na * 4));
    {
        void *a[] = {&dthr, &na, &da};
        CK(launch(f, (unsigned)((na + 127) / 128), 1, 128, 1, a));
    }
    CK(cuMemcpyDtoH(thr, dthr, (size_t)na * 4));
done:
    if (dthr) cuMemFree(dthr);
    rt_close(&rt);
    return rc;
}
