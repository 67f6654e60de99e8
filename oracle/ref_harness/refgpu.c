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
