/* Drives the reference's MPI RTM functions for ONE shot exactly as its
 * main() does inside the shot loop (2D-vti-fd+rtm-mpi/Toa_rtm_vti_adcig_cdp.c
 * :186-196 model read + pad, :310-337 aperture window, :339-344 forward with
 * boundary saving, :347-355 velocity back-transform, :357-358 mute,
 * :374-384 RTM correlation + stacking into mig_ns0), with the window width
 * nxs given per shot.  The model comes in memory instead of from files
 * (read_v_e_d_r with seismic=1 is a plain float read with rho=1).
 * Linked only into oracle/_ref/librefrtm.so, the parity pin of the oracle. */
#include <stdlib.h>
#include <string.h>
#include <math.h>

float **alloc2float(size_t n1, size_t n2);
float ***alloc3float(size_t n1, size_t n2, size_t n3);
void free2float(float **p);
void free3float(float ***p);
void zero2float(float **p, int n1, int n2);
void zero3float(float ***p, int n1, int n2, int n3);
void pad_vv(int nx, int nz, int npd, float **ee);
void model_vti_get_boundry(int nx, int nz, int vnx, int vnz, int nt, int npd, float dx, float dz,
                           float vdx, float vdz, float favg, float tmax, float dt, float dtout, float pfac,
                           float **vp, float **epsilu, float **deta, float **rho,
                           int ns_sxd, int ds_sxd, int fs_sxd, int zs_sxd, int is,
                           float **p_cal_x, float **p_cal_z,
                           float **p_top_x, float **p_bottom_x, float **p_left_x, float **p_right_x,
                           float **p_top_z, float **p_bottom_z, float **p_left_z, float **p_right_z, int _Circle_,
                           int mm, int wtype, int hsx, int myid, float *mu_v, int flag_snap, int seismic);
void mute_directwave(int flag_mu, int nx, int nt, float dt, float favg,
                     float dx, float dz, int fs_sxd, int ds_sxd, int zs_sxd, int is,
                     float mu_v, float **p_cal, int tt);
void RTM_corr_adcig(int nx, int nz, int vnx, int vnz, int nt, int npd, float dx, float dz,
                    float vdx, float vdz, float favg, float tmax, float dt, float dtout,
                    float pfac, float **vp, float **epsilu, float **deta, float **rho, char FN5[],
                    int ns_sxd, int ds_sxd, int fs_sxd, int ds_initial, int fs_initial, int zs_sxd, int is, int flag_cdp,
                    float **p_top_x, float **p_bottom_x, float **p_left_x, float **p_right_x,
                    float **p_top_z, float **p_bottom_z, float **p_left_z, float **p_right_z, float **p_obs_x, float **p_obs_z,
                    int mm, int wtype, int hsx, int myid, float **mig_is, float **mig_ns0,
                    float ***adcig_is, float ***adcig_ns0, float ***Ixhz_is, float ***Ixhz_ns0, int nh,
                    int flag_snap, int seismic, int flag_adcig);

/* v,e,d: unpadded nx*nz (x-major).  mig_ns0: nx*nz accumulator (stacked
 * image before the Laplacian), mig_is: nxs*nz, p_cal_x: nxs*nt muted record,
 * adcig_ns0_acc (optional): 90*nx*nz accumulator of the angle gathers
 * (adcig_ns0[ia][ix][iz]).
 * Returns 0, or 1 when the window leaves the model (the reference exits). */
int ref_rtm_mpi_shot(int nx, int nz, int npd, int nt, float dx, float dz, float dt_ms,
                     float favg, float pfac, int fs_sxd, int ds_sxd, int zs_sxd, int is, int nxs,
                     const float *v, const float *e, const float *d,
                     float *mig_ns0_acc, float *mig_is_out, float *p_cal_x_out, float *adcig_ns0_acc)
{
    int i, j, k, nnz = nz + 2 * npd, nnx = nx + 2 * npd, nnxs = nxs + 2 * npd;
    float mu_v, tmax = nt * dt_ms / 1000.0f;
    if (fs_sxd + (is - 1) * ds_sxd < nxs / 2 + 1 || fs_sxd + (is - 1) * ds_sxd + nxs / 2 > nx) return 1;
    float **vp = alloc2float(nnz, nnx), **rho = alloc2float(nnz, nnx), **eps = alloc2float(nnz, nnx), **del = alloc2float(nnz, nnx);
    zero2float(vp, nnz, nnx); zero2float(rho, nnz, nnx); zero2float(eps, nnz, nnx); zero2float(del, nnz, nnx);
    for (i = npd; i < nx + npd; i++)
        for (j = npd; j < nz + npd; j++) {
            vp[i][j] = v[(i - npd) * nz + (j - npd)];
            eps[i][j] = e[(i - npd) * nz + (j - npd)];
            del[i][j] = d[(i - npd) * nz + (j - npd)];
            rho[i][j] = 1.0f;
        }
    pad_vv(nx, nz, npd, vp); pad_vv(nx, nz, npd, rho); pad_vv(nx, nz, npd, eps); pad_vv(nx, nz, npd, del);
    float **vps = alloc2float(nnz, nnxs), **rhos = alloc2float(nnz, nnxs), **epss = alloc2float(nnz, nnxs), **dels = alloc2float(nnz, nnxs);
    zero2float(vps, nnz, nnxs); zero2float(rhos, nnz, nnxs); zero2float(epss, nnz, nnxs); zero2float(dels, nnz, nnxs);
    k = fs_sxd + (is - 1) * ds_sxd;
    for (i = k - nxs / 2 + npd; i <= k + nxs / 2 + npd; i++)
        for (j = npd; j < nz + npd; j++) {
            vps[i - k + nxs / 2][j] = vp[i][j];
            rhos[i - k + nxs / 2][j] = rho[i][j];
            dels[i - k + nxs / 2][j] = del[i][j];
            epss[i - k + nxs / 2][j] = eps[i][j];
        }
    pad_vv(nxs, nz, npd, vps); pad_vv(nxs, nz, npd, rhos); pad_vv(nxs, nz, npd, epss); pad_vv(nxs, nz, npd, dels);
    float **pcx = alloc2float(nt, nxs), **pcz = alloc2float(nt, nxs);
    float **tx = alloc2float(nt, nxs), **bx = alloc2float(nt, nxs), **tz = alloc2float(nt, nxs), **bz = alloc2float(nt, nxs);
    float **lx = alloc2float(nt, nz), **rx = alloc2float(nt, nz), **lz = alloc2float(nt, nz), **rz = alloc2float(nt, nz);
    zero2float(pcx, nt, nxs); zero2float(pcz, nt, nxs); zero2float(tx, nt, nxs); zero2float(bx, nt, nxs);
    zero2float(tz, nt, nxs); zero2float(bz, nt, nxs); zero2float(lx, nt, nz); zero2float(rx, nt, nz);
    zero2float(lz, nt, nz); zero2float(rz, nt, nz);
    int fs = nxs / 2 + 1, ds = 0;
    model_vti_get_boundry(nxs, nz, nxs, nz, nt, npd, dx, dz, dx, dz, favg, tmax, dt_ms, dt_ms, pfac,
                          vps, epss, dels, rhos, 1, ds, fs, zs_sxd, is,
                          pcx, pcz, tx, bx, lx, rx, tz, bz, lz, rz, 15, 4, 1, 1, 1, &mu_v, 0, 1);
    for (i = 0; i <= nxs + 2 * npd - 1; i++)
        for (j = 0; j <= nz + 2 * npd - 1; j++) {
            rhos[i][j] = 1.0 / rhos[i][j];
            vps[i][j] = sqrtf(vps[i][j] / rhos[i][j]);
        }
    mute_directwave(1, nxs, nt, dt_ms, favg, dx, dz, fs, ds, zs_sxd, is, mu_v, pcx, 285);
    mute_directwave(1, nxs, nt, dt_ms, favg, dx, dz, fs, ds, zs_sxd, is, mu_v, pcz, 285);
    if (p_cal_x_out) for (i = 0; i < nxs; i++) memcpy(p_cal_x_out + (size_t)i * nt, pcx[i], (size_t)nt * 4);
    float **mig_is = alloc2float(nz, nxs), **mig_ns0 = alloc2float(nz, nx);
    float ***adcig_is = alloc3float(nz, nxs, 90), ***adcig_ns0 = alloc3float(nz, nx, 90);
    zero2float(mig_is, nz, nxs); zero3float(adcig_is, nz, nxs, 90); zero3float(adcig_ns0, nz, nx, 90);
    for (i = 0; i < nx; i++) memcpy(mig_ns0[i], mig_ns0_acc + (size_t)i * nz, (size_t)nz * 4);
    if (adcig_ns0_acc)
        for (k = 0; k < 90; k++)
            for (i = 0; i < nx; i++)
                memcpy(adcig_ns0[k][i], adcig_ns0_acc + ((size_t)k * nx + i) * nz, (size_t)nz * 4);
    char fn5[16] = "unused";
    RTM_corr_adcig(nxs, nz, nxs, nz, nt, npd, dx, dz, dx, dz, favg, tmax, dt_ms, dt_ms, pfac,
                   vps, epss, dels, rhos, fn5, 1, ds, fs, ds_sxd, fs_sxd, zs_sxd, is, 1,
                   tx, bx, lx, rx, tz, bz, lz, rz, pcx, pcz, 4, 1, 1, 1, mig_is, mig_ns0,
                   adcig_is, adcig_ns0, NULL, NULL, nxs / 2 + 1, 0, 1, 1);
    for (i = 0; i < nx; i++) memcpy(mig_ns0_acc + (size_t)i * nz, mig_ns0[i], (size_t)nz * 4);
    if (adcig_ns0_acc)
        for (k = 0; k < 90; k++)
            for (i = 0; i < nx; i++)
                memcpy(adcig_ns0_acc + ((size_t)k * nx + i) * nz, adcig_ns0[k][i], (size_t)nz * 4);
    if (mig_is_out) for (i = 0; i < nxs; i++) memcpy(mig_is_out + (size_t)i * nz, mig_is[i], (size_t)nz * 4);
    free2float(vp); free2float(rho); free2float(eps); free2float(del);
    free2float(vps); free2float(rhos); free2float(epss); free2float(dels);
    free2float(pcx); free2float(pcz); free2float(tx); free2float(bx); free2float(tz); free2float(bz);
    free2float(lx); free2float(rx); free2float(lz); free2float(rz);
    free2float(mig_is); free2float(mig_ns0); free3float(adcig_is); free3float(adcig_ns0);
    return 0;
}
