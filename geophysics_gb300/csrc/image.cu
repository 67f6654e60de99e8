// Imaging-side kernels: direct-wave mute, record transpose, image
// normalisation, shot-ordered stacking and the adjoint Laplacian.
#include "geo_internal.h"

namespace geo {

// Zero samples lo[tr] <= it < hi[tr] of a time-major record (nt x ntr).
__global__ void k_mute(float *rec, int ntr, int nt, const int *lo, const int *hi) {
    const long n = (long)ntr * nt;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int tr = (int)(k % ntr), it = (int)(k / ntr);
        const int a = lo ? lo[tr] : 0;
        if (it >= a && it < hi[tr]) rec[k] = 0.0f;
    }
}

int launch_mute_records(float *rec, int ntr, int nt, const int *lo, const int *hi, cudaStream_t s) {
    const long n = (long)ntr * nt;
    int g = (int)((n + 255) / 256);
    if (g > 152 * 32) g = 152 * 32;
    k_mute<<<g, 256, 0, s>>>(rec, ntr, nt, lo, hi);
    return check_launch("mute");
}

// (nt x ntr) time-major -> (ntr x nt) trace-major through a 32x33 tile.
__global__ void k_transpose(const float *__restrict__ in, float *__restrict__ out, int ntr, int nt) {
    __shared__ float tile[32][33];
    const int tr0 = blockIdx.x * 32, t0 = blockIdx.y * 32;
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int it = t0 + j, tr = tr0 + threadIdx.x;
        if (it < nt && tr < ntr) tile[j][threadIdx.x] = in[(long)it * ntr + tr];
    }
    __syncthreads();
    for (int j = threadIdx.y; j < 32; j += blockDim.y) {
        const int tr = tr0 + j, it = t0 + threadIdx.x;
        if (it < nt && tr < ntr) out[(long)tr * nt + it] = tile[threadIdx.x][j];
    }
}

int launch_transpose_records(const float *tm, float *out, int ntr, int nt, cudaStream_t s) {
    dim3 g((ntr + 31) / 32, (nt + 31) / 32), b(32, 8);
    k_transpose<<<g, b, 0, s>>>(tm, out, ntr, nt);
    return check_launch("transpose");
}

// mig /= source illumination (Toa_rtm_vti_adcig_cdp.c:1101).
__global__ void k_normalize(float *mig, const float *ill, long n) {
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
        mig[k] = mig[k] / ill[k];
}

int launch_normalize_image(float *mig, const float *ill, size_t n, cudaStream_t s) {
    int g = (int)((n + 255) / 256);
    if (g > 152 * 32) g = 152 * 32;
    k_normalize<<<g, 256, 0, s>>>(mig, ill, (long)n);
    return check_launch("normalize");
}

__global__ void k_normalize_planes(float *a, const float *ill, long n, int planes) {
    const long tot = n * planes;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < tot; k += (long)gridDim.x * blockDim.x)
        a[k] = a[k] / ill[k % n];
}

int launch_normalize_planes(float *a, const float *ill, size_t n, int planes, cudaStream_t s) {
    const long tot = (long)n * planes;
    int g = (int)((tot + 255) / 256);
    if (g > 152 * 32) g = 152 * 32;
    k_normalize_planes<<<g, 256, 0, s>>>(a, ill, (long)n, planes);
    return check_launch("normalize_planes");
}

// Stack per-shot images into the full image.  Each output point sums the
// shots covering it in shot order, so the float sum equals the reference's
// sequential shot loop (Toa_rtm_vti_adcig_cdp.c:1102-1104: window column c
// lands on column c + offset of the full image).
__global__ void k_stack(float *full, int nz, int nx, const float *const *imgs, const int *offsets,
                        const int *widths, int nshots) {
    const long n = (long)nx * nz;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int gx = (int)(k / nz), iz = (int)(k % nz);
        float acc = full[k];
        for (int s = 0; s < nshots; s++) {
            const int c = gx - offsets[s];
            if (c >= 0 && c < widths[s]) acc = acc + imgs[s][(long)c * nz + iz];
        }
        full[k] = acc;
    }
}

int launch_stack_image(float *full, int nz, const float *const *imgs, const int *offsets, const int *widths,
                       int nshots, int nx, cudaStream_t s) {
    const long n = (long)nx * nz;
    int g = (int)((n + 255) / 256);
    if (g > 152 * 32) g = 152 * 32;
    k_stack<<<g, 256, 0, s>>>(full, nz, nx, imgs, offsets, widths, nshots);
    return check_launch("stack");
}

// Adjoint first-difference Laplacian.  The reference scatters from each
// input point in loop order (laplac2_lop adj=1, utils-Laplacian-filter/
// laplace.c:14-52); this gathers the same terms per output point in the
// order the scatter delivers them, so the float result is identical:
//   from (ix-1): -in[j-nz]; from (iz-1): -in[j-1]; own point: +in[j] once
//   per existing neighbour (z-, z+, x-, x+); from (iz+1): -in[j+1];
//   from (ix+1): -in[j+nz].
__global__ void k_laplace2d(int nx, int nz, const float *__restrict__ in, float *__restrict__ out) {
    const long n = (long)nx * nz;
    for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += (long)gridDim.x * blockDim.x) {
        const int ix = (int)(j / nz), iz = (int)(j % nz);
        const float c = in[j];
        float a = 0.0f;
        if (ix > 0) a = a - in[j - nz];
        if (iz > 0) a = a - in[j - 1];
        if (iz > 0) a = a + c;
        if (iz < nz - 1) a = a + c;
        if (ix > 0) a = a + c;
        if (ix < nx - 1) a = a + c;
        if (iz < nz - 1) a = a - in[j + 1];
        if (ix < nx - 1) a = a - in[j + nz];
        out[j] = a;
    }
}

int launch_laplace2d(int nx, int nz, const float *in, float *out, cudaStream_t s) {
    const long n = (long)nx * nz;
    int g = (int)((n + 255) / 256);
    if (g > 152 * 32) g = 152 * 32;
    k_laplace2d<<<g, 256, 0, s>>>(nx, nz, in, out);
    return check_launch("laplace2d");
}

// 3D form: scatter loop order (iy, ix, iz) with the z, x, y branches of
// laplace_3d_filter; gathered in delivery order.
__global__ void k_laplace3d(int nx, int ny, int nz, const float *__restrict__ in, float *__restrict__ out) {
    const long nxz = (long)nx * nz, n = nxz * ny;
    for (long j = blockIdx.x * (long)blockDim.x + threadIdx.x; j < n; j += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(j % nz), ix = (int)((j / nz) % nx), iy = (int)(j / nxz);
        const float c = in[j];
        float a = 0.0f;
        if (iy > 0) a = a - in[j - nxz];
        if (ix > 0) a = a - in[j - nz];
        if (iz > 0) a = a - in[j - 1];
        if (iz > 0) a = a + c;
        if (iz < nz - 1) a = a + c;
        if (ix > 0) a = a + c;
        if (ix < nx - 1) a = a + c;
        if (iy > 0) a = a + c;
        if (iy < ny - 1) a = a + c;
        if (iz < nz - 1) a = a - in[j + 1];
        if (ix < nx - 1) a = a - in[j + nz];
        if (iy < ny - 1) a = a - in[j + nxz];
        out[j] = a;
    }
}

int launch_laplace3d(int nx, int ny, int nz, const float *in, float *out, cudaStream_t s) {
    const long n = (long)nx * ny * nz;
    int g = (int)((n + 255) / 256);
    if (g > 152 * 64) g = 152 * 64;
    k_laplace3d<<<g, 256, 0, s>>>(nx, ny, nz, in, out);
    return check_launch("laplace3d");
}

}  // namespace geo
