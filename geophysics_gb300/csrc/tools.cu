// Post-processing and model tools around the RTM path.
//
//   geo_smooth_lines      repeated 3-point averaging along lines of a
//                         strided array: smooth1float of the MPI RTM program
//                         (2D-vti-fd+rtm-mpi/Toa_rtm_vti_adcig_cdp.c:1642-1664);
//   geo_smooth2d          smooth2float (:1607-1639): along x for every z, then
//                         along z for every x;
//   geo_adcig_smooth_stack the program's smoothed gathers and their stack
//                         (:416-437): every CDP's gathers smoothed along the
//                         angle axis, then summed over the angles;
//   geo_mute_direct       the direct-wave mute utility
//                         (2D-vti-fd+rtm-cuda/functions/shot_muteDirect.c:11-33).
//
// A smoothing pass is Jacobi: v[i] = (v0[i-1] + v0[i] + v0[i+1]) / 3.0 inside,
// v[0] = (v0[0] + v0[1]) / 2.0, v[n-1] = (v0[n-1] + v0[n-2]) / 2.0, from a copy
// v0 of the previous pass.  The programs divide the float sum by the double
// 3.0 (or 2.0) and store the float.  Both operands are floats, and double has
// more than 2*24+2 bits of precision, so rounding the quotient to double and
// then to float equals rounding it to float once (Figueroa, "When is double
// rounding innocuous?", SIGNUM Newsletter 30(3), 1995): the kernel's IEEE
// float division s / 3.0f gives the programs' value.
#include "geo_internal.h"
#include <cmath>
#include <vector>

namespace geo {

// One block per line: element k of line l sits at l*ls + k*ks.  The line and
// its previous pass live in shared memory (2n floats).
__global__ void k_smooth_lines(float *v, int n, long nlines, long ls, long ks, int passes) {
    extern __shared__ float sm[];
    float *a = sm, *b = sm + n;
    for (long l = blockIdx.x; l < nlines; l += gridDim.x) {
        float *base = v + l * ls;
        for (int k = threadIdx.x; k < n; k += blockDim.x) a[k] = base[k * ks];
        __syncthreads();
        for (int p = 0; p < passes; p++) {
            for (int k = threadIdx.x; k < n; k += blockDim.x) {
                float r;
                if (k == 0) r = (n > 1) ? (a[0] + a[1]) / 2.0f : a[0];
                else if (k == n - 1) r = (a[n - 1] + a[n - 2]) / 2.0f;
                else r = (a[k - 1] + a[k] + a[k + 1]) / 3.0f;
                b[k] = r;
            }
            __syncthreads();
            float *t = a;
            a = b;
            b = t;
        }
        for (int k = threadIdx.x; k < n; k += blockDim.x) base[k * ks] = a[k];
        __syncthreads();
    }
}

// stk[o] = sum over ia in order of g[ia*nline + o], from 0.
__global__ void k_stack_planes(const float *g, float *stk, long nline, int na) {
    for (long o = blockIdx.x * (long)blockDim.x + threadIdx.x; o < nline; o += (long)gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int ia = 0; ia < na; ia++) s += g[(long)ia * nline + o];
        stk[o] = s;
    }
}

// Zero shot[ix*nt + it] for lo[ix] <= it < hi[ix] (trace-major record).
__global__ void k_mute_traces(float *shot, int nx, int nt, const int *lo, const int *hi) {
    const long n = (long)nx * nt;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int ix = (int)(k / nt), it = (int)(k % nt);
        if (it >= lo[ix] && it < hi[ix]) shot[k] = 0.0f;
    }
}

constexpr int kMaxSmoothLine = 24 * 1024;   // 2 x 96 KB of shared memory per block

static int smooth_lines_dev(float *v, int n, long nlines, long ls, long ks, int passes, cudaStream_t s) {
    if (n < 1 || nlines < 1 || passes < 1) return GEO_OK;
    if (n > kMaxSmoothLine) return fail(GEO_ERR_ARG, "smoothing lines longer than %d samples", kMaxSmoothLine);
    const size_t smem = (size_t)2 * n * 4;
    if (smem > 48 * 1024)
        GEO_CUDA(cudaFuncSetAttribute(k_smooth_lines, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int threads = n >= 256 ? 256 : ((n + 31) / 32) * 32;
    const int blocks = (int)std::min<long>(nlines, 152L * 64);
    k_smooth_lines<<<blocks, threads, smem, s>>>(v, n, nlines, ls, ks, passes);
    return check_launch("smooth_lines");
}

// Copy a host or device array of n floats to a fresh device buffer.
static int to_device(DevBuf &b, const float *src, size_t n, int mem, cudaStream_t s) {
    GEO_TRY(b.alloc(n * 4));
    GEO_CUDA(cudaMemcpyAsync(b.p, src, n * 4, mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                             s));
    return GEO_OK;
}

static int from_device(float *dst, const DevBuf &b, size_t n, int mem, cudaStream_t s) {
    GEO_CUDA(cudaMemcpyAsync(dst, b.p, n * 4, mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                             s));
    return GEO_OK;
}

}  // namespace geo

using namespace geo;

extern "C" int geo_smooth_lines(float *v, int n, long long nlines, long long line_stride, long long elem_stride,
                                int passes, int mem, void *stream) {
    if (!v || n < 1 || nlines < 1 || passes < 0) return fail(GEO_ERR_ARG, "bad argument");
    if (line_stride < 0 || elem_stride < 1) return fail(GEO_ERR_ARG, "strides must be >= 0 (lines) and >= 1 (samples)");
    if (mem != GEO_MEM_HOST && mem != GEO_MEM_DEVICE) return fail(GEO_ERR_ARG, "bad mem kind");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t span = (size_t)((nlines - 1) * line_stride + (long long)(n - 1) * elem_stride + 1);
    if (mem == GEO_MEM_DEVICE) {
        GEO_TRY(smooth_lines_dev(v, n, nlines, line_stride, elem_stride, passes, s));
    } else {
        DevBuf d;
        GEO_TRY(to_device(d, v, span, mem, s));
        GEO_TRY(smooth_lines_dev(d.as<float>(), n, nlines, line_stride, elem_stride, passes, s));
        GEO_TRY(from_device(v, d, span, mem, s));
    }
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}

extern "C" int geo_smooth2d(int nx, int rx, int nz, int rz, float *v, int mem, void *stream) {
    if (!v || nx < 1 || nz < 1 || rx < 0 || rz < 0) return fail(GEO_ERR_ARG, "bad argument");
    if (mem != GEO_MEM_HOST && mem != GEO_MEM_DEVICE) return fail(GEO_ERR_ARG, "bad mem kind");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)nx * nz;
    DevBuf d;
    float *p = v;
    if (mem == GEO_MEM_HOST) {
        GEO_TRY(to_device(d, v, n, mem, s));
        p = d.as<float>();
    }
    GEO_TRY(smooth_lines_dev(p, nx, nz, 1, nz, rx, s));   // along x, one line per z
    GEO_TRY(smooth_lines_dev(p, nz, nx, nz, 1, rz, s));   // along z, one line per x
    if (mem == GEO_MEM_HOST) GEO_TRY(from_device(v, d, n, mem, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}

extern "C" int geo_adcig_smooth_stack(int nx, int nz, int na, int passes, float *adcig, float *stack, int mem,
                                      void *stream) {
    if (!adcig || nx < 1 || nz < 1 || na < 1 || passes < 0) return fail(GEO_ERR_ARG, "bad argument");
    if (mem != GEO_MEM_HOST && mem != GEO_MEM_DEVICE) return fail(GEO_ERR_ARG, "bad mem kind");
    cudaStream_t s = (cudaStream_t)stream;
    const long nline = (long)nx * nz;
    const size_t n = (size_t)na * nline;
    DevBuf d, st;
    float *p = adcig, *q = stack;
    if (mem == GEO_MEM_HOST) {
        GEO_TRY(to_device(d, adcig, n, mem, s));
        p = d.as<float>();
        if (stack) {
            GEO_TRY(st.alloc((size_t)nline * 4));
            q = st.as<float>();
        }
    }
    // gathers adcig[ia][ix][iz]: one line per (ix, iz) along ia
    GEO_TRY(smooth_lines_dev(p, na, nline, 1, nline, passes, s));
    if (stack) {
        k_stack_planes<<<(int)std::min<long>((nline + 255) / 256, 152L * 16), 256, 0, s>>>(p, q, nline, na);
        GEO_TRY(check_launch("stack_planes"));
    }
    if (mem == GEO_MEM_HOST) {
        GEO_TRY(from_device(adcig, d, n, mem, s));
        if (stack) GEO_TRY(from_device(stack, st, (size_t)nline, mem, s));
    }
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}

extern "C" int geo_mute_direct(int nx, int nt, float dt, float favg, float dx, float dz, int fs, int ds, int zs, int is,
                               float vp, float epsilon, int tt, float *shot, int mem, void *stream) {
    if (!shot || nx < 1 || nt < 1 || !(dt > 0) || !(favg > 0) || !(vp > 0)) return fail(GEO_ERR_ARG, "bad argument");
    if (mem != GEO_MEM_HOST && mem != GEO_MEM_DEVICE) return fail(GEO_ERR_ARG, "bad mem kind");
    cudaStream_t s = (cudaStream_t)stream;
    // window (t0/dt - tt, t0/dt + 2/(dt favg) + tt) per trace; t0 in double as the
    // utility forms it: sqrt(pow(x,2)+pow(z,2)) / (vp*sqrtf(1+2 eps))
    std::vector<int> lo(nx), hi(nx);
    for (int ix = 0; ix < nx; ix++) {
        const float mu_x = dx * std::abs(ix - fs - (is - 1) * ds), mu_z = dz * zs;
        const float mu_t0 = (float)(std::sqrt(std::pow(mu_x, 2) + std::pow(mu_z, 2)) / (vp * sqrtf(1 + 2 * epsilon)));
        const int mu_t = (int)(2.0 / (dt * favg));
        const int mu_nt = (int)(mu_t0 / dt) + mu_t + tt;
        lo[ix] = std::max(0, (int)(mu_t0 / dt) - tt + 1);
        hi[ix] = std::min(mu_nt, nt);
    }
    const size_t n = (size_t)nx * nt;
    DevBuf d, dl, dh;
    float *p = shot;
    if (mem == GEO_MEM_HOST) {
        GEO_TRY(to_device(d, shot, n, mem, s));
        p = d.as<float>();
    }
    GEO_TRY(dl.alloc((size_t)nx * 4));
    GEO_TRY(dh.alloc((size_t)nx * 4));
    GEO_CUDA(cudaMemcpyAsync(dl.p, lo.data(), (size_t)nx * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemcpyAsync(dh.p, hi.data(), (size_t)nx * 4, cudaMemcpyHostToDevice, s));
    k_mute_traces<<<(int)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(p, nx, nt, dl.as<int>(),
                                                                                   dh.as<int>());
    GEO_TRY(check_launch("mute_traces"));
    if (mem == GEO_MEM_HOST) GEO_TRY(from_device(shot, d, n, mem, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}

// ------------------------------------------------------------ model smoothers
// The two model smoothers of the reference update the model in place while
// they sweep it (Gauss-Seidel order), so each result depends on the visiting
// order; they run on the host, in the programs' order.

namespace geo {

// utils-3D-smooth-f95/Toa_smooth3D.c:50-161 on a model stored z fastest, then
// x, then y (the program's file order).  The program holds it as vel[x][y][z]
// (z fastest, then y), and its front/back faces read z = nz, one past a
// column, which in that layout is the next element in memory: (x, y+1, 0),
// or (x+1, 0, 0) from y = ny-1.  at() resolves every read through that layout.
// One read, at (nx-2, ny-1, nz-1), lands one float past the end of the
// program's allocation; for models of 128 KB and more the C library serves
// that allocation from fresh zero-filled pages with room after the end, so
// the program reads 0 there, and so does at().
struct Smooth3D {
    int nx, ny, nz;
    float *v;
    float &cell(long i, long j, long k) const { return v[k + (long)nz * (i + (long)nx * j)]; }
    float at(long i, long j, long k) const {
        const long m = k + (long)nz * (j + (long)ny * i);   // index in the program's vel[x][y][z]
        if (m >= (long)nx * ny * nz) return 0.0f;
        return cell(m / ((long)nz * ny), (m / nz) % ny, m % nz);
    }
    // nine samples of one z plane, x major then y, in the program's order
    float sum_xy(long i, long j, long k) const {
        float s = 0.0f;
        bool first = true;
        for (int di = -1; di <= 1; di++)
            for (int dj = -1; dj <= 1; dj++) {
                const float a = at(i + di, j + dj, k);
                s = first ? a : s + a;
                first = false;
            }
        return s;
    }
    // nine samples of one x plane (y major then z)
    float sum_yz(long i, long j, long k) const {
        float s = 0.0f;
        bool first = true;
        for (int dj = -1; dj <= 1; dj++)
            for (int dk = -1; dk <= 1; dk++) {
                const float a = at(i, j + dj, k + dk);
                s = first ? a : s + a;
                first = false;
            }
        return s;
    }
    // nine samples of one y plane (x major then z)
    float sum_xz(long i, long j, long k) const {
        float s = 0.0f;
        bool first = true;
        for (int di = -1; di <= 1; di++)
            for (int dk = -1; dk <= 1; dk++) {
                const float a = at(i + di, j, k + dk);
                s = first ? a : s + a;
                first = false;
            }
        return s;
    }
    // corner (I,J,K) with inward neighbours I2, J2, K2: the program's sum of
    // eight, (I2,J,K) (I,J2,K) (I2,J2,K) (I,J,K) then the same four at K2
    float corner(long I, long J, long K, long I2, long J2, long K2, bool swap_last) const {
        float s = at(I2, J, K) + at(I, J2, K) + at(I2, J2, K) + at(I, J, K) + at(I2, J, K2) + at(I, J2, K2);
        if (swap_last) s = s + at(I, J, K2) + at(I2, J2, K2);   // vel[0][ny-1][nz-1] lists these two the other way
        else s = s + at(I2, J2, K2) + at(I, J, K2);
        return s / 8;
    }
    // four samples of an edge cross-section: the in-section neighbours a, b,
    // their diagonal c, the edge point itself -- in that order
    float quad(long ia, long ja, long ka, long ib, long jb, long kb, long ic, long jc, long kc, long i, long j,
               long k) const {
        return at(ia, ja, ka) + at(ib, jb, kb) + at(ic, jc, kc) + at(i, j, k);
    }

    void pass(int mmz) {
        const long X = nx - 1, Y = ny - 1, Z = nz - 1;
        for (long i = 1; i < X; i++)                               // inner
            for (long j = 1; j < Y; j++)
                for (long k = mmz; k < Z; k++)
                    cell(i, j, k) = ((sum_xy(i, j, k - 1)) + (sum_xy(i, j, k)) + (sum_xy(i, j, k + 1))) / 27;
        for (long j = 1; j < Y; j++)                               // up and down
            for (long i = 1; i < X; i++) {
                cell(i, j, mmz) = ((sum_xy(i, j, mmz)) + (sum_xy(i, j, mmz + 1))) / 18;
                cell(i, j, Z) = ((sum_xy(i, j, Z)) + (sum_xy(i, j, Z - 1))) / 18;
            }
        for (long j = 1; j < Y; j++)                               // left and right
            for (long k = mmz; k < Z; k++) {
                cell(0, j, k) = ((sum_yz(0, j, k)) + (sum_yz(1, j, k))) / 18;
                cell(X, j, k) = ((sum_yz(X, j, k)) + (sum_yz(X - 1, j, k))) / 18;
            }
        for (long i = 1; i < X; i++)                               // front and back, z up to nz-1
            for (long k = mmz; k < nz; k++) {
                cell(i, 0, k) = ((sum_xz(i, 0, k)) + (sum_xz(i, 1, k))) / 18;
                cell(i, Y, k) = ((sum_xz(i, Y, k)) + (sum_xz(i, Y - 1, k))) / 18;
            }
        cell(0, 0, mmz) = corner(0, 0, mmz, 1, 1, mmz + 1, false);   // the eight points
        cell(0, 0, Z) = corner(0, 0, Z, 1, 1, Z - 1, false);
        cell(X, 0, mmz) = corner(X, 0, mmz, X - 1, 1, mmz + 1, false);
        cell(X, 0, Z) = corner(X, 0, Z, X - 1, 1, Z - 1, false);
        cell(0, Y, mmz) = corner(0, Y, mmz, 1, Y - 1, mmz + 1, false);
        cell(0, Y, Z) = corner(0, Y, Z, 1, Y - 1, Z - 1, true);
        cell(X, Y, mmz) = corner(X, Y, mmz, X - 1, Y - 1, mmz + 1, false);
        cell(X, Y, Z) = corner(X, Y, Z, X - 1, Y - 1, Z - 1, false);
        for (long k = mmz; k < Z; k++) {                           // edges along z: planes k, k-1, k+1
            const long cs[4][4] = {{0, 0, 1, 1}, {0, Y, 1, Y - 1}, {X, 0, X - 1, 1}, {X, Y, X - 1, Y - 1}};
            for (const auto &c : cs) {
                const long I = c[0], J = c[1], I2 = c[2], J2 = c[3];
                cell(I, J, k) = ((quad(I2, J, k, I, J2, k, I2, J2, k, I, J, k)) +
                                 (quad(I2, J, k - 1, I, J2, k - 1, I2, J2, k - 1, I, J, k - 1)) +
                                 (quad(I2, J, k + 1, I, J2, k + 1, I2, J2, k + 1, I, J, k + 1))) / 12;
            }
        }
        for (long i = 1; i < X; i++) {                             // edges along x: planes i, i-1, i+1
            const long cs[4][4] = {{0, mmz, 1, mmz + 1}, {0, Z, 1, Z - 1}, {Y, mmz, Y - 1, mmz + 1}, {Y, Z, Y - 1, Z - 1}};
            for (const auto &c : cs) {
                const long J = c[0], K = c[1], J2 = c[2], K2 = c[3];
                cell(i, J, K) = ((quad(i, J2, K, i, J, K2, i, J2, K2, i, J, K)) +
                                 (quad(i - 1, J2, K, i - 1, J, K2, i - 1, J2, K2, i - 1, J, K)) +
                                 (quad(i + 1, J2, K, i + 1, J, K2, i + 1, J2, K2, i + 1, J, K))) / 12;
            }
        }
        for (long j = 1; j < Y; j++) {                             // edges along y: planes j, j-1, j+1
            const long cs[4][4] = {{0, mmz, 1, mmz + 1}, {0, Z, 1, Z - 1}, {X, mmz, X - 1, mmz + 1}, {X, Z, X - 1, Z - 1}};
            for (const auto &c : cs) {
                const long I = c[0], K = c[1], I2 = c[2], K2 = c[3];
                cell(I, j, K) = ((quad(I2, j, K, I, j, K2, I2, j, K2, I, j, K)) +
                                 (quad(I2, j - 1, K, I, j - 1, K2, I2, j - 1, K2, I, j - 1, K)) +
                                 (quad(I2, j + 1, K, I, j + 1, K2, I2, j + 1, K2, I, j + 1, K))) / 12;
            }
        }
    }
};

// utils-3D-smooth-f95/smooth.f95:44-70 on v[ix*nz + iz]; z0 = nzs-1 (0-based).
static void smooth_model2d_host(int nx, int nz, int z0, int nsmooth, float *v) {
    auto P = [&](int i, int j) -> float & { return v[(long)i * nz + j]; };   // 0-based (x, z)
    const int X = nx - 1, Z = nz - 1;
    for (int it = 0; it < nsmooth; it++) {
        P(0, z0) = (2 * P(1, z0) + 2 * P(0, z0 + 1) + P(1, z0 + 1) + 4 * P(0, z0)) / 9;
        P(0, Z) = (2 * P(0, Z - 1) + 2 * P(1, Z) + P(1, Z - 1) + 4 * P(0, Z)) / 9;
        P(X, z0) = (2 * P(X - 1, z0) + P(X - 1, z0 + 1) + 2 * P(X, z0 + 1) + 4 * P(X, z0)) / 9;
        P(X, Z) = (P(X - 1, Z - 1) + 2 * P(X, Z - 1) + 2 * P(X - 1, Z) + 4 * P(X, Z)) / 9;
        for (int i = 1; i < X; i++) {
            P(i, z0) = (2 * P(i - 1, z0) + P(i - 1, z0 + 1) + 2 * P(i, z0 + 1) + P(i + 1, z0 + 1) + 2 * P(i + 1, z0) +
                        4 * P(i, z0)) / 12;
            P(i, Z) = (2 * P(i - 1, Z) + P(i - 1, Z - 1) + 2 * P(i, Z - 1) + P(i + 1, Z - 1) + 2 * P(i + 1, Z) +
                       4 * P(i, Z)) / 12;
        }
        for (int j = z0 + 1; j < Z; j++) {
            P(0, j) = (2 * P(0, j - 1) + P(1, j - 1) + 2 * P(1, j) + P(1, j + 1) + 2 * P(0, j + 1) + 4 * P(0, j)) / 12;
            P(X, j) = (2 * P(X, j - 1) + P(X - 1, j - 1) + 2 * P(X - 1, j) + P(X - 1, j + 1) + 2 * P(X, j + 1) +
                       4 * P(X, j)) / 12;
        }
        for (int i = 1; i < X; i++)
            for (int j = z0 + 1; j < Z; j++)
                P(i, j) = (P(i - 1, j - 1) + P(i, j - 1) * 2 + P(i + 1, j - 1) + P(i - 1, j) * 2 + P(i, j) * 4 +
                           P(i + 1, j) * 2 + P(i - 1, j + 1) + P(i, j + 1) * 2 + P(i + 1, j + 1)) / 16;
    }
}

// Host copy of a host or device model, run f on it, copy back.
template <class F>
static int on_host(float *v, size_t n, int mem, cudaStream_t s, F f) {
    if (mem == GEO_MEM_HOST) {
        f(v);
        return GEO_OK;
    }
    std::vector<float> h(n);
    GEO_CUDA(cudaMemcpyAsync(h.data(), v, n * 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    f(h.data());
    GEO_CUDA(cudaMemcpyAsync(v, h.data(), n * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}

}  // namespace geo

extern "C" int geo_smooth_model3d(int nx, int ny, int nz, int passes, int mmz, float *v, int mem, void *stream) {
    if (!v || nx < 3 || ny < 3 || nz < 3 || passes < 0) return fail(GEO_ERR_ARG, "bad argument (sizes >= 3)");
    if (mmz < 1 || mmz > nz - 2) return fail(GEO_ERR_ARG, "mmz must be 1..nz-2");
    if (mem != GEO_MEM_HOST && mem != GEO_MEM_DEVICE) return fail(GEO_ERR_ARG, "bad mem kind");
    return on_host(v, (size_t)nx * ny * nz, mem, (cudaStream_t)stream, [&](float *h) {
        Smooth3D sm{nx, ny, nz, h};
        for (int p = 0; p < passes; p++) sm.pass(mmz);
    });
}

extern "C" int geo_smooth_model2d(int nx, int nz, int z0, int passes, float *v, int mem, void *stream) {
    if (!v || nx < 3 || nz < 3 || passes < 0) return fail(GEO_ERR_ARG, "bad argument (sizes >= 3)");
    if (z0 < 0 || z0 > nz - 2) return fail(GEO_ERR_ARG, "z0 must be 0..nz-2");
    if (mem != GEO_MEM_HOST && mem != GEO_MEM_DEVICE) return fail(GEO_ERR_ARG, "bad mem kind");
    return on_host(v, (size_t)nx * nz, mem, (cudaStream_t)stream,
                   [&](float *h) { smooth_model2d_host(nx, nz, z0, passes, h); });
}
