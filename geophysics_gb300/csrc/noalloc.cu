// geo_fd2d_shot_noalloc: the 2D forward-modelling shot of geo_fd2d_shot for
// callers that cannot allocate GPU memory.
//
// Who needs it: code that runs where cudaMalloc is off limits -- a host
// application whose GPU memory is fully reserved up front by its own pool,
// an embedding framework that forbids allocation outside its allocator, or
// a real-time loop that must not hit the allocator's synchronisation.  Such
// a caller owns its input and output buffers but cannot let the library
// allocate the wavefields it works on.
//
// This entry point allocates nothing on the GPU (no cudaMalloc/cudaFree,
// no graph instantiation, no allocating library routine) and nothing on the
// host heap.  Its work memory is one file-scope device array, kScratchBytes
// long, that every GPU which loads the library holds until the process
// exits.  Host-side set-up quantities live in fixed-size static host arrays,
// one set per process, so concurrent calls (other threads, other devices)
// wait for one another on a mutex while they set up.  The array's device
// address is looked up once per device and kept: a process that resets a
// device (cudaDeviceReset) must not call this entry point on it afterwards.
#include "geo_internal.h"
#include <cmath>
#include <cstring>
#include <mutex>

namespace geo {

namespace {

constexpr size_t kScratchBytes = 32u << 20;  // 32 MiB per GPU
constexpr int kMaxDevices = 64;
constexpr int kMaxN = 8192;                   // padded extent along x or z
constexpr int kMaxNt = 1 << 16;               // time steps

// The scratch array.  In host code its name is only a host-side stand-in;
// the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

static void *g_scratch_addr[kMaxDevices];     // per device, filled once

// Host-side working storage (fixed size: no heap use).  One set for the
// process, so g_host_mu serialises the calls (from any thread, on any
// device) for as long as they use it.
static float h_prof[8 * kMaxN];
static float h_amp[kMaxNt];
static uint8_t h_on[kMaxNt];
static float h_box[2 * kTB * kTB], h_taper[2 * kTB * kTB];
static int h_mute[2 * kMaxN];
static std::mutex g_host_mu;

// Device address of the scratch array on the current device, resolved by the
// first call on that device and kept.
int scratch_address(void **out) {
    int dev = 0;
    GEO_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(GEO_ERR_ARG, "device ordinal %d beyond %d", dev, kMaxDevices);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p)
            return fail(GEO_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return GEO_OK;
}

// Pad the model into the scratch copy and form 1+2eps and sqrtf(1+2del),
// the same float operations the host path performs.
__global__ void k_pad_model(int nx, int nz, int npd, const float *__restrict__ v, const float *__restrict__ e,
                            const float *__restrict__ d, float *vp, float *e2, float *d2) {
    const int nnx = nx + 2 * npd, nnz = nz + 2 * npd;
    const long n = (long)nnx * nnz;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int ix = (int)(k / nnz), iz = (int)(k % nnz);
        const int sx = ix < npd ? 0 : (ix >= npd + nx ? nx - 1 : ix - npd);
        const int sz = iz < npd ? 0 : (iz >= npd + nz ? nz - 1 : iz - npd);
        const long s = (long)sx * nz + sz;
        vp[k] = v[s];
        e2[k] = 1 + 2 * e[s];
        d2[k] = sqrtf(1 + 2 * d[s]);
    }
}

// The raw eps/del values of the SV taper box (kTB x kTB points from padded
// cell (tx0, tz0)), read through the same edge clamp as the padded model;
// z outside the padded grid gives 0 (those taper entries are never read).
__global__ void k_gather_box(int nx, int nz, int npd, int tx0, int tz0, const float *__restrict__ e,
                             const float *__restrict__ d, float *out) {
    const int nnz = nz + 2 * npd;
    for (int k = threadIdx.x; k < kTB * kTB; k += blockDim.x) {
        const int bx = k / kTB, bz = k % kTB, ix = tx0 + bx, iz = tz0 + bz;
        float ev = 0.0f, dv = 0.0f;
        if (iz >= 0 && iz < nnz) {
            const int sx = ix < npd ? 0 : (ix >= npd + nx ? nx - 1 : ix - npd);
            const int sz = iz < npd ? 0 : (iz >= npd + nz ? nz - 1 : iz - npd);
            ev = e[(size_t)sx * nz + sz];
            dv = d[(size_t)sx * nz + sz];
        }
        out[k] = ev;
        out[kTB * kTB + k] = dv;
    }
}

// Largest velocity and the first velocity/epsilon (one block).
__global__ void k_model_stats(long n, const float *__restrict__ v, const float *__restrict__ e, float *out) {
    __shared__ float red[256];
    float m = v[0];
    for (long k = threadIdx.x; k < n; k += blockDim.x) m = fmaxf(m, v[k]);
    red[threadIdx.x] = m;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = red[0];
        out[1] = v[0];
        out[2] = e[0];
    }
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace
}  // namespace geo

using namespace geo;

extern "C" size_t geo_fd2d_noalloc_limit(void) { return kScratchBytes; }

extern "C" int geo_fd2d_shot_noalloc(const geo_fd2d_desc *desc, const float *v, const float *e, const float *d,
                                     float *shot, void *stream) {
    if (!desc || !v || !e || !d || !shot) return fail(GEO_ERR_ARG, "null argument");
    const geo_fd2d_desc &D = *desc;
    if (D.variant != GEO_VARIANT_CPU && D.variant != GEO_VARIANT_GPU)
        return fail(GEO_ERR_ARG, "no-allocation path supports the CPU and GPU variants");
    if (D.nx < 2 || D.nz < 2 || D.npd < 5 || D.nt < 1) return fail(GEO_ERR_ARG, "grid too small (npd >= 5)");
    if (!(D.dt > 0) || !(D.dx > 0) || !(D.dz > 0) || !(D.favg > 0)) return fail(GEO_ERR_ARG, "bad spacing");
    const int nnx = D.nx + 2 * D.npd, nnz = D.nz + 2 * D.npd;
    if (nnx > kMaxN || nnz > kMaxN || D.nt > kMaxNt || D.nx > kMaxN)
        return fail(GEO_ERR_ARG, "grid %dx%d or nt %d beyond the no-allocation limits (%d, %d)", nnx, nnz, D.nt,
                    kMaxN, kMaxNt);
    if (D.rec_iz < 4 || D.rec_iz >= nnz - 4) return fail(GEO_ERR_ARG, "receiver row outside grid");
    const Variant var = (Variant)D.variant;
    const float fsx = D.fs + (D.is - 1) * D.ds;
    const int ixs = (int)(fsx + 0.5) + D.npd - 1, izs = (int)(D.zs + 0.5) + D.npd - 1;
    if (ixs < 4 || ixs >= nnx - 4 || izs < 4 || izs >= nnz - 4) return fail(GEO_ERR_ARG, "source outside grid");
    if (var == V_CPU && (ixs - 3 < 0 || ixs + 3 >= nnx || izs - 3 < 0 || izs + 3 >= nnz))
        return fail(GEO_ERR_ARG, "source window outside grid");

    // scratch layout
    const size_t n = (size_t)nnx * nnz;
    const int by = 8;
    const int ntiles = ((nnz + 31) / 32) * ((nnx + by - 1) / by);
    size_t off = 0;
    const size_t o_model = off; off = align256(off + 3 * n * 4);
    const size_t o_fields = off; off = align256(off + 8 * n * 4);
    const size_t o_prof = off; off = align256(off + (4 * (size_t)nnx + 4 * (size_t)nnz) * 4);
    const size_t o_rec = off; off = align256(off + (size_t)D.nt * D.nx * 4);
    const size_t o_taper = off; off = align256(off + 2 * kTB * kTB * 4);
    const size_t o_mute = off; off = align256(off + 2 * (size_t)D.nx * 4);
    const size_t o_desc = off; off = align256(off + sizeof(Shot2D));
    const size_t o_items = off; off = align256(off + (size_t)ntiles * 4);
    const size_t o_stats = off; off = align256(off + 16);
    if (off > kScratchBytes)
        return fail(GEO_ERR_ARG, "shot needs %zu bytes of work memory; the no-allocation limit is %zu", off,
                    kScratchBytes);

    std::lock_guard<std::mutex> host_lock(g_host_mu);
    void *base = nullptr;
    GEO_TRY(scratch_address(&base));
    unsigned char *S = static_cast<unsigned char *>(base);
    cudaStream_t s = (cudaStream_t)stream;
    float *vp = (float *)(S + o_model), *e2 = vp + n, *d2 = vp + 2 * n;
    float *fields = (float *)(S + o_fields), *prof = (float *)(S + o_prof), *rec = (float *)(S + o_rec);
    float *taper = (float *)(S + o_taper), *stats = (float *)(S + o_stats);
    int *mute = (int *)(S + o_mute), *items = (int *)(S + o_items);
    Shot2D *dshot = (Shot2D *)(S + o_desc);

    // model: pad on the device; the scalars the set-up needs come back
    k_pad_model<<<152 * 4, 256, 0, s>>>(D.nx, D.nz, D.npd, v, e, d, vp, e2, d2);
    GEO_TRY(check_launch("pad_model"));
    k_model_stats<<<1, 256, 0, s>>>((long)D.nx * D.nz, v, e, stats);
    GEO_TRY(check_launch("model_stats"));
    float h_scalars[4];
    GEO_CUDA(cudaMemcpyAsync(h_scalars, stats, 3 * 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaMemcpyAsync(h_scalars + 3, vp + n / 2, 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    const float vpmax = h_scalars[0], v00 = h_scalars[1], e00 = h_scalars[2], vcenter = h_scalars[3];
    if (!std::isfinite(vpmax) || !(vpmax > 0)) return fail(GEO_ERR_MODEL, "velocity maximum %g", vpmax);

    // sponge profiles (host, fixed arrays) -> scratch
    const float d0 = sponge_d0(var, 2, vpmax, vcenter, D.npd, D.dx, D.dx, D.dz);
    float *px_ = h_prof, *pz_ = h_prof + 4 * nnx;
    sponge_profiles(var, D.nx, D.npd, D.dt, d0, px_, px_ + nnx, px_ + 2 * nnx, px_ + 3 * nnx);
    sponge_profiles(var, D.nz, D.npd, D.dt, d0, pz_, pz_ + nnz, pz_ + 2 * nnz, pz_ + 3 * nnz);
    GEO_CUDA(cudaMemcpyAsync(prof, h_prof, (4 * (size_t)nnx + 4 * (size_t)nnz) * 4, cudaMemcpyHostToDevice, s));

    // source amplitudes: pfac*w(t), float time accumulated from dt
    {
        const double pi = kPiGui;
        const float tdelay = (float)(1.0 / D.favg);
        float t = D.dt;
        for (int it = 0; it < D.nt; it++, t += D.dt) {
            const float ts = t - tdelay;
            h_on[it] = (t <= 2 * tdelay);
            h_amp[it] = 0.0f;
            if (!h_on[it]) continue;
            float w = 0.0f;
            if (D.wtype == 1) {
                const float x = D.favg * ts, xx = x * x;
                w = (float)((1 - 2 * pi * pi * (xx)) * std::exp(-(pi * pi * xx)));
            } else if (D.wtype == 2) {
                const double y = (-4) * D.favg * D.favg * pi * pi / std::log(0.1);
                w = (float)((-2) * pi * pi * ts * std::exp(-y * ts * ts));
            } else if (D.wtype == 3) {
                const double y = (-1) * D.favg * D.favg * pi * pi / std::log(0.1);
                w = (float)std::exp(-y * ts * ts);
            }
            h_amp[it] = D.pfac * w;
        }
    }

    // SV taper box around the circle centre, from the raw eps/del
    int tx0 = -100000, tz0 = -100000;
    if (D.sv) {
        const int cx = var == V_GPU ? ixs + 1 : ixs, cz = var == V_GPU ? izs + 1 : izs;
        tx0 = cx - kTB / 2;
        tz0 = cz - kTB / 2;
        k_gather_box<<<1, 256, 0, s>>>(D.nx, D.nz, D.npd, tx0, tz0, e, d, taper);
        GEO_TRY(check_launch("gather_box"));
        GEO_CUDA(cudaMemcpyAsync(h_box, taper, 2 * kTB * kTB * 4, cudaMemcpyDeviceToHost, s));
        GEO_CUDA(cudaStreamSynchronize(s));
        for (int bx = 0; bx < kTB; bx++)
            for (int bz = 0; bz < kTB; bz++) {
                const int rx = tx0 + bx - cx, rz = tz0 + bz - cz, r2 = rx * rx + rz * rz;
                float ee = h_box[bx * kTB + bz], dd = h_box[kTB * kTB + bx * kTB + bz];
                if (var == V_CPU) {
                    const int CR = 15;
                    if (r2 <= CR * CR) {
                        if (r2 <= (CR * CR / 16)) {
                            ee = 0.0f; dd = 0.0f;
                        } else {
                            const double g = 0.5 * (1 - std::cos(kPiGui * ((std::pow((double)r2, 0.5) - CR / 4.0) * 4.0 / (CR * 3.0 - 1))));
                            ee = (float)(g * ee); dd = (float)(g * dd);
                        }
                    }
                } else {
                    const int R = 15, r = 4;
                    if (r2 <= R * R) {
                        if (r2 <= r * r) {
                            ee = 0.0f; dd = 0.0f;
                        } else {
                            const double g = 0.5 * (1 - std::cos(kPiGui * ((sqrtf((float)r2) - r) * 4.0 / (R * 3.0 - 1))));
                            ee = (float)(g * ee); dd = (float)(g * dd);
                        }
                    }
                }
                h_taper[bx * kTB + bz] = 1 + 2 * ee;
                h_taper[kTB * kTB + bx * kTB + bz] = sqrtf(1 + 2 * dd);
            }
        GEO_CUDA(cudaMemcpyAsync(taper, h_taper, 2 * kTB * kTB * 4, cudaMemcpyHostToDevice, s));
    }

    // the array keeps the previous call's contents: clear the state
    GEO_CUDA(cudaMemsetAsync(fields, 0, 8 * n * 4, s));
    GEO_CUDA(cudaMemsetAsync(rec, 0, (size_t)D.nt * D.nx * 4, s));
    GEO_CUDA(cudaMemsetAsync(items, 0, (size_t)ntiles * 4, s));

    Shot2D H;
    memset(&H, 0, sizeof H);
    H.nnx = nnx; H.nnz = nnz; H.npd = D.npd; H.nx = D.nx; H.nz = D.nz;
    H.dtx = D.dt / D.dx; H.dtz = D.dt / D.dz;
    H.cx1 = prof; H.cx2 = prof + nnx; H.ax1 = prof + 2 * nnx; H.ax2 = prof + 3 * nnx;
    float *pz = prof + 4 * nnx;
    H.cz1 = pz; H.cz2 = pz + nnz; H.az1 = pz + 2 * nnz; H.az2 = pz + 3 * nnz;
    H.vp = vp; H.e2 = e2; H.d2 = d2; H.kz = nullptr; H.kx = nullptr;
    H.tx0 = tx0; H.tz0 = tz0; H.te2 = taper; H.td2 = taper + kTB * kTB; H.tkz = nullptr; H.tkx = nullptr;
    H.ixs = ixs; H.izs = izs;
    H.u[0] = fields; H.w[0] = fields + n; H.P[0] = fields + 2 * n; H.Q[0] = fields + 3 * n;
    H.px[0] = fields + 4 * n; H.pz[0] = fields + 5 * n; H.qx[0] = fields + 6 * n; H.qz[0] = fields + 7 * n;
    H.rec_iz = D.rec_iz; H.rec_scale = D.rec_scale;
    H.rec_p = rec; H.rec_q = nullptr;
    H.tile_base = 0; H.ntz = (nnz + 31) / 32;
    // from pageable memory: the copy has taken H before it returns
    GEO_CUDA(cudaMemcpyAsync(dshot, &H, sizeof(Shot2D), cudaMemcpyHostToDevice, s));

    int sms = 1, dev = 0;
    GEO_CUDA(cudaGetDevice(&dev));
    GEO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int grid = ntiles < sms * 8 ? ntiles : sms * 8;
    for (int it = 0; it < D.nt; it++) {
        Step2D st{};
        st.it = it; st.amp = h_amp[it]; st.src_on = h_on[it]; st.taper = D.sv ? 1 : 0; st.nf = 1;
        GEO_TRY(launch_vel2d(var, dshot, items, ntiles, by, grid, st, s));
        GEO_TRY(launch_stress2d(var, PH_FWD, dshot, items, ntiles, by, grid, st, s));
    }
    if (D.mute_tt > 0) {
        // GPU-form direct-wave mute (GPU_vti2dfd_kernels.cu:151-174)
        const float mu_v = v00 * sqrtf(1 + 2 * e00);
        for (int ix = 0; ix < D.nx; ix++) {
            const float mu_x = D.dx * std::abs(ix - (int)D.fs - (D.is - 1) * (int)D.ds), mu_z = D.dz * (int)D.zs;
            const float mu_t0 = sqrtf((float)(std::pow(mu_x, 2) + std::pow(mu_z, 2))) / mu_v;
            const int mu_t = (int)(2.0 / (D.dt * D.favg));
            const int mu_nt = (int)(mu_t0 / D.dt) + mu_t + D.mute_tt;
            int a = (int)(mu_t0 / D.dt) - D.mute_tt + 1;
            if (a < 0) a = 0;
            const int b = mu_nt < D.nt ? mu_nt : D.nt;
            h_mute[ix] = a;
            h_mute[D.nx + ix] = b > a ? b : a;
        }
        GEO_CUDA(cudaMemcpyAsync(mute, h_mute, 2 * (size_t)D.nx * 4, cudaMemcpyHostToDevice, s));
        GEO_TRY(launch_mute_records(rec, D.nx, D.nt, mute, mute + D.nx, s));
    }
    GEO_TRY(launch_transpose_records(rec, shot, D.nx, D.nt, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}
