// 2D RTM with the semantics of the 2D GPU RTM program
// (2D-vti-fd+rtm-cuda/Toa_gpu2DvtiFdRtmAdcigsLaplace.cu, RTM() :1184-1566).
// Per shot:
//   forward, SV taper on (R=18, r=7, update_stress :303-404): point source
//     before the velocity update (add_source :204), record P at row npml
//     (shot_record :498), save the ring of P,Q (wavefield_bndr :532: rows
//     npml-1 and npml+nz+1, columns npml-1 and npml+nx+1), source
//     illumination ill += P*P + Q*Q, then <= 0 -> 1 (cal_illumination :654);
//   direct-wave mute of the record (mute_directwave :614, tt = 20 in the
//     program) -- the program launches one thread per sample rounded up to
//     512 without a bound on the sample index, so the surplus threads zero
//     samples of later traces; those samples are zeroed too;
//   backward, SV taper off: restore the ring into the source field and step
//     it forward, write the record into P and Q of the receiver field at row
//     npml (shot_record with record = false) and step it, image mig += sP*gP
//     (cal_migration :679) and the Poynting angle gathers (Poynting_Adcigs
//     :718-766).
// After the shots: mig /= ill, gathers /= ill (migration_illum :700,
// adcigs_illum :768), the adjoint Laplacian of the image and of the angle
// stack (stk_adcigs :799).  The image kernels of the program run over
// nnx*nnz threads on nx*nz arrays (an overrun); here they cover nx*nz.
// Fields are single buffers updated in place (the program's u0 = u1
// pointer assignment).
//
// The 2D TTI GPU RTM program (2D-tti-fd+rtm-cuda/
// Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu, main :500-800) has the same
// shot structure and runs through the same driver with its own choices:
// the TTI update_vel / update_stress (:126-228) over the tilt field, SV taper
// R=15, r=4, a mute with a sample bound whose direct-wave velocity is
// vp[1]*(1+(sqrtf(1+2 eps[1])-1)*cos(theta[1])) (:336-358, tt = 30 in the
// program), its own sponge (d0 with 3.0 in place of 10.0, whole-cell
// distances for both profile pairs; :230-233, :289-320), gathers at every
// dcdp-th CDP (Poynting_Adcigs :454-486,
// adcigs_illum :488-498), no angle stack and no readFile checks.  Where the
// program's adcigs_illum bound ((nx*nz)/dcdp*na) runs past its gathers
// array (nx not a multiple of dcdp) it divides floats beyond the array;
// here only the nx/dcdp gathers are divided.
#include "geo_internal.h"
#include "adcig.cuh"
#include "tti2d.cuh"
#include "gridsync.cuh"
#include <cmath>
#include <cstring>
#include <vector>

namespace geo {

__constant__ float c_grtm[4] = {1.196289f, -0.0797526f, 0.009570313f, -0.0006975447f};
__constant__ float c_gthr[128];   // angle-bin thresholds (largest cosine of bins >= k)
__constant__ float c_gcos[128];   // cosf(ia*pi/180) per bin

struct GRtm {
    int nnx, nnz, nx, nz, npml, nangle, dcdp;
    float dtx, dtz;
    const float *cx1, *cx2, *cz1, *cz2, *ax1, *ax2, *az1, *az2;
    const float *vp;
    const float *ct, *st;   // cos, sin of the tilt (TTI program)
};

struct GField {
    float *u, *w, *P, *Q, *px, *pz, *qx, *qz;
};

static TtiGrid tti_grid(const GRtm &g) {
    TtiGrid t;
    t.nnx = g.nnx; t.nnz = g.nnz; t.dtx = g.dtx; t.dtz = g.dtz;
    t.cx1 = g.cx1; t.cx2 = g.cx2; t.cz1 = g.cz1; t.cz2 = g.cz2;
    t.ax1 = g.ax1; t.ax2 = g.ax2; t.az1 = g.az1; t.az2 = g.az2;
    t.vp = g.vp; t.ct = g.ct; t.st = g.st;
    return t;
}

static TtiField tti_field(const GField &f) {
    TtiField t;
    t.u = f.u; t.w = f.w; t.px = f.px; t.pz = f.pz; t.qx = f.qx; t.qz = f.qz; t.P = f.P; t.Q = f.Q;
    return t;
}

// Everything one persistent launch of a pass needs.
struct GCoop {
    GRtm g;
    TtiGrid tg;
    GField S, R;                 // source-side and receiver-side fields
    TtiField tS, tR;
    const float *e2, *d2;        // stress model of the pass (SV taper forward)
    const float *amp;            // pfac*w(t) of every step
    const unsigned char *on;     // source active at every step
    long src;                    // source cell
    int ixs, izs;
    float *rec;                  // nt*nx, time-major
    float *bp, *bq;              // ring of P and Q, nt*L each
    float *ill, *mig, *adcig;
    int L;
    int it0, it1;                // forward: steps it0..it1-1; backward: it0 down to it1
    unsigned *bar;               // grid-barrier arrival counter, zeroed before the launch
    int *err;                    // set when a barrier wait gave up
};

// The VTI program's update_vel (Toa_gpu2DvtiFdRtmAdcigsLaplace.cu:256-289)
// at one point; SRC folds the step's point source (add_source :204, P,Q +=
// amp at the source cell before the update) into the taps that read it.
template <bool SRC>
__device__ __forceinline__ void g_vel_at(const GRtm &g, const GField &f, long id, int ix, int iz, long src, float amp) {
    const long s = g.nnz;
    float xx = 0.0f, zz = 0.0f;
#pragma unroll
    for (int im = 0; im < 4; im++) {
        xx += c_grtm[im] * (tti_tap<true, SRC>(f.P, id + (im + 1) * s, src, amp) - tti_tap<true, SRC>(f.P, id - im * s, src, amp));
        zz += c_grtm[im] * (tti_tap<true, SRC>(f.Q, id + im + 1, src, amp) - tti_tap<true, SRC>(f.Q, id - im, src, amp));
    }
    f.u[id] = g.cx2[ix] * __ldcg(f.u + id) - g.cx1[ix] * g.dtx * xx;
    f.w[id] = g.cz2[iz] * __ldcg(f.w + id) - g.cz1[iz] * g.dtz * zz;
}

// The VTI program's update_stress (:303-404) at one point; returns P and Q.
__device__ __forceinline__ float2 g_stress_at(const GRtm &g, const GField &f, const float *e2, const float *d2,
                                              long id, int ix, int iz) {
    const long s = g.nnz;
    float xx = 0.0f, zz = 0.0f;
#pragma unroll
    for (int im = 0; im < 4; im++) {
        xx += c_grtm[im] * (__ldcg(f.u + id + im * s) - __ldcg(f.u + id - (im + 1) * s));
        zz += c_grtm[im] * (__ldcg(f.w + id + im) - __ldcg(f.w + id - im - 1));
    }
    const float vp = g.vp[id];
    const float px = g.ax2[ix] * __ldcg(f.px + id) - g.ax1[ix] * vp * vp * e2[id] * g.dtx * xx;
    const float pz = g.az2[iz] * __ldcg(f.pz + id) - g.az1[iz] * vp * vp * d2[id] * g.dtz * zz;
    const float qx = g.ax2[ix] * __ldcg(f.qx + id) - g.ax1[ix] * vp * vp * d2[id] * g.dtx * xx;
    const float qz = g.az2[iz] * __ldcg(f.qz + id) - g.az1[iz] * vp * vp * g.dtz * zz;
    f.px[id] = px; f.pz[id] = pz; f.qx[id] = qx; f.qz[id] = qz;
    const float P = px + pz, Q = qx + qz;
    f.P[id] = P;
    f.Q[id] = Q;
    return make_float2(P, Q);
}

// One program's velocity / stress update: the TTI program's
// (Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu:126-228) over the tilt field,
// or the VTI program's.
template <bool TTI, bool SRC>
__device__ __forceinline__ void vel_at(const GCoop &a, const GField &f, const TtiField &tf, long id, int ix, int iz,
                                       float amp) {
    if constexpr (TTI) tti_vel_at<true, SRC>(a.tg, tf, c_grtm, id, ix, iz, a.src, amp);
    else g_vel_at<SRC>(a.g, f, id, ix, iz, a.src, amp);
}

template <bool TTI>
__device__ __forceinline__ float2 stress_at(const GCoop &a, const GField &f, const TtiField &tf, long id, int ix,
                                            int iz) {
    if constexpr (TTI) return tti_stress_at<true>(a.tg, tf, a.e2, a.d2, c_grtm, id, ix, iz);
    else return g_stress_at(a.g, f, a.e2, a.d2, id, ix, iz);
}

// Position of (ix, iz) in the ring of wavefield_bndr (:532): rows npml-1
// (top) and npml+nz+1 (bottom) over the nx interior columns, then columns
// npml-1 (left) and npml+nx+1 (right) over the nz interior rows; -1 off it.
__device__ __forceinline__ int ring_index(const GRtm &g, int ix, int iz) {
    const int npml = g.npml, nx = g.nx, nz = g.nz;
    if (ix >= npml && ix < npml + nx) {
        if (iz == npml - 1) return ix - npml;
        if (iz == npml + nz + 1) return nx + ix - npml;
    }
    if (iz >= npml && iz < npml + nz) {
        if (ix == npml - 1) return 2 * nx + iz - npml;
        if (ix == npml + nx + 1) return 2 * nx + nz + iz - npml;
    }
    return -1;
}

__device__ __forceinline__ bool g_updated(const GRtm &g, int ix, int iz) {
    return ix >= 4 && ix < g.nnx - 4 && iz >= 4 && iz < g.nnz - 4;
}

// Forward pass, steps it0..it1-1, one cooperative launch: per step the
// velocity half-step (source folded in), a grid barrier, the stress
// half-step with the SV taper and, per point, the surface record
// (shot_record :498), the ring save (wavefield_bndr :532) and the source
// illumination (cal_illumination :654: ill += P*P + Q*Q, <= 0 -> 1), a grid
// barrier.  The ring covers cells outside the updated band too (their
// unchanged values).
template <bool TTI>
// Four blocks per SM (64 registers): the passes are bound by the latency of
// their L2 round trips and the gathers' scattered updates, and at 1700x601
// that ran the TTI program 1.3x and the VTI program 1.1x faster than with
// the two blocks its 128 registers allowed.
__global__ void __launch_bounds__(256, 4) k_grtm_fwd(const GCoop a) {
    if (ld_acquire_u32(reinterpret_cast<const unsigned *>(a.err))) return;   // an earlier run gave up
    const GRtm &g = a.g;
    const long n = (long)g.nnx * g.nnz, stride = (long)gridDim.x * blockDim.x;
    const long first = blockIdx.x * (long)blockDim.x + threadIdx.x;
    unsigned k = 0;
    for (int it = a.it0; it < a.it1; it++) {
        const bool on = a.on[it] != 0;
        const float amp = a.amp[it];
        for (long id = first; id < n; id += stride) {
            const int ix = (int)(id / g.nnz), iz = (int)(id % g.nnz);
            if (!g_updated(g, ix, iz)) continue;
            const bool near = on && ((iz == a.izs && abs(ix - a.ixs) <= 4) || (ix == a.ixs && abs(iz - a.izs) <= 4));
            if (near) vel_at<TTI, true>(a, a.S, a.tS, id, ix, iz, amp);
            else vel_at<TTI, false>(a, a.S, a.tS, id, ix, iz, 0.0f);
        }
        if (!grid_barrier(a.bar, ++k * gridDim.x, a.err)) return;
        for (long id = first; id < n; id += stride) {
            const int ix = (int)(id / g.nnz), iz = (int)(id % g.nnz);
            const int r = ring_index(g, ix, iz), gx = ix - g.npml, gz = iz - g.npml;
            const bool inner = gx >= 0 && gx < g.nx && gz >= 0 && gz < g.nz;
            if (!g_updated(g, ix, iz)) {
                if (r >= 0) {
                    a.bp[(long)it * a.L + r] = __ldcg(a.S.P + id);
                    a.bq[(long)it * a.L + r] = __ldcg(a.S.Q + id);
                }
                continue;
            }
            const float2 pq = stress_at<TTI>(a, a.S, a.tS, id, ix, iz);
            if (gz == 0 && inner) a.rec[(long)it * g.nx + gx] = pq.x;
            if (r >= 0) {
                a.bp[(long)it * a.L + r] = pq.x;
                a.bq[(long)it * a.L + r] = pq.y;
            }
            if (inner) {
                const long o = (long)gx * g.nz + gz;
                float v = a.ill[o] + (pq.x * pq.x + pq.y * pq.y);
                if (v <= 0.0f) v = 1.0f;
                a.ill[o] = v;
            }
        }
        if (it + 1 < a.it1 && !grid_barrier(a.bar, ++k * gridDim.x, a.err)) return;
    }
}

// Before backward step it: the saved ring into the source-side P,Q and the
// muted record into the receiver-side P,Q at row npml (shot_record with
// record = false).
__device__ __forceinline__ void restore_inject(const GCoop &a, long id, int ix, int iz, int it) {
    const GRtm &g = a.g;
    const int r = ring_index(g, ix, iz);
    if (r >= 0) {
        a.S.P[id] = a.bp[(long)it * a.L + r];
        a.S.Q[id] = a.bq[(long)it * a.L + r];
    }
    const int gx = ix - g.npml;
    if (iz == g.npml && gx >= 0 && gx < g.nx) {
        const float v = a.rec[(long)it * g.nx + gx];
        a.R.P[id] = v;
        a.R.Q[id] = v;
    }
}

// Backward pass, steps it0 down to it1, one cooperative launch: the ring
// restore and record injection of step it0, a grid barrier, then per step
// both fields' velocity half-steps, a grid barrier, both stress half-steps
// with, per image point, the cross-correlation image (cal_migration :679)
// and the Poynting gathers (:718-766), then the restore and injection of
// the next step at the same point, a grid barrier.  A ring or surface cell
// is read by no other point of the phase that writes it.
template <bool TTI>
__global__ void __launch_bounds__(256, 4) k_grtm_bwd(const GCoop a) {
    if (ld_acquire_u32(reinterpret_cast<const unsigned *>(a.err))) return;
    const GRtm &g = a.g;
    const long n = (long)g.nnx * g.nnz, stride = (long)gridDim.x * blockDim.x;
    const long first = blockIdx.x * (long)blockDim.x + threadIdx.x;
    unsigned k = 0;
    for (long id = first; id < n; id += stride) restore_inject(a, id, (int)(id / g.nnz), (int)(id % g.nnz), a.it0);
    if (!grid_barrier(a.bar, ++k * gridDim.x, a.err)) return;
    for (int it = a.it0; it >= a.it1; it--) {
        for (long id = first; id < n; id += stride) {
            const int ix = (int)(id / g.nnz), iz = (int)(id % g.nnz);
            if (!g_updated(g, ix, iz)) continue;
            vel_at<TTI, false>(a, a.S, a.tS, id, ix, iz, 0.0f);
            vel_at<TTI, false>(a, a.R, a.tR, id, ix, iz, 0.0f);
        }
        if (!grid_barrier(a.bar, ++k * gridDim.x, a.err)) return;
        for (long id = first; id < n; id += stride) {
            const int ix = (int)(id / g.nnz), iz = (int)(id % g.nnz);
            if (g_updated(g, ix, iz)) {
                const float2 s = stress_at<TTI>(a, a.S, a.tS, id, ix, iz);
                const float2 r = stress_at<TTI>(a, a.R, a.tR, id, ix, iz);
                const int gx = ix - g.npml, gz = iz - g.npml;
                if (gx >= 0 && gx < g.nx && gz >= 0 && gz < g.nz) {
                    const long o = (long)gx * g.nz + gz;
                    const float sP = s.x, gP = r.x;
                    a.mig[o] = a.mig[o] + sP * gP;
                    // gathers at ix = 0, dcdp, ... below nx / dcdp * dcdp (Poynting_Adcigs
                    // :473 runs id < nx/dcdp*nz; the array holds nx/dcdp gathers)
                    if (a.adcig && gx % g.dcdp == 0 && gx / g.dcdp < g.nx / g.dcdp) {
                        const float Ssx = -sP * __ldcg(a.S.u + id), Ssz = -s.y * __ldcg(a.S.w + id);
                        const float Sgx = gP * __ldcg(a.R.u + id), Sgz = r.y * __ldcg(a.R.w + id);
                        const float b1 = Ssx * Ssx + Ssz * Ssz, b2 = Sgx * Sgx + Sgz * Sgz;
                        const int ia = poynting_bin(Ssx * Sgx + Ssz * Sgz, b1, b2, c_gthr, g.nangle);
                        if (ia >= 0) {
                            const float c = c_gcos[ia];
                            float *ag = a.adcig + gz + (long)g.nz * ia + (long)g.nz * g.nangle * (gx / g.dcdp);
                            *ag = *ag + sP * gP * c * c * c;
                        }
                    }
                }
            }
            if (it > a.it1) restore_inject(a, id, ix, iz, it - 1);
        }
        if (it > a.it1 && !grid_barrier(a.bar, ++k * gridDim.x, a.err)) return;
    }
}

__global__ void k_g_mask(float *rec, const uint8_t *keep, long n) {
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
        if (!keep[k]) rec[k] = 0.0f;
}

// gathers [ixa][ia][iz] /= ill[ixa*dcdp][iz]
__global__ void k_g_adcig_norm(float *adcig, const float *ill, int nxa, int nz, int nangle, int dcdp) {
    const long n = (long)nxa * nz * nangle;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int ix = (int)(k / ((long)nz * nangle)) * dcdp, iz = (int)(k % nz);
        adcig[k] = adcig[k] / ill[iz + (long)nz * ix];
    }
}

// angle stack (stk_adcigs :799-818): stk = 0, += over the angles in order
__global__ void k_g_stack_angles(const float *adcig, float *stk, int nx, int nz, int nangle) {
    const long n = (long)nx * nz;
    for (long o = blockIdx.x * (long)blockDim.x + threadIdx.x; o < n; o += (long)gridDim.x * blockDim.x) {
        const int ix = (int)(o / nz), iz = (int)(o % nz);
        float s = 0.0f;
        for (int ia = 0; ia < nangle; ia++) s += adcig[(long)ix * nangle * nz + (long)ia * nz + iz];
        stk[o] = s;
    }
}

// The programs' bin of a cosine a: (int)((float)(0.5*acosf(a)*180.0/pi) / (dangle*1.0)),
// with the device's acosf, as their Poynting_Adcigs kernels evaluate it.
__device__ int ref_gpu_bin(float a, int dangle) {
    const float deg = (float)(0.5 * acosf(a) * 180.0 / kPiGui);
    return (int)(deg / (dangle * 1.0));
}

// Float keys ordered like the floats they encode.
__device__ uint32_t okey(float f) {
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ float kfloat(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// One thread per bin k < kMaxAngles: thr[k] = largest float a in [-1,1]
// with bin(a) >= k+1 (binary search over the ordered float keys; bin is
// non-increasing in a), -2 where none is; cs[k] = cosf(k*pi/180).  Both
// come from the device's acosf and cosf, the functions the programs'
// kernels call, so the tables give their bins and weights bit for bit.
__global__ void k_angle_tables(float *thr, float *cs, int nangle, int dangle) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= kMaxAngles) return;
    cs[k] = k < nangle ? cosf((float)(k * kPiGui / 180.0)) : 0.0f;
    float t = -2.0f;
    if (k < nangle && ref_gpu_bin(-1.0f, dangle) >= k + 1) {
        uint32_t a = okey(-1.0f), b = okey(1.0f);
        while (a < b) {
            const uint32_t m = a + (b - a + 1) / 2;
            if (ref_gpu_bin(kfloat(m), dangle) >= k + 1) a = m;
            else b = m - 1;
        }
        t = kfloat(a);
    }
    thr[k] = t;
}

int adcig_angle_tables(int nangle, int dangle, float *thr, float *cs, cudaStream_t s) {
    k_angle_tables<<<1, kMaxAngles, 0, s>>>(thr, cs, nangle, dangle);
    return check_launch("angle_tables");
}

__device__ float g_angle_stage[2 * kMaxAngles];

static int gpu_adcig_tables(int nangle, int dangle, cudaStream_t s) {
    void *stage = nullptr;
    GEO_CUDA(cudaGetSymbolAddress(&stage, g_angle_stage));
    float *st = static_cast<float *>(stage);
    GEO_TRY(adcig_angle_tables(nangle, dangle, st, st + kMaxAngles, s));
    GEO_CUDA(cudaMemcpyToSymbolAsync(c_gthr, st, kMaxAngles * 4, 0, cudaMemcpyDeviceToDevice, s));
    GEO_CUDA(cudaMemcpyToSymbolAsync(c_gcos, st + kMaxAngles, kMaxAngles * 4, 0, cudaMemcpyDeviceToDevice, s));
    return GEO_OK;
}

// readFile's checks (:930-965): grid spacing for the frequency, dt, dispersion, stability.
static int gpu_rtm_checks(const geo_rtm2d_gpu_desc &D, const std::vector<float> &v) {
    float vmin = 999999.9f, vmax = -999999.9f;
    for (float x : v) {
        vmin = std::min(vmin, x);
        vmax = std::max(vmax, x);
    }
    const float H_min = D.dx < D.dz ? D.dx : D.dz;
    const float dt_max = (float)(0.5 * H_min / vmin), dxz_max = (float)(vmax / D.favg * 0.2);
    if (dxz_max < D.dz || dxz_max < D.dx) return fail(GEO_ERR_CFL, "grid spacing too coarse for favg (redefine dx, dz)");
    if (dt_max < D.dt) return fail(GEO_ERR_CFL, "dt too large (redefine dt)");
    if (D.favg >= vmin / (5.0 * (D.dx > D.dz ? D.dx : D.dz))) return fail(GEO_ERR_CFL, "non-dispersion relation not satisfied");
    const float tmp = (float)(D.dt * vmax * sqrtf((float)(1.0 / (D.dx * D.dx) + 1.0 / (D.dz * D.dz))));
    if (tmp >= 0.777f) return fail(GEO_ERR_CFL, "stability condition not satisfied (%g >= 0.777)", tmp);
    return GEO_OK;
}

static int grid_of_n(long n) { return (int)std::min<long>((n + 255) / 256, 152L * 16); }

}  // namespace geo

namespace geo {

// What differs between the two GPU RTM programs that share this driver.
struct GpuRtmProgram {
    bool tti;            // TTI stencil over a tilt field (theta, degrees)
    int taper_R, taper_r;  // SV taper radii of the forward stress update
    bool mute_overrun;   // the mute launch has no sample bound (VTI program)
    bool checks;         // readFile's dispersion / stability checks (VTI program)
};

static int gpu_rtm_run(const GpuRtmProgram &prog, const geo_rtm2d_gpu_desc &D, const float *v, const float *e,
                       const float *d, const float *theta, const float *obs, float *mig_lap, float *illum,
                       float *adcigs, float *stk_lap, float *shots, int mem, void *stream) {
    if (D.nx < 2 || D.nz < 2 || D.npml < 5 || D.nt < 1 || D.ns < 1) return fail(GEO_ERR_ARG, "bad sizes");
    if (!(D.dt > 0) || !(D.dx > 0) || !(D.dz > 0) || !(D.favg > 0)) return fail(GEO_ERR_ARG, "bad spacing");
    if (D.nangle < 1 || D.nangle > 128 || D.dangle < 1) return fail(GEO_ERR_ARG, "nangle must be 1..128, dangle >= 1");
    const int dcdp = D.dcdp > 0 ? D.dcdp : 1;
    if (dcdp > D.nx) return fail(GEO_ERR_ARG, "dcdp exceeds nx");
    if (dcdp != 1 && !prog.tti) return fail(GEO_ERR_ARG, "the VTI program forms gathers at every CDP (dcdp 0 or 1)");
    if (mem != GEO_MEM_HOST && mem != GEO_MEM_DEVICE) return fail(GEO_ERR_ARG, "bad mem kind");
    const int nx = D.nx, nz = D.nz, npml = D.npml, nt = D.nt, nnx = nx + 2 * npml, nnz = nz + 2 * npml;
    const size_t n0 = (size_t)nx * nz, n = (size_t)nnx * nnz;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<float> hv(n0), he(n0), hd(n0), ht(prog.tti ? n0 : 0);
    const float *src[4] = {v, e, d, theta};
    float *dst[4] = {hv.data(), he.data(), hd.data(), ht.data()};
    for (int k = 0; k < (prog.tti ? 4 : 3); k++) {
        if (mem == GEO_MEM_DEVICE) GEO_CUDA(cudaMemcpyAsync(dst[k], src[k], n0 * 4, cudaMemcpyDeviceToHost, s));
        else memcpy(dst[k], src[k], n0 * 4);
    }
    GEO_CUDA(cudaStreamSynchronize(s));
    GEO_TRY(check_model(hv.data(), he.data(), hd.data(), n0));
    if (prog.tti)
        for (size_t k = 0; k < n0; k++)
            if (!std::isfinite(ht[k])) return fail(GEO_ERR_MODEL, "theta[%zu] not finite", k);
    if (prog.checks) GEO_TRY(gpu_rtm_checks(D, hv));
    for (int is = 1; is <= D.ns; is++) {
        const int ixs = D.fs + (is - 1) * D.ds + npml - 1, izs = D.zs + npml - 1;
        if (ixs < 4 || ixs >= nnx - 4 || izs < 4 || izs >= nnz - 4) return fail(GEO_ERR_ARG, "shot %d outside the grid", is);
    }
    std::vector<float> pv(n), pe(n), pd(n);
    pad_model_2d(nx, nz, npml, hv.data(), pv.data());
    pad_model_2d(nx, nz, npml, he.data(), pe.data());
    pad_model_2d(nx, nz, npml, hd.data(), pd.data());
    // get_d0 and initial_coffe of the program (VTI :110-118; TTI :230-233, :289-320)
    const Variant sp = prog.tti ? V_TTIRTM : V_GPU;
    const float d0 = sponge_d0(sp, 2, 0.0f, pv[n / 2], npml, D.dx, D.dx, D.dz);
    std::vector<float> prof(4 * (size_t)(nnx + nnz));
    float *q = prof.data();
    sponge_profiles(sp, nx, npml, D.dt, d0, q, q + nnx, q + 2 * nnx, q + 3 * nnx);
    q += 4 * nnx;
    sponge_profiles(sp, nz, npml, D.dt, d0, q, q + nnz, q + 2 * nnz, q + 3 * nnz);
    std::vector<float> amp;
    std::vector<uint8_t> on;
    source_amplitudes(V_GPU, nt, D.dt, D.favg, D.pfac, D.wtype, amp, on);
    // untapered 1+2eps, sqrtf(1+2del)
    std::vector<float> e2(n), d2(n);
    for (size_t k = 0; k < n; k++) {
        e2[k] = 1 + 2 * pe[k];
        d2[k] = sqrtf(1 + 2 * pd[k]);
    }
    // tilt in radians as read_file converts it (theta *= pi/180); its cos and
    // sin are formed on the device below, as the program's kernels form them
    std::vector<float> ct;
    float mu_v = pv[1] * sqrtf(1 + 2 * pe[1]);   // direct-wave velocity of the VTI program's mute
    if (prog.tti) {
        std::vector<float> pt(n);
        pad_model_2d(nx, nz, npml, ht.data(), pt.data());
        ct.resize(n);
        for (size_t k = 0; k < n; k++) ct[k] = (float)((double)pt[k] * (kPiGui / 180.0));
    }
    const int L = 2 * nx + 2 * nz;

    DevBuf dvp, dprof, de2, dd2, dte2, dtd2, fs_, fr_, ring, rec, mig, ill, ag, lap, stk, mkeep, trs, dct, dst_;
    GEO_TRY(dvp.alloc(n * 4));
    if (prog.tti) {
        GEO_TRY(dct.alloc(n * 4));
        GEO_TRY(dst_.alloc(n * 4));
        GEO_CUDA(cudaMemcpyAsync(dct.p, ct.data(), n * 4, cudaMemcpyHostToDevice, s));
        GEO_TRY(launch_tilt_trig(dct.as<float>(), dst_.as<float>(), n, s));
        // mute_directwave of the TTI program: vp[1]*(1+(sqrtf(1+2 eps[1])-1)*cos(theta[1]))
        float c1 = 0.0f;
        GEO_CUDA(cudaMemcpyAsync(&c1, dct.as<float>() + 1, 4, cudaMemcpyDeviceToHost, s));
        GEO_CUDA(cudaStreamSynchronize(s));
        mu_v = pv[1] * (1 + (sqrtf(1 + 2 * pe[1]) - 1) * c1);
    }
    GEO_TRY(dprof.alloc(prof.size() * 4));
    GEO_TRY(de2.alloc(n * 4));
    GEO_TRY(dd2.alloc(n * 4));
    GEO_TRY(dte2.alloc(n * 4));
    GEO_TRY(dtd2.alloc(n * 4));
    GEO_TRY(fs_.alloc(8 * n * 4));
    GEO_TRY(fr_.alloc(8 * n * 4));
    GEO_TRY(ring.alloc((size_t)2 * nt * L * 4));
    GEO_TRY(rec.alloc((size_t)nt * nx * 4));
    GEO_TRY(mig.alloc(n0 * 4));
    GEO_TRY(ill.alloc(n0 * 4));
    GEO_TRY(mkeep.alloc((size_t)nt * nx));
    const int nxa = nx / dcdp;
    const size_t nag = (size_t)D.nangle * nz * nxa;
    if (adcigs || stk_lap) {
        GEO_TRY(ag.alloc(nag * 4));
        GEO_TRY(ag.zero(s));
        GEO_TRY(gpu_adcig_tables(D.nangle, D.dangle, s));
    }
    GEO_CUDA(cudaMemcpyAsync(dvp.p, pv.data(), n * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemcpyAsync(dprof.p, prof.data(), prof.size() * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemcpyAsync(de2.p, e2.data(), n * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemcpyAsync(dd2.p, d2.data(), n * 4, cudaMemcpyHostToDevice, s));
    GEO_TRY(mig.zero(s));
    GEO_TRY(ill.zero(s));
    GRtm g{};
    g.nnx = nnx; g.nnz = nnz; g.nx = nx; g.nz = nz; g.npml = npml; g.nangle = D.nangle; g.dcdp = dcdp;
    g.ct = dct.as<float>();
    g.st = dst_.as<float>();
    g.dtx = D.dt / D.dx;
    g.dtz = D.dt / D.dz;
    const float *pp = dprof.as<float>();
    g.cx1 = pp; g.cx2 = pp + nnx; g.ax1 = pp + 2 * nnx; g.ax2 = pp + 3 * nnx;
    pp += 4 * nnx;
    g.cz1 = pp; g.cz2 = pp + nnz; g.az1 = pp + 2 * nnz; g.az2 = pp + 3 * nnz;
    g.vp = dvp.as<float>();
    auto fields = [&](DevBuf &b) {
        GField f;
        float *p = b.as<float>();
        f.u = p; f.w = p + n; f.P = p + 2 * n; f.Q = p + 3 * n;
        f.px = p + 4 * n; f.pz = p + 5 * n; f.qx = p + 6 * n; f.qz = p + 7 * n;
        return f;
    };
    const GField S = fields(fs_), R = fields(fr_);
    float *bp = ring.as<float>(), *bq = bp + (size_t)nt * L;
    const int gi = grid_of_n((long)n0);
    const cudaMemcpyKind kout = mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const cudaMemcpyKind kin = mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    if (shots || obs) GEO_TRY(trs.alloc((size_t)nt * nx * 4));
    DevBuf d_amp, d_on, d_sync;
    GEO_TRY(d_amp.alloc((size_t)nt * 4));
    GEO_TRY(d_on.alloc((size_t)nt));
    GEO_TRY(d_sync.alloc(8));
    GEO_TRY(d_sync.zero(s));
    GEO_CUDA(cudaMemcpyAsync(d_amp.p, amp.data(), (size_t)nt * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemcpyAsync(d_on.p, on.data(), (size_t)nt, cudaMemcpyHostToDevice, s));
    GCoop a{};
    a.g = g;
    a.tg = tti_grid(g);
    a.S = S;
    a.R = R;
    a.tS = tti_field(S);
    a.tR = tti_field(R);
    a.amp = d_amp.as<float>();
    a.on = d_on.as<unsigned char>();
    a.rec = rec.as<float>();
    a.bp = bp;
    a.bq = bq;
    a.ill = ill.as<float>();
    a.mig = mig.as<float>();
    a.adcig = ag.p ? ag.as<float>() : nullptr;
    a.L = L;
    a.bar = d_sync.as<unsigned>();
    a.err = d_sync.as<int>() + 1;
    // every block resident at once (the grid barrier needs it; the
    // cooperative launch checks it), threads striding over the points
    const void *kf = prog.tti ? (const void *)k_grtm_fwd<true> : (const void *)k_grtm_fwd<false>;
    const void *kb = prog.tti ? (const void *)k_grtm_bwd<true> : (const void *)k_grtm_bwd<false>;
    int grid_f = 0, grid_b = 0;
    {
        int dev = 0, sms = 0, occ_f = 0, occ_b = 0, coop = 0;
        GEO_CUDA(cudaGetDevice(&dev));
        GEO_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        GEO_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
        GEO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_f, kf, 256, 0));
        GEO_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_b, kb, 256, 0));
        if (!coop || occ_f < 1 || occ_b < 1) return fail(GEO_ERR_CUDA, "cooperative launch unavailable");
        grid_f = (int)std::min<size_t>((n + 255) / 256, (size_t)occ_f * sms);
        grid_b = (int)std::min<size_t>((n + 255) / 256, (size_t)occ_b * sms);
        if ((long long)std::max(grid_f, grid_b) * (2LL * nt + 2) >= 4000000000LL)
            return fail(GEO_ERR_ARG, "too many steps for one launch");
    }
    auto launch = [&](const void *fn, int grid, int it0, int it1) -> int {
        a.it0 = it0;
        a.it1 = it1;
        GEO_CUDA(cudaMemsetAsync(a.bar, 0, 4, s));
        void *args[] = {(void *)&a};
        GEO_CUDA(cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(256), args, 0, s));
        return check_launch("grtm_pass");
    };
    Watchdog wd;
    GEO_TRY(wd.open());
    for (int is = 1; is <= D.ns; is++) {
        // SV taper box of this shot (centre fs+(is-1)ds+npml, zs+npml)
        std::vector<float> te2(e2), td2(d2);
        {
            const int TR = prog.taper_R, tr = prog.taper_r;
            const int cx = D.fs + (is - 1) * D.ds + npml, cz = D.zs + npml, R2 = TR * TR, r2 = tr * tr;
            for (int ix = std::max(0, cx - TR); ix <= std::min(nnx - 1, cx + TR); ix++)
                for (int iz = std::max(0, cz - TR); iz <= std::min(nnz - 1, cz + TR); iz++) {
                    const int rx = ix - cx, rz = iz - cz, q2 = rx * rx + rz * rz;
                    if (q2 > R2) continue;
                    const size_t id = (size_t)ix * nnz + iz;
                    float ee = 0.0f, dd = 0.0f;
                    if (q2 > r2) {
                        const double gq = 0.5 * (1 - std::cos(kPiGui * ((sqrtf((float)q2) - tr) * 4.0 / (TR * 3.0 - 1))));
                        ee = (float)(gq * pe[id]);
                        dd = (float)(gq * pd[id]);
                    }
                    te2[id] = 1 + 2 * ee;
                    td2[id] = sqrtf(1 + 2 * dd);
                }
        }
        GEO_CUDA(cudaMemcpyAsync(dte2.p, te2.data(), n * 4, cudaMemcpyHostToDevice, s));
        GEO_CUDA(cudaMemcpyAsync(dtd2.p, td2.data(), n * 4, cudaMemcpyHostToDevice, s));
        GEO_TRY(fs_.zero(s));
        GEO_TRY(fr_.zero(s));
        GEO_TRY(rec.zero(s));
        GEO_TRY(ring.zero(s));
        a.ixs = D.fs + (is - 1) * D.ds + npml - 1;
        a.izs = D.zs + npml - 1;
        a.src = (long)a.ixs * nnz + a.izs;
        a.e2 = dte2.as<float>();
        a.d2 = dtd2.as<float>();
        // runs of steps between the watchdog's scans, one launch each
        for (int it0 = 0; it0 < nt;) {
            int it1 = it0 + 1;
            while (it1 < nt && !(wd.every > 0 && it1 % wd.every == 0)) it1++;
            GEO_TRY(launch(kf, grid_f, it0, it1));
            const int w = wd.check(S.P, n, it1 - 1, it1 == nt, s);
            if (w == GEO_ERR_NAN) break;
            GEO_TRY(w);
            it0 = it1;
        }
        GEO_TRY(wd.verdict(s, "2D RTM forward pass"));
        // direct-wave mute (GPU form, tt), exactly as the program's kernel
        // writes it.  VTI program: thread it < nt rounded up to 512 zeroes
        // flat sample ix*nt + it of the trace-major record for every trace
        // ix whose window holds it -- past nt that lands on later traces.
        // TTI program: one thread per sample, bounded.
        {
            std::vector<uint8_t> keep((size_t)nt * nx, 1);   // time-major
            const int nt512 = prog.mute_overrun ? (nt + 511) / 512 * 512 : nt;
            for (int ix = 0; ix < nx; ix++) {
                const float mu_x = D.dx * std::abs(ix - D.fs - (is - 1) * D.ds), mu_z = D.dz * D.zs;
                const float mu_t0 = sqrtf((float)(std::pow(mu_x, 2) + std::pow(mu_z, 2))) / mu_v;
                const int mu_t = (int)(2.0 / (D.dt * D.favg));
                const int mu_nt = (int)(mu_t0 / D.dt) + mu_t + D.mute_tt;
                const int first = std::max(0, (int)(mu_t0 / D.dt) - D.mute_tt + 1);
                for (int it = first; it < std::min(mu_nt, nt512); it++) {
                    const long j = (long)ix * nt + it;          // trace-major flat index
                    if (j >= (long)nx * nt) break;
                    keep[(size_t)(j % nt) * nx + (size_t)(j / nt)] = 0;
                }
            }
            GEO_CUDA(cudaMemcpyAsync(mkeep.p, keep.data(), keep.size(), cudaMemcpyHostToDevice, s));
            k_g_mask<<<grid_of_n((long)nt * nx), 256, 0, s>>>(rec.as<float>(), mkeep.as<uint8_t>(), (long)nt * nx);
            GEO_TRY(check_launch("grtm_mute"));
            GEO_CUDA(cudaStreamSynchronize(s));
        }
        if (shots) {
            GEO_TRY(launch_transpose_records(rec.as<float>(), trs.as<float>(), nx, nt, s));
            GEO_CUDA(cudaMemcpyAsync(shots + (size_t)(is - 1) * nx * nt, trs.p, (size_t)nx * nt * 4, kout, s));
        }
        if (obs) {
            // observed shot (trace-major nx*nt) replaces the modelled record
            GEO_CUDA(cudaMemcpyAsync(trs.p, obs + (size_t)(is - 1) * nx * nt, (size_t)nx * nt * 4, kin, s));
            GEO_TRY(launch_transpose_records(trs.as<float>(), rec.as<float>(), nt, nx, s));
        }
        a.e2 = de2.as<float>();
        a.d2 = dd2.as<float>();
        // runs of steps between the watchdog's scans (after backward step
        // it when (nt - it) is a multiple of the interval), one launch each
        for (int hi = nt - 1; hi >= 0;) {
            int lo = hi;
            while (lo > 0 && !(wd.every > 0 && (nt - lo) % wd.every == 0)) lo--;
            GEO_TRY(launch(kb, grid_b, hi, lo));
            const int w = wd.check(R.P, n, nt - 1 - lo, lo == 0, s);
            if (w == GEO_ERR_NAN) break;
            GEO_TRY(w);
            hi = lo - 1;
        }
        GEO_TRY(wd.verdict(s, "2D RTM backward pass"));
    }
    {
        int err = 0;
        GEO_CUDA(cudaMemcpyAsync(&err, a.err, 4, cudaMemcpyDeviceToHost, s));
        GEO_CUDA(cudaStreamSynchronize(s));
        if (err) return fail(GEO_ERR_CUDA, "2D RTM: a grid barrier wait timed out");
    }
    GEO_TRY(launch_normalize_image(mig.as<float>(), ill.as<float>(), n0, s));
    GEO_TRY(lap.alloc(n0 * 4));
    GEO_TRY(launch_laplace2d(nx, nz, mig.as<float>(), lap.as<float>(), s));
    GEO_CUDA(cudaMemcpyAsync(mig_lap, lap.p, n0 * 4, kout, s));
    if (illum) GEO_CUDA(cudaMemcpyAsync(illum, ill.p, n0 * 4, kout, s));
    if (ag.p) {
        k_g_adcig_norm<<<grid_of_n((long)nag), 256, 0, s>>>(ag.as<float>(), ill.as<float>(), nxa, nz, D.nangle, dcdp);
        GEO_TRY(check_launch("grtm_adcig_norm"));
        if (adcigs) GEO_CUDA(cudaMemcpyAsync(adcigs, ag.p, nag * 4, kout, s));
        if (stk_lap) {
            GEO_TRY(stk.alloc(n0 * 4));
            k_g_stack_angles<<<gi, 256, 0, s>>>(ag.as<float>(), stk.as<float>(), nx, nz, D.nangle);
            GEO_TRY(check_launch("grtm_stack_angles"));
            GEO_TRY(launch_laplace2d(nx, nz, stk.as<float>(), lap.as<float>(), s));
            GEO_CUDA(cudaMemcpyAsync(stk_lap, lap.p, n0 * 4, kout, s));
        }
    }
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}

}  // namespace geo

using namespace geo;

extern "C" int geo_rtm2d_gpu(const geo_rtm2d_gpu_desc *desc, const float *v, const float *e, const float *d,
                             const float *obs, float *mig_lap, float *illum, float *adcigs, float *stk_lap,
                             float *shots, int mem, void *stream) {
    if (!desc || !v || !e || !d || !mig_lap) return fail(GEO_ERR_ARG, "null argument");
    const GpuRtmProgram vti{false, 18, 7, true, true};
    return gpu_rtm_run(vti, *desc, v, e, d, nullptr, obs, mig_lap, illum, adcigs, stk_lap, shots, mem, stream);
}

extern "C" int geo_rtm2d_tti(const geo_rtm2d_gpu_desc *desc, const float *v, const float *e, const float *d,
                             const float *theta, const float *obs, float *mig_lap, float *illum, float *adcigs,
                             float *shots, int mem, void *stream) {
    if (!desc || !v || !e || !d || !theta || !mig_lap) return fail(GEO_ERR_ARG, "null argument");
    const GpuRtmProgram tti{true, 15, 4, false, false};
    return gpu_rtm_run(tti, *desc, v, e, d, theta, obs, mig_lap, illum, adcigs, nullptr, shots, mem, stream);
}
