// Point updates of the 2D TTI staggered-grid scheme of the GPU TTI programs
// (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:81-183, the same
// kernels as Toa_gpu_2dtti_rtm_adcigs_iorderfunciton.cu:126-228):
//   u <- cx2 cz2 u - cx1 cz1 (cos t dtx dP/dx - sin t dtz dP/dz)
//   w <- cx2 cz2 w - cx1 cz1 (sin t dtx dQ/dx + cos t dtz dQ/dz)
//   px,pz,qx,qz <- ax2 az2 (.) - ax1 az1 vp^2 {1+2e, sqrtf(1+2d), sqrtf(1+2d), 1} (rotated derivative)
//   P = px + pz, Q = qx + qz
// in the programs' operation order.  Fields are updated in place (the
// programs' u0 = u1 pointer assignment leaves one buffer per field); each
// point writes only itself and reads only neighbours of the other field, so
// one launch (or one phase of a persistent launch) per half-step is
// race-free.  cos and sin of the tilt are tables (ct, st) formed with the
// device's cosf/sinf, as the programs' kernels evaluate them.
#pragma once

namespace geo {

struct TtiGrid {
    int nnx, nnz;
    float dtx, dtz;
    const float *cx1, *cx2, *cz1, *cz2, *ax1, *ax2, *az1, *az2;
    const float *vp, *ct, *st;
};

struct TtiField {
    float *u, *w, *px, *pz, *qx, *qz, *P, *Q;
};

// Field loads: plain, or through L2 (CG) when other blocks of a persistent
// launch wrote the values before a grid barrier (L1 is not coherent with
// them).
template <bool CG>
__device__ __forceinline__ float tti_ld(const float *p) {
    if constexpr (CG) return __ldcg(p);
    else return *p;
}

// P/Q tap of the velocity update.  SRC folds in the point source of the
// step (P,Q += amp at cell src before the velocity update): the tap that
// reads the source cell gets the same single float addition.
template <bool CG, bool SRC>
__device__ __forceinline__ float tti_tap(const float *a, long idx, long src, float amp) {
    float v = tti_ld<CG>(a + idx);
    if (SRC && idx == src) v = v + amp;
    return v;
}

// c: the four staggered coefficients (a __constant__ array of the caller's file)
template <bool CG = false, bool SRC = false>
__device__ __forceinline__ void tti_vel_at(const TtiGrid &g, const TtiField &f, const float *c, long id, int ix,
                                           int iz, long src = -1, float amp = 0.0f) {
    const long s = g.nnz;
    float Px = 0.0f, Pz = 0.0f, Qz = 0.0f, Qx = 0.0f;
#pragma unroll
    for (int im = 0; im < 4; im++) {
        Px += c[im] * (tti_tap<CG, SRC>(f.P, id + (im + 1) * s, src, amp) - tti_tap<CG, SRC>(f.P, id - im * s, src, amp));
        Pz += c[im] * (tti_tap<CG, SRC>(f.P, id + im + 1, src, amp) - tti_tap<CG, SRC>(f.P, id - im, src, amp));
        Qz += c[im] * (tti_tap<CG, SRC>(f.Q, id + im + 1, src, amp) - tti_tap<CG, SRC>(f.Q, id - im, src, amp));
        Qx += c[im] * (tti_tap<CG, SRC>(f.Q, id + (im + 1) * s, src, amp) - tti_tap<CG, SRC>(f.Q, id - im * s, src, amp));
    }
    const float ct = g.ct[id], st = g.st[id];
    const float k2 = g.cx2[ix] * g.cz2[iz], k1 = g.cx1[ix] * g.cz1[iz];
    f.u[id] = k2 * tti_ld<CG>(f.u + id) - k1 * (ct * g.dtx * Px - st * g.dtz * Pz);
    f.w[id] = k2 * tti_ld<CG>(f.w + id) - k1 * (st * g.dtx * Qx + ct * g.dtz * Qz);
}

// e2 = 1+2*eps, d2 = sqrtf(1+2*del) (tapered or not, as the caller's step
// needs).  Returns the new P and Q.
template <bool CG = false>
__device__ __forceinline__ float2 tti_stress_at(const TtiGrid &g, const TtiField &f, const float *e2,
                                               const float *d2, const float *c, long id, int ix, int iz) {
    const long s = g.nnz;
    float ux = 0.0f, uz = 0.0f, wz = 0.0f, wx = 0.0f;
#pragma unroll
    for (int im = 0; im < 4; im++) {
        ux += c[im] * (tti_ld<CG>(f.u + id + im * s) - tti_ld<CG>(f.u + id - (im + 1) * s));
        uz += c[im] * (tti_ld<CG>(f.u + id + im) - tti_ld<CG>(f.u + id - im - 1));
        wz += c[im] * (tti_ld<CG>(f.w + id + im) - tti_ld<CG>(f.w + id - im - 1));
        wx += c[im] * (tti_ld<CG>(f.w + id + im * s) - tti_ld<CG>(f.w + id - (im + 1) * s));
    }
    const float ct = g.ct[id], st = g.st[id], vp = g.vp[id];
    const float A = ct * g.dtx * ux - st * g.dtz * uz, B = st * g.dtx * wx + ct * g.dtz * wz;
    const float k2 = g.ax2[ix] * g.az2[iz], k1 = g.ax1[ix] * g.az1[iz];
    const float px = k2 * tti_ld<CG>(f.px + id) - k1 * vp * vp * e2[id] * A;
    const float pz = k2 * tti_ld<CG>(f.pz + id) - k1 * vp * vp * d2[id] * B;
    const float qx = k2 * tti_ld<CG>(f.qx + id) - k1 * vp * vp * d2[id] * A;
    const float qz = k2 * tti_ld<CG>(f.qz + id) - k1 * vp * vp * B;
    f.px[id] = px; f.pz[id] = pz; f.qx[id] = qx; f.qz[id] = qz;
    const float P = px + pz, Q = qx + qz;
    f.P[id] = P;
    f.Q[id] = Q;
    return make_float2(P, Q);
}

}  // namespace geo
