// 3D TTI time step: tilt t (from the vertical) and azimuth f of the symmetry
// axis per grid point.  No reference program has a 3D TTI scheme; this one
// extends the 2D TTI GPU programs' rotated-derivative scheme
// (2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:81-183) to a tilted
// and rotated axis.  With the rotated frame
//   x' = (cos t cos f, cos t sin f, -sin t), y' = (-sin f, cos f, 0),
//   z' = (sin t cos f, sin t sin f, cos t):
//   u <- k2 u - k1 dP/dx',  v <- k2 v - k1 dP/dy',  w <- k2 w - k1 dQ/dz'
//   P <- k2 P - k1 (A a + B b),  Q <- k2 Q - k1 (B a + C b)
// a = du/dx' + dv/dy', b = dw/dz', A = vp^2(1+2eps), B = vp^2 sqrtf(1+2del),
// C = vp^2 (the plan's premultiplied model), k the 2D programs' product
// sponge (half-grid profiles for the velocities, integer-grid for the
// stresses).  Each axis derivative has the 2D programs' stagger (forward for
// the velocities, backward for the stresses).  With t = f = 0 the
// derivatives are the VTI step's; with f = 0 and no y the 2D programs'.
//
// Two kernels per step over one thread per point (z fastest, 32 x 4 blocks,
// every tap through the read-only path): velocities from P,Q of level c
// into level n, then stresses from the new velocities and P,Q of level c
// into level n, with the receivers and the RTM imaging epilogue of the VTI
// step.  Measured at 600x600x400 + 40: 7.62 ms per step against 9.26 ms
// with 32 x 8 blocks and plain loads (shared x/z tiles and y-marching blocks
// were no faster).  The point source is added to P,Q of level c
// before the velocity kernel (the cell's old values kept in `save`), so it
// reaches the velocities only, as in the VTI step.  The operation order is
// the oracle's (orc_tti3d), so FP32 results are bit-identical to it.
#include "geo_internal.h"
#include "fd3d.cuh"

namespace geo {

__constant__ float c_tti3d[4] = {1.196289f, -0.0797526f, 0.009570313f, -0.0006975447f};

// Source cell: keep P,Q of level c, then add the amplitude.
__global__ void k_tti3d_source(float *P, float *Q, long src, float amp, float *save) {
    save[0] = P[src];
    save[1] = Q[src];
    P[src] += amp;
    Q[src] += amp;
}

__global__ void __launch_bounds__(128) k_tti3d_vel(const Tti3DStep t) {
    const int iz = blockIdx.x * 32 + threadIdx.x, ix = blockIdx.y * 4 + threadIdx.y, iy = blockIdx.z;
    const Grid3D &g = t.g;
    if (iz < 4 || iz >= g.nnz - 4 || ix < 4 || ix >= g.nnx - 4 || iy < 4 || iy >= g.nny - 4) return;
    const long sx = g.ldz, sy = g.sxy;
    const long id = iz + sx * ix + sy * iy;
    const float *P = t.P0, *Q = t.Q0;
    float Px = 0.0f, Py = 0.0f, Pz = 0.0f, Qx = 0.0f, Qy = 0.0f, Qz = 0.0f;
#pragma unroll
    for (int im = 0; im < 4; im++) {
        const float c = c_tti3d[im];
        Px += c * (__ldg(P + id + (im + 1) * sx) - __ldg(P + id - im * sx));
        Py += c * (__ldg(P + id + (im + 1) * sy) - __ldg(P + id - im * sy));
        Pz += c * (__ldg(P + id + im + 1) - __ldg(P + id - im));
        Qx += c * (__ldg(Q + id + (im + 1) * sx) - __ldg(Q + id - im * sx));
        Qy += c * (__ldg(Q + id + (im + 1) * sy) - __ldg(Q + id - im * sy));
        Qz += c * (__ldg(Q + id + im + 1) - __ldg(Q + id - im));
    }
    const float a = __ldg(t.ct + id), b = __ldg(t.st + id), c = __ldg(t.cp + id), sn = __ldg(t.sp + id);
    const float k2 = g.cx2[ix] * g.cy2[iy] * g.cz2[iz];
    const float k1 = g.cx1[ix] * g.cy1[iy] * g.cz1[iz];
    const float gx = a * c * g.dtx * Px + a * sn * g.dty * Py - b * g.dtz * Pz;
    const float gy = c * g.dty * Py - sn * g.dtx * Px;
    const float gz = b * c * g.dtx * Qx + b * sn * g.dty * Qy + a * g.dtz * Qz;
    t.u1[id] = k2 * t.u0[id] - k1 * gx;
    t.v1[id] = k2 * t.v0[id] - k1 * gy;
    t.w1[id] = k2 * t.w0[id] - k1 * gz;
}

__global__ void __launch_bounds__(128) k_tti3d_stress(const Tti3DStep t, const StepArgs3D st) {
    const int iz = blockIdx.x * 32 + threadIdx.x, ix = blockIdx.y * 4 + threadIdx.y, iy = blockIdx.z;
    const Grid3D &g = t.g;
    if (iz < 4 || iz >= g.nnz - 4 || ix < 4 || ix >= g.nnx - 4 || iy < 4 || iy >= g.nny - 4) return;
    const long sx = g.ldz, sy = g.sxy;
    const long id = iz + sx * ix + sy * iy;
    const float *u = t.u1, *v = t.v1, *w = t.w1;
    float ux = 0.0f, uy = 0.0f, uz = 0.0f, vx = 0.0f, vy = 0.0f, wx = 0.0f, wy = 0.0f, wz = 0.0f;
#pragma unroll
    for (int im = 0; im < 4; im++) {
        const float c = c_tti3d[im];
        ux += c * (__ldg(u + id + im * sx) - __ldg(u + id - (im + 1) * sx));
        uy += c * (__ldg(u + id + im * sy) - __ldg(u + id - (im + 1) * sy));
        uz += c * (__ldg(u + id + im) - __ldg(u + id - im - 1));
        vx += c * (__ldg(v + id + im * sx) - __ldg(v + id - (im + 1) * sx));
        vy += c * (__ldg(v + id + im * sy) - __ldg(v + id - (im + 1) * sy));
        wx += c * (__ldg(w + id + im * sx) - __ldg(w + id - (im + 1) * sx));
        wy += c * (__ldg(w + id + im * sy) - __ldg(w + id - (im + 1) * sy));
        wz += c * (__ldg(w + id + im) - __ldg(w + id - im - 1));
    }
    const float a = __ldg(t.ct + id), b = __ldg(t.st + id), c = __ldg(t.cp + id), sn = __ldg(t.sp + id);
    const float ha = (a * c * g.dtx * ux + a * sn * g.dty * uy - b * g.dtz * uz) + (c * g.dty * vy - sn * g.dtx * vx);
    const float hb = b * c * g.dtx * wx + b * sn * g.dty * wy + a * g.dtz * wz;
    const float k2 = g.ax2[ix] * g.ay2[iy] * g.az2[iz];
    const float k1 = g.ax1[ix] * g.ay1[iy] * g.az1[iz];
    float p0 = t.P0[id], q0 = t.Q0[id];
    if (st.src_on && id == st.src) {
        p0 = t.save[0];
        q0 = t.save[1];
    }
    const float mA = __ldg(g.vp + id), mB = __ldg(g.e2 + id), mC = __ldg(g.d2 + id);
    const float P = k2 * p0 - k1 * (mA * ha + mB * hb);
    const float Q = k2 * q0 - k1 * (mB * ha + mC * hb);
    t.P1[id] = P;
    t.Q1[id] = Q;
    // receivers at depth rec_iz on the (rx0 + k drx, ry0 + j dry) grid
    if (st.rec && iz == st.rec_iz) {
        const int rx = ix - g.npd - st.rx0, ry = iy - g.npd - st.ry0;
        if (rx >= 0 && rx % st.drx == 0 && rx / st.drx < st.nrx && ry >= 0 && ry % st.dry == 0 &&
            ry / st.dry < st.nry)
            st.rec[(long)st.it * st.nrx * st.nry + rx / st.drx + (long)st.nrx * (ry / st.dry)] =
                st.rec_pq ? P + Q : P;
    }
    // RTM imaging on the physical box (cal_illumination / cal_migration)
    if ((st.ill || st.mig) && iz >= g.npd && iz < g.npd + g.nz && ix >= g.npd && ix < g.npd + g.nx &&
        iy >= g.npd && iy < g.npd + g.ny) {
        const long o = (long)(iz - g.npd) + (long)g.nz * ((ix - g.npd) + (long)g.nx * (iy - g.npd));
        if (st.ill) st.ill[o] = st.ill[o] + (P * P + Q * Q);
        if (st.mig) st.mig[o] = st.mig[o] + st.other_P[id] * P;
    }
}

int launch_tti3d(const Tti3DStep &t, const StepArgs3D &args, cudaStream_t s) {
    StepArgs3D st = args;
    const Grid3D &g = t.g;
    st.src = st.izs + (long)g.ldz * (st.ixs + (long)g.nnx * st.iys);
    if (st.src_on) {
        k_tti3d_source<<<1, 1, 0, s>>>(const_cast<float *>(t.P0), const_cast<float *>(t.Q0), st.src, st.amp, t.save);
        GEO_TRY(check_launch("tti3d_source"));
    }
    const dim3 block(32, 4), grid((g.nnz + 31) / 32, (g.nnx + 3) / 4, g.nny);
    k_tti3d_vel<<<grid, block, 0, s>>>(t);
    GEO_TRY(check_launch("tti3d_vel"));
    k_tti3d_stress<<<grid, block, 0, s>>>(t, st);
    return check_launch("tti3d_stress");
}

}  // namespace geo
