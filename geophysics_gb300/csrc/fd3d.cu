// 3D VTI staggered-grid FD: plan, kernels and shot driver.
//
// Semantics follow the GUI GPU program GPU_vti3dfd
// (2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti3dfd_kernels.cu): point source added to
// P,Q before the velocity update (:53-88), velocity (:90-129) and
// split-sponge stress (:131-201) updates on [4, nn-4) in every axis.  Two
// stress formulations:
//   GEO_MODE_EXACT  split fields everywhere -- the reference's arithmetic,
//                   bit-identical to it and to the oracle;
//   GEO_MODE_FAST   inside the physical box (all sponge factors 1) P and Q
//                   are updated unsplit, P -= X; P -= Y; P -= Z; the sponge
//                   keeps the split form.  Saves 12 floats of traffic per
//                   interior point and differs from EXACT only by rounding.
// Layout: id = iz + nnz*(ix + nnx*iy), z fastest, as the reference.
#include "geo_internal.h"
#include "fd3d.cuh"
#include <cmath>
#include <cstring>
#include <vector>

using namespace geo;

namespace geo {

__constant__ float c3_fd[4] = {1.196289f, -0.0797526f, 0.009570313f, -0.0006975447f};

// ---------------------------------------------------------------- kernels
// Velocity update, one thread per point; the point source is applied on the
// fly to the taps that read the source cell (P,Q += amp before the update,
// GPU_vti3dfd_kernels.cu:135).
__global__ void __launch_bounds__(256) k_vel3d(Grid3D g, StepArgs3D st) {
    const int iz = blockIdx.x * 32 + threadIdx.x, ix = blockIdx.y * blockDim.y + threadIdx.y, iy = blockIdx.z;
    if (iz < 4 || iz >= g.nnz - 4 || ix < 4 || ix >= g.nnx - 4 || iy < 4 || iy >= g.nny - 4) return;
    const long sxy = g.sxy, id = iz + (long)g.ldz * ix + sxy * iy;
    const float *P = g.P, *Q = g.Q;
    float xx = 0.0f, yy = 0.0f, zz = 0.0f;
    const bool near = st.src_on && ((iz == st.izs && ix == st.ixs && abs(iy - st.iys) <= 4) ||
                                    (iz == st.izs && iy == st.iys && abs(ix - st.ixs) <= 4) ||
                                    (ix == st.ixs && iy == st.iys && abs(iz - st.izs) <= 4));
    if (!near) {
#pragma unroll
        for (int im = 0; im < 4; im++) {
            yy += c3_fd[im] * (__ldg(P + id + (im + 1) * sxy) - __ldg(P + id - im * sxy));
            xx += c3_fd[im] * (__ldg(P + id + (im + 1) * g.ldz) - __ldg(P + id - im * g.ldz));
            zz += c3_fd[im] * (__ldg(Q + id + im + 1) - __ldg(Q + id - im));
        }
    } else {
        auto ldp = [&](long k) { float v = P[k]; if (k == st.src) v = v + st.amp; return v; };
        auto ldq = [&](long k) { float v = Q[k]; if (k == st.src) v = v + st.amp; return v; };
#pragma unroll
        for (int im = 0; im < 4; im++) {
            yy += c3_fd[im] * (ldp(id + (im + 1) * sxy) - ldp(id - im * sxy));
            xx += c3_fd[im] * (ldp(id + (im + 1) * g.ldz) - ldp(id - im * g.ldz));
            zz += c3_fd[im] * (ldq(id + im + 1) - ldq(id - im));
        }
    }
    g.u[id] = g.cx2[ix] * g.u[id] - g.cx1[ix] * g.dtx * xx;
    g.v[id] = g.cy2[iy] * g.v[id] - g.cy1[iy] * g.dty * yy;
    g.w[id] = g.cz2[iz] * g.w[id] - g.cz1[iz] * g.dtz * zz;
}

template <int MODE>
__global__ void __launch_bounds__(256) k_stress3d(Grid3D g, StepArgs3D st) {
    const int iz = blockIdx.x * 32 + threadIdx.x, ix = blockIdx.y * blockDim.y + threadIdx.y, iy = blockIdx.z;
    if (iz < 4 || iz >= g.nnz - 4 || ix < 4 || ix >= g.nnx - 4 || iy < 4 || iy >= g.nny - 4) return;
    const long sxy = g.sxy, id = iz + (long)g.ldz * ix + sxy * iy;
    float xx = 0.0f, yy = 0.0f, zz = 0.0f;
#pragma unroll
    for (int im = 0; im < 4; im++) {
        yy += c3_fd[im] * (__ldg(g.v + id + im * sxy) - __ldg(g.v + id - (im + 1) * sxy));
        xx += c3_fd[im] * (__ldg(g.u + id + im * g.ldz) - __ldg(g.u + id - (im + 1) * g.ldz));
        zz += c3_fd[im] * (__ldg(g.w + id + im) - __ldg(g.w + id - im - 1));
    }
    const float vp = __ldg(g.vp + id), e2 = __ldg(g.e2 + id), d2 = __ldg(g.d2 + id);
    const bool inside = MODE == GEO_MODE_FAST && ix >= g.npd && ix < g.npd + g.nx && iy >= g.npd &&
                        iy < g.npd + g.ny && iz >= g.npd && iz < g.npd + g.nz;
    float P, Q;
    if (inside) {
        // all sponge factors are 1: acoff*vp == vp exactly, so each term is
        // the reference's product chain; only the split sum is replaced
        P = g.P[id] - vp * vp * e2 * g.dtx * xx - vp * vp * e2 * g.dty * yy - vp * vp * d2 * g.dtz * zz;
        Q = g.Q[id] - vp * vp * d2 * g.dtx * xx - vp * vp * d2 * g.dty * yy - vp * vp * g.dtz * zz;
    } else {
        const float ax1 = g.ax1[ix], ax2 = g.ax2[ix], ay1 = g.ay1[iy], ay2 = g.ay2[iy], az1 = g.az1[iz], az2 = g.az2[iz];
        const float px = ax2 * g.px[id] - ax1 * vp * vp * e2 * g.dtx * xx;
        const float py = ay2 * g.py[id] - ay1 * vp * vp * e2 * g.dty * yy;
        const float pz = az2 * g.pz[id] - az1 * vp * vp * d2 * g.dtz * zz;
        const float qx = ax2 * g.qx[id] - ax1 * vp * vp * d2 * g.dtx * xx;
        const float qy = ay2 * g.qy[id] - ay1 * vp * vp * d2 * g.dty * yy;
        const float qz = az2 * g.qz[id] - az1 * vp * vp * g.dtz * zz;
        g.px[id] = px; g.py[id] = py; g.pz[id] = pz;
        g.qx[id] = qx; g.qy[id] = qy; g.qz[id] = qz;
        P = px + py + pz;
        Q = qx + qy + qz;
    }
    g.P[id] = P;
    g.Q[id] = Q;
    // receiver gather, time-major (shot_record3d, GPU_vti3dfd_kernels.cu:316-327)
    if (st.rec && iz == st.rec_iz) {
        const int rx = ix - g.npd - st.rx0, ry = iy - g.npd - st.ry0;
        if (rx >= 0 && ry >= 0 && rx % st.drx == 0 && ry % st.dry == 0) {
            const int irx = rx / st.drx, iry = ry / st.dry;
            if (irx < st.nrx && iry < st.nry) st.rec[(long)st.it * st.nrx * st.nry + irx + (long)st.nrx * iry] = P;
        }
    }
}

// Write a B^3 box of (1+2eps, sqrtf(1+2del)) into the model, clipped.
__global__ void k_box3d(Grid3D g, float *e2, float *d2, long x0, long y0, long z0, int B, const float *src) {
    const long n = (long)B * B * B;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const long bz = k % B, bx = (k / B) % B, by = k / ((long)B * B);
        const long iz = z0 + bz, ix = x0 + bx, iy = y0 + by;
        if (iz < 0 || iz >= g.nnz || ix < 0 || ix >= g.nnx || iy < 0 || iy >= g.nny) continue;
        const long id = iz + (long)g.ldz * ix + g.sxy * iy;
        e2[id] = src[k];
        d2[id] = src[n + k];
    }
}

}  // namespace geo

struct geo_fd3d_plan {
    geo_fd3d_desc d;
    int nnx, nny, nnz;
    size_t n;
    DevBuf vp, e2, d2, prof;
    DevBuf u, v, w, P, Q, px, py, pz, qx, qy, qz;
    DevBuf rec_tm, rec_tr, mute_hi, box;
    std::vector<float> amp;
    std::vector<uint8_t> on;
    std::vector<float> h_eps, h_del;   // padded raw eps/del, kept for the SV taper
    float vp1 = 0, eps1 = 0;           // padded model at linear index 1 (mute)
    bool model_set = false;
};

namespace geo {

Grid3D make_grid(const geo_fd3d_plan *p) {
    Grid3D g;
    g.nnx = p->nnx; g.nny = p->nny; g.nnz = p->nnz;
    g.ldz = p->nnz;
    g.sxy = (long)p->nnz * p->nnx;
    g.npd = p->d.npd;
    g.nx = p->d.nx; g.ny = p->d.ny; g.nz = p->d.nz;
    g.dtx = p->d.dt / p->d.dx;
    g.dty = p->d.dt / p->d.dy;
    g.dtz = p->d.dt / p->d.dz;
    const float *pr = p->prof.as<float>();
    size_t o = 0;
    g.cx1 = pr + o; o += p->nnx; g.cx2 = pr + o; o += p->nnx; g.ax1 = pr + o; o += p->nnx; g.ax2 = pr + o; o += p->nnx;
    g.cy1 = pr + o; o += p->nny; g.cy2 = pr + o; o += p->nny; g.ay1 = pr + o; o += p->nny; g.ay2 = pr + o; o += p->nny;
    g.cz1 = pr + o; o += p->nnz; g.cz2 = pr + o; o += p->nnz; g.az1 = pr + o; o += p->nnz; g.az2 = pr + o;
    g.vp = p->vp.as<float>(); g.e2 = p->e2.as<float>(); g.d2 = p->d2.as<float>();
    g.u = p->u.as<float>(); g.v = p->v.as<float>(); g.w = p->w.as<float>();
    g.P = p->P.as<float>(); g.Q = p->Q.as<float>();
    g.px = p->px.as<float>(); g.py = p->py.as<float>(); g.pz = p->pz.as<float>();
    g.qx = p->qx.as<float>(); g.qy = p->qy.as<float>(); g.qz = p->qz.as<float>();
    return g;
}

static int step3d(const geo_fd3d_plan *p, const Grid3D &g, const StepArgs3D &st, cudaStream_t s) {
    dim3 block(32, 8), grid((p->nnz + 31) / 32, (p->nnx + 7) / 8, p->nny);
    k_vel3d<<<grid, block, 0, s>>>(g, st);
    GEO_TRY(check_launch("vel3d"));
    if (p->d.mode == GEO_MODE_FAST) k_stress3d<GEO_MODE_FAST><<<grid, block, 0, s>>>(g, st);
    else k_stress3d<GEO_MODE_EXACT><<<grid, block, 0, s>>>(g, st);
    return check_launch("stress3d");
}

static int zero_state(geo_fd3d_plan *p, cudaStream_t s) {
    DevBuf *f[] = {&p->u, &p->v, &p->w, &p->P, &p->Q, &p->px, &p->py, &p->pz, &p->qx, &p->qy, &p->qz};
    for (DevBuf *b : f) GEO_TRY(b->zero(s));
    return GEO_OK;
}

// SV taper box for shot `is` (GPU_vti3dfd_kernels.cu:155-174: R=15, r=4,
// centre fs+is*ds+npml-1): tapered=true writes the tapered coefficients,
// false restores the untapered ones.
static int taper_box_3d(geo_fd3d_plan *p, int is, bool tapered, cudaStream_t s) {
    const geo_fd3d_desc &D = p->d;
    const long cx = D.fsx + (long)is * D.dsx + D.npd - 1, cy = D.fsy + (long)is * D.dsy + D.npd - 1,
               cz = D.fsz + (long)is * D.dsz + D.npd - 1;
    const int B = 31, R = 15, r = 4;
    const long n = (long)B * B * B;
    std::vector<float> h(2 * n, 1.0f);
    for (int by = 0; by < B; by++)
        for (int bx = 0; bx < B; bx++)
            for (int bz = 0; bz < B; bz++) {
                const long iz = cz - 15 + bz, ix = cx - 15 + bx, iy = cy - 15 + by;
                if (iz < 0 || iz >= p->nnz || ix < 0 || ix >= p->nnx || iy < 0 || iy >= p->nny) continue;
                const size_t id = iz + (size_t)p->nnz * (ix + (size_t)p->nnx * iy);
                float ee = p->h_eps[id], dd = p->h_del[id];
                if (tapered) {
                    const int rx = (int)(ix - cx), ry = (int)(iy - cy), rz = (int)(iz - cz);
                    const int r2 = rx * rx + ry * ry + rz * rz;
                    if (r2 <= R * R) {
                        if (r2 <= r * r) {
                            ee = 0.0f; dd = 0.0f;
                        } else {
                            const double gq = 0.5 * (1 - std::cos(kPiGui * ((sqrtf((float)r2) - r) * 4.0 / (R * 3.0 - 1))));
                            ee = (float)(gq * ee); dd = (float)(gq * dd);
                        }
                    }
                }
                const long k = bz + (long)B * (bx + (long)B * by);
                h[k] = 1 + 2 * ee;
                h[n + k] = sqrtf(1 + 2 * dd);
            }
    GEO_CUDA(cudaMemcpyAsync(p->box.p, h.data(), h.size() * 4, cudaMemcpyHostToDevice, s));
    Grid3D g = make_grid(p);
    k_box3d<<<(int)((n + 255) / 256), 256, 0, s>>>(g, p->e2.as<float>(), p->d2.as<float>(), cx - 15, cy - 15, cz - 15, B,
                                                 p->box.as<float>());
    GEO_TRY(check_launch("box3d"));
    return GEO_OK;
}

// Forward run of shot `is` into the plan's time-major record buffer;
// `on_step(it)` (optional) runs after each step (snapshots).
int run_shot_3d(geo_fd3d_plan *p, int is, cudaStream_t s, int (*on_step)(void *, int), void *ctx) {
    if (!p->model_set) return fail(GEO_ERR_ARG, "model not set");
    const geo_fd3d_desc &D = p->d;
    const long ixs = D.fsx + (long)is * D.dsx + D.npd - 1, iys = D.fsy + (long)is * D.dsy + D.npd - 1,
               izs = D.fsz + (long)is * D.dsz + D.npd - 1;
    if (ixs < 4 || ixs >= p->nnx - 4 || iys < 4 || iys >= p->nny - 4 || izs < 4 || izs >= p->nnz - 4)
        return fail(GEO_ERR_ARG, "source outside the updated grid");
    GEO_TRY(zero_state(p, s));
    if (D.sv) GEO_TRY(taper_box_3d(p, is, true, s));
    Grid3D g = make_grid(p);
    StepArgs3D st{};
    st.ixs = (int)ixs; st.iys = (int)iys; st.izs = (int)izs;
    st.src = izs + (long)p->nnz * (ixs + (long)p->nnx * iys);
    st.rec = p->rec_tm.as<float>();
    st.rec_iz = D.rec_iz; st.rx0 = D.rx0; st.drx = D.drx; st.nrx = D.nrx; st.ry0 = D.ry0; st.dry = D.dry; st.nry = D.nry;
    for (int it = 0; it < D.nt; it++) {
        st.it = it;
        st.src_on = p->on[it];
        st.amp = p->amp[it];
        GEO_TRY(step3d(p, g, st, s));
        if (on_step) GEO_TRY(on_step(ctx, it));
    }
    if (D.sv) GEO_TRY(taper_box_3d(p, is, false, s));
    const int ntr = D.nrx * D.nry;
    if (D.mute_tt > 0) {
        std::vector<int> hi;
        // the mute formula indexes receivers as model cells (every node)
        mute_window_3d(D.nrx, D.nry, D.nt, D.dt, D.favg, D.dx, D.dy, D.dz, D.fsx, D.fsy, D.dsx, D.dsy, D.fsz, is,
                       p->vp1, p->eps1, D.mute_tt, hi);
        GEO_CUDA(cudaMemcpyAsync(p->mute_hi.p, hi.data(), hi.size() * 4, cudaMemcpyHostToDevice, s));
        GEO_TRY(launch_mute_records(p->rec_tm.as<float>(), ntr, D.nt, nullptr, p->mute_hi.as<int>(), s));
    }
    return GEO_OK;
}

const float *plan3d_P(const geo_fd3d_plan *p) { return p->P.as<float>(); }
int plan3d_dims(const geo_fd3d_plan *p, int *nnx, int *nny, int *nnz) {
    *nnx = p->nnx; *nny = p->nny; *nnz = p->nnz;
    return GEO_OK;
}

}  // namespace geo

extern "C" int geo_fd3d_plan_create(geo_fd3d_plan **out, const geo_fd3d_desc *desc) {
    if (!out || !desc) return fail(GEO_ERR_ARG, "null argument");
    const geo_fd3d_desc &d = *desc;
    if (d.nx < 2 || d.ny < 2 || d.nz < 2 || d.npd < 5 || d.nt < 1)
        return fail(GEO_ERR_ARG, "grid too small (npd must be >= 5)");
    if (!(d.dt > 0) || !(d.dx > 0) || !(d.dy > 0) || !(d.dz > 0)) return fail(GEO_ERR_ARG, "bad spacing");
    if (d.nrx < 1 || d.nry < 1 || d.drx < 1 || d.dry < 1) return fail(GEO_ERR_ARG, "bad receiver grid");
    if (d.rx0 < 0 || d.rx0 + (d.nrx - 1) * d.drx >= d.nx) return fail(GEO_ERR_ARG, "receivers outside x");
    if (d.ry0 < 0 || d.ry0 + (d.nry - 1) * d.dry >= d.ny) return fail(GEO_ERR_ARG, "receivers outside y");
    if (d.rec_iz < 4 || d.rec_iz >= d.nz + 2 * d.npd - 4) return fail(GEO_ERR_ARG, "receiver depth outside grid");
    if (d.mode != GEO_MODE_EXACT && d.mode != GEO_MODE_FAST) return fail(GEO_ERR_ARG, "bad mode");
    if (!(d.favg > 0)) return fail(GEO_ERR_ARG, "favg must be > 0");
    geo_fd3d_plan *p = new geo_fd3d_plan();
    p->d = d;
    p->nnx = d.nx + 2 * d.npd;
    p->nny = d.ny + 2 * d.npd;
    p->nnz = d.nz + 2 * d.npd;
    p->n = (size_t)p->nnx * p->nny * p->nnz;
    const size_t n = p->n, ntr = (size_t)d.nrx * d.nry;
    int st = GEO_OK;
    DevBuf *fields[] = {&p->vp, &p->e2, &p->d2, &p->u, &p->v, &p->w, &p->P, &p->Q,
                        &p->px, &p->py, &p->pz, &p->qx, &p->qy, &p->qz};
    for (DevBuf *b : fields)
        if (st == GEO_OK) st = b->alloc(n * 4);
    if (st == GEO_OK) st = p->prof.alloc((size_t)4 * (p->nnx + p->nny + p->nnz) * 4);
    if (st == GEO_OK) st = p->rec_tm.alloc(ntr * d.nt * 4);
    if (st == GEO_OK) st = p->rec_tr.alloc(ntr * d.nt * 4);
    if (st == GEO_OK) st = p->mute_hi.alloc(ntr * 4);
    if (st == GEO_OK) st = p->box.alloc((size_t)2 * 31 * 31 * 31 * 4);
    if (st != GEO_OK) {
        delete p;
        return st;
    }
    source_amplitudes(V_GPU, d.nt, d.dt, d.favg, d.pfac, d.wtype, p->amp, p->on);
    *out = p;
    return GEO_OK;
}

extern "C" int geo_fd3d_plan_destroy(geo_fd3d_plan *p) {
    delete p;
    return GEO_OK;
}

// Model upload: pad on the host, build vp, 1+2eps, sqrtf(1+2del) and the
// sponge profiles (d0 from the padded centre velocity, GPU_vti3dfd_kernels.cu:203-206).
extern "C" int geo_fd3d_set_model(geo_fd3d_plan *p, const float *v, const float *e, const float *d, int mem,
                                  void *stream) {
    if (!p || !v || !e || !d) return fail(GEO_ERR_ARG, "null argument");
    cudaStream_t s = (cudaStream_t)stream;
    const geo_fd3d_desc &D = p->d;
    const size_t n0 = (size_t)D.nx * D.ny * D.nz;
    std::vector<float> hv, he, hd;
    const float *sv = v, *se = e, *sd = d;
    if (mem == GEO_MEM_DEVICE) {
        hv.resize(n0); he.resize(n0); hd.resize(n0);
        GEO_CUDA(cudaMemcpyAsync(hv.data(), v, n0 * 4, cudaMemcpyDeviceToHost, s));
        GEO_CUDA(cudaMemcpyAsync(he.data(), e, n0 * 4, cudaMemcpyDeviceToHost, s));
        GEO_CUDA(cudaMemcpyAsync(hd.data(), d, n0 * 4, cudaMemcpyDeviceToHost, s));
        GEO_CUDA(cudaStreamSynchronize(s));
        sv = hv.data(); se = he.data(); sd = hd.data();
    } else if (mem != GEO_MEM_HOST) {
        return fail(GEO_ERR_ARG, "bad mem kind");
    }
    GEO_TRY(check_model(sv, se, sd, n0));
    std::vector<float> pv(p->n), pe(p->n), pd(p->n);
    pad_model_3d(D.nx, D.ny, D.nz, D.npd, sv, pv.data());
    pad_model_3d(D.nx, D.ny, D.nz, D.npd, se, pe.data());
    pad_model_3d(D.nx, D.ny, D.nz, D.npd, sd, pd.data());
    p->vp1 = pv[1];
    p->eps1 = pe[1];
    const float d0 = sponge_d0(V_GPU, 3, 0.0f, pv[(size_t)p->nny * p->nnx * p->nnz / 2], D.npd, D.dx, D.dy, D.dz);
    std::vector<float> prof((size_t)4 * (p->nnx + p->nny + p->nnz));
    float *q = prof.data();
    sponge_profiles(V_GPU, D.nx, D.npd, D.dt, d0, q, q + p->nnx, q + 2 * p->nnx, q + 3 * p->nnx);
    q += 4 * p->nnx;
    sponge_profiles(V_GPU, D.ny, D.npd, D.dt, d0, q, q + p->nny, q + 2 * p->nny, q + 3 * p->nny);
    q += 4 * p->nny;
    sponge_profiles(V_GPU, D.nz, D.npd, D.dt, d0, q, q + p->nnz, q + 2 * p->nnz, q + 3 * p->nnz);
    if (D.sv) {
        p->h_eps = pe;
        p->h_del = pd;
    }
    // 1+2*eps and sqrtf(1+2*del) in float, as the stress kernel forms them
    for (size_t k = 0; k < p->n; k++) {
        pe[k] = 1 + 2 * pe[k];
        pd[k] = sqrtf(1 + 2 * pd[k]);
    }
    GEO_CUDA(cudaMemcpyAsync(p->vp.p, pv.data(), p->n * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemcpyAsync(p->e2.p, pe.data(), p->n * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemcpyAsync(p->d2.p, pd.data(), p->n * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemcpyAsync(p->prof.p, prof.data(), prof.size() * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    p->model_set = true;
    return GEO_OK;
}

namespace geo {
// Transpose the time-major record into the caller's trace-major buffer.
int fetch_shot_3d(geo_fd3d_plan *p, float *shot, int mem, cudaStream_t s) {
    const int ntr = p->d.nrx * p->d.nry;
    const size_t bytes = (size_t)ntr * p->d.nt * 4;
    if (mem == GEO_MEM_DEVICE) {
        GEO_TRY(launch_transpose_records(p->rec_tm.as<float>(), shot, ntr, p->d.nt, s));
    } else {
        GEO_TRY(launch_transpose_records(p->rec_tm.as<float>(), p->rec_tr.as<float>(), ntr, p->d.nt, s));
        GEO_CUDA(cudaMemcpyAsync(shot, p->rec_tr.p, bytes, cudaMemcpyDeviceToHost, s));
    }
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}
}  // namespace geo

extern "C" int geo_fd3d_run_shot(geo_fd3d_plan *p, int is, float *shot, int mem, void *stream) {
    if (!p || !shot) return fail(GEO_ERR_ARG, "null argument");
    if (mem != GEO_MEM_HOST && mem != GEO_MEM_DEVICE) return fail(GEO_ERR_ARG, "bad mem kind");
    cudaStream_t s = (cudaStream_t)stream;
    GEO_TRY(run_shot_3d(p, is, s, nullptr, nullptr));
    return fetch_shot_3d(p, shot, mem, s);
}

extern "C" int geo_fd3d_time_steps(geo_fd3d_plan *p, int nsteps, float *ms, void *stream) {
    if (!p || nsteps < 1) return fail(GEO_ERR_ARG, "bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    Grid3D g = make_grid(p);
    StepArgs3D st{};
    st.src = -1;
    cudaEvent_t a, b;
    GEO_CUDA(cudaEventCreate(&a));
    GEO_CUDA(cudaEventCreate(&b));
    GEO_CUDA(cudaEventRecord(a, s));
    for (int k = 0; k < nsteps; k++) GEO_TRY(step3d(p, g, st, s));
    GEO_CUDA(cudaEventRecord(b, s));
    GEO_CUDA(cudaEventSynchronize(b));
    float t = 0;
    GEO_CUDA(cudaEventElapsedTime(&t, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (ms) *ms = t;
    return GEO_OK;
}

extern "C" int geo_fd3d_get_fields(geo_fd3d_plan *p, float *P, float *Q, int mem, void *stream) {
    if (!p) return fail(GEO_ERR_ARG, "null plan");
    cudaStream_t s = (cudaStream_t)stream;
    const cudaMemcpyKind k = mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (P) GEO_CUDA(cudaMemcpyAsync(P, p->P.p, p->n * 4, k, s));
    if (Q) GEO_CUDA(cudaMemcpyAsync(Q, p->Q.p, p->n * 4, k, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}

extern "C" int geo_fd3d_shot(const geo_fd3d_desc *desc, int is, const float *v, const float *e, const float *d,
                             float *shot, int mem, void *stream) {
    geo_fd3d_plan *p = nullptr;
    GEO_TRY(geo_fd3d_plan_create(&p, desc));
    int st = geo_fd3d_set_model(p, v, e, d, mem, stream);
    if (st == GEO_OK) st = geo_fd3d_run_shot(p, is, shot, mem, stream);
    geo_fd3d_plan_destroy(p);
    return st;
}
