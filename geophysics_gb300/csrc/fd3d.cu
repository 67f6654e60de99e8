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
#include "fd3d_fused.cuh"
#include "ae.cuh"
#include "adcig.cuh"
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <vector>
#include <memory>
#include <thread>

using namespace geo;

namespace geo {

// ---------------------------------------------------------------- kernels
// Write a B^3 box of two model arrays (the SV taper), clipped to the grid.
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

// One ring of P,Q just outside the physical box (faces z=npml-1, z=npml+nz,
// x=npml-1, x=npml+nx, y=npml-1, y=npml+ny in the 3D RTM program's order,
// wavefield_bndr :405-506): save after a forward step or restore before a
// backward step.  Faces do not overlap.
__global__ void k_ring3d(Grid3D g, float *P, float *Q, float *bp, float *bq, long L, int it, int save) {
    const int nx = g.nx, ny = g.ny, nz = g.nz, npd = g.npd;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < L; k += (long)gridDim.x * blockDim.x) {
        long r = k;
        int iz, ix, iy;
        const long fxy = (long)nx * ny, fzy = (long)nz * ny, fxz = (long)nx * nz;
        if (r < fxy) { iz = npd - 1; ix = npd + (int)(r % nx); iy = npd + (int)(r / nx); }
        else if ((r -= fxy) < fxy) { iz = npd + nz; ix = npd + (int)(r % nx); iy = npd + (int)(r / nx); }
        else if ((r -= fxy) < fzy) { iz = npd + (int)(r % nz); ix = npd - 1; iy = npd + (int)(r / nz); }
        else if ((r -= fzy) < fzy) { iz = npd + (int)(r % nz); ix = npd + nx; iy = npd + (int)(r / nz); }
        else if ((r -= fzy) < fxz) { iz = npd + (int)(r % nz); ix = npd + (int)(r / nz); iy = npd - 1; }
        else { r -= fxz; iz = npd + (int)(r % nz); ix = npd + (int)(r / nz); iy = npd + ny; }
        const long id = iz + (long)g.ldz * ix + g.sxy * iy, b = (long)it * L + k;
        if (save) { bp[b] = P[id]; bq[b] = Q[id]; }
        else { P[id] = bp[b]; Q[id] = bq[b]; }
    }
}

// Receiver injection before a backward step: the muted record into P and Q
// of the receiver field at z = npml-1 (shot_record, flag false, :319-334).
// Receivers (rx0 + jx*drx, ry0 + jy*dry), jx < nrx, jy < nry, take the
// time-major record back at depth npml-1.
__global__ void k_inject3d(Grid3D g, float *P, float *Q, const float *rec_tm, int it, int rx0, int drx, int nrx,
                           int ry0, int dry, int nry) {
    const int npd = g.npd;
    const long n = (long)nrx * nry;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int ix = rx0 + (int)(k % nrx) * drx, iy = ry0 + (int)(k / nrx) * dry;
        const long id = (npd - 1) + (long)g.ldz * (npd + ix) + g.sxy * (npd + iy);
        const float r = rec_tm[(long)it * n + k];
        P[id] = r;
        Q[id] = r;
    }
}

// migration_illum (:539-553): mig /= illum where illum != 0.
__global__ void k_image_illum(float *mig, const float *ill, long n) {
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
        if (ill[k] != 0.0f) mig[k] = mig[k] / ill[k];
}

static int grid_blocks(long n) { return (int)std::min<long>((n + 255) / 256, 152L * 16); }

// Model set-up on the device.  First failing point of the host check
// check_model (velocity, then eps/del finiteness, then 1+2 del >= 0), as
// key = index*4 + kind; the smallest key is the host loop's first report.
__global__ void k_check_model3d(const float *v, const float *e, const float *d, long n,
                                unsigned long long *first) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        int kind = 0;
        if (!isfinite(v[i]) || !(v[i] > 0.0f)) kind = 1;
        else if (!isfinite(e[i]) || !isfinite(d[i])) kind = 2;
        else if (1 + 2 * d[i] < 0) kind = 3;
        if (kind) atomicMin(first, (unsigned long long)i * 4 + (kind - 1));
    }
}

// Edge-replicated padding (pad_vv3d, GPU_vti3dfd_kernels.cu:208-255: each
// axis clamped to the interior) and the stencil's model arrays in
// one pass, into the pitched layout: exact vp, 1+2eps, sqrtf(1+2del); fast
// A = vp^2(1+2eps), B = vp^2 sqrtf(1+2del), C = vp^2 -- the host formulas,
// float for float.
__global__ void k_model3d(const float *v, const float *e, const float *d, int nx, int ny, int nz, int npd,
                          int nnx, int nny, int nnz, int ldz, int fast, float *o0, float *o1, float *o2) {
    const long n = (long)nnx * nny * nnz;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(k % nnz), ix = (int)((k / nnz) % nnx), iy = (int)(k / ((long)nnz * nnx));
        const int sz = min(max(iz - npd, 0), nz - 1), sx = min(max(ix - npd, 0), nx - 1),
                  sy = min(max(iy - npd, 0), ny - 1);
        const long r = sz + (long)nz * (sx + (long)nx * sy);
        const float pv = v[r], e2 = 1 + 2 * e[r], d2 = sqrtf(1 + 2 * d[r]);
        const long o = iz + (long)ldz * (ix + (long)nnx * iy);
        if (fast) {
            const float c2 = pv * pv;
            o0[o] = c2 * e2;
            o1[o] = c2 * d2;
            o2[o] = c2;
        } else {
            o0[o] = pv;
            o1[o] = e2;
            o2[o] = d2;
        }
    }
}

// Edge-replicated padding of one unpadded array into the pitched layout
// (the same clamping as k_model3d).
__global__ void k_pad3d(const float *src, int nx, int ny, int nz, int npd, int nnx, int nny, int nnz, int ldz,
                        float *dst) {
    const long n = (long)nnx * nny * nnz;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(k % nnz), ix = (int)((k / nnz) % nnx), iy = (int)(k / ((long)nnz * nnx));
        const int sz = min(max(iz - npd, 0), nz - 1), sx = min(max(ix - npd, 0), nx - 1),
                  sy = min(max(iy - npd, 0), ny - 1);
        dst[iz + (long)ldz * (ix + (long)nnx * iy)] = src[sz + (long)nz * (sx + (long)nx * sy)];
    }
}

// The padded raw model on a B^3 box at (x0, y0, z0) (padded coordinates),
// gathered from the unpadded arrays with the same edge replication; box
// points outside the padded grid are left alone.
__global__ void k_gather_box3d(const float *raw, int nx, int ny, int nz, int npd, int nnx, int nny, int nnz, long x0,
                               long y0, long z0, int B, float *out) {
    const long nb = (long)B * B * B, n0 = (long)nx * ny * nz;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < nb; k += (long)gridDim.x * blockDim.x) {
        const long iz = z0 + k % B, ix = x0 + (k / B) % B, iy = y0 + k / ((long)B * B);
        if (iz < 0 || iz >= nnz || ix < 0 || ix >= nnx || iy < 0 || iy >= nny) continue;
        const long sz = min(max(iz - npd, 0L), (long)nz - 1), sx = min(max(ix - npd, 0L), (long)nx - 1),
                   sy = min(max(iy - npd, 0L), (long)ny - 1);
        const long r = sz + (long)nz * (sx + (long)nx * sy);
        for (int a = 0; a < 3; a++) out[a * nb + k] = raw[a * n0 + r];
    }
}

}  // namespace geo

// One wavefield set: u,v,w,P,Q at two time levels (ping-pong), split stresses
// in place, and the tensor maps of both levels.
struct FieldSet3D {
    DevBuf lev[2][5];
    DevBuf px, py, pz, qx, qy, qz;
    StepMaps maps[2];
    int cur = 0;
};

// Device state of one 3D grid.  Fields use the reference layout with the z
// stride ldz rounded up to 4 floats (16 bytes, the TMA stride rule); points
// iz >= nnz of a column are padding and never read or written.
struct geo_fd3d_plan {
    geo_fd3d_desc d;
    int nnx, nny, nnz, ldz;
    size_t n, nalloc;                  // padded points, allocated floats per field
    DevBuf vp, e2, d2, prof;           // model (exact: vp,1+2eps,sqrtf(1+2del); fast: A,B,C)
    FieldSet3D fs[2];                  // [0] forward / source side, [1] receiver side (RTM)
    int nfs = 1;
    DevBuf rec_tm, rec_tr, mute_lo, mute_hi, box, err;
    int chunk = 0, nitems = 0, ntz = 0, ntx = 0;
    std::vector<float> amp;
    std::vector<uint8_t> on;
    DevBuf raw;                        // unpadded vp, eps, del (3 x nx*ny*nz), kept for the SV taper
    float vp1 = 0, eps1 = 0;           // padded model at linear index 1 (mute)
    bool model_set = false;
    bool tuned = false;
    // 3D TTI medium (geo_fd3d_set_tilt): cos/sin of tilt and azimuth, 4 x nalloc
    DevBuf tilt, save;
    bool tti = false;
    geo::Watchdog wd;                  // non-finite wavefield detector
};

namespace geo {

// Extents, profiles and the current level of field set f.
static Grid3D grid_of(const geo_fd3d_plan *p, int f) {
    Grid3D g;
    g.nnx = p->nnx; g.nny = p->nny; g.nnz = p->nnz;
    g.ldz = p->ldz;
    g.sxy = (long)p->ldz * p->nnx;
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
    const FieldSet3D &F = p->fs[f];
    const int c = F.cur;
    g.u = F.lev[c][0].as<float>(); g.v = F.lev[c][1].as<float>(); g.w = F.lev[c][2].as<float>();
    g.P = F.lev[c][3].as<float>(); g.Q = F.lev[c][4].as<float>();
    g.px = F.px.as<float>(); g.py = F.py.as<float>(); g.pz = F.pz.as<float>();
    g.qx = F.qx.as<float>(); g.qy = F.qy.as<float>(); g.qz = F.qz.as<float>();
    return g;
}

Grid3D make_grid(const geo_fd3d_plan *p) { return grid_of(p, 0); }

// Fused-kernel view of field set f: reads level cur (through the maps),
// writes level 1-cur.
static Fused3D make_fused(const geo_fd3d_plan *p, int f) {
    const Grid3D g = grid_of(p, f);
    const FieldSet3D &F = p->fs[f];
    Fused3D r;
    r.nnx = g.nnx; r.nny = g.nny; r.nnz = g.nnz; r.ldz = g.ldz; r.sxy = g.sxy;
    r.npd = g.npd; r.nx = g.nx; r.ny = g.ny; r.nz = g.nz;
    r.dtx = g.dtx; r.dty = g.dty; r.dtz = g.dtz;
    r.cx1 = g.cx1; r.cx2 = g.cx2; r.ax1 = g.ax1; r.ax2 = g.ax2;
    r.cy1 = g.cy1; r.cy2 = g.cy2; r.ay1 = g.ay1; r.ay2 = g.ay2;
    r.cz1 = g.cz1; r.cz2 = g.cz2; r.az1 = g.az1; r.az2 = g.az2;
    r.m0 = g.vp; r.m1 = g.e2; r.m2 = g.d2;
    r.P0 = g.P; r.Q0 = g.Q;
    const int n = 1 - F.cur;
    r.u1 = F.lev[n][0].as<float>(); r.v1 = F.lev[n][1].as<float>(); r.w1 = F.lev[n][2].as<float>();
    r.P1 = F.lev[n][3].as<float>(); r.Q1 = F.lev[n][4].as<float>();
    r.px = g.px; r.py = g.py; r.pz = g.pz; r.qx = g.qx; r.qy = g.qy; r.qz = g.qz;
    r.ntz = p->ntz; r.ntx = p->ntx; r.ntiles = p->ntz * p->ntx; r.chunk = p->chunk; r.nitems = p->nitems;
    r.err = p->err.as<int>();
    return r;
}

static int alloc_fields(geo_fd3d_plan *p, int f) {
    FieldSet3D &F = p->fs[f];
    const size_t n = p->nalloc;
    for (int c = 0; c < 2; c++)
        for (int k = 0; k < 5; k++) GEO_TRY(F.lev[c][k].alloc(n * 4));
    DevBuf *sp[6] = {&F.px, &F.py, &F.pz, &F.qx, &F.qy, &F.qz};
    for (DevBuf *b : sp) GEO_TRY(b->alloc(n * 4));
    for (int c = 0; c < 2; c++) {
        StepMaps &M = F.maps[c];
        const int nz = p->nnz, ld = p->ldz, nx = p->nnx, ny = p->nny;
        GEO_TRY(encode_map(&M.m[0], F.lev[c][3].as<float>(), nz, ld, nx, ny, kTZ, kTXF + 14));  // P halo
        GEO_TRY(encode_map(&M.m[1], F.lev[c][3].as<float>(), nz, ld, nx, ny, kTZ, kTXF));       // P own
        GEO_TRY(encode_map(&M.m[2], F.lev[c][4].as<float>(), nz, ld, nx, ny, 48, kTXF));        // Q
        GEO_TRY(encode_map(&M.m[3], F.lev[c][0].as<float>(), nz, ld, nx, ny, kTZ, kTXF + 8));   // u
        GEO_TRY(encode_map(&M.m[4], F.lev[c][2].as<float>(), nz, ld, nx, ny, 48, kTXF));        // w
        GEO_TRY(encode_map(&M.m[5], F.lev[c][1].as<float>(), nz, ld, nx, ny, kTZ, kTXF));       // v
        const DevBuf *own[9] = {&p->vp, &p->e2, &p->d2, &F.px, &F.py, &F.pz, &F.qx, &F.qy, &F.qz};
        for (int r = 0; r < 9; r++) GEO_TRY(encode_map(&M.m[6 + r], own[r]->as<float>(), nz, ld, nx, ny, kTZ, kTXF));
    }
    return GEO_OK;
}

// y chunking: a block marches over one chunk of y planes and recomputes 14
// warm-up planes of its queues, so more chunks mean more blocks in flight at
// different depths (better DRAM and L2 spread, shorter tails) at the price of
// the warm-up.  The best count varies with the grid (measured on GB300: 4
// for 480^3, 6 for 592x592x464, 8 for 272^3), so set_model times the
// candidates (autotune_chunks); this is the starting guess.
static void set_chunks(geo_fd3d_plan *p, int c) {
    const int planes = p->nny - 8, ntiles = p->ntz * p->ntx;
    c = std::max(1, std::min(c, planes / 8));
    p->chunk = (planes + c - 1) / c;
    p->nitems = ntiles * ((planes + p->chunk - 1) / p->chunk);
}

static bool g_chunks_fixed() { return getenv("GEO_FD3D_CHUNKS") != nullptr; }

static void choose_chunks(geo_fd3d_plan *p) {
    int c = 4;
    if (const char *e = getenv("GEO_FD3D_CHUNKS")) c = std::max(1, atoi(e));
    set_chunks(p, c);
}

// One time step of field set f: the fused kernel reads level cur and writes
// level 1-cur.
static int step3d(geo_fd3d_plan *p, int f, const StepArgs3D &st, cudaStream_t s) {
    if (p->tti) {
        const FieldSet3D &F = p->fs[f];
        const int c = F.cur, n = 1 - c;
        Tti3DStep t;
        t.g = grid_of(p, f);
        t.u0 = F.lev[c][0].as<float>(); t.v0 = F.lev[c][1].as<float>(); t.w0 = F.lev[c][2].as<float>();
        t.P0 = F.lev[c][3].as<float>(); t.Q0 = F.lev[c][4].as<float>();
        t.u1 = F.lev[n][0].as<float>(); t.v1 = F.lev[n][1].as<float>(); t.w1 = F.lev[n][2].as<float>();
        t.P1 = F.lev[n][3].as<float>(); t.Q1 = F.lev[n][4].as<float>();
        const float *tl = p->tilt.as<float>();
        t.ct = tl; t.st = tl + p->nalloc; t.cp = tl + 2 * p->nalloc; t.sp = tl + 3 * p->nalloc;
        t.save = p->save.as<float>();
        t.err = p->err.as<int>();
        GEO_TRY(launch_tti3d(t, st, s));
    } else {
        const Fused3D r = make_fused(p, f);
        GEO_TRY(launch_fused3d(p->fs[f].maps[p->fs[f].cur], r, p->d.mode, st, s));
    }
    p->fs[f].cur ^= 1;
    return GEO_OK;
}

// Current level of P of field set f (the watchdog's input, nalloc floats).
static const float *cur_P(const geo_fd3d_plan *p, int f) { return p->fs[f].lev[p->fs[f].cur][3].as<float>(); }

static int zero_state(geo_fd3d_plan *p, int f, cudaStream_t s) {
    FieldSet3D &F = p->fs[f];
    for (int c = 0; c < 2; c++)
        for (int k = 0; k < 5; k++) GEO_TRY(F.lev[c][k].zero(s));
    DevBuf *sp[6] = {&F.px, &F.py, &F.pz, &F.qx, &F.qy, &F.qz};
    for (DevBuf *b : sp) GEO_TRY(b->zero(s));
    F.cur = 0;
    return GEO_OK;
}

static int check_err(geo_fd3d_plan *p, cudaStream_t s) {
    int e = 0;
    GEO_CUDA(cudaMemcpyAsync(&e, p->err.p, 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    if (e) return fail(GEO_ERR_CUDA, "3D step: a TMA pipeline stage timed out");
    return GEO_OK;
}

// Autotuner for the y chunking: bare steps of the zeroed field set 0 (which
// stays zero) timed with events for each candidate chunk count.
static int autotune_chunks(geo_fd3d_plan *p, cudaStream_t s) {
    if (g_chunks_fixed()) return GEO_OK;
    GEO_TRY(zero_state(p, 0, s));
    GEO_TRY(p->err.zero(s));
    cudaEvent_t a, b;
    GEO_CUDA(cudaEventCreate(&a));
    GEO_CUDA(cudaEventCreate(&b));
    StepArgs3D st{};
    float best = 1e30f;
    int best_c = 4;
    const int planes = p->nny - 8;
    for (int c : {2, 3, 4, 5, 6, 8, 10}) {
        if (planes / c < 16) break;
        set_chunks(p, c);
        int rc = step3d(p, 0, st, s);
        if (rc == GEO_OK && cudaEventRecord(a, s) != cudaSuccess) rc = fail(GEO_ERR_CUDA, "event record");
        for (int k = 0; k < 3 && rc == GEO_OK; k++) rc = step3d(p, 0, st, s);
        float ms = 0;
        if (rc == GEO_OK && (cudaEventRecord(b, s) != cudaSuccess || cudaEventSynchronize(b) != cudaSuccess ||
                             cudaEventElapsedTime(&ms, a, b) != cudaSuccess))
            rc = fail(GEO_ERR_CUDA, "chunk autotune timing");
        if (rc != GEO_OK) {
            cudaEventDestroy(a);
            cudaEventDestroy(b);
            return rc;
        }
        if (ms < best) {
            best = ms;
            best_c = c;
        }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    set_chunks(p, best_c);
    p->fs[0].cur = 0;
    return check_err(p, s);
}

// SV taper box for shot `is` (GPU_vti3dfd_kernels.cu:155-174: R=15, r=4,
// centre fs+is*ds+npml-1): tapered=true writes the tapered coefficients,
// false restores the untapered ones.  Exact mode holds 1+2eps and
// sqrtf(1+2del); fast mode A = vp^2(1+2eps) and B = vp^2 sqrtf(1+2del).
static int taper_box_3d(geo_fd3d_plan *p, int is, bool tapered, cudaStream_t s) {
    const geo_fd3d_desc &D = p->d;
    const long cx = D.fsx + (long)is * D.dsx + D.npd - 1, cy = D.fsy + (long)is * D.dsy + D.npd - 1,
               cz = D.fsz + (long)is * D.dsz + D.npd - 1;
    const int B = 31, R = 15, r = 4;
    const long n = (long)B * B * B;
    std::vector<float> h(2 * n, 1.0f), raw(3 * n, 0.0f);   // raw: padded vp, eps, del on the box
    k_gather_box3d<<<(int)((n + 255) / 256), 256, 0, s>>>(p->raw.as<float>(), D.nx, D.ny, D.nz, D.npd, p->nnx, p->nny,
                                                          p->nnz, cx - 15, cy - 15, cz - 15, B, p->box.as<float>());
    GEO_TRY(check_launch("gather_box3d"));
    GEO_CUDA(cudaMemcpyAsync(raw.data(), p->box.p, 3 * n * 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    for (int by = 0; by < B; by++)
        for (int bx = 0; bx < B; bx++)
            for (int bz = 0; bz < B; bz++) {
                const long iz = cz - 15 + bz, ix = cx - 15 + bx, iy = cy - 15 + by;
                if (iz < 0 || iz >= p->nnz || ix < 0 || ix >= p->nnx || iy < 0 || iy >= p->nny) continue;
                const long k = bz + (long)B * (bx + (long)B * by);
                float ee = raw[n + k], dd = raw[2 * n + k];
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
                const float e2 = 1 + 2 * ee, d2 = sqrtf(1 + 2 * dd);
                if (p->d.mode == GEO_MODE_FAST) {
                    const float c2 = raw[k] * raw[k];
                    h[k] = c2 * e2;
                    h[n + k] = c2 * d2;
                } else {
                    h[k] = e2;
                    h[n + k] = d2;
                }
            }
    GEO_CUDA(cudaMemcpyAsync(p->box.p, h.data(), h.size() * 4, cudaMemcpyHostToDevice, s));
    Grid3D g = make_grid(p);
    float *a0 = p->d.mode == GEO_MODE_FAST ? p->vp.as<float>() : p->e2.as<float>();
    float *a1 = p->d.mode == GEO_MODE_FAST ? p->e2.as<float>() : p->d2.as<float>();
    k_box3d<<<(int)((n + 255) / 256), 256, 0, s>>>(g, a0, a1, cx - 15, cy - 15, cz - 15, B, p->box.as<float>());
    GEO_TRY(check_launch("box3d"));
    GEO_CUDA(cudaStreamSynchronize(s));  // h goes out of scope
    return GEO_OK;
}

static int source_cell(const geo_fd3d_plan *p, int is, StepArgs3D &st) {
    const geo_fd3d_desc &D = p->d;
    const long ixs = D.fsx + (long)is * D.dsx + D.npd - 1, iys = D.fsy + (long)is * D.dsy + D.npd - 1,
               izs = D.fsz + (long)is * D.dsz + D.npd - 1;
    if (ixs < 4 || ixs >= p->nnx - 4 || iys < 4 || iys >= p->nny - 4 || izs < 4 || izs >= p->nnz - 4)
        return fail(GEO_ERR_ARG, "source outside the updated grid");
    st.ixs = (int)ixs; st.iys = (int)iys; st.izs = (int)izs;
    return GEO_OK;
}

// Forward run of shot `is` into the plan's time-major record buffer;
// `on_step(it)` (optional) runs after each step (snapshots).
int run_shot_3d(geo_fd3d_plan *p, int is, cudaStream_t s, int (*on_step)(void *, int), void *ctx) {
    if (!p->model_set) return fail(GEO_ERR_ARG, "model not set");
    const geo_fd3d_desc &D = p->d;
    StepArgs3D st{};
    GEO_TRY(source_cell(p, is, st));
    GEO_TRY(zero_state(p, 0, s));
    GEO_TRY(p->err.zero(s));
    if (D.sv) GEO_TRY(taper_box_3d(p, is, true, s));
    st.rec = p->rec_tm.as<float>();
    st.rec_iz = D.rec_iz; st.rx0 = D.rx0; st.drx = D.drx; st.nrx = D.nrx; st.ry0 = D.ry0; st.dry = D.dry; st.nry = D.nry;
    GEO_TRY(p->wd.open());
    p->wd.arm();
    for (int it = 0; it < D.nt; it++) {
        st.it = it;
        st.src_on = p->on[it];
        st.amp = p->amp[it];
        GEO_TRY(step3d(p, 0, st, s));
        if (on_step) GEO_TRY(on_step(ctx, it));
        const int w = p->wd.check(cur_P(p, 0), p->nalloc, it, it == D.nt - 1, s);
        if (w == GEO_ERR_NAN) break;
        GEO_TRY(w);
    }
    GEO_TRY(p->wd.verdict(s, "3D shot"));
    if (D.sv) GEO_TRY(taper_box_3d(p, is, false, s));
    GEO_TRY(check_err(p, s));
    const int ntr = D.nrx * D.nry;
    if (D.mute_tt > 0) {
        std::vector<int> hi;
        // the mute formula indexes receivers as model cells (every node)
        mute_window_3d(D.nrx, D.nry, D.nt, D.dt, D.favg, D.dx, D.dy, D.dz, D.fsx, D.fsy, D.dsx, D.dsy, D.fsz, is,
                       p->vp1, p->eps1, D.mute_tt, hi);
        GEO_CUDA(cudaMemcpyAsync(p->mute_hi.p, hi.data(), hi.size() * 4, cudaMemcpyHostToDevice, s));
        GEO_TRY(launch_mute_records(p->rec_tm.as<float>(), ntr, D.nt, nullptr, p->mute_hi.as<int>(), s));
        GEO_CUDA(cudaStreamSynchronize(s));
    }
    return GEO_OK;
}

int plan3d_dims(const geo_fd3d_plan *p, int *nnx, int *nny, int *nnz) {
    *nnx = p->nnx; *nny = p->nny; *nnz = p->nnz;
    return GEO_OK;
}

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

static int check_desc(const geo_fd3d_desc &d) {
    if (d.nx < 2 || d.ny < 2 || d.nz < 2 || d.npd < 5 || d.nt < 1)
        return fail(GEO_ERR_ARG, "grid too small (npd must be >= 5)");
    if (!(d.dt > 0) || !(d.dx > 0) || !(d.dy > 0) || !(d.dz > 0)) return fail(GEO_ERR_ARG, "bad spacing");
    if (d.nrx < 1 || d.nry < 1 || d.drx < 1 || d.dry < 1) return fail(GEO_ERR_ARG, "bad receiver grid");
    if (d.rx0 < 0 || d.rx0 + (d.nrx - 1) * d.drx >= d.nx) return fail(GEO_ERR_ARG, "receivers outside x");
    if (d.ry0 < 0 || d.ry0 + (d.nry - 1) * d.dry >= d.ny) return fail(GEO_ERR_ARG, "receivers outside y");
    if (d.rec_iz < 4 || d.rec_iz >= d.nz + 2 * d.npd - 4) return fail(GEO_ERR_ARG, "receiver depth outside grid");
    if (d.mode != GEO_MODE_EXACT && d.mode != GEO_MODE_FAST) return fail(GEO_ERR_ARG, "bad mode");
    if (!(d.favg > 0)) return fail(GEO_ERR_ARG, "favg must be > 0");
    return GEO_OK;
}

// Plan with nfs wavefield sets.
int plan3d_create(geo_fd3d_plan **out, const geo_fd3d_desc *desc, int nfs) {
    if (!out || !desc) return fail(GEO_ERR_ARG, "null argument");
    const geo_fd3d_desc &d = *desc;
    GEO_TRY(check_desc(d));
    geo_fd3d_plan *p = new geo_fd3d_plan();
    p->d = d;
    p->nfs = nfs;
    p->nnx = d.nx + 2 * d.npd;
    p->nny = d.ny + 2 * d.npd;
    p->nnz = d.nz + 2 * d.npd;
    p->ldz = (p->nnz + 3) & ~3;
    p->n = (size_t)p->nnx * p->nny * p->nnz;
    p->nalloc = (size_t)p->nnx * p->nny * p->ldz;
    if (p->nalloc >= (size_t)1 << 31) {
        delete p;
        return fail(GEO_ERR_ARG, "grid of %zu points per field exceeds 2^31", (size_t)d.nx * d.ny * d.nz);
    }
    p->ntz = (p->nnz + kTZ - 1) / kTZ;
    p->ntx = (p->nnx + kTXF - 1) / kTXF;
    const size_t n = p->nalloc, ntr = (size_t)d.nrx * d.nry;
    int st = GEO_OK;
    DevBuf *model[3] = {&p->vp, &p->e2, &p->d2};
    for (DevBuf *b : model)
        if (st == GEO_OK) st = b->alloc(n * 4);
    for (int f = 0; f < nfs && st == GEO_OK; f++) st = alloc_fields(p, f);
    if (st == GEO_OK) st = p->prof.alloc((size_t)4 * (p->nnx + p->nny + p->nnz) * 4);
    if (st == GEO_OK) st = p->rec_tm.alloc(ntr * d.nt * 4);
    if (st == GEO_OK) st = p->rec_tr.alloc(ntr * d.nt * 4);
    if (st == GEO_OK) st = p->mute_lo.alloc(ntr * 4);
    if (st == GEO_OK) st = p->mute_hi.alloc(ntr * 4);
    if (st == GEO_OK) st = p->box.alloc((size_t)3 * 31 * 31 * 31 * 4);   // gathered raw box (3), tapered box (2)
    if (st == GEO_OK) st = p->err.alloc(16);
    if (st == GEO_OK) st = p->err.zero(nullptr);
    if (st != GEO_OK) {
        delete p;
        return st;
    }
    choose_chunks(p);
    source_amplitudes(V_GPU, d.nt, d.dt, d.favg, d.pfac, d.wtype, p->amp, p->on);
    *out = p;
    return GEO_OK;
}

}  // namespace geo

extern "C" int geo_fd3d_plan_create(geo_fd3d_plan **out, const geo_fd3d_desc *desc) {
    return plan3d_create(out, desc, 1);
}

extern "C" int geo_fd3d_plan_destroy(geo_fd3d_plan *p) {
    delete p;
    return GEO_OK;
}

// Copy a padded nnz-contiguous host volume into an ldz-strided device field.

// Model upload: pad on the host, build the model arrays of the chosen form
// and the sponge profiles (d0 from the padded centre velocity,
// GPU_vti3dfd_kernels.cu:203-206).
// Tilt and azimuth (degrees, interior layout) of a 3D TTI medium: from now
// on the plan steps with the 3D TTI scheme (tti3d.cu).  Their cosines and
// sines are formed on the host as cosf(deg * 0.017453292519943295f) and
// padded by edge replication on the device.
extern "C" int geo_fd3d_set_tilt(geo_fd3d_plan *p, const float *theta, const float *phi, int mem, void *stream) {
    if (!p || !theta || !phi) return fail(GEO_ERR_ARG, "null argument");
    if (mem != GEO_MEM_HOST && mem != GEO_MEM_DEVICE) return fail(GEO_ERR_ARG, "bad mem kind");
    if (p->d.mode != GEO_MODE_FAST) return fail(GEO_ERR_ARG, "the TTI step needs the fast (premultiplied) model form");
    cudaStream_t s = (cudaStream_t)stream;
    const geo_fd3d_desc &D = p->d;
    const size_t n0 = (size_t)D.nx * D.ny * D.nz;
    std::vector<float> ang;
    const float *th = theta, *ph = phi;
    if (mem == GEO_MEM_DEVICE) {
        ang.resize(2 * n0);
        GEO_CUDA(cudaMemcpyAsync(ang.data(), theta, n0 * 4, cudaMemcpyDeviceToHost, s));
        GEO_CUDA(cudaMemcpyAsync(ang.data() + n0, phi, n0 * 4, cudaMemcpyDeviceToHost, s));
        GEO_CUDA(cudaStreamSynchronize(s));
        th = ang.data();
        ph = ang.data() + n0;
    }
    for (size_t k = 0; k < n0; k++)
        if (!std::isfinite(th[k]) || !std::isfinite(ph[k])) return fail(GEO_ERR_MODEL, "tilt/azimuth[%zu] not finite", k);
    std::vector<float> trig(4 * n0);
    {
        const unsigned nth = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        const size_t chunk = (n0 + nth - 1) / nth;
        for (unsigned t = 0; t < nth; t++)
            pool.emplace_back([&, t]() {
                const size_t lo = t * chunk, hi = std::min(n0, lo + chunk);
                for (size_t k = lo; k < hi; k++) {
                    const float a = th[k] * 0.017453292519943295f, b = ph[k] * 0.017453292519943295f;
                    trig[k] = cosf(a);
                    trig[n0 + k] = sinf(a);
                    trig[2 * n0 + k] = cosf(b);
                    trig[3 * n0 + k] = sinf(b);
                }
            });
        for (auto &t : pool) t.join();
    }
    DevBuf tmp;
    GEO_TRY(tmp.alloc(4 * n0 * 4));
    GEO_CUDA(cudaMemcpyAsync(tmp.p, trig.data(), 4 * n0 * 4, cudaMemcpyHostToDevice, s));
    if (p->tilt.bytes != 4 * p->nalloc * 4) GEO_TRY(p->tilt.alloc(4 * p->nalloc * 4));
    if (!p->save.p) GEO_TRY(p->save.alloc(16));
    for (int r = 0; r < 4; r++) {
        k_pad3d<<<grid_blocks((long)p->n), 256, 0, s>>>(tmp.as<float>() + r * n0, D.nx, D.ny, D.nz, D.npd, p->nnx,
                                                        p->nny, p->nnz, p->ldz, p->tilt.as<float>() + r * p->nalloc);
        GEO_TRY(check_launch("pad3d"));
    }
    GEO_CUDA(cudaStreamSynchronize(s));
    p->tti = true;
    return GEO_OK;
}

extern "C" int geo_fd3d_set_model(geo_fd3d_plan *p, const float *v, const float *e, const float *d, int mem,
                                  void *stream) {
    if (!p || !v || !e || !d) return fail(GEO_ERR_ARG, "null argument");
    if (mem != GEO_MEM_HOST && mem != GEO_MEM_DEVICE) return fail(GEO_ERR_ARG, "bad mem kind");
    cudaStream_t s = (cudaStream_t)stream;
    const geo_fd3d_desc &D = p->d;
    const size_t n0 = (size_t)D.nx * D.ny * D.nz;
    // the unpadded model on the device (kept: the SV taper gathers from it)
    if (p->raw.bytes != 3 * n0 * 4) GEO_TRY(p->raw.alloc(3 * n0 * 4));
    float *raw = p->raw.as<float>();
    const cudaMemcpyKind kin = mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    GEO_CUDA(cudaMemcpyAsync(raw, v, n0 * 4, kin, s));
    GEO_CUDA(cudaMemcpyAsync(raw + n0, e, n0 * 4, kin, s));
    GEO_CUDA(cudaMemcpyAsync(raw + 2 * n0, d, n0 * 4, kin, s));
    // model check on the device, reported like check_model
    GEO_CUDA(cudaMemsetAsync(p->box.p, 0xff, 8, s));
    unsigned long long *first = reinterpret_cast<unsigned long long *>(p->box.p);
    k_check_model3d<<<grid_blocks((long)n0), 256, 0, s>>>(raw, raw + n0, raw + 2 * n0, (long)n0, first);
    GEO_TRY(check_launch("check_model3d"));
    unsigned long long key = 0;
    GEO_CUDA(cudaMemcpyAsync(&key, first, 8, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    if (key != ~0ull) {
        const size_t i = (size_t)(key >> 2);
        float bad = 0;
        GEO_CUDA(cudaMemcpy(&bad, raw + i, 4, cudaMemcpyDeviceToHost));
        if ((key & 3) == 0) return fail(GEO_ERR_MODEL, "velocity[%zu]=%g", i, bad);
        if ((key & 3) == 1) return fail(GEO_ERR_MODEL, "eps/del[%zu] not finite", i);
        return fail(GEO_ERR_MODEL, "1+2*delta[%zu] < 0", i);
    }
    // the stability number of the set-up code (dt*vmax*sqrt(sum 1/d^2) < 0.777)
    {
        unsigned *mm = reinterpret_cast<unsigned *>(p->box.p) + 4;
        GEO_TRY(launch_minmax(raw, n0, mm, s));
        unsigned b[2];
        GEO_CUDA(cudaMemcpyAsync(b, mm, 8, cudaMemcpyDeviceToHost, s));
        GEO_CUDA(cudaStreamSynchronize(s));
        float vmin, vmax;
        memcpy(&vmin, &b[0], 4);
        memcpy(&vmax, &b[1], 4);
        GEO_TRY(check_stability(V_GPU, 3, vmin, vmax, D.dt, D.dx, D.dy, D.dz, D.favg));
    }
    // padded model arrays, written straight into the pitched layout
    k_model3d<<<grid_blocks((long)p->n), 256, 0, s>>>(raw, raw + n0, raw + 2 * n0, D.nx, D.ny, D.nz, D.npd, p->nnx,
                                                      p->nny, p->nnz, p->ldz, D.mode == GEO_MODE_FAST ? 1 : 0,
                                                      p->vp.as<float>(), p->e2.as<float>(), p->d2.as<float>());
    GEO_TRY(check_launch("model3d"));
    // the few padded values the host set-up needs: vp, eps at padded index 1
    // (the mute) and vp at the padded centre (d0); edge replication maps a
    // padded index to the unpadded one
    auto raw_index = [&](size_t k) {
        const long iz = (long)(k % p->nnz), ix = (long)((k / p->nnz) % p->nnx), iy = (long)(k / ((size_t)p->nnz * p->nnx));
        const long sz = std::min(std::max(iz - D.npd, 0L), (long)D.nz - 1);
        const long sx = std::min(std::max(ix - D.npd, 0L), (long)D.nx - 1);
        const long sy = std::min(std::max(iy - D.npd, 0L), (long)D.ny - 1);
        return (size_t)(sz + (long)D.nz * (sx + (long)D.nx * sy));
    };
    float pick[3];
    const size_t r1 = raw_index(1), rc = raw_index((size_t)p->nny * p->nnx * p->nnz / 2);
    GEO_CUDA(cudaMemcpyAsync(&pick[0], raw + r1, 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaMemcpyAsync(&pick[1], raw + n0 + r1, 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaMemcpyAsync(&pick[2], raw + rc, 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    p->vp1 = pick[0];
    p->eps1 = pick[1];
    const float d0 = sponge_d0(V_GPU, 3, 0.0f, pick[2], D.npd, D.dx, D.dy, D.dz);
    std::vector<float> prof((size_t)4 * (p->nnx + p->nny + p->nnz));
    float *q = prof.data();
    sponge_profiles(V_GPU, D.nx, D.npd, D.dt, d0, q, q + p->nnx, q + 2 * p->nnx, q + 3 * p->nnx);
    q += 4 * p->nnx;
    sponge_profiles(V_GPU, D.ny, D.npd, D.dt, d0, q, q + p->nny, q + 2 * p->nny, q + 3 * p->nny);
    q += 4 * p->nny;
    sponge_profiles(V_GPU, D.nz, D.npd, D.dt, d0, q, q + p->nnz, q + 2 * p->nnz, q + 3 * p->nnz);
    GEO_CUDA(cudaMemcpyAsync(p->prof.p, prof.data(), prof.size() * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    if (!p->tuned) {
        GEO_TRY(autotune_chunks(p, s));
        p->tuned = true;
    }
    p->model_set = true;
    return GEO_OK;
}

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
    StepArgs3D st{};
    cudaEvent_t a, b;
    GEO_CUDA(cudaEventCreate(&a));
    GEO_CUDA(cudaEventCreate(&b));
    GEO_CUDA(cudaEventRecord(a, s));
    for (int k = 0; k < nsteps; k++) {
        st.it = k;
        GEO_TRY(step3d(p, 0, st, s));
    }
    GEO_CUDA(cudaEventRecord(b, s));
    GEO_CUDA(cudaEventSynchronize(b));
    float t = 0;
    GEO_CUDA(cudaEventElapsedTime(&t, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (ms) *ms = t;
    return check_err(p, s);
}

extern "C" int geo_fd3d_get_fields(geo_fd3d_plan *p, float *P, float *Q, int mem, void *stream) {
    if (!p) return fail(GEO_ERR_ARG, "null plan");
    cudaStream_t s = (cudaStream_t)stream;
    const cudaMemcpyKind k = mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    float *dst[2] = {P, Q};
    const FieldSet3D &F = p->fs[0];
    for (int f = 0; f < 2; f++)
        if (dst[f])
            GEO_CUDA(cudaMemcpy2DAsync(dst[f], (size_t)p->nnz * 4, F.lev[F.cur][3 + f].p, (size_t)p->ldz * 4,
                                       (size_t)p->nnz * 4, (size_t)p->nnx * p->nny, k, s));
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

// ---------------------------------------------------------------- RTM 3D
namespace geo {

// Source P of the interior box into a dense snapshot (iz + nz*(ix + nx*iy)).
__global__ void k_snap_store(Grid3D g, const float *P, float *snap) {
    const long n = (long)g.nx * g.ny * g.nz;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(k % g.nz), ix = (int)((k / g.nz) % g.nx), iy = (int)(k / ((long)g.nz * g.nx));
        snap[k] = P[(g.npd + iz) + (long)g.ldz * (g.npd + ix) + g.sxy * (g.npd + iy)];
    }
}

// mig += w * snap * gP on the interior box (the codec's imaging, same order).
__global__ void k_snap_image(Grid3D g, const float *snap, const float *gP, float *mig, float w) {
    const long n = (long)g.nx * g.ny * g.nz;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(k % g.nz), ix = (int)((k / g.nz) % g.nx), iy = (int)(k / ((long)g.nz * g.nx));
        mig[k] = mig[k] + w * snap[k] * gP[(g.npd + iz) + (long)g.ldz * (g.npd + ix) + g.sxy * (g.npd + iy)];
    }
}

// Poynting angle gathers after a backward step (Poynting_Adcigs :618-661):
// s, r are the source and receiver fields at their new time level; tab holds
// the bin thresholds then cosf(ia*pi/180), kMaxAngles each.  One thread per
// gather column point (iz fastest); each point adds to one bin of its own
// column, so there are no write conflicts.
__global__ void k_adcig3d(Grid3D s, Grid3D r, float *adcig, const float *tab, int na, int dcdp, int nxa, int nya) {
    __shared__ float thr[kMaxAngles], cs[kMaxAngles];
    for (int i = threadIdx.x; i < kMaxAngles; i += blockDim.x) {
        thr[i] = tab[i];
        cs[i] = tab[kMaxAngles + i];
    }
    __syncthreads();
    const int nz = s.nz;
    const long n = (long)nz * nxa * nya;
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(k % nz);
        const long c = k / nz;
        const int ix = (int)(c % nxa), iy = (int)(c / nxa);
        const long id = (s.npd + iz) + s.ldz * (long)(s.npd + ix * dcdp) + s.sxy * (long)(s.npd + iy * dcdp);
        const float sP = s.P[id], gP = r.P[id];
        const float Ssx = -sP * s.u[id], Ssy = -sP * s.v[id], Ssz = -s.Q[id] * s.w[id];
        const float Sgx = gP * r.u[id], Sgy = gP * r.v[id], Sgz = r.Q[id] * r.w[id];
        const float b1 = Ssx * Ssx + Ssy * Ssy + Ssz * Ssz, b2 = Sgx * Sgx + Sgy * Sgy + Sgz * Sgz;
        const int ia = poynting_bin(Ssx * Sgx + Ssy * Sgy + Ssz * Sgz, b1, b2, thr, na);
        if (ia < 0) continue;
        const float w = cs[ia];
        float *o = adcig + iz + (long)nz * (ia + (long)na * (ix + (long)nxa * iy));
        *o = *o + sP * gP * w * w * w;
    }
}

// adcigs_illum (:663-684): gathers /= illum at (iz, ix*dcdp, iy*dcdp) where non-zero.
__global__ void k_adcig3d_illum(float *adcig, const float *ill, int nx, int nz, int na, int dcdp, int nxa, long n) {
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        const int iz = (int)(k % nz);
        const long c = k / ((long)nz * na);
        const int ix = (int)(c % nxa), iy = (int)(c / nxa);
        const float w = ill[iz + (long)ix * dcdp * nz + (long)iy * dcdp * nx * nz];
        if (w != 0.0f) adcig[k] = adcig[k] / w;
    }
}

}  // namespace geo

// 3D RTM.  Method GEO_RTM_BOUNDARY follows the 3D GPU RTM program
// (3D-vti-fd+rtm-cuda/Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:882-981):
// ring save in the forward pass, source re-propagation driven by the ring in
// the backward pass.  GEO_RTM_SNAPSHOT and GEO_RTM_LEARNED keep snapshots of
// the source P instead and propagate only the receiver field backwards.
// GEO_RTM_CHECKPOINT saves the source field's full state every K steps and,
// in the backward pass, re-propagates each K-step segment from its
// checkpoint to hold that segment's snapshots: three propagations per step
// like the boundary method, the snapshot method's image bit for bit, and
// memory of K/snap_every snapshots plus nt/K states.
extern "C" int geo_rtm3d_adcig(const geo_rtm3d_desc *desc, const float *v, const float *e, const float *d,
                               float *mig_out, float *lap_out, float *illum_out, float *adcig_out, int mem,
                               void *stream) {
    if (!desc || !v || !e || !d || !mig_out) return fail(GEO_ERR_ARG, "null argument");
    if (mem != GEO_MEM_HOST && mem != GEO_MEM_DEVICE) return fail(GEO_ERR_ARG, "bad mem kind");
    const geo_rtm3d_desc &R = *desc;
    if (R.ns < 1) return fail(GEO_ERR_ARG, "ns must be >= 1");
    const int method = R.method;
    if (method != GEO_RTM_BOUNDARY && method != GEO_RTM_SNAPSHOT && method != GEO_RTM_LEARNED &&
        method != GEO_RTM_CHECKPOINT)
        return fail(GEO_ERR_ARG, "unknown RTM method %d", method);
    if (method != GEO_RTM_BOUNDARY && R.snap_every < 1) return fail(GEO_ERR_ARG, "snap_every must be >= 1");
    if (method == GEO_RTM_LEARNED && !R.ae) return fail(GEO_ERR_ARG, "the learned method needs a codec");
    // angle gathers: the program's na = 65, da = 1, dcdp = 1 by default
    const int na = R.na > 0 ? R.na : 65, da = R.da > 0 ? R.da : 1, dcdp = R.dcdp > 0 ? R.dcdp : 1;
    if (R.theta && !R.phi) return fail(GEO_ERR_ARG, "tilt without azimuth");
    if (adcig_out) {
        if (R.theta) return fail(GEO_ERR_ARG, "no angle gathers on a TTI medium");
        if (method != GEO_RTM_BOUNDARY) return fail(GEO_ERR_ARG, "angle gathers need the boundary method");
        if (na > kMaxAngles) return fail(GEO_ERR_ARG, "na must be 1..%d", kMaxAngles);
        if (dcdp > R.fd.nx || dcdp > R.fd.ny) return fail(GEO_ERR_ARG, "dcdp exceeds the model");
    }
    geo_fd3d_desc D = R.fd;
    // every surface node records P+Q at z = npml (shot_record :319-334), or
    // the caller's receiver grid (checked with the plan)
    D.rec_iz = D.npd;
    if (!R.rec_grid) {
        D.rx0 = 0; D.drx = 1; D.nrx = D.nx; D.ry0 = 0; D.dry = 1; D.nry = D.ny;
    }
    D.mute_tt = 0;
    cudaStream_t s = (cudaStream_t)stream;
    geo_fd3d_plan *p = nullptr;
    GEO_TRY(plan3d_create(&p, &D, 2));
    std::unique_ptr<geo_fd3d_plan, int (*)(geo_fd3d_plan *)> guard(p, geo_fd3d_plan_destroy);
    GEO_TRY(geo_fd3d_set_model(p, v, e, d, mem, stream));
    if (R.theta) GEO_TRY(geo_fd3d_set_tilt(p, R.theta, R.phi, mem, stream));
    const long nimg = (long)D.nx * D.ny * D.nz;
    const long L = 2L * D.nx * D.ny + 2L * D.nz * D.ny + 2L * D.nx * D.nz;
    const int k = method == GEO_RTM_BOUNDARY ? 1 : R.snap_every;
    const int nsnap = method == GEO_RTM_BOUNDARY ? 0 : D.nt / k;
    // checkpoint method: the full state of the source field every K steps
    // (u,v,w,P,Q of the current level, plus the six split stresses of the
    // VTI step), a segment's snapshots at a time in the backward pass
    int K = 0, nck = 0, narr = 0;
    if (method == GEO_RTM_CHECKPOINT) {
        narr = R.theta ? 5 : 11;
        // automatic interval: minimises nt/K states (narr padded arrays each)
        // plus K/snap_every snapshots (interior arrays)
        const double ratio = (double)narr * p->nalloc / (double)((long)D.nx * D.ny * D.nz);
        K = R.ckpt_every;
        if (K <= 0) K = k * std::max(1, (int)std::lround(std::sqrt((double)D.nt / k * ratio)));
        if (K % k) return fail(GEO_ERR_ARG, "ckpt_every must be a multiple of snap_every");
        nck = (D.nt + K - 1) / K;
    }
    DevBuf ring, mig, ill, lap, snaps, codes, scales, escs, resid, nesc, ckpt;
    const Grid3D g0 = grid_of(p, 0);
    const AeVolume box = ae_volume(nullptr, g0.ldz, g0.sxy, D.npd, D.npd, D.npd, D.nz, D.nx, D.ny);
    const int crow = ae_code_rows(box);
    const int ecap = method == GEO_RTM_LEARNED ? ae_escape_cap(R.ae, box) : 0;
    if (method == GEO_RTM_BOUNDARY) {
        GEO_TRY(ring.alloc((size_t)2 * D.nt * L * 4));
    } else if (method == GEO_RTM_CHECKPOINT) {
        GEO_TRY(ckpt.alloc((size_t)nck * narr * p->nalloc * 4));
        GEO_TRY(snaps.alloc((size_t)std::max(K / k, 1) * nimg * 4));
    } else if (method == GEO_RTM_SNAPSHOT) {
        GEO_TRY(snaps.alloc((size_t)std::max(nsnap, 1) * nimg * 4));
    } else {
        const size_t ns1 = (size_t)std::max(nsnap, 1);
        GEO_TRY(codes.alloc(ns1 * crow * kAeLat * 2));
        GEO_TRY(scales.alloc(ns1 * crow * 4));
        GEO_TRY(escs.alloc(ns1 * crow * 4));
        GEO_TRY(resid.alloc(ns1 * std::max(ecap, 1) * kAePts * 2));
        GEO_TRY(nesc.alloc(ns1 * 4));
    }
    GEO_TRY(mig.alloc(nimg * 4));
    GEO_TRY(ill.alloc(nimg * 4));
    GEO_TRY(mig.zero(s));
    GEO_TRY(ill.zero(s));
    const int nxa = D.nx / dcdp, nya = D.ny / dcdp;
    const long nag = (long)D.nz * na * nxa * nya;
    DevBuf ag, atab;
    if (adcig_out) {
        GEO_TRY(ag.alloc(nag * 4));
        GEO_TRY(ag.zero(s));
        GEO_TRY(atab.alloc(2 * kMaxAngles * 4));
        GEO_TRY(adcig_angle_tables(na, da, atab.as<float>(), atab.as<float>() + kMaxAngles, s));
    }
    float *bp = ring.as<float>(), *bq = bp + (size_t)D.nt * L;
    const int ntr = D.nrx * D.nry;
    auto launch_ring = [&](int it, int save) -> int {
        Grid3D g = grid_of(p, 0);
        k_ring3d<<<grid_blocks(L), 256, 0, s>>>(g, g.P, g.Q, bp, bq, L, it, save);
        return check_launch("ring3d");
    };
    auto is_snap = [&](int it) { return method != GEO_RTM_BOUNDARY && it % k == k - 1 && it / k < nsnap; };
    // copy the source field's state into checkpoint c (save) or back
    auto state_copy = [&](int c, bool save) -> int {
        FieldSet3D &F = p->fs[0];
        DevBuf *arr[11] = {&F.lev[F.cur][0], &F.lev[F.cur][1], &F.lev[F.cur][2], &F.lev[F.cur][3], &F.lev[F.cur][4],
                           &F.px, &F.py, &F.pz, &F.qx, &F.qy, &F.qz};
        for (int a = 0; a < narr; a++) {
            float *slot = ckpt.as<float>() + ((size_t)c * narr + a) * p->nalloc;
            if (save)
                GEO_CUDA(cudaMemcpyAsync(slot, arr[a]->p, p->nalloc * 4, cudaMemcpyDeviceToDevice, s));
            else
                GEO_CUDA(cudaMemcpyAsync(arr[a]->p, slot, p->nalloc * 4, cudaMemcpyDeviceToDevice, s));
        }
        return GEO_OK;
    };
    for (int is = 0; is < R.ns; is++) {
        StepArgs3D st{};
        GEO_TRY(source_cell(p, is, st));
        GEO_TRY(zero_state(p, 0, s));
        GEO_TRY(zero_state(p, 1, s));
        if (D.sv) GEO_TRY(taper_box_3d(p, is, true, s));
        if (method == GEO_RTM_LEARNED) GEO_TRY(nesc.zero(s));
        // forward: record P+Q, source illumination, keep the ring or the snapshots
        st.rec = p->rec_tm.as<float>();
        st.rec_iz = D.rec_iz; st.rx0 = D.rx0; st.drx = D.drx; st.nrx = D.nrx; st.ry0 = D.ry0; st.dry = D.dry;
        st.nry = D.nry;
        st.rec_pq = 1;
        st.ill = ill.as<float>();
        GEO_TRY(p->wd.open());
        p->wd.arm();
        bool diverged = false;
        for (int it = 0; it < D.nt && !diverged; it++) {
            st.it = it;
            st.src_on = p->on[it];
            st.amp = p->amp[it];
            if (method == GEO_RTM_CHECKPOINT && it % K == 0) GEO_TRY(state_copy(it / K, true));
            GEO_TRY(step3d(p, 0, st, s));
            if (method == GEO_RTM_BOUNDARY) {
                GEO_TRY(launch_ring(it, 1));
            } else if (is_snap(it) && method != GEO_RTM_CHECKPOINT) {
                const Grid3D g = grid_of(p, 0);
                const int j = it / k;
                if (method == GEO_RTM_SNAPSHOT) {
                    k_snap_store<<<grid_blocks(nimg), 256, 0, s>>>(g, g.P, snaps.as<float>() + (size_t)j * nimg);
                    GEO_TRY(check_launch("snap_store"));
                } else {
                    AeVolume vb = box;
                    vb.src = g.P;
                    GEO_TRY(ae_encode_volume(R.ae, vb, codes.as<__nv_bfloat16>() + (size_t)j * crow * kAeLat,
                                             scales.as<float>() + (size_t)j * crow, escs.as<int>() + (size_t)j * crow,
                                             resid.as<__nv_bfloat16>() + (size_t)j * ecap * kAePts,
                                             nesc.as<int>() + j, s));
                }
            }
            const int w = p->wd.check(cur_P(p, 0), p->nalloc, it, it == D.nt - 1, s);
            if (w == GEO_ERR_NAN) diverged = true;
            else GEO_TRY(w);
        }
        GEO_TRY(p->wd.verdict(s, "3D RTM forward pass"));
        // direct-wave mute, window form (mute_directwave :352-390)
        if (R.mute_tt > 0) {
            std::vector<int> flo, fhi, lo(ntr), hi(ntr);
            mute_window_3d_band(D.nx, D.ny, D.nt, D.dt, D.favg, D.dx, D.dy, D.dz, D.fsx, D.fsy, D.dsx, D.dsy, D.fsz,
                                is, p->vp1, p->eps1, R.mute_tt, flo, fhi);
            // the window of each receiver of the grid, by its model cell
            for (int jy = 0; jy < D.nry; jy++)
                for (int jx = 0; jx < D.nrx; jx++) {
                    const size_t c = (size_t)(D.ry0 + jy * D.dry) * D.nx + (D.rx0 + jx * D.drx);
                    lo[(size_t)jy * D.nrx + jx] = flo[c];
                    hi[(size_t)jy * D.nrx + jx] = fhi[c];
                }
            GEO_CUDA(cudaMemcpyAsync(p->mute_lo.p, lo.data(), lo.size() * 4, cudaMemcpyHostToDevice, s));
            GEO_CUDA(cudaMemcpyAsync(p->mute_hi.p, hi.data(), hi.size() * 4, cudaMemcpyHostToDevice, s));
            GEO_TRY(launch_mute_records(p->rec_tm.as<float>(), ntr, D.nt, p->mute_lo.as<int>(), p->mute_hi.as<int>(), s));
            GEO_CUDA(cudaStreamSynchronize(s));
        }
        // backward: propagate the record from the surface, image
        StepArgs3D sb{}, gb{};
        sb.ixs = gb.ixs = st.ixs; sb.iys = gb.iys = st.iys; sb.izs = gb.izs = st.izs;
        gb.ill = ill.as<float>();
        if (method == GEO_RTM_BOUNDARY) gb.mig = mig.as<float>();
        for (int it = D.nt - 1; it >= 0 && !diverged; it--) {
            sb.it = gb.it = it;
            if (method == GEO_RTM_BOUNDARY) {
                GEO_TRY(launch_ring(it, 0));
                GEO_TRY(step3d(p, 0, sb, s));
            }
            if (method == GEO_RTM_CHECKPOINT && (it == D.nt - 1 || it % K == K - 1)) {
                // entering segment c from its end: restore its checkpoint and
                // re-propagate it (source on, nothing recorded), keeping
                // its snapshots
                const int c = it / K;
                GEO_TRY(state_copy(c, false));
                StepArgs3D sr{};
                sr.ixs = st.ixs; sr.iys = st.iys; sr.izs = st.izs;
                for (int j = c * K; j <= it; j++) {
                    sr.it = j;
                    sr.src_on = p->on[j];
                    sr.amp = p->amp[j];
                    GEO_TRY(step3d(p, 0, sr, s));
                    if (is_snap(j)) {
                        const Grid3D g = grid_of(p, 0);
                        k_snap_store<<<grid_blocks(nimg), 256, 0, s>>>(
                            g, g.P, snaps.as<float>() + (size_t)((j - c * K) / k) * nimg);
                        GEO_TRY(check_launch("snap_store"));
                    }
                }
            }
            {
                Grid3D gg = grid_of(p, 1);
                k_inject3d<<<grid_blocks(ntr), 256, 0, s>>>(gg, gg.P, gg.Q, p->rec_tm.as<float>(), it, D.rx0, D.drx,
                                                             D.nrx, D.ry0, D.dry, D.nry);
                GEO_TRY(check_launch("inject3d"));
            }
            if (method == GEO_RTM_BOUNDARY) gb.other_P = grid_of(p, 0).P;  // the source side's new level
            GEO_TRY(step3d(p, 1, gb, s));
            if (adcig_out) {
                k_adcig3d<<<grid_blocks((long)D.nz * nxa * nya), 256, 0, s>>>(
                    grid_of(p, 0), grid_of(p, 1), ag.as<float>(), atab.as<float>(), na, dcdp, nxa, nya);
                GEO_TRY(check_launch("adcig3d"));
            }
            if (is_snap(it)) {
                const Grid3D g = grid_of(p, 1);
                const int j = it / k;
                if (method == GEO_RTM_SNAPSHOT || method == GEO_RTM_CHECKPOINT) {
                    const size_t slot = method == GEO_RTM_SNAPSHOT ? (size_t)j : (size_t)((it % K) / k);
                    k_snap_image<<<grid_blocks(nimg), 256, 0, s>>>(g, snaps.as<float>() + slot * nimg, g.P,
                                                                    mig.as<float>(), (float)k);
                    GEO_TRY(check_launch("snap_image"));
                } else {
                    GEO_TRY(ae_decode_volume(R.ae, box, codes.as<__nv_bfloat16>() + (size_t)j * crow * kAeLat,
                                             scales.as<float>() + (size_t)j * crow, escs.as<int>() + (size_t)j * crow,
                                             resid.as<__nv_bfloat16>() + (size_t)j * ecap * kAePts, 1, nullptr, g.P,
                                             mig.as<float>(), (float)k, s));
                }
            }
            const int w = p->wd.check(cur_P(p, 1), p->nalloc, D.nt - 1 - it, it == 0, s);
            if (w == GEO_ERR_NAN) diverged = true;
            else GEO_TRY(w);
        }
        GEO_TRY(p->wd.verdict(s, "3D RTM backward pass"));
        if (D.sv) GEO_TRY(taper_box_3d(p, is, false, s));
        GEO_TRY(check_err(p, s));
        if (method == GEO_RTM_LEARNED) {
            GEO_TRY(ae_check_err(R.ae, s));
            std::vector<int> ne(std::max(nsnap, 1));
            GEO_CUDA(cudaMemcpy(ne.data(), nesc.p, ne.size() * 4, cudaMemcpyDeviceToHost));
            long long tot = 0;
            for (int j = 0; j < nsnap; j++) tot += std::min(ne[j], ecap);
            ae_note_run(R.ae, (long long)nsnap * (D.nx / 16 + (D.nx % 16 != 0)) * (D.ny / 16 + (D.ny % 16 != 0)) *
                                  (D.nz / 16 + (D.nz % 16 != 0)), tot);
        }
    }
    k_image_illum<<<grid_blocks(nimg), 256, 0, s>>>(mig.as<float>(), ill.as<float>(), nimg);
    GEO_TRY(check_launch("image_illum"));
    const cudaMemcpyKind kind = mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    GEO_CUDA(cudaMemcpyAsync(mig_out, mig.p, nimg * 4, kind, s));
    if (illum_out) GEO_CUDA(cudaMemcpyAsync(illum_out, ill.p, nimg * 4, kind, s));
    if (adcig_out) {
        k_adcig3d_illum<<<grid_blocks(nag), 256, 0, s>>>(ag.as<float>(), ill.as<float>(), D.nx, D.nz, na, dcdp, nxa,
                                                         nag);
        GEO_TRY(check_launch("adcig3d_illum"));
        GEO_CUDA(cudaMemcpyAsync(adcig_out, ag.p, nag * 4, kind, s));
    }
    if (lap_out) {
        GEO_TRY(lap.alloc(nimg * 4));
        GEO_TRY(launch_laplace3d(D.nx, D.ny, D.nz, mig.as<float>(), lap.as<float>(), s));
        GEO_CUDA(cudaMemcpyAsync(lap_out, lap.p, nimg * 4, kind, s));
    }
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}

extern "C" int geo_rtm3d(const geo_rtm3d_desc *desc, const float *v, const float *e, const float *d, float *mig_out,
                         float *lap_out, float *illum_out, int mem, void *stream) {
    return geo_rtm3d_adcig(desc, v, e, d, mig_out, lap_out, illum_out, nullptr, mem, stream);
}
