// 2D drivers: single-shot forward modelling and batched RTM.
//
// Both build per-shot Shot2D descriptors and step them with the batched
// kernels of fd2d.cu.  A batch time step is one persistent launch per phase
// (velocity, stress) covering every shot's tiles; the time loops are
// captured once into CUDA graphs and replayed.
#include "geo_internal.h"
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <tuple>

namespace geo {

static int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

// Host-side working set of one shot (window) plus its device buffers.
struct ShotHost {
    int nx, nz, npd, nnx, nnz;
    Variant var;
    std::vector<float> vp, e2, d2, cx1, cx2, cz1, cz2, ax1, ax2, az1, az2;
    std::vector<double> kz, kx;     // MPI exact form: the chains' double factors per point
    Taper2D taper;
    std::vector<float> te2, td2;
    std::vector<double> tkz, tkx;   // the same on the taper box
    int ixs, izs;
    float mu_v;
    DevBuf d_model, d_k, d_prof, d_taper, d_tk, d_fields, d_rec, d_edge, d_img, d_adcig;
};

// Build the propagation coefficients of one (padded) window from its
// unpadded model; Variant picks the reference program's formulas.
static void build_shot_host(ShotHost &h, Variant var, int nx, int nz, int npd, float dx, float dz, float dt,
                            const float *v, const float *e, const float *d, float srcx, float srcz, bool taper,
                            bool fast = false) {
    h.var = var;
    h.nx = nx; h.nz = nz; h.npd = npd;
    h.nnx = nx + 2 * npd; h.nnz = nz + 2 * npd;
    const size_t n = (size_t)h.nnx * h.nnz;
    std::vector<float> pv(n), pe(n), pd(n);
    pad_model_2d(nx, nz, npd, v, pv.data());
    pad_model_2d(nx, nz, npd, e, pe.data());
    pad_model_2d(nx, nz, npd, d, pd.data());
    float vpmax = v[0];
    for (size_t k = 0; k < (size_t)nx * nz; k++) vpmax = std::max(vpmax, v[k]);
    const float d0 = sponge_d0(var, 2, vpmax, pv[(size_t)h.nnx * h.nnz / 2], npd, dx, dx, dz);
    h.cx1.resize(h.nnx); h.cx2.resize(h.nnx); h.ax1.resize(h.nnx); h.ax2.resize(h.nnx);
    h.cz1.resize(h.nnz); h.cz2.resize(h.nnz); h.az1.resize(h.nnz); h.az2.resize(h.nnz);
    sponge_profiles(var, nx, npd, dt, d0, h.cx1.data(), h.cx2.data(), h.ax1.data(), h.ax2.data());
    sponge_profiles(var, nz, npd, dt, d0, h.cz1.data(), h.cz2.data(), h.az1.data(), h.az2.data());
    // source cell: (int)(fs+0.5)+npd-1 (CPU_vti2dfd_kernels.c:65-66)
    h.ixs = (int)(srcx + 0.5) + npd - 1;
    h.izs = (int)(srcz + 0.5) + npd - 1;
    h.vp.resize(n); h.e2.resize(n); h.d2.resize(n);
    // the MPI program's pz and qx chains are
    //   (double)(az2*pz) - (double)(az1*vp) * pow(1+2del,0.5) * (double)dtz * (double)zz
    // (and with ax, dtx, xx for qx), evaluated left to right; every factor but
    // zz is fixed for the shot, so the product of the first three is formed
    // here once, in the same order and precision, and the kernel issues one
    // double multiply and one double subtraction per chain
    const bool kchain = var == V_MPI && !fast;
    const double ddtx = (double)(dt / dx), ddtz = (double)(dt / dz);
    if (kchain) {
        h.kz.resize(n);
        h.kx.resize(n);
    }
    for (size_t k = 0; k < n; k++) {
        // MPI program: vp <- rho*vp^2 with rho == 1 (Toa_rtm_vti_adcig_cdp.c:641)
        h.vp[k] = (var == V_MPI) ? 1.0f * (pv[k] * pv[k]) : pv[k];
        h.e2[k] = 1 + 2 * pe[k];
        h.d2[k] = sqrtf(1 + 2 * pd[k]);
        if (kchain) {
            const double pw = std::pow((double)(1 + 2 * pd[k]), 0.5);
            const size_t ix = k / h.nnz, iz = k % h.nnz;
            h.kz[k] = (double)(h.az1[iz] * h.vp[k]) * pw * ddtz;
            h.kx[k] = (double)(h.ax1[ix] * h.vp[k]) * pw * ddtx;
        }
    }
    h.mu_v = pv[(size_t)(1 + npd) * h.nnz + 1 + npd] * sqrtf(1 + 2 * pe[(size_t)(1 + npd) * h.nnz + 1 + npd]);
    if (taper) {
        // CPU/MPI circle centre = the source cell; GPU form centre is
        // (fs+(is-1)ds+npd, zs+npd), one cell right/down of it
        const int cx = (var == V_GPU) ? h.ixs + 1 : h.ixs, cz = (var == V_GPU) ? h.izs + 1 : h.izs;
        sv_taper_2d(var, h.nnx, h.nnz, npd, cx, cz, pe.data(), pd.data(), h.taper);
        h.te2.assign(kTB * kTB, 1.0f); h.td2.assign(kTB * kTB, 1.0f);
        if (kchain) {
            h.tkz.assign(kTB * kTB, 0.0);
            h.tkx.assign(kTB * kTB, 0.0);
        }
        for (int k = 0; k < kTB * kTB; k++) {
            const float ee = h.taper.e[k], dd = h.taper.d[k];
            h.te2[k] = 1 + 2 * ee;
            h.td2[k] = sqrtf(1 + 2 * dd);
            const int ix = h.taper.x0 + k / kTB, iz = h.taper.z0 + k % kTB;
            if (kchain && ix >= 0 && ix < h.nnx && iz >= 0 && iz < h.nnz) {
                const double pw = std::pow((double)(1 + 2 * dd), 0.5);
                const float vpk = h.vp[(size_t)ix * h.nnz + iz];
                h.tkz[k] = (double)(h.az1[iz] * vpk) * pw * ddtz;
                h.tkx[k] = (double)(h.ax1[ix] * vpk) * pw * ddtx;
            }
        }
    }
}

// Upload one shot and fill its device descriptor.
static int upload_shot(ShotHost &h, Shot2D &S, int nfields, int nt, bool records, bool edges, bool image,
                       float dtx, float dtz, cudaStream_t s) {
    const size_t n = (size_t)h.nnx * h.nnz;
    GEO_TRY(h.d_model.alloc(3 * n * 4));
    float *m = h.d_model.as<float>();
    GEO_CUDA(cudaMemcpyAsync(m, h.vp.data(), n * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemcpyAsync(m + n, h.e2.data(), n * 4, cudaMemcpyHostToDevice, s));
    GEO_CUDA(cudaMemcpyAsync(m + 2 * n, h.d2.data(), n * 4, cudaMemcpyHostToDevice, s));
    if (!h.kz.empty()) {
        GEO_TRY(h.d_k.alloc(2 * n * 8));
        GEO_CUDA(cudaMemcpyAsync(h.d_k.p, h.kz.data(), n * 8, cudaMemcpyHostToDevice, s));
        GEO_CUDA(cudaMemcpyAsync(h.d_k.as<double>() + n, h.kx.data(), n * 8, cudaMemcpyHostToDevice, s));
    }
    const size_t np = 4 * (size_t)h.nnx + 4 * (size_t)h.nnz;
    GEO_TRY(h.d_prof.alloc(np * 4));
    float *pr = h.d_prof.as<float>();
    const std::vector<float> *prof[8] = {&h.cx1, &h.cx2, &h.ax1, &h.ax2, &h.cz1, &h.cz2, &h.az1, &h.az2};
    size_t o = 0;
    const float *dp[8];
    for (int k = 0; k < 8; k++) {
        GEO_CUDA(cudaMemcpyAsync(pr + o, prof[k]->data(), prof[k]->size() * 4, cudaMemcpyHostToDevice, s));
        dp[k] = pr + o;
        o += prof[k]->size();
    }
    memset(&S, 0, sizeof S);
    S.nnx = h.nnx; S.nnz = h.nnz; S.npd = h.npd; S.nx = h.nx; S.nz = h.nz;
    S.dtx = dtx; S.dtz = dtz;
    S.cx1 = dp[0]; S.cx2 = dp[1]; S.ax1 = dp[2]; S.ax2 = dp[3];
    S.cz1 = dp[4]; S.cz2 = dp[5]; S.az1 = dp[6]; S.az2 = dp[7];
    S.vp = m; S.e2 = m + n; S.d2 = m + 2 * n;
    S.kz = h.kz.empty() ? nullptr : h.d_k.as<double>();
    S.kx = h.kz.empty() ? nullptr : h.d_k.as<double>() + n;
    if (!h.te2.empty()) {
        GEO_TRY(h.d_taper.alloc(2 * kTB * kTB * 4));
        GEO_CUDA(cudaMemcpyAsync(h.d_taper.p, h.te2.data(), kTB * kTB * 4, cudaMemcpyHostToDevice, s));
        GEO_CUDA(cudaMemcpyAsync(h.d_taper.as<float>() + kTB * kTB, h.td2.data(), kTB * kTB * 4, cudaMemcpyHostToDevice, s));
        if (!h.tkz.empty()) {
            GEO_TRY(h.d_tk.alloc(2 * kTB * kTB * 8));
            GEO_CUDA(cudaMemcpyAsync(h.d_tk.p, h.tkz.data(), kTB * kTB * 8, cudaMemcpyHostToDevice, s));
            GEO_CUDA(cudaMemcpyAsync(h.d_tk.as<double>() + kTB * kTB, h.tkx.data(), kTB * kTB * 8,
                                     cudaMemcpyHostToDevice, s));
        }
        S.tx0 = h.taper.x0; S.tz0 = h.taper.z0;
        S.te2 = h.d_taper.as<float>(); S.td2 = h.d_taper.as<float>() + kTB * kTB;
        S.tkz = h.tkz.empty() ? nullptr : h.d_tk.as<double>();
        S.tkx = h.tkz.empty() ? nullptr : h.d_tk.as<double>() + kTB * kTB;
    } else {
        S.tx0 = -100000; S.tz0 = -100000;
    }
    S.ixs = h.ixs; S.izs = h.izs;
    GEO_TRY(h.d_fields.alloc((size_t)8 * nfields * n * 4));
    GEO_TRY(h.d_fields.zero(s));
    float *f = h.d_fields.as<float>();
    for (int k = 0; k < nfields; k++) {
        float *b = f + (size_t)8 * k * n;
        S.u[k] = b; S.w[k] = b + n; S.P[k] = b + 2 * n; S.Q[k] = b + 3 * n;
        S.px[k] = b + 4 * n; S.pz[k] = b + 5 * n; S.qx[k] = b + 6 * n; S.qz[k] = b + 7 * n;
    }
    S.rec_iz = h.npd;
    S.rec_scale = 1.0f;
    if (records) {
        GEO_TRY(h.d_rec.alloc((size_t)2 * nt * h.nx * 4));
        GEO_TRY(h.d_rec.zero(s));
        S.rec_p = h.d_rec.as<float>();
        S.rec_q = S.rec_p + (size_t)nt * h.nx;
    }
    if (edges) {
        const size_t L = 2 * (size_t)h.nx + 2 * (size_t)h.nz;
        GEO_TRY(h.d_edge.alloc((size_t)2 * nt * L * 4));
        S.edge_p = h.d_edge.as<float>();
        S.edge_q = S.edge_p + (size_t)nt * L;
    }
    if (image) {
        GEO_TRY(h.d_img.alloc((size_t)2 * h.nx * h.nz * 4));
        GEO_TRY(h.d_img.zero(s));
        S.mig = h.d_img.as<float>();
        S.ill = S.mig + (size_t)h.nx * h.nz;
    }
    return GEO_OK;
}

// Work list: item -> shot.  Tiles are 32 (z) x by (x).
static void build_items(std::vector<Shot2D> &S, int by, std::vector<int> &item_shot) {
    item_shot.clear();
    for (size_t k = 0; k < S.size(); k++) {
        S[k].ntz = (S[k].nnz + 31) / 32;
        const int ntx = (S[k].nnx + by - 1) / by;
        S[k].tile_base = (int)item_shot.size();
        item_shot.insert(item_shot.end(), (size_t)S[k].ntz * ntx, (int)k);
    }
}

struct Batch2D {
    std::vector<Shot2D> S;
    std::vector<int> items;
    DevBuf d_S, d_items;
    int by = 8, grid = 1, variant = V_CPU;
    int upload(int by_, int blocks_per_sm, cudaStream_t s) {
        by = by_;
        build_items(S, by, items);
        const int nitems = (int)items.size();
        grid = std::max(1, std::min(nitems, sm_count() * blocks_per_sm));
        GEO_TRY(d_S.alloc(S.size() * sizeof(Shot2D)));
        GEO_TRY(d_items.alloc(items.size() * 4));
        GEO_CUDA(cudaMemcpyAsync(d_S.p, S.data(), S.size() * sizeof(Shot2D), cudaMemcpyHostToDevice, s));
        GEO_CUDA(cudaMemcpyAsync(d_items.p, items.data(), items.size() * 4, cudaMemcpyHostToDevice, s));
        GEO_CUDA(cudaStreamSynchronize(s));
        return GEO_OK;
    }
    int vel(Step2D st, cudaStream_t s) {
        return launch_vel2d(variant, d_S.as<Shot2D>(), d_items.as<int>(), (int)items.size(), by, grid, st, s);
    }
    int stress(int phase, Step2D st, cudaStream_t s) {
        return launch_stress2d(variant, phase, d_S.as<Shot2D>(), d_items.as<int>(), (int)items.size(), by, grid, st, s);
    }

    // Skewed schedule (MPI form, two or more shots): the shots are split
    // into groups A = [0, split) and B = [split, ns) of about equal tiles,
    // B half a step behind A, so that every launch pairs one group's stress
    // tiles with the other's velocity tiles (launch_mix2d).  Every shot
    // still runs velocity then stress of each step in order.  Tables, as
    // (shot | kind << 30, tile) items with the kinds interleaved:
    //   VA: velocity of A;  MX: stress of A + velocity of B;
    //   MY: velocity of A + stress of B;  SB: stress of B.
    enum { VA = 0, MX = 1, MY = 2, SB = 3 };
    DevBuf d_mix;
    int split = 0, mix_n[4] = {0, 0, 0, 0};
    size_t mix_o[4] = {0, 0, 0, 0};
    int build_mix(cudaStream_t s) {
        const int ns = (int)S.size();
        std::vector<long> tiles(ns);
        long total = 0;
        for (int k = 0; k < ns; k++) {
            tiles[k] = (long)S[k].ntz * ((S[k].nnx + by - 1) / by);
            total += tiles[k];
        }
        long acc = 0;
        split = 1;
        for (int k = 0; k < ns - 1; k++) {
            acc += tiles[k];
            split = k + 1;
            if (2 * acc >= total) break;
        }
        auto list = [&](int k0, int k1, int kind) {
            std::vector<int2> v;
            for (int k = k0; k < k1; k++)
                for (long t = 0; t < tiles[k]; t++) v.push_back(make_int2(k | (kind << 30), (int)t));
            return v;
        };
        auto merge = [](const std::vector<int2> &a, const std::vector<int2> &b) {
            std::vector<int2> v;
            v.reserve(a.size() + b.size());
            size_t i = 0, j = 0;
            while (i < a.size() || j < b.size()) {
                if (j >= b.size() || (i < a.size() && i * b.size() <= j * a.size())) v.push_back(a[i++]);
                else v.push_back(b[j++]);
            }
            return v;
        };
        const std::vector<int2> vA = list(0, split, 0), sA = list(0, split, 1), vB = list(split, ns, 0),
                                sB = list(split, ns, 1);
        const std::vector<int2> tab[4] = {vA, merge(sA, vB), merge(vA, sB), sB};
        size_t off = 0;
        for (int t = 0; t < 4; t++) {
            mix_o[t] = off;
            mix_n[t] = (int)tab[t].size();
            off += tab[t].size();
        }
        GEO_TRY(d_mix.alloc(off * sizeof(int2)));
        for (int t = 0; t < 4; t++)
            GEO_CUDA(cudaMemcpyAsync(d_mix.as<int2>() + mix_o[t], tab[t].data(), tab[t].size() * sizeof(int2),
                                     cudaMemcpyHostToDevice, s));
        GEO_CUDA(cudaStreamSynchronize(s));
        return GEO_OK;
    }
    int mix(int table, int phase, int fast, Step2D sv, Step2D ss, cudaStream_t s) {
        return launch_mix2d(phase, fast, d_S.as<Shot2D>(), d_mix.as<int2>() + mix_o[table], mix_n[table], by, grid,
                            sv, ss, s);
    }
};

// Graph of a range of steps; capture on a private stream.
struct Graph {
    cudaGraph_t g = nullptr;
    cudaGraphExec_t x = nullptr;
    long long kernels = 0;     // kernel nodes, counted once per replay
    int launch(cudaStream_t s) {
        GEO_CUDA(cudaGraphLaunch(x, s));
        count_launch(kernels);
        return GEO_OK;
    }
    ~Graph() {
        if (x) cudaGraphExecDestroy(x);
        if (g) cudaGraphDestroy(g);
    }
};

template <class F>
static int capture(Graph &G, cudaStream_t cs, F &&body) {
    GEO_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    const long long before = launches_so_far();
    int st = body();
    G.kernels = launches_so_far() - before;
    count_launch(-G.kernels);   // captured, not yet run
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(cs, &g);
    if (st != GEO_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return fail(GEO_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    G.g = g;
    GEO_CUDA(cudaGraphInstantiate(&G.x, g, 0));
    return GEO_OK;
}

// Autotuner: time a few forward steps for each (rows per tile, blocks per
// SM) candidate on the real batch and keep the fastest.  Results are cached
// per (grid extents, shot count, device) for the life of the process.
static std::map<std::tuple<int, int, int, int>, std::pair<int, int>> g_tune_cache;

static int autotune(Batch2D &B, int nf, int key_nx, int key_nz, cudaStream_t s, int *by_out, int *bps_out) {
    int dev = 0;
    cudaGetDevice(&dev);
    auto key = std::make_tuple(key_nx, key_nz, (int)B.S.size() * 16 + nf, dev);
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
        *by_out = it->second.first;
        *bps_out = it->second.second;
        return GEO_OK;
    }
    const int bys[] = {4, 8};
    const int bpss[] = {4, 8, 16};
    float best = 1e30f;
    int bb = 8, bp = 8;
    cudaEvent_t a, b;
    GEO_CUDA(cudaEventCreate(&a));
    GEO_CUDA(cudaEventCreate(&b));
    Step2D st{};
    st.nf = nf;
    for (int by : bys)
        for (int bps : bpss) {
            GEO_TRY(B.upload(by, bps, s));
            GEO_TRY(B.vel(st, s));
            GEO_TRY(B.stress(PH_BWD, st, s));
            GEO_CUDA(cudaEventRecord(a, s));
            for (int k = 0; k < 4; k++) {
                GEO_TRY(B.vel(st, s));
                GEO_TRY(B.stress(PH_BWD, st, s));
            }
            GEO_CUDA(cudaEventRecord(b, s));
            GEO_CUDA(cudaEventSynchronize(b));
            float ms = 0;
            GEO_CUDA(cudaEventElapsedTime(&ms, a, b));
            if (ms < best) {
                best = ms;
                bb = by;
                bp = bps;
            }
        }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    g_tune_cache[key] = {bb, bp};
    *by_out = bb;
    *bps_out = bp;
    return GEO_OK;
}

static int host_model(const float *v, const float *e, const float *d, size_t n, int mem, cudaStream_t s,
                      std::vector<float> &hv, std::vector<float> &he, std::vector<float> &hd) {
    hv.resize(n); he.resize(n); hd.resize(n);
    const cudaMemcpyKind k = mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost;
    if (mem != GEO_MEM_DEVICE && mem != GEO_MEM_HOST) return fail(GEO_ERR_ARG, "bad mem kind");
    GEO_CUDA(cudaMemcpyAsync(hv.data(), v, n * 4, k, s));
    GEO_CUDA(cudaMemcpyAsync(he.data(), e, n * 4, k, s));
    GEO_CUDA(cudaMemcpyAsync(hd.data(), d, n * 4, k, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    return check_model(hv.data(), he.data(), hd.data(), n);
}

// Event-ordered hand-off between the caller's stream and a private one.
struct SideStream {
    cudaStream_t cs = nullptr;
    cudaEvent_t ev = nullptr;
    int open(cudaStream_t user) {
        GEO_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        GEO_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        GEO_CUDA(cudaEventRecord(ev, user));
        GEO_CUDA(cudaStreamWaitEvent(cs, ev, 0));
        return GEO_OK;
    }
    ~SideStream() {
        if (cs) {
            cudaStreamSynchronize(cs);
            cudaStreamDestroy(cs);
        }
        if (ev) cudaEventDestroy(ev);
    }
};

}  // namespace geo

using namespace geo;

// ---------------------------------------------------------------- FD 2D
extern "C" int geo_fd2d_shot(const geo_fd2d_desc *desc, const float *v, const float *e, const float *d,
                             float *shot, float *snap, int snap_every, int mem, void *stream) {
    if (!desc || !v || !e || !d || !shot) return fail(GEO_ERR_ARG, "null argument");
    const geo_fd2d_desc &D = *desc;
    if (D.nx < 2 || D.nz < 2 || D.npd < 5 || D.nt < 1) return fail(GEO_ERR_ARG, "grid too small (npd >= 5)");
    if (D.variant < GEO_VARIANT_CPU || D.variant > GEO_VARIANT_MPI) return fail(GEO_ERR_ARG, "bad variant");
    if (!(D.dt > 0) || !(D.dx > 0) || !(D.dz > 0) || !(D.favg > 0)) return fail(GEO_ERR_ARG, "bad spacing");
    const int nnx = D.nx + 2 * D.npd, nnz = D.nz + 2 * D.npd;
    if (D.rec_iz < 4 || D.rec_iz >= nnz - 4) return fail(GEO_ERR_ARG, "receiver row outside grid");
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<float> hv, he, hd;
    GEO_TRY(host_model(v, e, d, (size_t)D.nx * D.nz, mem, s, hv, he, hd));
    const Variant var = (Variant)D.variant;
    {
        const auto mm = std::minmax_element(hv.begin(), hv.end());
        GEO_TRY(check_stability(var, 2, *mm.first, *mm.second, D.dt, D.dx, D.dx, D.dz, D.favg));
    }
    const float fsx = D.fs + (D.is - 1) * D.ds;
    ShotHost h;
    const bool taper = var == V_MPI || D.sv;
    build_shot_host(h, var, D.nx, D.nz, D.npd, D.dx, D.dz, D.dt, hv.data(), he.data(), hd.data(), fsx, D.zs, taper);
    if (h.ixs < 4 || h.ixs >= nnx - 4 || h.izs < 4 || h.izs >= nnz - 4)
        return fail(GEO_ERR_ARG, "source outside the updated grid");
    if (var == V_CPU || var == V_MPI)
        if (h.ixs - 3 < 0 || h.ixs + 3 >= nnx || h.izs - 3 < 0 || h.izs + 3 >= nnz)
            return fail(GEO_ERR_ARG, "source window outside grid");
    SideStream ss;
    GEO_TRY(ss.open(s));
    Batch2D B;
    B.variant = var;
    B.S.resize(1);
    GEO_TRY(upload_shot(h, B.S[0], 1, D.nt, true, false, false, D.dt / D.dx, D.dt / D.dz, ss.cs));
    B.S[0].rec_iz = D.rec_iz;
    B.S[0].rec_scale = D.rec_scale;
    B.S[0].rec_q = nullptr;
    const bool persistent = !(snap && snap_every > 0);
    GEO_TRY(B.upload(persistent ? 16 : 8, 8, ss.cs));
    std::vector<float> amp;
    std::vector<uint8_t> on;
    source_amplitudes(var, D.nt, D.dt, D.favg, D.pfac, D.wtype, amp, on);
    auto step = [&](int it) -> int {
        Step2D st{};
        st.it = it;
        st.amp = amp[it];
        st.src_on = on[it];
        st.taper = taper ? 1 : 0;
        st.nf = 1;
        GEO_TRY(B.vel(st, ss.cs));
        return B.stress(PH_FWD, st, ss.cs);
    };
    const size_t nn = (size_t)nnx * nnz;
    Watchdog wd;
    GEO_TRY(wd.open());
    const cudaMemcpyKind ksnap = mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    // CPU and GPU forms: every block keeps its tile of the fields in shared
    // memory for the run (launch_fd2d_tile), one launch per run of steps
    // between snapshots, when the grid fits on the device that way
    bool tiled = false;
    if (var == V_CPU || var == V_GPU) {
        DevBuf xch, d_amp, d_on, d_sync;
        GEO_TRY(xch.alloc(8 * nn * 4));
        GEO_TRY(xch.zero(ss.cs));
        GEO_TRY(d_amp.alloc((size_t)D.nt * 4));
        GEO_TRY(d_on.alloc((size_t)D.nt));
        GEO_TRY(d_sync.alloc(8));
        GEO_TRY(d_sync.zero(ss.cs));
        GEO_CUDA(cudaMemcpyAsync(d_amp.p, amp.data(), (size_t)D.nt * 4, cudaMemcpyHostToDevice, ss.cs));
        GEO_CUDA(cudaMemcpyAsync(d_on.p, on.data(), (size_t)D.nt, cudaMemcpyHostToDevice, ss.cs));
        unsigned *bar = d_sync.as<unsigned>();
        int *errw = d_sync.as<int>() + 1;
        for (int it0 = 0; it0 < D.nt;) {
            int it1 = it0 + 1;
            if (snap && snap_every > 0)
                while (it1 < D.nt && (it1 - 1) % snap_every != 0) it1++;
            else
                it1 = D.nt;
            bool fits = false;
            GEO_TRY(launch_fd2d_tile(var, B.S[0], xch.as<float>(), d_amp.as<float>(), d_on.as<unsigned char>(),
                                     taper ? 1 : 0, it0, it1, bar, errw, &fits, ss.cs));
            if (!fits) {   // decided by the grid alone, so on the first run of steps
                if (tiled) return fail(GEO_ERR_CUDA, "2D shot: tile-resident launch refused mid-run");
                break;
            }
            tiled = true;
            const int it = it1 - 1;
            if (snap && snap_every > 0 && it % snap_every == 0)
                GEO_CUDA(cudaMemcpyAsync(snap + (size_t)(it / snap_every) * nn, B.S[0].P[0], nn * 4, ksnap, ss.cs));
            if (wd.every > 0) {
                GEO_TRY(launch_watch_shots(B.d_S.as<Shot2D>(), 1, 1, wd.d, it + 1, ss.cs));
                if (wd.tripped()) break;
            }
            it0 = it1;
        }
        if (tiled) {
            int err = 0;
            GEO_CUDA(cudaMemcpyAsync(&err, errw, 4, cudaMemcpyDeviceToHost, ss.cs));
            GEO_CUDA(cudaStreamSynchronize(ss.cs));
            if (err) return fail(GEO_ERR_CUDA, "2D shot: a grid barrier wait timed out");
            if (wd.every > 0) GEO_TRY(wd.scan(B.S[0].rec_p, (size_t)D.nx * D.nt, D.nt, ss.cs));
        }
    }
    if (!tiled && snap && snap_every > 0) {
        for (int it = 0; it < D.nt; it++) {
            GEO_TRY(step(it));
            if (it % snap_every == 0)
                GEO_CUDA(cudaMemcpyAsync(snap + (size_t)(it / snap_every) * nn, B.S[0].P[0], nn * 4, ksnap, ss.cs));
            if (wd.every > 0 && ((it + 1) % wd.every == 0 || it == D.nt - 1)) {
                GEO_TRY(launch_watch_shots(B.d_S.as<Shot2D>(), 1, 1, wd.d, it + 1, ss.cs));
                if (wd.tripped()) break;
            }
        }
    } else if (!tiled) {
        // the whole shot in one cooperative launch (grid barriers between the
        // half-steps, bounded waits reported through an error word)
        DevBuf d_amp, d_on, d_sync;
        GEO_TRY(d_amp.alloc((size_t)D.nt * 4));
        GEO_TRY(d_on.alloc((size_t)D.nt));
        GEO_TRY(d_sync.alloc(8));
        GEO_TRY(d_sync.zero(ss.cs));
        GEO_CUDA(cudaMemcpyAsync(d_amp.p, amp.data(), (size_t)D.nt * 4, cudaMemcpyHostToDevice, ss.cs));
        GEO_CUDA(cudaMemcpyAsync(d_on.p, on.data(), (size_t)D.nt, cudaMemcpyHostToDevice, ss.cs));
        Persist2D a{};
        a.nt = D.nt;
        a.taper = taper ? 1 : 0;
        a.amp = d_amp.as<float>();
        a.on = d_on.as<unsigned char>();
        a.bar = d_sync.as<unsigned>();
        a.err = d_sync.as<int>() + 1;
        GEO_TRY(launch_fd2d_shot(var, B.d_S.as<Shot2D>(), B.d_items.as<int>(), (int)B.items.size(), B.by, a, ss.cs));
        int err = 0;
        GEO_CUDA(cudaMemcpyAsync(&err, a.err, 4, cudaMemcpyDeviceToHost, ss.cs));
        GEO_CUDA(cudaStreamSynchronize(ss.cs));
        if (err) return fail(GEO_ERR_CUDA, "2D shot: a grid barrier wait timed out");
        // the shot ran in one launch: scan its final P and its record
        if (wd.every > 0) {
            GEO_TRY(launch_watch_shots(B.d_S.as<Shot2D>(), 1, 1, wd.d, D.nt, ss.cs));
            GEO_TRY(wd.scan(B.S[0].rec_p, (size_t)D.nx * D.nt, D.nt, ss.cs));
        }
    }
    GEO_TRY(wd.verdict(ss.cs, "2D shot"));
    DevBuf mlo, mhi, out;
    if (D.mute_tt > 0) {
        std::vector<int> lo, hi;
        // vp[1]*sqrtf(1+2*eps[1]) of the padded model (GPU_vti2dfd_kernels.cu:167)
        {
            std::vector<float> pv((size_t)nnx * nnz), pe((size_t)nnx * nnz);
            pad_model_2d(D.nx, D.nz, D.npd, hv.data(), pv.data());
            pad_model_2d(D.nx, D.nz, D.npd, he.data(), pe.data());
            const float mu_v = pv[1] * sqrtf(1 + 2 * pe[1]);
            mute_window_gpu2d(D.nx, D.nt, D.dt, D.favg, D.dx, D.dz, (int)D.fs, (int)D.ds, (int)D.zs, D.is, mu_v,
                              D.mute_tt, lo, hi);
        }
        GEO_TRY(mlo.alloc(lo.size() * 4));
        GEO_TRY(mhi.alloc(hi.size() * 4));
        GEO_CUDA(cudaMemcpyAsync(mlo.p, lo.data(), lo.size() * 4, cudaMemcpyHostToDevice, ss.cs));
        GEO_CUDA(cudaMemcpyAsync(mhi.p, hi.data(), hi.size() * 4, cudaMemcpyHostToDevice, ss.cs));
        GEO_TRY(launch_mute_records(B.S[0].rec_p, D.nx, D.nt, mlo.as<int>(), mhi.as<int>(), ss.cs));
    }
    const size_t rbytes = (size_t)D.nx * D.nt * 4;
    if (mem == GEO_MEM_DEVICE) {
        GEO_TRY(launch_transpose_records(B.S[0].rec_p, shot, D.nx, D.nt, ss.cs));
    } else {
        GEO_TRY(out.alloc(rbytes));
        GEO_TRY(launch_transpose_records(B.S[0].rec_p, out.as<float>(), D.nx, D.nt, ss.cs));
        GEO_CUDA(cudaMemcpyAsync(shot, out.p, rbytes, cudaMemcpyDeviceToHost, ss.cs));
    }
    GEO_CUDA(cudaStreamSynchronize(ss.cs));
    return GEO_OK;
}

// ---------------------------------------------------------------- RTM 2D
extern "C" int geo_rtm2d_batch(const geo_rtm2d_desc *desc, const float *v, const float *e, const float *d,
                               float *image, float *per_shot, int mem, void *stream) {
    return geo_rtm2d_batch_adcig(desc, v, e, d, image, per_shot, nullptr, mem, stream);
}

extern "C" int geo_rtm2d_batch_adcig(const geo_rtm2d_desc *desc, const float *v, const float *e, const float *d,
                                     float *image, float *per_shot, float *adcig, int mem, void *stream) {
    if (!desc || !v || !e || !d || !image || !desc->shot_x || !desc->shot_nxs) return fail(GEO_ERR_ARG, "null argument");
    const geo_rtm2d_desc &D = *desc;
    if (D.nx < 2 || D.nz < 2 || D.npd < 5 || D.nt < 1 || D.ns < 1) return fail(GEO_ERR_ARG, "bad sizes");
    if (!(D.dt_ms > 0) || !(D.dx > 0) || !(D.dz > 0) || !(D.favg > 0)) return fail(GEO_ERR_ARG, "bad spacing");
    for (int k = 0; k < D.ns; k++) {
        const int nxs = D.shot_nxs[k], kk = D.shot_x[k];
        if (nxs < 3 || nxs % 2 == 0) return fail(GEO_ERR_ARG, "shot %d: window width must be odd and >= 3", k);
        // the reference exits when a window leaves the model (Toa_rtm_vti_adcig_cdp.c:283-292)
        if (kk < nxs / 2 + 1 || kk + nxs / 2 > D.nx) return fail(GEO_ERR_WINDOW, "shot %d window leaves model", k);
    }
    if (D.zs < 1 || D.zs + D.npd - 1 + 3 >= D.nz + 2 * D.npd) return fail(GEO_ERR_ARG, "bad source depth");
    if (D.mode != GEO_MODE_EXACT && D.mode != GEO_MODE_FAST) return fail(GEO_ERR_ARG, "bad mode %d", D.mode);
    const int fast = D.mode == GEO_MODE_FAST;
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<float> hv, he, hd;
    GEO_TRY(host_model(v, e, d, (size_t)D.nx * D.nz, mem, s, hv, he, hd));
    SideStream ss;
    GEO_TRY(ss.open(s));
    const float dt = D.dt_ms / 1000;
    const int nt = D.nt, nz = D.nz, npd = D.npd;
    {
        const auto mm = std::minmax_element(hv.begin(), hv.end());
        GEO_TRY(check_stability(V_MPI, 2, *mm.first, *mm.second, dt, D.dx, D.dx, D.dz, D.favg));
    }
    std::vector<std::unique_ptr<ShotHost>> H(D.ns);
    Batch2D B;
    B.variant = V_MPI;
    B.S.resize(D.ns);
    int maxline = 0;
    for (int k = 0; k < D.ns; k++) {
        const int nxs = D.shot_nxs[k], kk = D.shot_x[k];
        // window column c <- model column c + k - nxs/2, clamped into the pad
        std::vector<float> wv((size_t)nxs * nz), we((size_t)nxs * nz), wd((size_t)nxs * nz);
        for (int c = 0; c < nxs; c++) {
            int col = c + kk - nxs / 2;
            col = std::min(col, D.nx - 1);
            memcpy(&wv[(size_t)c * nz], &hv[(size_t)col * nz], nz * 4);
            memcpy(&we[(size_t)c * nz], &he[(size_t)col * nz], nz * 4);
            memcpy(&wd[(size_t)c * nz], &hd[(size_t)col * nz], nz * 4);
        }
        H[k].reset(new ShotHost());
        // shot position inside its window: fs = nxs/2+1, ds = 0
        build_shot_host(*H[k], V_MPI, nxs, nz, npd, D.dx, D.dz, dt, wv.data(), we.data(), wd.data(),
                        (float)(nxs / 2 + 1), (float)D.zs, true, fast != 0);
        GEO_TRY(upload_shot(*H[k], B.S[k], 2, nt, true, true, true, dt / D.dx, dt / D.dz, ss.cs));
        if (adcig) {
            GEO_TRY(H[k]->d_adcig.alloc((size_t)kAdcigAngles * nxs * nz * 4));
            B.S[k].adcig = H[k]->d_adcig.as<float>();
        }
        maxline = std::max(maxline, 2 * nxs + 2 * nz);
    }
    // tile shape: caller's choice or the autotuner's
    int by = D.tile_x, bps = 8;
    if (by != 4 && by != 8) GEO_TRY(autotune(B, 2, D.nx, D.nz, ss.cs, &by, &bps));
    GEO_TRY(B.upload(by, bps, ss.cs));
    // the autotuner stepped the state: start from zero again
    for (int k = 0; k < D.ns; k++) {
        GEO_TRY(H[k]->d_fields.zero(ss.cs));
        GEO_TRY(H[k]->d_img.zero(ss.cs));
        if (adcig) GEO_TRY(H[k]->d_adcig.zero(ss.cs));
    }
    if (adcig) GEO_TRY(load_adcig_tables(ss.cs));

    std::vector<float> amp;
    std::vector<uint8_t> on;
    source_amplitudes(V_MPI, nt, dt, D.favg, D.pfac, 1, amp, on);
    // non-finite detector: every wd.every steps (and the last) the graphs
    // scan every shot's P; the verdict follows each pass
    Watchdog wd;
    GEO_TRY(wd.open());
    auto watch = [&](int k, bool last, int nf) -> int {
        if (wd.every <= 0 || ((k + 1) % wd.every && !last)) return GEO_OK;
        return launch_watch_shots(B.d_S.as<Shot2D>(), D.ns, nf, wd.d, k + 1, ss.cs);
    };
    // forward: source side only, with records and edge lines; with two or
    // more shots on the skewed schedule (Batch2D::build_mix)
    const bool skew = D.ns >= 2;
    if (skew) GEO_TRY(B.build_mix(ss.cs));
    auto fwd_st = [&](int it) {
        Step2D st{};
        st.it = it; st.amp = amp[it]; st.src_on = on[it]; st.taper = 1; st.nf = 1; st.fast = fast;
        return st;
    };
    {
        Graph G;
        GEO_TRY(capture(G, ss.cs, [&]() -> int {
            if (skew) {
                GEO_TRY(B.mix(Batch2D::VA, PH_FWD, fast, fwd_st(0), fwd_st(0), ss.cs));
                for (int it = 0; it < nt; it++) {
                    GEO_TRY(B.mix(Batch2D::MX, PH_FWD, fast, fwd_st(it), fwd_st(it), ss.cs));
                    if (it + 1 < nt) GEO_TRY(B.mix(Batch2D::MY, PH_FWD, fast, fwd_st(it + 1), fwd_st(it), ss.cs));
                    else GEO_TRY(B.mix(Batch2D::SB, PH_FWD, fast, fwd_st(it), fwd_st(it), ss.cs));
                    GEO_TRY(watch(it, it == nt - 1, 1));
                }
                return GEO_OK;
            }
            for (int it = 0; it < nt; it++) {
                const Step2D st = fwd_st(it);
                GEO_TRY(B.vel(st, ss.cs));
                GEO_TRY(B.stress(PH_FWD, st, ss.cs));
                GEO_TRY(watch(it, it == nt - 1, 1));
            }
            return GEO_OK;
        }));
        GEO_TRY(G.launch(ss.cs));
    }
    GEO_TRY(wd.verdict(ss.cs, "batched 2D RTM forward pass"));
    // mute both records (tt = 285) and restart the source side from zero
    std::vector<DevBuf> mute(D.ns);
    for (int k = 0; k < D.ns; k++) {
        const int nxs = D.shot_nxs[k];
        std::vector<int> lo, hi;
        mute_window_mpi(nxs, nt, D.dt_ms, D.favg, D.dx, D.dz, nxs / 2 + 1, 0, D.zs, k + 1, H[k]->mu_v, 285, lo, hi);
        GEO_TRY(mute[k].alloc(hi.size() * 4));
        GEO_CUDA(cudaMemcpyAsync(mute[k].p, hi.data(), hi.size() * 4, cudaMemcpyHostToDevice, ss.cs));
        GEO_TRY(launch_mute_records(B.S[k].rec_p, nxs, nt, nullptr, mute[k].as<int>(), ss.cs));
        GEO_TRY(launch_mute_records(B.S[k].rec_q, nxs, nt, nullptr, mute[k].as<int>(), ss.cs));
        const size_t n = (size_t)H[k]->nnx * H[k]->nnz;
        GEO_CUDA(cudaMemsetAsync(B.S[k].u[0], 0, 8 * n * 4, ss.cs));
    }
    // backward: inject, both propagations, fused imaging
    {
        Graph G;
        auto bwd_st = [&](int it) {
            Step2D st{};
            st.it = it; st.nf = 2; st.fast = fast;
            return st;
        };
        const Shot2D *dA = B.d_S.as<Shot2D>(), *dB = dA + B.split;
        const int nA = B.split, nB = D.ns - B.split;
        GEO_TRY(capture(G, ss.cs, [&]() -> int {
            if (skew) {
                GEO_TRY(launch_inject2d(dA, nA, maxline, nt - 1, ss.cs));
                GEO_TRY(B.mix(Batch2D::VA, PH_BWD, fast, bwd_st(nt - 1), bwd_st(nt - 1), ss.cs));
                for (int it = nt - 1; it >= 0; it--) {
                    GEO_TRY(launch_inject2d(dB, nB, maxline, it, ss.cs));
                    GEO_TRY(B.mix(Batch2D::MX, PH_BWD, fast, bwd_st(it), bwd_st(it), ss.cs));
                    if (it > 0) {
                        GEO_TRY(launch_inject2d(dA, nA, maxline, it - 1, ss.cs));
                        GEO_TRY(B.mix(Batch2D::MY, PH_BWD, fast, bwd_st(it - 1), bwd_st(it), ss.cs));
                    } else {
                        GEO_TRY(B.mix(Batch2D::SB, PH_BWD, fast, bwd_st(it), bwd_st(it), ss.cs));
                    }
                    GEO_TRY(watch(nt - 1 - it, it == 0, 2));
                }
                return GEO_OK;
            }
            for (int it = nt - 1; it >= 0; it--) {
                GEO_TRY(launch_inject2d(B.d_S.as<Shot2D>(), D.ns, maxline, it, ss.cs));
                const Step2D st = bwd_st(it);
                GEO_TRY(B.vel(st, ss.cs));
                GEO_TRY(B.stress(PH_BWD, st, ss.cs));
                GEO_TRY(watch(nt - 1 - it, it == 0, 2));
            }
            return GEO_OK;
        }));
        GEO_TRY(G.launch(ss.cs));
    }
    GEO_TRY(wd.verdict(ss.cs, "batched 2D RTM backward pass"));
    // normalise per shot, stack in shot order, Laplacian
    std::vector<const float *> imgs(D.ns);
    std::vector<int> offs(D.ns), wid(D.ns);
    for (int k = 0; k < D.ns; k++) {
        GEO_TRY(launch_normalize_image(B.S[k].mig, B.S[k].ill, (size_t)D.shot_nxs[k] * nz, ss.cs));
        imgs[k] = B.S[k].mig;
        offs[k] = D.shot_x[k] - D.shot_nxs[k] / 2 - 1;
        wid[k] = D.shot_nxs[k];
    }
    DevBuf d_imgs, d_offs, d_wid, stack, lap;
    GEO_TRY(d_imgs.alloc(D.ns * sizeof(float *)));
    GEO_TRY(d_offs.alloc(D.ns * 4));
    GEO_TRY(d_wid.alloc(D.ns * 4));
    GEO_CUDA(cudaMemcpyAsync(d_imgs.p, imgs.data(), D.ns * sizeof(float *), cudaMemcpyHostToDevice, ss.cs));
    GEO_CUDA(cudaMemcpyAsync(d_offs.p, offs.data(), D.ns * 4, cudaMemcpyHostToDevice, ss.cs));
    GEO_CUDA(cudaMemcpyAsync(d_wid.p, wid.data(), D.ns * 4, cudaMemcpyHostToDevice, ss.cs));
    const size_t nimg = (size_t)D.nx * nz;
    GEO_TRY(stack.alloc(nimg * 4));
    GEO_TRY(stack.zero(ss.cs));
    GEO_TRY(launch_stack_image(stack.as<float>(), nz, d_imgs.as<const float *const>(), d_offs.as<int>(),
                               d_wid.as<int>(), D.ns, D.nx, ss.cs));
    const float *result = stack.as<float>();
    if (D.laplace) {
        GEO_TRY(lap.alloc(nimg * 4));
        GEO_TRY(launch_laplace2d(D.nx, nz, stack.as<float>(), lap.as<float>(), ss.cs));
        result = lap.as<float>();
    }
    const cudaMemcpyKind k = mem == GEO_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    GEO_CUDA(cudaMemcpyAsync(image, result, nimg * 4, k, ss.cs));
    DevBuf gathers, d_aptr;
    if (adcig) {
        // per shot: divide by the source illumination (Toa_rtm_vti_adcig_cdp.c:1083-1090), then stack
        // every angle plane in shot order into [90][nx][nz] (adcig_ns0)
        std::vector<const float *> ap((size_t)kAdcigAngles * D.ns);
        for (int q = 0; q < D.ns; q++) {
            const size_t m = (size_t)D.shot_nxs[q] * nz;
            GEO_TRY(launch_normalize_planes(B.S[q].adcig, B.S[q].ill, m, kAdcigAngles, ss.cs));
            for (int ia = 0; ia < kAdcigAngles; ia++) ap[(size_t)ia * D.ns + q] = B.S[q].adcig + ia * m;
        }
        GEO_TRY(d_aptr.alloc(ap.size() * sizeof(float *)));
        GEO_CUDA(cudaMemcpyAsync(d_aptr.p, ap.data(), ap.size() * sizeof(float *), cudaMemcpyHostToDevice, ss.cs));
        GEO_TRY(gathers.alloc((size_t)kAdcigAngles * nimg * 4));
        GEO_TRY(gathers.zero(ss.cs));
        for (int ia = 0; ia < kAdcigAngles; ia++)
            GEO_TRY(launch_stack_image(gathers.as<float>() + ia * nimg, nz,
                                       d_aptr.as<const float *const>() + (size_t)ia * D.ns, d_offs.as<int>(),
                                       d_wid.as<int>(), D.ns, D.nx, ss.cs));
        GEO_CUDA(cudaMemcpyAsync(adcig, gathers.p, (size_t)kAdcigAngles * nimg * 4, k, ss.cs));
    }
    if (per_shot) {
        size_t o = 0;
        for (int q = 0; q < D.ns; q++) {
            const size_t m = (size_t)D.shot_nxs[q] * nz;
            GEO_CUDA(cudaMemcpyAsync(per_shot + o, B.S[q].mig, m * 4, k, ss.cs));
            o += m;
        }
    }
    GEO_CUDA(cudaStreamSynchronize(ss.cs));
    return GEO_OK;
}
