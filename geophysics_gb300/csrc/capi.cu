// C ABI: the reference's drop-in entry points, the Laplacian calls, the par
// file reader and status strings.
#include "geo_internal.h"
#include "fd3d.cuh"
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

using namespace geo;

extern "C" const char *geo_version(void) { return "geofd-gb300 0.1 (sm_103a)"; }

extern "C" const char *geo_strerror(int status) {
    switch (status) {
        case GEO_OK: return "ok";
        case GEO_ERR_ARG: return "invalid argument";
        case GEO_ERR_CUDA: return "CUDA error";
        case GEO_ERR_IO: return "file I/O error";
        case GEO_ERR_MODEL: return "invalid model values";
        case GEO_ERR_CFL: return "stability check failed";
        case GEO_ERR_WINDOW: return "aperture window leaves the model";
        case GEO_ERR_NOMEM: return "device allocation failed";
        case GEO_ERR_NAN: return "wavefield became non-finite";
        default: return "unknown status";
    }
}

// Detail of the last failure on this thread (not part of the header's
// stable surface; used by the Python wrapper for messages).
extern "C" const char *geo_last_error(void) { return g_last_error; }

namespace geo { long long launches_so_far(); }
extern "C" long long geo_launch_count(void) { return geo::launches_so_far(); }

// ---------------------------------------------------------------- Laplacian
static int lap_common(size_t n, const float *in, float *out, int mem, cudaStream_t s, DevBuf &din, DevBuf &dout,
                      const float **pin, float **pout) {
    if (!in || !out) return fail(GEO_ERR_ARG, "null argument");
    if (mem == GEO_MEM_DEVICE) {
        *pin = in;
        *pout = out;
        return GEO_OK;
    }
    if (mem != GEO_MEM_HOST) return fail(GEO_ERR_ARG, "bad mem kind");
    GEO_TRY(din.alloc(n * 4));
    GEO_TRY(dout.alloc(n * 4));
    GEO_CUDA(cudaMemcpyAsync(din.p, in, n * 4, cudaMemcpyHostToDevice, s));
    *pin = din.as<float>();
    *pout = dout.as<float>();
    return GEO_OK;
}

extern "C" int geo_laplace2d(int nx, int nz, const float *in, float *out, int mem, void *stream) {
    if (nx < 1 || nz < 1) return fail(GEO_ERR_ARG, "bad sizes");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)nx * nz;
    DevBuf a, b;
    const float *pi;
    float *po;
    GEO_TRY(lap_common(n, in, out, mem, s, a, b, &pi, &po));
    GEO_TRY(launch_laplace2d(nx, nz, pi, po, s));
    if (mem == GEO_MEM_HOST) GEO_CUDA(cudaMemcpyAsync(out, po, n * 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}

extern "C" int geo_laplace3d(int nx, int ny, int nz, const float *in, float *out, int mem, void *stream) {
    if (nx < 1 || ny < 1 || nz < 1) return fail(GEO_ERR_ARG, "bad sizes");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)nx * ny * nz;
    DevBuf a, b;
    const float *pi;
    float *po;
    GEO_TRY(lap_common(n, in, out, mem, s, a, b, &pi, &po));
    GEO_TRY(launch_laplace3d(nx, ny, nz, pi, po, s));
    if (mem == GEO_MEM_HOST) GEO_CUDA(cudaMemcpyAsync(out, po, n * 4, cudaMemcpyDeviceToHost, s));
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}

// ---------------------------------------------------------------- file I/O
namespace geo {

int read_floats(const char *fn, size_t n, std::vector<float> &out) {
    FILE *fp = fopen(fn, "rb");
    if (!fp) return fail(GEO_ERR_IO, "cannot open <%s>", fn);
    out.resize(n);
    size_t got = fread(out.data(), 4, n, fp);
    fclose(fp);
    if (got != n) return fail(GEO_ERR_IO, "<%s>: expected %zu floats, read %zu", fn, n, got);
    return GEO_OK;
}

int write_at(FILE *fp, size_t offset_bytes, const float *a, size_t n) {
    if (fseek(fp, (long)offset_bytes, SEEK_SET) != 0) return fail(GEO_ERR_IO, "seek failed");
    if (fwrite(a, 4, n, fp) != n) return fail(GEO_ERR_IO, "write failed");
    return GEO_OK;
}

}  // namespace geo

static void report(const char *who, int st) {
    if (st != GEO_OK) fprintf(stderr, "%s: %s (%s)\n", who, geo_strerror(st), g_last_error);
}

// 2D drop-in body shared by GPU_vti2dfd and CPU_vti2dfd: read the three
// model files (nx*nz float32, x-major), run ns shots, write the shot file
// (shot is at byte offset (is-1)*nt*nx*4) and the padded P snapshot of shot
// 1 every 50 steps (GPU_vti2dfd_kernels.cu:404-444; CPU_vti2dfd_kernels.c:465-510).
static int vti2d_files(int variant, int nx, int nz, int dx, int dz, int npd, int SV, const char *FNv,
                       const char *FNe, const char *FNd, int favg, int ns, int fs, int ds, int zs,
                       const char *FNshot, const char *FNsnap, int nt, int dt) {
    if (!FNv || !FNe || !FNd || !FNshot || !FNsnap) return fail(GEO_ERR_ARG, "null file name");
    std::vector<float> v, e, d;
    const size_t n = (size_t)nx * nz;
    GEO_TRY(read_floats(FNv, n, v));
    GEO_TRY(read_floats(FNe, n, e));
    GEO_TRY(read_floats(FNd, n, d));
    FILE *fshot = fopen(FNshot, "wb");
    if (!fshot) return fail(GEO_ERR_IO, "cannot open <%s>", FNshot);
    FILE *fsnap = fopen(FNsnap, "wb");
    if (!fsnap) {
        fclose(fshot);
        return fail(GEO_ERR_IO, "cannot open <%s>", FNsnap);
    }
    const int nnx = nx + 2 * npd, nnz = nz + 2 * npd;
    const int nsnap = (nt - 1) / 50 + 1;
    std::vector<float> shot((size_t)nt * nx), snap((size_t)nsnap * nnx * nnz);
    int st = GEO_OK;
    for (int is = 1; is <= ns && st == GEO_OK; is++) {
        geo_fd2d_desc D{};
        D.nx = nx; D.nz = nz; D.npd = npd; D.nt = nt;
        D.dx = (float)dx; D.dz = (float)dz; D.dt = (float)(dt * 1.0 / 1000000);
        D.favg = (float)favg; D.pfac = 10.0f; D.wtype = 1;
        D.fs = (float)fs; D.ds = (float)ds; D.zs = (float)zs; D.is = is;
        D.variant = variant; D.sv = SV; D.rec_iz = npd;
        D.rec_scale = variant == GEO_VARIANT_CPU ? 2.0f : 1.0f;
        D.mute_tt = variant == GEO_VARIANT_GPU ? 100 : 0;
        st = geo_fd2d_shot(&D, v.data(), e.data(), d.data(), shot.data(), is == 1 ? snap.data() : nullptr,
                           is == 1 ? 50 : 0, GEO_MEM_HOST, nullptr);
        if (st == GEO_OK && is == 1) st = write_at(fsnap, 0, snap.data(), snap.size());
        if (st == GEO_OK) st = write_at(fshot, (size_t)(is - 1) * nt * nx * 4, shot.data(), shot.size());
    }
    fclose(fshot);
    fclose(fsnap);
    return st;
}

extern "C" void GPU_vti2dfd(int nx, int nz, int dx, int dz, int npd, int SV, const char FNv[], const char FNe[],
                            const char FNd[], int favg, int ns, int fs, int ds, int zs, const char FNshot[],
                            const char FNsnap[], int nt, int dt, int run_count) {
    (void)run_count;
    report("GPU_vti2dfd", vti2d_files(GEO_VARIANT_GPU, nx, nz, dx, dz, npd, SV, FNv, FNe, FNd, favg, ns, fs, ds, zs,
                                      FNshot, FNsnap, nt, dt));
}

extern "C" void CPU_vti2dfd(int nx, int nz, int dx, int dz, int npd, int SV, const char FNv[], const char FNe[],
                            const char FNd[], int favg, int ns, int fs, int ds, int zs, const char FNshot[],
                            const char FNsnap[], int nt, int dt, int run_count) {
    (void)run_count;
    report("CPU_vti2dfd", vti2d_files(GEO_VARIANT_CPU, nx, nz, dx, dz, npd, SV, FNv, FNe, FNd, favg, ns, fs, ds, zs,
                                      FNshot, FNsnap, nt, dt));
}

// 3D drop-in (GPU_vti3dfd_kernels.cu:371-573): shots 0..ns-1, every surface
// node a receiver, direct-wave mute tt=100, the interior window of P for
// shot 0 every 300 steps (it != 0) into the snapshot file.
struct Snap3D {
    geo_fd3d_plan *plan;
    FILE *fp;
    int nx, ny, nz, npd;
    std::vector<float> full, win;
};

static int snap3d_cb(void *ctx, int it) {
    Snap3D *S = (Snap3D *)ctx;
    if (it == 0 || it % 300 != 0) return GEO_OK;
    int nnx, nny, nnz;
    plan3d_dims(S->plan, &nnx, &nny, &nnz);
    S->full.resize((size_t)nnx * nny * nnz);
    GEO_TRY(geo_fd3d_get_fields(S->plan, S->full.data(), nullptr, GEO_MEM_HOST, nullptr));
    S->win.resize((size_t)S->nx * S->ny * S->nz);
    for (int iy = 0; iy < S->ny; iy++)
        for (int ix = 0; ix < S->nx; ix++)
            memcpy(&S->win[(size_t)S->nz * (ix + (size_t)S->nx * iy)],
                   &S->full[(size_t)S->npd + nnz * ((size_t)(ix + S->npd) + (size_t)nnx * (iy + S->npd))], S->nz * 4);
    return write_at(S->fp, (size_t)(it / 300 - 1) * S->win.size() * 4, S->win.data(), S->win.size());
}

static int vti3d_files(int nx, int ny, int nz, int dx, int dy, int dz, int npml, int SV, const char *FNv,
                       const char *FNe, const char *FNd, int favg, int ns, int fsx, int dsx, int fsy, int dsy, int fsz,
                       int dsz, const char *FNshot, const char *FNsnap, int nt, int dt) {
    if (!FNv || !FNe || !FNd || !FNshot || !FNsnap) return fail(GEO_ERR_ARG, "null file name");
    const size_t n = (size_t)nx * ny * nz;
    std::vector<float> v, e, d;
    GEO_TRY(read_floats(FNv, n, v));
    GEO_TRY(read_floats(FNe, n, e));
    GEO_TRY(read_floats(FNd, n, d));
    geo_fd3d_desc D{};
    D.nx = nx; D.ny = ny; D.nz = nz; D.npd = npml; D.nt = nt;
    D.dx = (float)dx; D.dy = (float)dy; D.dz = (float)dz; D.dt = (float)(dt * 1.0 / 1000000);
    D.favg = (float)favg; D.pfac = 10.0f; D.wtype = 1; D.sv = SV;
    const char *mode = getenv("GEO_FD3D_MODE");
    D.mode = (mode && !strcmp(mode, "fast")) ? GEO_MODE_FAST : GEO_MODE_EXACT;
    D.fsx = fsx; D.fsy = fsy; D.fsz = fsz; D.dsx = dsx; D.dsy = dsy; D.dsz = dsz;
    D.rec_iz = npml; D.rx0 = 0; D.drx = 1; D.nrx = nx; D.ry0 = 0; D.dry = 1; D.nry = ny;
    D.mute_tt = 100;
    geo_fd3d_plan *p = nullptr;
    GEO_TRY(geo_fd3d_plan_create(&p, &D));
    int st = geo_fd3d_set_model(p, v.data(), e.data(), d.data(), GEO_MEM_HOST, nullptr);
    FILE *fshot = st == GEO_OK ? fopen(FNshot, "wb") : nullptr;
    FILE *fsnap = fshot ? fopen(FNsnap, "wb") : nullptr;
    if (st == GEO_OK && (!fshot || !fsnap)) st = fail(GEO_ERR_IO, "cannot open output files");
    std::vector<float> shot((size_t)nt * nx * ny);
    for (int is = 0; is < ns && st == GEO_OK; is++) {
        Snap3D S{p, fsnap, nx, ny, nz, npml, {}, {}};
        st = run_shot_3d(p, is, nullptr, is == 0 ? snap3d_cb : nullptr, &S);
        if (st == GEO_OK) st = fetch_shot_3d(p, shot.data(), GEO_MEM_HOST, nullptr);
        if (st == GEO_OK) st = write_at(fshot, (size_t)is * nt * nx * ny * 4, shot.data(), shot.size());
    }
    if (fshot) fclose(fshot);
    if (fsnap) fclose(fsnap);
    geo_fd3d_plan_destroy(p);
    return st;
}

extern "C" void GPU_vti3dfd(int nx, int ny, int nz, int dx, int dy, int dz, int npml, int SV, const char FNv[],
                            const char FNe[], const char FNd[], int favg, int ns, int fsx, int dsx, int fsy, int dsy,
                            int fsz, int dsz, const char FNshot[], const char FNsnap[], int nt, int dt,
                            int run_count) {
    (void)run_count;
    report("GPU_vti3dfd", vti3d_files(nx, ny, nz, dx, dy, dz, npml, SV, FNv, FNe, FNd, favg, ns, fsx, dsx, fsy, dsy,
                                      fsz, dsz, FNshot, FNsnap, nt, dt));
}

// ---------------------------------------------------------------- par file
struct geo_par {
    std::map<std::string, std::string> kv;
};

static std::string trim(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && isspace((unsigned char)s[a])) a++;
    while (b > a && isspace((unsigned char)s[b - 1])) b--;
    return s.substr(a, b - a);
}

// `key= value` per line (leading blanks allowed, '#' starts a comment), the
// layout of the reference's .par files (2D-ISO-tomography-inversion-c-0.0/tomo-1.par).
extern "C" int geo_par_load(const char *path, geo_par **par) {
    if (!path || !par) return fail(GEO_ERR_ARG, "null argument");
    FILE *fp = fopen(path, "r");
    if (!fp) return fail(GEO_ERR_IO, "cannot open <%s>", path);
    geo_par *p = new geo_par();
    char line[1024];
    while (fgets(line, sizeof line, fp)) {
        std::string l(line);
        const size_t h = l.find('#');
        if (h != std::string::npos) l = l.substr(0, h);
        const size_t eq = l.find('=');
        if (eq == std::string::npos) continue;
        const std::string k = trim(l.substr(0, eq)), v = trim(l.substr(eq + 1));
        if (!k.empty()) p->kv[k] = v;
    }
    fclose(fp);
    *par = p;
    return GEO_OK;
}

static const std::string *par_find(const geo_par *p, const char *key) {
    if (!p || !key) return nullptr;
    auto it = p->kv.find(key);
    return it == p->kv.end() ? nullptr : &it->second;
}

extern "C" int geo_par_get_int(const geo_par *p, const char *key, int *out) {
    const std::string *v = par_find(p, key);
    if (!v || !out) return fail(GEO_ERR_ARG, "missing key %s", key ? key : "(null)");
    char *end = nullptr;
    const long x = strtol(v->c_str(), &end, 10);
    if (end == v->c_str()) return fail(GEO_ERR_ARG, "key %s is not an integer", key);
    *out = (int)x;
    return GEO_OK;
}

extern "C" int geo_par_get_float(const geo_par *p, const char *key, float *out) {
    const std::string *v = par_find(p, key);
    if (!v || !out) return fail(GEO_ERR_ARG, "missing key %s", key ? key : "(null)");
    char *end = nullptr;
    const double x = strtod(v->c_str(), &end);
    if (end == v->c_str()) return fail(GEO_ERR_ARG, "key %s is not a number", key);
    *out = (float)x;
    return GEO_OK;
}

extern "C" int geo_par_get_string(const geo_par *p, const char *key, char *out, int cap) {
    const std::string *v = par_find(p, key);
    if (!v || !out || cap < 1) return fail(GEO_ERR_ARG, "missing key %s", key ? key : "(null)");
    if ((int)v->size() >= cap) return fail(GEO_ERR_ARG, "value of %s longer than %d", key, cap - 1);
    memcpy(out, v->c_str(), v->size() + 1);
    return GEO_OK;
}

extern "C" void geo_par_free(geo_par *p) { delete p; }
