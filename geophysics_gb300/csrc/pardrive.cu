// Par-file driven runs: geo_fd2d, geo_fd3d, geo_rtm2d.
//
// Each takes a loaded par file (geo_par_load, the key= value format of
// 2D-ISO-tomography-inversion-c-0.0/tomo-1.par), an optional device ordinal
// and an optional caller-owned device buffer for the result, and runs what
// the reference's programs run from their parameters:
//
//   geo_fd2d   the shots of GPU_vti2dfd / CPU_vti2dfd
//              (2D-3D-vti-fd-cuda-gtk-GUI/GPU_vti2dfd_kernels.cu:301-444,
//              CPU_vti2dfd_kernels.c:366-510), keys named after their
//              arguments (nx nz dx dz npd SV FNv FNe FNd favg ns fs ds zs
//              FNshot FNsnap nt dt, dt in microseconds);
//   geo_fd3d   the shots of GPU_vti3dfd (GPU_vti3dfd_kernels.cu:371-573),
//              keys nx ny nz dx dy dz npml SV FNv FNe FNd favg ns fsx dsx
//              fsy dsy fsz dsz FNshot nt dt;
//   geo_rtm2d  the MPI RTM program's main (2D-vti-fd+rtm-mpi/
//              Toa_rtm_vti_adcig_cdp.c:59-481), whose parameters are fixed
//              in its source; the keys carry their names (nx nz dx dz npd
//              nt dt favg pfac ns_sxd fs_sxd ds_sxd zs_sxd nxs seismic
//              FN1 FN2 FN3 and the outputs FN6 FN7 FN8 FN9 FN10).
//
// Everything runs through the library's own entry points (geo_fd2d_shot,
// the 3D plan, geo_rtm2d_batch_adcig, geo_adcig_smooth_stack); this file
// only reads parameters and files and writes results.
//
// Resume by shot (geo_fd2d, geo_fd3d; key resume= 1).  The reference writes
// every shot's record at its own offset of the shot file
// (GPU_vti2dfd_kernels.cu:441, GPU_vti3dfd_kernels.cu:560), so a run can be
// continued shot by shot.  With resume on, the shot file is updated in place
// and a manifest (key FNdone, default <FNshot>.done) gets one line per shot
// once that shot's record (and, for shot 1, its snapshots) is on disk
// (fflush + fsync before the line is written).  A rerun with the same par
// file skips the shots the manifest lists -- their records are read back
// from the shot file when a device buffer is given -- and runs the rest.
// The manifest's first line holds the run's parameters; a manifest from a
// different run is refused (GEO_ERR_ARG).
#include "geo_internal.h"
#include <cstring>
#include <memory>
#include <unistd.h>
#include <string>
#include <vector>

namespace geo {

static int par_i(const geo_par *p, const char *k, int *o) {
    if (geo_par_get_int(p, k, o) != GEO_OK) return fail(GEO_ERR_ARG, "par: integer key '%s' missing", k);
    return GEO_OK;
}
static int par_f(const geo_par *p, const char *k, float *o) {
    if (geo_par_get_float(p, k, o) != GEO_OK) return fail(GEO_ERR_ARG, "par: number key '%s' missing", k);
    return GEO_OK;
}
static int par_s(const geo_par *p, const char *k, std::string &o) {
    char buf[1024];
    if (geo_par_get_string(p, k, buf, sizeof buf) != GEO_OK) return fail(GEO_ERR_ARG, "par: key '%s' missing", k);
    o = buf;
    return GEO_OK;
}
static int opt_i(const geo_par *p, const char *k, int def) {
    int v;
    return geo_par_get_int(p, k, &v) == GEO_OK ? v : def;
}
static float opt_f(const geo_par *p, const char *k, float def) {
    float v;
    return geo_par_get_float(p, k, &v) == GEO_OK ? v : def;
}
static std::string opt_s(const geo_par *p, const char *k) {
    char buf[1024];
    return geo_par_get_string(p, k, buf, sizeof buf) == GEO_OK ? std::string(buf) : std::string();
}

// Make `device` current for the call (when >= 0) and restore the caller's
// device afterwards.
struct DeviceScope {
    int prev = -1;
    bool set = false;
    int enter(int device) {
        if (device < 0) return GEO_OK;
        int n = 0;
        GEO_CUDA(cudaGetDeviceCount(&n));
        if (device >= n) return fail(GEO_ERR_ARG, "device %d out of range (%d devices)", device, n);
        GEO_CUDA(cudaGetDevice(&prev));
        GEO_CUDA(cudaSetDevice(device));
        set = true;
        return GEO_OK;
    }
    ~DeviceScope() {
        if (set) cudaSetDevice(prev);
    }
};

struct FileCloser {
    void operator()(FILE *f) const {
        if (f) fclose(f);
    }
};
using File = std::unique_ptr<FILE, FileCloser>;

static int open_out(const std::string &fn, File &f) {
    f.reset(fopen(fn.c_str(), "wb"));
    if (!f) return fail(GEO_ERR_IO, "cannot create <%s>", fn.c_str());
    return GEO_OK;
}

// Open for update in place (resume), creating the file when absent.
static int open_update(const std::string &fn, File &f) {
    f.reset(fopen(fn.c_str(), "r+b"));
    if (!f) f.reset(fopen(fn.c_str(), "w+b"));
    if (!f) return fail(GEO_ERR_IO, "cannot open <%s> for update", fn.c_str());
    return GEO_OK;
}

static int flush_to_disk(FILE *f, const char *what) {
    if (fflush(f) != 0 || fsync(fileno(f)) != 0) return fail(GEO_ERR_IO, "cannot flush %s", what);
    return GEO_OK;
}

// Manifest of completed shots: header line = the run's parameters, then one
// "shot <is>" line per completed shot.
struct Manifest {
    std::string path, header;
    std::vector<char> done;        // by shot index (0-based)
    File f;
    int open(const std::string &p, const std::string &hdr, int ns) {
        path = p;
        header = hdr;
        done.assign(ns, 0);
        FILE *r = fopen(p.c_str(), "r");
        if (r) {
            char line[4096];
            bool first = true, ok = true;
            while (fgets(line, sizeof line, r)) {
                std::string l(line);
                while (!l.empty() && (l.back() == '\n' || l.back() == '\r')) l.pop_back();
                if (first) {
                    ok = l == hdr;
                    first = false;
                    continue;
                }
                int k = -1;
                if (sscanf(l.c_str(), "shot %d", &k) == 1 && k >= 0 && k < ns) done[k] = 1;
            }
            fclose(r);
            if (!first && !ok) return fail(GEO_ERR_ARG, "manifest <%s> belongs to another run", p.c_str());
            if (first) r = nullptr;   // empty file: start over
        }
        f.reset(fopen(p.c_str(), r ? "a" : "w"));
        if (!f) return fail(GEO_ERR_IO, "cannot write manifest <%s>", p.c_str());
        if (!r) {
            fprintf(f.get(), "%s\n", hdr.c_str());
            GEO_TRY(flush_to_disk(f.get(), "manifest"));
        }
        return GEO_OK;
    }
    int mark(int k) {
        fprintf(f.get(), "shot %d\n", k);
        GEO_TRY(flush_to_disk(f.get(), "manifest"));
        done[k] = 1;
        return GEO_OK;
    }
};

// Read n floats at a byte offset (a completed shot's record on resume).
static int read_at(FILE *fp, size_t offset_bytes, float *a, size_t n) {
    if (fseeko(fp, (off_t)offset_bytes, SEEK_SET) != 0 || fread(a, 4, n, fp) != n)
        return fail(GEO_ERR_IO, "short read of a completed shot's record");
    return GEO_OK;
}

// Three model files of n floats each: raw native floats, or (seismic = 2)
// SU traces of nz big-endian samples (read_v_e_d_r, Toa_rtm_vti_adcig_cdp.c:1415-1453).
static int read_model(const std::string fn[3], size_t ntr, size_t ns, int seismic, std::vector<float> out[3]) {
    for (int k = 0; k < 3; k++) {
        if (seismic == 2) {
            out[k].resize(ntr * ns);
            GEO_TRY(geo_su_read(fn[k].c_str(), (int)ntr, (int)ns, 1, out[k].data(), nullptr));
        } else {
            GEO_TRY(read_floats(fn[k].c_str(), ntr * ns, out[k]));
        }
    }
    return GEO_OK;
}

static int variant_of(const std::string &s, int *v) {
    if (s.empty() || s == "gpu" || s == "1") *v = GEO_VARIANT_GPU;
    else if (s == "cpu" || s == "0") *v = GEO_VARIANT_CPU;
    else if (s == "mpi" || s == "2") *v = GEO_VARIANT_MPI;
    else return fail(GEO_ERR_ARG, "par: variant must be gpu, cpu or mpi");
    return GEO_OK;
}

}  // namespace geo

using namespace geo;

extern "C" int geo_fd2d(const geo_par *par, int device, float *d_shots, void *stream) {
    if (!par) return fail(GEO_ERR_ARG, "null par");
    geo_fd2d_desc D{};
    int ns = 0;
    float dt_us = 0;
    std::string fn[3], fshot, fsnap;
    GEO_TRY(par_i(par, "nx", &D.nx));
    GEO_TRY(par_i(par, "nz", &D.nz));
    GEO_TRY(par_f(par, "dx", &D.dx));
    GEO_TRY(par_f(par, "dz", &D.dz));
    GEO_TRY(par_i(par, "npd", &D.npd));
    GEO_TRY(par_i(par, "nt", &D.nt));
    GEO_TRY(par_f(par, "dt", &dt_us));
    GEO_TRY(par_f(par, "favg", &D.favg));
    GEO_TRY(par_i(par, "ns", &ns));
    GEO_TRY(par_f(par, "fs", &D.fs));
    GEO_TRY(par_f(par, "ds", &D.ds));
    GEO_TRY(par_f(par, "zs", &D.zs));
    GEO_TRY(par_s(par, "FNv", fn[0]));
    GEO_TRY(par_s(par, "FNe", fn[1]));
    GEO_TRY(par_s(par, "FNd", fn[2]));
    GEO_TRY(variant_of(opt_s(par, "variant"), &D.variant));
    fshot = opt_s(par, "FNshot");
    fsnap = opt_s(par, "FNsnap");
    if (ns < 1) return fail(GEO_ERR_ARG, "par: ns must be >= 1");
    if (!d_shots && fshot.empty()) return fail(GEO_ERR_ARG, "par: FNshot missing and no device buffer given");
    D.dt = (float)(dt_us * 1.0 / 1000000);
    D.pfac = opt_f(par, "pfac", 10.0f);
    D.wtype = opt_i(par, "wtype", 1);
    D.sv = opt_i(par, "SV", 0);
    D.rec_iz = opt_i(par, "rec_iz", D.npd);
    D.rec_scale = D.variant == GEO_VARIANT_CPU ? 2.0f : 1.0f;
    D.mute_tt = opt_i(par, "mute_tt", D.variant == GEO_VARIANT_GPU ? 100 : 0);
    const int snap_every = opt_i(par, "snap_every", 50);
    DeviceScope dev;
    GEO_TRY(dev.enter(device));
    std::vector<float> m[3];
    GEO_TRY(read_model(fn, (size_t)D.nx, (size_t)D.nz, 1, m));
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n0 = (size_t)D.nx * D.nz, nrec = (size_t)D.nx * D.nt;
    const size_t nsnap = snap_every > 0 ? (size_t)((D.nt - 1) / snap_every + 1) * (D.nx + 2 * D.npd) * (D.nz + 2 * D.npd)
                                        : 0;
    const int resume = opt_i(par, "resume", 0);
    if (resume && fshot.empty()) return fail(GEO_ERR_ARG, "par: resume needs FNshot");
    File fs_, fsn;
    Manifest man;
    if (resume) {
        char hdr[512];
        snprintf(hdr, sizeof hdr, "geo_fd2d nx=%d nz=%d npd=%d nt=%d ns=%d variant=%d dx=%g dz=%g dt=%g favg=%g "
                 "fs=%g ds=%g zs=%g SV=%d", D.nx, D.nz, D.npd, D.nt, ns, D.variant, D.dx, D.dz, D.dt, D.favg, D.fs,
                 D.ds, D.zs, D.sv);
        std::string dn = opt_s(par, "FNdone");
        GEO_TRY(man.open(dn.empty() ? fshot + ".done" : dn, hdr, ns));
        GEO_TRY(open_update(fshot, fs_));
        if (!fsnap.empty()) GEO_TRY(open_update(fsnap, fsn));
    } else {
        if (!fshot.empty()) GEO_TRY(open_out(fshot, fs_));
        if (!fsnap.empty()) GEO_TRY(open_out(fsnap, fsn));
    }
    std::vector<float> rec(fshot.empty() ? 0 : nrec), snap(fsnap.empty() ? 0 : nsnap);
    DevBuf dm;
    if (d_shots) {   // the model on the device, as geo_fd2d_shot takes one memory kind
        GEO_TRY(dm.alloc(3 * n0 * 4));
        for (int k = 0; k < 3; k++)
            GEO_CUDA(cudaMemcpyAsync(dm.as<float>() + k * n0, m[k].data(), n0 * 4, cudaMemcpyHostToDevice, s));
    }
    for (int is = 1; is <= ns; is++) {
        D.is = is;
        if (resume && man.done[is - 1]) {
            if (d_shots) {
                GEO_TRY(read_at(fs_.get(), (size_t)(is - 1) * nrec * 4, rec.data(), nrec));
                GEO_CUDA(cudaMemcpyAsync(d_shots + (size_t)(is - 1) * nrec, rec.data(), nrec * 4,
                                         cudaMemcpyHostToDevice, s));
                GEO_CUDA(cudaStreamSynchronize(s));
            }
            continue;
        }
        const bool want_snap = is == 1 && !fsnap.empty() && snap_every > 0;
        if (d_shots) {
            float *out = d_shots + (size_t)(is - 1) * nrec;
            const float *dv = dm.as<float>();
            GEO_TRY(geo_fd2d_shot(&D, dv, dv + n0, dv + 2 * n0, out, nullptr, 0, GEO_MEM_DEVICE, stream));
            if (fs_) {
                GEO_CUDA(cudaMemcpyAsync(rec.data(), out, nrec * 4, cudaMemcpyDeviceToHost, s));
                GEO_CUDA(cudaStreamSynchronize(s));
            }
            if (want_snap) {   // frames of shot 1 come from a host run of the same shot
                std::vector<float> tmp(nrec);
                GEO_TRY(geo_fd2d_shot(&D, m[0].data(), m[1].data(), m[2].data(), tmp.data(), snap.data(), snap_every,
                                      GEO_MEM_HOST, nullptr));
            }
        } else {
            GEO_TRY(geo_fd2d_shot(&D, m[0].data(), m[1].data(), m[2].data(), rec.data(),
                                  want_snap ? snap.data() : nullptr, want_snap ? snap_every : 0, GEO_MEM_HOST, nullptr));
        }
        if (fs_) GEO_TRY(write_at(fs_.get(), (size_t)(is - 1) * nrec * 4, rec.data(), nrec));
        if (want_snap) GEO_TRY(write_at(fsn.get(), 0, snap.data(), snap.size()));
        if (resume) {
            if (want_snap) GEO_TRY(flush_to_disk(fsn.get(), "snapshot file"));
            GEO_TRY(flush_to_disk(fs_.get(), "shot file"));
            GEO_TRY(man.mark(is - 1));
        }
    }
    if (d_shots) GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}

extern "C" int geo_fd3d(const geo_par *par, int device, float *d_shots, void *stream) {
    if (!par) return fail(GEO_ERR_ARG, "null par");
    geo_fd3d_desc D{};
    int ns = 0;
    float dt_us = 0;
    std::string fn[3], fshot;
    GEO_TRY(par_i(par, "nx", &D.nx));
    GEO_TRY(par_i(par, "ny", &D.ny));
    GEO_TRY(par_i(par, "nz", &D.nz));
    GEO_TRY(par_f(par, "dx", &D.dx));
    GEO_TRY(par_f(par, "dy", &D.dy));
    GEO_TRY(par_f(par, "dz", &D.dz));
    GEO_TRY(par_i(par, "npml", &D.npd));
    GEO_TRY(par_i(par, "nt", &D.nt));
    GEO_TRY(par_f(par, "dt", &dt_us));
    GEO_TRY(par_f(par, "favg", &D.favg));
    GEO_TRY(par_i(par, "ns", &ns));
    GEO_TRY(par_i(par, "fsx", &D.fsx));
    GEO_TRY(par_i(par, "fsy", &D.fsy));
    GEO_TRY(par_i(par, "fsz", &D.fsz));
    GEO_TRY(par_s(par, "FNv", fn[0]));
    GEO_TRY(par_s(par, "FNe", fn[1]));
    GEO_TRY(par_s(par, "FNd", fn[2]));
    fshot = opt_s(par, "FNshot");
    if (ns < 1) return fail(GEO_ERR_ARG, "par: ns must be >= 1");
    if (!d_shots && fshot.empty()) return fail(GEO_ERR_ARG, "par: FNshot missing and no device buffer given");
    const std::string mode = opt_s(par, "mode");
    if (!mode.empty() && mode != "exact" && mode != "fast") return fail(GEO_ERR_ARG, "par: mode must be exact or fast");
    D.mode = mode == "fast" ? GEO_MODE_FAST : GEO_MODE_EXACT;
    D.dsx = opt_i(par, "dsx", 0);
    D.dsy = opt_i(par, "dsy", 0);
    D.dsz = opt_i(par, "dsz", 0);
    D.dt = (float)(dt_us * 1.0 / 1000000);
    D.pfac = opt_f(par, "pfac", 10.0f);
    D.wtype = opt_i(par, "wtype", 1);
    D.sv = opt_i(par, "SV", 0);
    D.rec_iz = opt_i(par, "rec_iz", D.npd);
    D.rx0 = opt_i(par, "rx0", 0);
    D.drx = opt_i(par, "drx", 1);
    D.ry0 = opt_i(par, "ry0", 0);
    D.dry = opt_i(par, "dry", 1);
    D.nrx = opt_i(par, "nrx", D.drx > 0 ? (D.nx - D.rx0 + D.drx - 1) / D.drx : D.nx);
    D.nry = opt_i(par, "nry", D.dry > 0 ? (D.ny - D.ry0 + D.dry - 1) / D.dry : D.ny);
    D.mute_tt = opt_i(par, "mute_tt", 100);
    DeviceScope dev;
    GEO_TRY(dev.enter(device));
    std::vector<float> m[3];
    for (int k = 0; k < 3; k++) GEO_TRY(read_floats(fn[k].c_str(), (size_t)D.nx * D.ny * D.nz, m[k]));
    geo_fd3d_plan *plan = nullptr;
    GEO_TRY(geo_fd3d_plan_create(&plan, &D));
    std::unique_ptr<geo_fd3d_plan, int (*)(geo_fd3d_plan *)> guard(plan, geo_fd3d_plan_destroy);
    GEO_TRY(geo_fd3d_set_model(plan, m[0].data(), m[1].data(), m[2].data(), GEO_MEM_HOST, stream));
    // optional 3D TTI medium: tilt and azimuth files in degrees (FNtheta, FNphi)
    const std::string fth = opt_s(par, "FNtheta"), fph = opt_s(par, "FNphi");
    if (fth.empty() != fph.empty()) return fail(GEO_ERR_ARG, "par: FNtheta and FNphi go together");
    if (!fth.empty()) {
        std::vector<float> th, ph;
        GEO_TRY(read_floats(fth.c_str(), (size_t)D.nx * D.ny * D.nz, th));
        GEO_TRY(read_floats(fph.c_str(), (size_t)D.nx * D.ny * D.nz, ph));
        GEO_TRY(geo_fd3d_set_tilt(plan, th.data(), ph.data(), GEO_MEM_HOST, stream));
    }
    const size_t nrec = (size_t)D.nt * D.nrx * D.nry;
    const int resume = opt_i(par, "resume", 0);
    if (resume && fshot.empty()) return fail(GEO_ERR_ARG, "par: resume needs FNshot");
    File f;
    Manifest man;
    if (resume) {
        char hdr[512];
        snprintf(hdr, sizeof hdr, "geo_fd3d nx=%d ny=%d nz=%d npml=%d nt=%d ns=%d mode=%d dx=%g dy=%g dz=%g dt=%g "
                 "favg=%g fsx=%d fsy=%d fsz=%d dsx=%d dsy=%d dsz=%d SV=%d rec=%d,%d,%d,%d,%d,%d,%d tilt=%d",
                 D.nx, D.ny, D.nz, D.npd, D.nt, ns, D.mode, D.dx, D.dy, D.dz, D.dt, D.favg, D.fsx, D.fsy, D.fsz,
                 D.dsx, D.dsy, D.dsz, D.sv, D.rec_iz, D.rx0, D.drx, D.nrx, D.ry0, D.dry, D.nry, fth.empty() ? 0 : 1);
        std::string dn = opt_s(par, "FNdone");
        GEO_TRY(man.open(dn.empty() ? fshot + ".done" : dn, hdr, ns));
        GEO_TRY(open_update(fshot, f));
    } else if (!fshot.empty()) {
        GEO_TRY(open_out(fshot, f));
    }
    std::vector<float> rec(f ? nrec : 0);
    cudaStream_t s = (cudaStream_t)stream;
    for (int is = 0; is < ns; is++) {   // 0-based shots, as the 3D program counts them
        if (resume && man.done[is]) {
            if (d_shots) {
                GEO_TRY(read_at(f.get(), (size_t)is * nrec * 4, rec.data(), nrec));
                GEO_CUDA(cudaMemcpyAsync(d_shots + (size_t)is * nrec, rec.data(), nrec * 4, cudaMemcpyHostToDevice,
                                         s));
                GEO_CUDA(cudaStreamSynchronize(s));
            }
            continue;
        }
        if (d_shots) {
            float *out = d_shots + (size_t)is * nrec;
            GEO_TRY(geo_fd3d_run_shot(plan, is, out, GEO_MEM_DEVICE, stream));
            if (f) {
                GEO_CUDA(cudaMemcpyAsync(rec.data(), out, nrec * 4, cudaMemcpyDeviceToHost, s));
                GEO_CUDA(cudaStreamSynchronize(s));
            }
        } else {
            GEO_TRY(geo_fd3d_run_shot(plan, is, rec.data(), GEO_MEM_HOST, stream));
        }
        if (f) GEO_TRY(write_at(f.get(), (size_t)is * nrec * 4, rec.data(), nrec));
        if (resume) {
            GEO_TRY(flush_to_disk(f.get(), "shot file"));
            GEO_TRY(man.mark(is));
        }
    }
    GEO_CUDA(cudaStreamSynchronize(s));
    return GEO_OK;
}

extern "C" int geo_rtm2d(const geo_par *par, int device, float *d_image, void *stream) {
    if (!par) return fail(GEO_ERR_ARG, "null par");
    geo_rtm2d_desc D{};
    int ns = 0, fs = 0, ds = 0, zs = 0, nxs = 0;
    std::string fn[3];
    GEO_TRY(par_i(par, "nx", &D.nx));
    GEO_TRY(par_i(par, "nz", &D.nz));
    GEO_TRY(par_f(par, "dx", &D.dx));
    GEO_TRY(par_f(par, "dz", &D.dz));
    GEO_TRY(par_i(par, "npd", &D.npd));
    GEO_TRY(par_i(par, "nt", &D.nt));
    GEO_TRY(par_f(par, "dt", &D.dt_ms));
    GEO_TRY(par_f(par, "favg", &D.favg));
    GEO_TRY(par_f(par, "pfac", &D.pfac));
    GEO_TRY(par_i(par, "ns_sxd", &ns));
    GEO_TRY(par_i(par, "fs_sxd", &fs));
    GEO_TRY(par_i(par, "ds_sxd", &ds));
    GEO_TRY(par_i(par, "zs_sxd", &zs));
    GEO_TRY(par_i(par, "nxs", &nxs));
    GEO_TRY(par_s(par, "FN1", fn[0]));
    GEO_TRY(par_s(par, "FN2", fn[1]));
    GEO_TRY(par_s(par, "FN3", fn[2]));
    const int seismic = opt_i(par, "seismic", 1);
    const std::string fmig = opt_s(par, "FN6"), fper = opt_s(par, "FN7"), fag = opt_s(par, "FN8"),
                      fags = opt_s(par, "FN9"), fstk = opt_s(par, "FN10");
    if (ns < 1) return fail(GEO_ERR_ARG, "par: ns_sxd must be >= 1");
    if (seismic != 1 && seismic != 2) return fail(GEO_ERR_ARG, "par: seismic must be 1 (.dat) or 2 (.su)");
    if (!d_image && fmig.empty()) return fail(GEO_ERR_ARG, "par: FN6 missing and no device buffer given");
    D.zs = zs;
    D.ns = ns;
    D.laplace = opt_i(par, "laplace", 0);
    D.tile_x = opt_i(par, "tile_x", 0);
    std::vector<int> sx(ns), sw(ns, nxs);
    for (int k = 0; k < ns; k++) sx[k] = fs + k * ds;   // shot is = k+1 at fs_sxd + (is-1)*ds_sxd (:295)
    D.shot_x = sx.data();
    D.shot_nxs = sw.data();
    DeviceScope dev;
    GEO_TRY(dev.enter(device));
    std::vector<float> m[3];
    GEO_TRY(read_model(fn, (size_t)D.nx, (size_t)D.nz, seismic, m));
    const size_t n0 = (size_t)D.nx * D.nz;
    const bool gathers = !fag.empty() || !fags.empty() || !fstk.empty();
    std::vector<float> img(n0), per(fper.empty() ? 0 : (size_t)ns * nxs * D.nz), ag(gathers ? 90 * n0 : 0);
    GEO_TRY(geo_rtm2d_batch_adcig(&D, m[0].data(), m[1].data(), m[2].data(), img.data(),
                                  per.empty() ? nullptr : per.data(), gathers ? ag.data() : nullptr, GEO_MEM_HOST,
                                  stream));
    if (d_image)
        GEO_CUDA(cudaMemcpyAsync(d_image, img.data(), n0 * 4, cudaMemcpyHostToDevice, (cudaStream_t)stream));
    File f;
    if (!fmig.empty()) {
        GEO_TRY(open_out(fmig, f));
        GEO_TRY(write_at(f.get(), 0, img.data(), n0));
    }
    if (!fper.empty()) {
        GEO_TRY(open_out(fper, f));
        GEO_TRY(write_at(f.get(), 0, per.data(), per.size()));
    }
    // gathers go to file x-major: for ix, for ia, for iz (:405-409, 430-433)
    auto write_gathers = [&](const std::string &name, const std::vector<float> &g) -> int {
        std::vector<float> t(g.size());
        for (int ix = 0; ix < D.nx; ix++)
            for (int ia = 0; ia < 90; ia++)
                memcpy(&t[((size_t)ix * 90 + ia) * D.nz], &g[(size_t)ia * n0 + (size_t)ix * D.nz], (size_t)D.nz * 4);
        GEO_TRY(open_out(name, f));
        return write_at(f.get(), 0, t.data(), t.size());
    };
    if (!fag.empty()) GEO_TRY(write_gathers(fag, ag));
    if (!fags.empty() || !fstk.empty()) {
        std::vector<float> stk(n0);
        GEO_TRY(geo_adcig_smooth_stack(D.nx, D.nz, 90, 10, ag.data(), stk.data(), GEO_MEM_HOST, nullptr));
        if (!fags.empty()) GEO_TRY(write_gathers(fags, ag));
        if (!fstk.empty()) {
            GEO_TRY(open_out(fstk, f));
            GEO_TRY(write_at(f.get(), 0, stk.data(), n0));
        }
    }
    if (d_image) GEO_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    return GEO_OK;
}
