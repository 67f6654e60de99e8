// SU / SEG-Y trace files (host code).
//
// A trace is a 240-byte header followed by ns 4-byte float samples.  The
// MPI RTM program reads models this way when seismic == 2 (read_v_e_d_r,
// 2D-vti-fd+rtm-mpi/Toa_rtm_vti_adcig_cdp.c:1415-1453: trace i of nz samples
// starts at byte (i+1)*240 + i*nz*4, samples big-endian, swapped on read).
// The binary2segy utility (utils-binary2segy/binary2segy.c:47-85) copies
// each 240-byte header of a template SU file unchanged and replaces the
// samples by those of a raw native-endian file, byte-swapped.  Header fields
// written here (the segy struct of hc/cjbsegy.h): tracl @0, tracr @4 (int),
// trid @28 (short), ns @114, dt @116 (unsigned short, microseconds).
#include "geo_internal.h"
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>

namespace geo {

constexpr int kSuHdr = 240;

static uint32_t bswap32(uint32_t x) {
    return (x >> 24) | ((x >> 8) & 0xff00u) | ((x << 8) & 0xff0000u) | (x << 24);
}
static uint16_t bswap16(uint16_t x) { return (uint16_t)((x >> 8) | (x << 8)); }

static void put32(unsigned char *h, int off, uint32_t v, bool be) {
    if (be) v = bswap32(v);
    memcpy(h + off, &v, 4);
}
static void put16(unsigned char *h, int off, uint16_t v, bool be) {
    if (be) v = bswap16(v);
    memcpy(h + off, &v, 2);
}

static void swap_floats(float *a, size_t n) {
    for (size_t k = 0; k < n; k++) {
        uint32_t u;
        memcpy(&u, a + k, 4);
        u = bswap32(u);
        memcpy(a + k, &u, 4);
    }
}

struct FileCloser {
    void operator()(FILE *f) const {
        if (f) fclose(f);
    }
};
using File = std::unique_ptr<FILE, FileCloser>;

}  // namespace geo

using namespace geo;

extern "C" int geo_su_read(const char *path, int ntr, int ns, int big_endian, float *data, void *headers) {
    if (!path || !data || ntr < 1 || ns < 1) return fail(GEO_ERR_ARG, "bad argument");
    File f(fopen(path, "rb"));
    if (!f) return fail(GEO_ERR_IO, "cannot open %s", path);
    unsigned char h[kSuHdr];
    for (int i = 0; i < ntr; i++) {
        if (fread(h, 1, kSuHdr, f.get()) != (size_t)kSuHdr)
            return fail(GEO_ERR_IO, "%s: short header at trace %d", path, i);
        if (headers) memcpy(static_cast<unsigned char *>(headers) + (size_t)i * kSuHdr, h, kSuHdr);
        float *t = data + (size_t)i * ns;
        if (fread(t, 4, (size_t)ns, f.get()) != (size_t)ns)
            return fail(GEO_ERR_IO, "%s: short trace %d", path, i);
        if (big_endian) swap_floats(t, (size_t)ns);
    }
    return GEO_OK;
}

extern "C" int geo_su_write(const char *path, int ntr, int ns, float dt_us, int big_endian, const float *data,
                            const void *headers) {
    if (!path || !data || ntr < 1 || ns < 1 || ns > 65535) return fail(GEO_ERR_ARG, "bad argument");
    if (!headers && !(dt_us > 0 && dt_us <= 65535)) return fail(GEO_ERR_ARG, "dt must be 1..65535 microseconds");
    File f(fopen(path, "wb"));
    if (!f) return fail(GEO_ERR_IO, "cannot create %s", path);
    unsigned char h[kSuHdr];
    std::vector<float> t((size_t)ns);
    for (int i = 0; i < ntr; i++) {
        if (headers) {
            memcpy(h, static_cast<const unsigned char *>(headers) + (size_t)i * kSuHdr, kSuHdr);
        } else {
            memset(h, 0, kSuHdr);
            put32(h, 0, (uint32_t)(i + 1), big_endian);     // tracl
            put32(h, 4, (uint32_t)(i + 1), big_endian);     // tracr
            put16(h, 28, 1, big_endian);                    // trid: seismic data
            put16(h, 114, (uint16_t)ns, big_endian);        // ns
            put16(h, 116, (uint16_t)(dt_us + 0.5f), big_endian);  // dt
        }
        memcpy(t.data(), data + (size_t)i * ns, (size_t)ns * 4);
        if (big_endian) swap_floats(t.data(), (size_t)ns);
        if (fwrite(h, 1, kSuHdr, f.get()) != (size_t)kSuHdr || fwrite(t.data(), 4, (size_t)ns, f.get()) != (size_t)ns)
            return fail(GEO_ERR_IO, "%s: write failed at trace %d", path, i);
    }
    return GEO_OK;
}

extern "C" int geo_su_replace_data(const char *template_path, const char *raw_path, const char *out_path, int ntr,
                                   int ns) {
    if (!template_path || !raw_path || !out_path || ntr < 1 || ns < 1) return fail(GEO_ERR_ARG, "bad argument");
    File ft(fopen(template_path, "rb")), fr(fopen(raw_path, "rb")), fo(fopen(out_path, "wb"));
    if (!ft || !fr || !fo) return fail(GEO_ERR_IO, "cannot open the template, raw or output file");
    unsigned char h[kSuHdr];
    std::vector<float> t((size_t)ns);
    for (int i = 0; i < ntr; i++) {
        if (fread(h, 1, kSuHdr, ft.get()) != (size_t)kSuHdr || fseek(ft.get(), (long)ns * 4, SEEK_CUR) != 0)
            return fail(GEO_ERR_IO, "%s: short trace %d", template_path, i);
        if (fread(t.data(), 4, (size_t)ns, fr.get()) != (size_t)ns)
            return fail(GEO_ERR_IO, "%s: short trace %d", raw_path, i);
        swap_floats(t.data(), (size_t)ns);
        if (fwrite(h, 1, kSuHdr, fo.get()) != (size_t)kSuHdr || fwrite(t.data(), 4, (size_t)ns, fo.get()) != (size_t)ns)
            return fail(GEO_ERR_IO, "%s: write failed at trace %d", out_path, i);
    }
    return GEO_OK;
}
