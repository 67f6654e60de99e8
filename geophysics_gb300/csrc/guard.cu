// Failure detection during propagation: the wavefield watchdog and the
// stability checks of the reference's set-up code.
//
// Watchdog.  Every `every` time steps a run launches k_watch over its
// current pressure field(s); the first non-finite value (NaN or +-Inf: a
// diverging run, e.g. a pseudo-acoustic VTI medium with delta > epsilon,
// overflows within a few hundred steps) makes the block write the step's
// tag into a word of mapped pinned host memory.  The host reads that word
// while it queues the next steps, stops queueing as soon as it is set and
// returns GEO_ERR_NAN once the stream has drained, so a blown-up shot ends
// early with a status instead of running to its end.  Nothing faults and
// nothing waits on the device.  GEO_WATCH_EVERY=K sets the interval
// (default 100 steps; 0 turns the watchdog off).
//
// Stability.  stability_number() is the Madagascar-derived check the
// reference's RTM set-up applies (Toa_gpu2DvtiFdRtmAdcigsLaplace.cu:952-965,
// C = 0.777 for the 8th-order operator, mm = 4): dt*vmax*sqrt(sum 1/d^2).
// Every entry point refuses a run whose number reaches C (GEO_ERR_CFL);
// the CPU program's get_constant limits (CPU_vti2dfd_kernels.c:179-219),
// whose failure leaves its sponge constant undefined, are checked for the
// CPU variant as well.
#include "geo_internal.h"
#include <cfloat>
#include <cmath>
#include <cstdlib>

namespace geo {

namespace {

__global__ void k_watch(const float *__restrict__ a, size_t n, int *flag, int tag) {
    bool bad = false;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
        bad |= !(fabsf(a[k]) <= FLT_MAX);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicCAS(flag, 0, tag);
}

__global__ void k_minmax(const float *__restrict__ a, size_t n, unsigned *out) {
    unsigned lo = 0x7f800000u, hi = 0u;
    for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x) {
        const unsigned b = __float_as_uint(a[k]);
        lo = min(lo, b);
        hi = max(hi, b);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(out, lo);
        atomicMax(out + 1, hi);
    }
}

}  // namespace

int launch_minmax(const float *a, size_t n, unsigned *out, cudaStream_t s) {
    const unsigned init[2] = {0x7f800000u, 0u};
    GEO_CUDA(cudaMemcpyAsync(out, init, sizeof init, cudaMemcpyHostToDevice, s));
    const int grid = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
    k_minmax<<<grid, 256, 0, s>>>(a, n, out);
    return check_launch("minmax");
}

int watch_every() {
    const char *s = getenv("GEO_WATCH_EVERY");
    if (!s || !*s) return 100;
    const int k = atoi(s);
    return k > 0 ? k : 0;
}

int Watchdog::open() {
    every = watch_every();
    if (h) return GEO_OK;
    GEO_CUDA(cudaHostAlloc((void **)&h, sizeof(int), cudaHostAllocMapped));
    GEO_CUDA(cudaHostGetDevicePointer((void **)&d, h, 0));
    *(volatile int *)h = 0;
    return GEO_OK;
}

void Watchdog::close() {
    if (h) cudaFreeHost(h);
    h = d = nullptr;
}

void Watchdog::arm() {
    every = watch_every();
    if (h) *(volatile int *)h = 0;
}

bool Watchdog::tripped() const { return h && *(volatile const int *)h != 0; }

int Watchdog::check(const float *a, size_t n, int it, bool last, cudaStream_t s) {
    if (!h || every <= 0 || ((it + 1) % every && !last)) return GEO_OK;
    const int grid = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
    k_watch<<<grid, 256, 0, s>>>(a, n, d, it + 1);
    GEO_TRY(check_launch("watch"));
    return tripped() ? GEO_ERR_NAN : GEO_OK;
}

int Watchdog::scan(const float *a, size_t n, int tag, cudaStream_t s) {
    if (!h || every <= 0) return GEO_OK;
    const int grid = (int)std::min<size_t>((n + 255) / 256, 152 * 8);
    k_watch<<<grid, 256, 0, s>>>(a, n, d, tag);
    return check_launch("watch");
}

int Watchdog::verdict(cudaStream_t s, const char *what) {
    if (!h) return GEO_OK;
    GEO_CUDA(cudaStreamSynchronize(s));
    const int tag = *(volatile int *)h;
    if (tag > 0) return fail(GEO_ERR_NAN, "%s: wavefield non-finite by time step %d", what, tag);
    if (tag < 0) return fail(GEO_ERR_NAN, "%s: non-finite values in the result", what);
    return GEO_OK;
}

double stability_number(int dims, float vmax, float dt, float dx, float dy, float dz) {
    double s = 1.0 / ((double)dx * dx) + 1.0 / ((double)dz * dz);
    if (dims == 3) s += 1.0 / ((double)dy * dy);
    return (double)dt * vmax * std::sqrt(s);
}

int check_stability(Variant v, int dims, float vmin, float vmax, float dt, float dx, float dy, float dz,
                    float favg) {
    if (!(vmax > 0) || !std::isfinite(vmax)) return fail(GEO_ERR_MODEL, "velocity maximum %g", vmax);
    const double c = stability_number(dims, vmax, dt, dx, dy, dz);
    if (!(c < kStabilityC))
        return fail(GEO_ERR_CFL, "stability condition not satisfied: dt*vmax*sqrt(sum 1/d^2) = %.4f >= %.3f", c,
                    kStabilityC);
    if (v == V_CPU) {
        // get_constant (CPU_vti2dfd_kernels.c:179-219): five points per
        // shortest wavelength and dt <= 0.5*min(dx,dz)/vmax
        const float hmin = dx < dz ? dx : dz;
        const float dmax = vmin / favg * 0.2f;
        if (dmax < dx || dmax < dz)
            return fail(GEO_ERR_CFL, "grid spacing above vmin/favg*0.2 = %g (redefine dx, dz)", dmax);
        if ((float)(0.5 * hmin / vmax) < dt) return fail(GEO_ERR_CFL, "dt above 0.5*min(dx,dz)/vmax (redefine dt)");
    }
    return GEO_OK;
}

}  // namespace geo
