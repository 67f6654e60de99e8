// The device's single-precision cos and sin of n angles (radians): the
// values the reference's GPU TTI programs compute for their tilt inside
// their kernels (cos(theta[id]), sin(theta[id]) of a float,
// 2D-tti-fd+rtm-cuda/Toa_gpu_2dtti_fd_1orderfunction.cu:106-107).  Test
// infrastructure: the CPU oracle cannot reproduce the device's cosf/sinf
// bit for bit, so the tests hand it these values (oracle/refgpu.py,
// cuda_trig).  Built with contraction off, as the library is.
extern "C" __global__ void k_ref_trig(const float *th, float *c, float *s, long n) {
    for (long k = blockIdx.x * (long)blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) {
        c[k] = cosf(th[k]);
        s[k] = sinf(th[k]);
    }
}

// The GPU RTM programs' Poynting angle bin of a cosine a, with the device's
// acosf (Poynting_Adcigs, 2D-vti-fd+rtm-cuda/Toa_gpu2DvtiFdRtmAdcigsLaplace.cu:718-766):
//   ia = (int)((float)(0.5*acosf(a)*180/pi) / (da*1.0)),  pi = 3.141592653.
// k_ref_bin_thresholds finds the cosines where that bin steps;
// k_ref_bin_check evaluates the bin for every float in [-1, 1] and counts
// the floats whose bin (capped at na, "not kept") differs from the number
// of thresholds thr[0..na) at or above a.  Zero for the device's own
// thresholds means the thresholds reproduce the device's bins for every
// possible cosine (the bin does not go back up anywhere); for thresholds a
// host computed from its acosf, the count is the floats the two acosf put
// in different bins.
__device__ static unsigned ord_key(float f) {
    const unsigned b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__device__ static float key_float(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

__device__ static int ref_bin(float a, int da) {
    const float deg = (float)(0.5 * acosf(a) * 180.0 / 3.141592653);
    return (int)(deg / (da * 1.0));
}

// thr[k] = largest float a in [-1, 1] whose device bin is >= k+1 (binary
// search over the ordered floats), -2 where none is; one thread per k < na.
extern "C" __global__ void k_ref_bin_thresholds(float *thr, int na, int da) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= na) return;
    float t = -2.0f;
    if (ref_bin(-1.0f, da) >= k + 1) {
        unsigned lo = ord_key(-1.0f), hi = ord_key(1.0f);
        while (lo < hi) {
            const unsigned m = lo + (hi - lo + 1) / 2;
            if (ref_bin(key_float(m), da) >= k + 1) lo = m;
            else hi = m - 1;
        }
        t = key_float(lo);
    }
    thr[k] = t;
}

extern "C" __global__ void k_ref_bin_check(const float *thr, int na, int da, unsigned long long *bad) {
    const unsigned lo = ord_key(-1.0f), hi = ord_key(1.0f);
    const unsigned long long n = (unsigned long long)(hi - lo) + 1;
    unsigned long long nbad = 0;
    for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
         k += (unsigned long long)gridDim.x * blockDim.x) {
        const float a = key_float(lo + (unsigned)k);
        int ia = ref_bin(a, da);
        if (ia > na) ia = na;
        int c = 0;
        while (c < na && a <= thr[c]) c++;
        nbad += (ia != c);
    }
    atomicAdd(bad, nbad);
}
