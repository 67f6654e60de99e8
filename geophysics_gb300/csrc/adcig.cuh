// Poynting opening-angle bin of the GPU RTM programs' angle gathers
// (Poynting_Adcigs, 3D-vti-fd+rtm-cuda/Toa_gpu_3dvti_rtm_adcigs_1orderfunction.cu:642-650;
// the 2D program's Poynting_Adcigs, 2D-vti-fd+rtm-cuda/Toa_gpu2DvtiFdRtmAdcigsLaplace.cu):
//   a = (S.G) / (sqrtf(b1*b2) * (1 - 0.1))   -- a double quotient stored as float
//   if -1 <= a <= 1:  ia = (int)((float)(0.5*acosf(a)*180/pi) / (da*1.0)),  kept if ia < na.
// The acosf expression becomes thresholds, found once per run on the device
// with the device's acosf (k_angle_tables): thr[k-1] is the largest float a
// with bin(a) >= k (non-increasing in k, -2 where no float in [-1,1]
// reaches bin k), so the bin of a is the number of thresholds at or above a
// and no acosf runs per point.  The host's acosf would not do: it bins a
// few dozen of the floats in [-1,1] next to a bin edge differently.
//
// The quotient is first formed in float.  Against the exact quotient its
// relative error is below 2.1e-7 (0.9f against 0.9, one product and one
// division, each within half an ulp), so when the float value lies farther
// than 1e-6*(|a|+|t|) from the thresholds t on either side of it and farther
// than 2e-6 from +-1, it gives the same decisions as the rounded double
// quotient.  Otherwise -- and for a denominator outside [1e-30, 1e30], where
// the float product could lose precision -- the double quotient is formed as
// the programs form it.  Only a few points in a million take that path.
#pragma once

namespace geo {

constexpr int kMaxAngles = 128;

// Number of thresholds thr[0..na) at or above a (a prefix, thr non-increasing).
__device__ __forceinline__ int angle_count(float a, const float *thr, int na) {
    int lo = 0, hi = na;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a <= thr[mid - 1]) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ bool angle_near(float a, float t) {
    return fabsf(a - t) <= 1e-6f * (fabsf(a) + fabsf(t));
}

// Bin of the pair (S.G, |S|^2, |G|^2), or -1 when the program adds nothing.
__device__ __forceinline__ int poynting_bin(float dot, float b1, float b2, const float *thr, int na) {
    const float den = sqrtf(b1 * b2);
    if (den >= 1e-30f && den <= 1e30f) {
        const float a = dot / (den * 0.9f);
        const float m = fabsf(a);
        if (!(m <= 1.0f + 2e-6f)) return -1;          // out of range (also inf, NaN)
        if (m < 1.0f - 2e-6f) {
            const int k = angle_count(a, thr, na);
            const bool edge = (k > 0 && angle_near(a, thr[k - 1])) || (k < na && angle_near(a, thr[k]));
            if (!edge) return k < na ? k : -1;
        }
    }
    const float a = (float)((double)dot / ((double)den * (1 - 0.1)));
    if (!(a >= -1.0f && a <= 1.0f)) return -1;
    const int k = angle_count(a, thr, na);
    return k < na ? k : -1;
}

}  // namespace geo
