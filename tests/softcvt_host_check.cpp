// Host build of the library's integer float <-> double conversions
// (geophysics_gb300/csrc/softcvt.cuh) checked against the host's IEEE 754
// conversions (round to nearest even): the widening over every binary32
// pattern except NaNs, the narrowing over random binary64 values from below
// the binary32 subnormal range to above its overflow threshold, exact ties
// of normal and subnormal results, and the binary64 images of random
// binary32 values.  Prints "f2d_bad d2f_bad".
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "softcvt.cuh"

using namespace geo;

static uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

int main(int argc, char **argv) {
    const long long n = argc > 1 ? atoll(argv[1]) : (1ll << 24);
    unsigned long long f2d_bad = 0, d2f_bad = 0;
    for (uint64_t i = 0; i < (1ull << 32); i++) {
        const uint32_t u = (uint32_t)i;
        if (((u >> 23) & 0xffu) == 0xffu && (u & 0x7fffffu)) continue;   // NaN: the hardware path
        const float f = sc_u2f(u);
        f2d_bad += sc_d2u(f2d_exact(f)) != sc_d2u((double)f);
    }
    for (long long k = 0; k < n; k++) {
        const uint64_t h = mix64(12345 ^ mix64((uint64_t)k)), h2 = mix64(h);
        const uint64_t sign = (h & 1ull) << 63, man = h2 & 0xfffffffffffffull;
        uint64_t b;
        switch (k & 3) {
            case 0: b = sign | ((uint64_t)(860 + (h >> 8) % 301) << 52) | man; break;
            case 1: b = sign | ((uint64_t)(897 + (h >> 8) % 254) << 52) | (man & ~((1ull << 29) - 1)) | (1ull << 28); break;
            case 2: {
                const uint64_t ex = 873 + (h >> 8) % 24;
                const int s = 926 - (int)ex;
                const uint64_t sig = ((man | (1ull << 52)) & ~((1ull << s) - 1)) | (1ull << (s - 1));
                b = sign | (ex << 52) | (sig & 0xfffffffffffffull);
                break;
            }
            default: {
                uint32_t u = (uint32_t)(h >> 16);
                if (((u >> 23) & 0xffu) == 0xffu) u &= 0xbfffffffu;
                b = sc_d2u((double)sc_u2f(u));
            }
        }
        const double d = sc_u2d(b);
        d2f_bad += sc_f2u(d2f_rn(d)) != sc_f2u((float)d);
    }
    printf("%llu %llu\n", f2d_bad, d2f_bad);
    return 0;
}
