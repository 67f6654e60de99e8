// Exact float <-> double conversions on the integer pipe.
//
// GB300 issues the hardware conversions F32->F64 and F64->F32 on its FP64
// pipe at about the FP64 add rate (measured: about 600 G conversions/s
// against 500 G double adds/s and 36 T float adds/s), so the MPI program's
// double chains (a float product widened, a double product and difference,
// the result narrowed) spend more of that pipe on conversions than on
// arithmetic.  These two functions give the same bits from integer
// operations, following the IEEE 754-2008 definitions:
//   widen:  every binary32 value is exactly representable in binary64
//           (normals rebias the exponent, subnormals are normalised, zeros
//           and infinities keep their sign);
//   narrow: round to nearest, ties to even (roundTiesToEven, §4.3.1), with
//           overflow to infinity, gradual underflow to subnormals and zero.
// A NaN (which a finite run never produces) takes the hardware conversion.
// geo_selftest_conversions() checks both against the hardware conversions:
// every binary32 for the widening, and random and boundary binary64 values
// (ties, subnormal and overflow edges) for the narrowing.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define GEO_SC_FN __host__ __device__ __forceinline__
#else
#define GEO_SC_FN inline
#endif

namespace geo {

// bit casts and the leading-zero count on either side (the host build is
// the CPU check of the same code)
GEO_SC_FN uint32_t sc_f2u(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
#endif
}
GEO_SC_FN float sc_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(u);
#else
    float f;
    memcpy(&f, &u, 4);
    return f;
#endif
}
GEO_SC_FN uint64_t sc_d2u(double d) {
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t u;
    memcpy(&u, &d, 8);
    return u;
#endif
}
GEO_SC_FN double sc_u2d(uint64_t u) {
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)u);
#else
    double d;
    memcpy(&d, &u, 8);
    return d;
#endif
}
GEO_SC_FN int sc_clz(uint32_t x) {   // x != 0
#if defined(__CUDA_ARCH__)
    return __clz(x);
#else
    return __builtin_clz(x);
#endif
}

GEO_SC_FN double f2d_exact(float f) {
    const uint32_t u = sc_f2u(f);
    const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
    const uint32_t ex = (u >> 23) & 0xffu, man = u & 0x7fffffu;
    uint64_t bits;
    if (ex != 0 && ex != 0xffu) {
        bits = sign | ((uint64_t)(ex + (1023 - 127)) << 52) | ((uint64_t)man << 29);
    } else if (ex == 0xffu) {
        if (man) return (double)f;   // NaN: the hardware's own quieting (never on a finite run)
        bits = sign | (0x7ffull << 52);
    } else if (man == 0) {
        bits = sign;
    } else {
        // subnormal: man * 2^-149 = 1.f * 2^(p - 149), p the leading one's position
        const int p = 31 - sc_clz(man);
        bits = sign | ((uint64_t)(p - 149 + 1023) << 52) | (((uint64_t)man << (52 - p)) & 0xfffffffffffffull);
    }
    return sc_u2d(bits);
}

GEO_SC_FN float d2f_rn(double d) {
    const uint64_t b = sc_d2u(d);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const int ex = (int)((b >> 52) & 0x7ffu);
    const uint64_t m = b & 0xfffffffffffffull;
    if (ex == 0x7ff) {
        if (m) return (float)d;   // NaN: the hardware's own quieting (never on a finite run)
        return sc_u2f(sign | 0x7f800000u);
    }
    const uint64_t sig = ex ? (m | (1ull << 52)) : m;   // 53-bit significand (value = sig * 2^(ex-1075))
    const int e = ex - 1023 + 127;                       // binary32 biased exponent of a normal result
    uint32_t q;
    uint64_t rem, half;
    if (e >= 1) {
        q = (uint32_t)(sig >> 29);
        rem = sig & ((1ull << 29) - 1);
        half = 1ull << 28;
    } else {
        // subnormal or zero result: units of 2^-149, sig * 2^(ex-1075) / 2^-149 = sig >> s
        const int s = 926 - ex;   // >= 29 + (1 - e)
        if (s >= 64) return sc_u2f(sign);
        q = (uint32_t)(sig >> s);
        rem = sig & ((1ull << s) - 1);
        half = 1ull << (s - 1);
    }
    if (rem > half || (rem == half && (q & 1u))) q++;
    if (e >= 1) {
        // a carry out of the 24-bit significand moves to the next binade
        uint32_t E = (uint32_t)e;
        if (q == (1u << 24)) {
            q >>= 1;
            E++;
        }
        if (E >= 0xffu) return sc_u2f(sign | 0x7f800000u);
        return sc_u2f(sign | (E << 23) | (q & 0x7fffffu));
    }
    // q <= 2^23: a carry into bit 23 is the smallest normal, which the
    // bit pattern already encodes
    return sc_u2f(sign | q);
}

}  // namespace geo
