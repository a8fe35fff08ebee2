// boids_softfp.h -- exact (float)((double)a + b) with integer arithmetic.
//
// The reference shifts a float coordinate by the double field size and
// stores the result back into a float (src/boid_simulation_grid.cpp:200-214
// for the periodic image, :274-289 for the wrap), i.e. it rounds twice:
// first to double, then to float.  GB300 executes FP64 at a small fraction of
// its FP32 rate, so the kernels never use double: this header reproduces
// the two roundings bit for bit with 64-bit integer operations.  The same
// code compiles for the host, where tests compare it with real double
// arithmetic.
#pragma once

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define BOIDS_HD __host__ __device__
#define BOIDS_HD_NOINLINE __host__ __device__ __noinline__
#else
#define BOIDS_HD
#define BOIDS_HD_NOINLINE
#endif

namespace boidsgpu {

// A positive finite double in integer form: value = mant * 2^exp with mant in
// [2^52, 2^53) (or a subnormal mantissa with exp = -1074).
struct SoftDouble {
    uint64_t mant;
    int32_t exp;
    int32_t pad;
};

BOIDS_HD inline uint32_t f32_bits(float x)
{
#ifdef __CUDA_ARCH__
    return __float_as_uint(x);
#else
    uint32_t u;
    memcpy(&u, &x, 4);
    return u;
#endif
}

BOIDS_HD inline float f32_from_bits(uint32_t u)
{
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float x;
    memcpy(&x, &u, 4);
    return x;
#endif
}

BOIDS_HD inline int clz64(uint64_t x)
{
#ifdef __CUDA_ARCH__
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

inline SoftDouble soft_double(double d)  // host only; d > 0 and finite
{
    uint64_t u;
    memcpy(&u, &d, 8);
    const int E = (int)((u >> 52) & 0x7ff);
    const uint64_t f = u & ((1ULL << 52) - 1);
    SoftDouble s;
    if (E == 0) {
        s.mant = f;
        s.exp = -1074;
    } else {
        s.mant = f | (1ULL << 52);
        s.exp = E - 1075;
    }
    s.pad = 0;
    return s;
}

// (float)((double)a + (neg_b ? -b : b)) with round-to-nearest-even at both
// steps.  a must be finite (a NaN or infinity is returned unchanged).
BOIDS_HD_NOINLINE inline float add_f32_f64_rn(float a, SoftDouble b, int neg_b)
{
    const uint32_t ua = f32_bits(a);
    const int Ea = (int)((ua >> 23) & 0xff);
    if (Ea == 0xff) return a;
    const int sa = (int)(ua >> 31);
    uint64_t ma = ua & 0x7fffffu;
    int ea;
    if (Ea == 0) {
        ea = -149;
    } else {
        ma |= 0x800000u;
        ea = Ea - 150;
    }
    // normalise both mantissas to [2^52, 2^53)
    uint64_t mb = b.mant;
    int eb = b.exp;
    if (mb == 0 && ma == 0) return f32_from_bits((uint32_t)(sa & neg_b) << 31);
    if (ma) {
        const int sh = clz64(ma) - 11;
        ma <<= sh;
        ea -= sh;
    }
    if (mb) {
        const int sh = clz64(mb) - 11;
        mb <<= sh;
        eb -= sh;
    }
    // x: the operand of larger magnitude
    uint64_t mx, my;
    int ex, ey, sx, sy;
    const bool a_big = ma != 0 && (mb == 0 || ea > eb || (ea == eb && ma >= mb));
    if (a_big) {
        mx = ma; ex = ea; sx = sa; my = mb; ey = eb; sy = neg_b;
    } else {
        mx = mb; ex = eb; sx = neg_b; my = ma; ey = ea; sy = sa;
    }
    // 8 guard bits; the smaller operand keeps a sticky bit when shifted
    uint64_t X = mx << 8, Y = my << 8;
    const int d = ex - ey;
    if (my == 0) {
        Y = 0;
    } else if (d >= 62) {
        Y = 1;
    } else if (d > 0) {
        const uint64_t lost = Y & ((1ULL << d) - 1);
        Y = (Y >> d) | (lost != 0);
    }
    uint64_t S = sx == sy ? X + Y : X - Y;  // X >= Y by construction
    if (S == 0) return 0.0f;                // exact cancellation: +0 under RN
    int e = ex - 8;                         // value = S * 2^e
    const int L = 64 - clz64(S);
    if (L > 61) {
        const int sh = L - 61;
        const uint64_t lost = S & ((1ULL << sh) - 1);
        S = (S >> sh) | (lost != 0);
        e += sh;
    } else if (L < 61) {
        const int sh = 61 - L;
        S <<= sh;
        e -= sh;
    }
    // first rounding: 61 -> 53 bits (double)
    uint64_t m = S >> 8;
    const uint32_t g = (uint32_t)(S & 0xff);
    if (g > 0x80 || (g == 0x80 && (m & 1))) {
        if (++m == (1ULL << 53)) {
            m >>= 1;
            e += 1;
        }
    }
    e += 8;  // value = m * 2^e, m in [2^52, 2^53)
    // second rounding: 53 bits -> float (24 bits, fewer for a subnormal)
    const uint32_t sign = (uint32_t)sx << 31;
    int E = e + 179;  // float exponent field of m * 2^e when normal
    int drop = 29;
    if (E <= 0) {
        drop += 1 - E;
        E = 0;
        if (drop > 54) return f32_from_bits(sign);
    }
    uint64_t q = m >> drop;
    const uint64_t rem = m & ((1ULL << drop) - 1), half = 1ULL << (drop - 1);
    if (rem > half || (rem == half && (q & 1))) ++q;
    if (E == 0) return f32_from_bits(sign | (uint32_t)q);  // q == 2^23 encodes the smallest normal
    if (q == (1ULL << 24)) {
        q >>= 1;
        ++E;
    }
    if (E >= 0xff) return f32_from_bits(sign | 0x7f800000u);
    return f32_from_bits(sign | ((uint32_t)E << 23) | ((uint32_t)q & 0x7fffffu));
}

}  // namespace boidsgpu
