// Float-float ("double-single") arithmetic on the FP32 pipe.
//
// On GB300 the FP64 pipe issues at 1/64 of the FP32 rate, so the element
// kernels carry their inner products as unevaluated sums hi + lo of two
// floats (Dekker 1971; error-free transformations TwoSum (Knuth) and
// TwoProd via FMA), which gives about 44-48 significant bits.  Conversions
// between double and float-float are done with integer operations so that
// they do not occupy the FP64 pipe.
//
// Range: values must stay within the normal float range (about 1e-38 to
// 3e38); callers check their inputs and fall back to FP64 otherwise.
#pragma once
#include <stdint.h>

namespace fe3d {

struct ff {
    float h, l;
};

__device__ __forceinline__ ff ff_make(float h) { return {h, 0.f}; }

// a * b (TwoProd with FMA, plus the cross terms)
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    const float s = p + e;
    return {s, e - (s - p)};
}

// a * b + c
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c) {
    const float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    const float s = p + c.h;
    const float v = s - p;
    float t = (p - (s - v)) + (c.h - v);
    t += e + c.l;
    const float hs = s + t;
    return {hs, t - (hs - s)};
}

__device__ __forceinline__ ff ff_add(ff a, ff b) {
    const float s = a.h + b.h;
    const float v = s - a.h;
    float t = (a.h - (s - v)) + (b.h - v);
    t += a.l + b.l;
    const float hs = s + t;
    return {hs, t - (hs - s)};
}

__device__ __forceinline__ ff ff_neg(ff a) { return {-a.h, -a.l}; }

// exact scaling by a power of two
__device__ __forceinline__ ff ff_scale(ff a, float pow2) { return {a.h * pow2, a.l * pow2}; }

// 1 / a: float reciprocal refined by one Newton step in float-float
__device__ __forceinline__ ff ff_rcp(ff a) {
    const float r = 1.f / a.h;
    // e = 1 - a * r (in float-float), r' = r + r e
    const ff ar = ff_mul(a, ff_make(r));
    const ff e = ff_add(ff_make(1.f), ff_neg(ar));
    return ff_fma(ff_make(r), e, ff_make(r));
}

// double -> float-float with integer operations (round-to-nearest hi, the
// remainder rounded to float).  Zero and values outside the normal float
// range map to {x as float, 0}; callers range-check beforehand.
__device__ __forceinline__ ff ff_from_double(double x) {
    const uint64_t b = (uint64_t)__double_as_longlong(x);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const int ed = (int)((b >> 52) & 0x7ffu);
    const int ef = ed - 1023 + 127;
    if (ed == 0 || ef <= 1 || ef >= 254) return {__uint_as_float(sign), 0.f};
    const uint64_t m = (b & 0xfffffffffffffull) | (1ull << 52);  // 53 bits
    uint64_t mh = m >> 29;                                        // 24 bits
    const uint64_t rem = m & ((1ull << 29) - 1);
    const uint64_t half = 1ull << 28;
    if (rem > half || (rem == half && (mh & 1ull))) mh += 1;
    // remainder d = m - mh * 2^29, |d| <= 2^28, scaled like m
    const int64_t d = (int64_t)m - (int64_t)(mh << 29);
    int eh = ef;
    if (mh >> 24) {  // rounding carried into a new binade
        mh >>= 1;
        eh += 1;
    }
    const float hi = __uint_as_float(sign | ((uint32_t)eh << 23) | ((uint32_t)mh & 0x7fffffu));
    if (d == 0) return {hi, 0.f};
    // lo = d * 2^(ed - 1023 - 52), built from |d| (<= 29 bits) with RN to 24 bits
    uint64_t ad = (uint64_t)(d < 0 ? -d : d);
    const int lz = __clzll((long long)ad);  // leading zeros in 64 bits
    const int msb = 63 - lz;                // position of the leading one
    int el = (ed - 1023 - 52) + msb + 127;  // biased float exponent of lo
    uint32_t ml;
    if (msb > 23) {
        const int sh = msb - 23;
        uint64_t q = ad >> sh;
        const uint64_t r = ad & ((1ull << sh) - 1), hf = 1ull << (sh - 1);
        if (r > hf || (r == hf && (q & 1ull))) q += 1;
        if (q >> 24) {
            q >>= 1;
            el += 1;
        }
        ml = (uint32_t)q;
    } else {
        ml = (uint32_t)(ad << (23 - msb));
    }
    if (el <= 0) return {hi, 0.f};
    const uint32_t lsign = (d < 0) ? (sign ^ 0x80000000u) : sign;
    const float lo = __uint_as_float(lsign | ((uint32_t)el << 23) | (ml & 0x7fffffu));
    return {hi, lo};
}

// float-float -> double with integer operations, rounded to nearest.
// Requires a normalised pair (|l| <= ulp(h) / 2).
__device__ __forceinline__ double ff_to_double(ff a) {
    const uint32_t hb = __float_as_uint(a.h);
    const uint32_t eh = (hb >> 23) & 0xffu;
    if (eh == 0u) return __longlong_as_double((long long)((uint64_t)(hb & 0x80000000u) << 32));
    const uint32_t lb = __float_as_uint(a.l);
    const uint32_t el = (lb >> 23) & 0xffu;
    uint64_t S = (uint64_t)((hb & 0x7fffffu) | 0x800000u) << 40;  // leading one at bit 63
    if (el != 0u && eh > el) {
        const uint32_t sh = eh - el;
        if (sh < 64u) {
            const uint64_t L = ((uint64_t)((lb & 0x7fffffu) | 0x800000u) << 40) >> sh;
            S = ((hb ^ lb) >> 31) ? S - L : S + L;
        }
    }
    int e = (int)eh;
    if (!(S >> 63)) {
        S <<= 1;
        e -= 1;
    }
    uint64_t m = S >> 11;  // 53 bits with the implicit one at bit 52
    const uint64_t r = S & 0x7ffull;
    if (r > 0x400ull || (r == 0x400ull && (m & 1ull))) m += 1;
    const uint64_t bits = ((uint64_t)(hb >> 31) << 63) + ((uint64_t)(e + 1023 - 127 - 1) << 52) + m;
    return __longlong_as_double((long long)bits);
}

// true when |x| is zero or inside [2^-100, 2^100]: products of a few such
// values stay in the normal float range
__device__ __forceinline__ bool ff_safe(double x) {
    const int ed = (int)(((uint64_t)__double_as_longlong(x) >> 52) & 0x7ffu);
    return ed == 0 ? (x == 0.) : (ed >= 1023 - 100 && ed <= 1023 + 100);
}

}  // namespace fe3d
