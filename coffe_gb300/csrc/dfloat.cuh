// Double-float ("df") arithmetic: a value is the unevaluated sum hi + lo of
// two floats, |lo| <= ulp(hi)/2, giving about 48 significant bits on the FP32
// pipes.  Error-free transformations after Knuth (two-sum), Dekker
// (quick-two-sum) and the FMA-based exact product; the addition is the
// "sloppy" variant whose error is bounded relative to |x| + |y|, which is what
// FFT butterflies need.  Used by the mixed-precision FFTLog, where a plain
// FP32 transform is not accurate enough (its absolute error at high Fourier
// modes is amplified by the growing Gamma-ratio kernel).
#pragma once

#include <cuda_runtime.h>

struct dfl {
    float hi, lo;
};

__device__ __forceinline__ dfl df_quick_two_sum(float a, float b)
{
    const float s = a + b;
    return dfl{s, b - (s - a)};
}

__device__ __forceinline__ dfl df_two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return dfl{s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ dfl df_add(dfl x, dfl y)
{
    dfl s = df_two_sum(x.hi, y.hi);
    return df_quick_two_sum(s.hi, s.lo + (x.lo + y.lo));
}

__device__ __forceinline__ dfl df_neg(dfl x) { return dfl{-x.hi, -x.lo}; }
__device__ __forceinline__ dfl df_sub(dfl x, dfl y) { return df_add(x, df_neg(y)); }

__device__ __forceinline__ dfl df_mul(dfl x, dfl y)
{
    const float p = x.hi * y.hi;
    float e = fmaf(x.hi, y.hi, -p);
    e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, e));
    return df_quick_two_sum(p, e);
}

__device__ __forceinline__ dfl df_scale(dfl x, float f) // exact power-of-two scaling when f is one
{
    const float p = x.hi * f;
    const float e = fmaf(x.hi, f, -p) + x.lo * f;
    return df_quick_two_sum(p, e);
}

__device__ __forceinline__ dfl df_from_double(double d)
{
    const float hi = (float)d;
    return dfl{hi, (float)(d - (double)hi)};
}

__device__ __forceinline__ double df_to_double(dfl x) { return (double)x.hi + (double)x.lo; }

// The same split with integer operations only (a double-to-float conversion
// runs on the FP64 pipe, 1/64 of the FP32 rate): hi = the leading 24
// significant bits rounded half up, lo = the remainder kept to 22 bits, so
// |hi + lo - d| <= 2^-46 |d| and |lo| <= ulp(hi) / 2 for 2^-80 <= |d| < 2^128
// (hi rounds to infinity as a float conversion does).  Outside that range
// lo = 0 and hi is what a float keeps: the same leading bits down to 2^-126,
// zero below, infinity above, NaN for NaN.
__device__ __forceinline__ dfl df_from_double_bits(double d)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const unsigned top = (unsigned)(u >> 32);
    const int e = (int)((top >> 20) & 0x7ffu);
    const int E = e - 1023;
    const unsigned long long mant = u & 0xFFFFFFFFFFFFFull;
    const unsigned rbit = (unsigned)(mant >> 28) & 1u;
    const unsigned sign = top & 0x80000000u;
    // exponent and top 23 fraction bits; a rounding carry moves into the exponent
    const int Ec = E < -126 ? -126 : (E > 127 ? 127 : E);
    const unsigned hb = ((unsigned)(Ec + 127) << 23) + (unsigned)(mant >> 29) + rbit;
    // remainder in units of 2^(E - 52), in (-2^28, 2^28]; floor to units of 2^(E - 46)
    const int rem = ((int)(mant & 0x1FFFFFFFull) - (int)(rbit << 29)) >> 6;
    // |rem| <= 2^22: exact as a float through the 1.5 * 2^23 offset
    const float x = __int_as_float(0x4B400000 + rem) - 12582912.f;
    const int Es = E < -80 ? -80 : (E > 127 ? 127 : E);
    float lo = x * __int_as_float((Es - 46 + 127) << 23);
    unsigned hi = hb;
    if (E < -126) hi = 0u;                                        // zero, subnormal double
    if (E > 127) hi = e == 2047 && mant ? 0x7FC00000u : 0x7F800000u; // NaN / overflow
    if (E < -80 || E > 127) lo = 0.f;
    return dfl{__int_as_float((int)(hi | sign)), __int_as_float(__float_as_int(lo) ^ (int)sign)};
}

// float of a double (the high part above) and the exact double of a float,
// both with integer operations only
__device__ __forceinline__ float f32_of_bits(double d) { return df_from_double_bits(d).hi; }
__device__ __forceinline__ double f64_of_bits(float f)
{
    const unsigned u = __float_as_uint(f);
    const unsigned long long sign = (unsigned long long)(u & 0x80000000u) << 32;
    const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
    unsigned long long bits;
    if (e == 0xffu) // infinity / NaN
        bits = sign | (0x7ffull << 52) | ((unsigned long long)m << 29);
    else if (e != 0u) // normal
        bits = sign | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    else if (m == 0u) // zero
        bits = sign;
    else { // subnormal: m 2^-149 with the leading one of m at bit p
        const int p = 31 - __clz((int)m);
        bits = sign | ((unsigned long long)(p - 149 + 1023) << 52) |
               ((unsigned long long)(m ^ (1u << p)) << (52 - p));
    }
    return __longlong_as_double((long long)bits);
}

// complex double-float, stored as float4 (re.hi, re.lo, im.hi, im.lo)
struct dfc {
    dfl re, im;
};

__device__ __forceinline__ dfc dfc_load(const float4 v) { return dfc{{v.x, v.y}, {v.z, v.w}}; }
__device__ __forceinline__ float4 dfc_pack(dfc a) { return make_float4(a.re.hi, a.re.lo, a.im.hi, a.im.lo); }
__device__ __forceinline__ dfc dfc_add(dfc a, dfc b) { return dfc{df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ dfc dfc_sub(dfc a, dfc b) { return dfc{df_sub(a.re, b.re), df_sub(a.im, b.im)}; }
// Unnormalised intermediates for chains that end in a normalising df_add:
// the product x y as p + e with p = fl(x.hi y.hi) and e its error plus the
// cross terms (|e| may exceed ulp(p)/2), and the sum x + y as the exact
// two-sum of the high parts with the low parts added to its error.
__device__ __forceinline__ dfl df_mul_raw(dfl x, dfl y)
{
    const float p = x.hi * y.hi;
    const float e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, fmaf(x.hi, y.hi, -p)));
    return dfl{p, e};
}
__device__ __forceinline__ dfl df_add_raw(dfl x, dfl y)
{
    const dfl s = df_two_sum(x.hi, y.hi);
    return dfl{s.hi, s.lo + (x.lo + y.lo)};
}
__device__ __forceinline__ dfc dfc_add_raw(dfc a, dfc b)
{
    return dfc{df_add_raw(a.re, b.re), df_add_raw(a.im, b.im)};
}
__device__ __forceinline__ dfc dfc_sub_raw(dfc a, dfc b)
{
    return dfc{df_add_raw(a.re, df_neg(b.re)), df_add_raw(a.im, df_neg(b.im))};
}

// complex product: each component one normalising sum of two raw products
__device__ __forceinline__ dfc dfc_mul(dfc a, dfc b)
{
    return dfc{df_add(df_mul_raw(a.re, b.re), df_neg(df_mul_raw(a.im, b.im))),
               df_add(df_mul_raw(a.re, b.im), df_mul_raw(a.im, b.re))};
}
__device__ __forceinline__ dfc dfc_conj(dfc a) { return dfc{a.re, df_neg(a.im)}; }
__device__ __forceinline__ dfc dfc_neg(dfc a) { return dfc{df_neg(a.re), df_neg(a.im)}; }
__device__ __forceinline__ dfc dfc_from_double2(double2 v) { return dfc{df_from_double(v.x), df_from_double(v.y)}; }
