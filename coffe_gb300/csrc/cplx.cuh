// Minimal FP64 complex arithmetic for the FFTLog Gamma-ratio coefficients.
#pragma once

#include "common.cuh"

struct cplx {
    double re, im;
};

__device__ __forceinline__ cplx cx(double r, double i) { return cplx{r, i}; }
__device__ __forceinline__ cplx operator+(cplx a, cplx b) { return cx(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ cplx operator-(cplx a, cplx b) { return cx(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ cplx operator+(cplx a, double b) { return cx(a.re + b, a.im); }
__device__ __forceinline__ cplx operator-(double a, cplx b) { return cx(a - b.re, -b.im); }
__device__ __forceinline__ cplx operator*(cplx a, cplx b)
{
    return cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ __forceinline__ cplx operator*(double a, cplx b) { return cx(a * b.re, a * b.im); }
__device__ __forceinline__ cplx operator/(cplx a, double b) { return cx(a.re / b, a.im / b); }
// Smith's algorithm
__device__ __forceinline__ cplx operator/(cplx a, cplx b)
{
    if (fabs(b.re) >= fabs(b.im)) {
        const double r = b.im / b.re, den = b.re + b.im * r;
        return cx((a.re + a.im * r) / den, (a.im - a.re * r) / den);
    }
    const double r = b.re / b.im, den = b.re * r + b.im;
    return cx((a.re * r + a.im) / den, (a.im * r - a.re) / den);
}
__device__ __forceinline__ cplx cx_log(cplx z) { return cx(log(hypot(z.re, z.im)), atan2(z.im, z.re)); }
__device__ __forceinline__ cplx cx_exp(cplx z)
{
    double s, c;
    sincos(z.im, &s, &c);
    const double e = exp(z.re);
    return cx(e * c, e * s);
}
// base^w for a real positive base: exp(w log(base))
__device__ __forceinline__ cplx cx_rpow(double base, cplx w)
{
    const double lb = log(base);
    return cx_exp(cx(w.re * lb, w.im * lb));
}

#define CG_LN_DBL_MAX 709.782712893384
#define CG_LN2 0.693147180559945309417232121458176568

// log(sin(pi z)) as clog(csin(pi z)) would return it; *overflow is set when
// either component of csin(pi z) exceeds the double range (the reference's
// csin then returns an infinity and its lnGamma becomes -inf).
__device__ __forceinline__ cplx cx_log_sinpi(cplx z, bool *overflow)
{
    const double ar = CG_PI * z.re, ai = CG_PI * z.im;
    double s, c;
    sincos(ar, &s, &c);
    *overflow = false;
    if (fabs(ai) <= 20.0) {
        const cplx w = cx(s * cosh(ai), c * sinh(ai));
        return cx_log(w);
    }
    // |ai| > 20: cosh ~ sinh ~ e^|ai| / 2 to better than 1e-17
    const double lmag = fabs(ai) - CG_LN2;
    if ((s != 0.0 && lmag + log(fabs(s)) > CG_LN_DBL_MAX) ||
        (c != 0.0 && lmag + log(fabs(c)) > CG_LN_DBL_MAX)) {
        *overflow = true;
        return cx(0, 0);
    }
    const double ci = ai > 0 ? c : -c;
    return cx(lmag + log(hypot(s, c)), atan2(ci, s));
}

// Lanczos log-Gamma, g = 7, 9 terms (twofast_lgamma, twofast.c:97-144).
// Returns false (and nothing usable) when the reflection overflowed.
__device__ __forceinline__ bool cx_lgamma_lanczos(cplx z, cplx *out)
{
    const double coeff[8] = {676.5203681218851,     -1259.1392167224028,  771.32342877765313,
                             -176.61502916214059,   12.507343278686905,   -0.13857109526572012,
                             9.9843695780195716e-6, 1.5056327351493116e-7};
    cplx refl = cx(0, 0);
    bool reflect = false;
    if (z.re < 0.5) {
        bool ovf;
        const cplx ls = cx_log_sinpi(z, &ovf);
        if (ovf) return false;
        refl = cx(log(CG_PI), 0) - ls;
        reflect = true;
        z = 1. - z;
    }
    cplx x = cx(0.99999999999980993, 0);
    z = cx(z.re - 1, z.im);
#pragma unroll
    for (int i = 0; i < 8; ++i) x = x + cx(coeff[i], 0) / (z + ((double)i + 1.));
    const cplx t = z + (8 - 0.5);
    const cplx r = cx(log(2 * CG_PI) / 2., 0) + (z + 0.5) * cx_log(t) - t + cx_log(x);
    *out = reflect ? refl - r : r;
    return true;
}
