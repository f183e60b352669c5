// Forward-mode dual numbers over six seed values (FP64): the value of an
// expression and its partials with respect to six consecutive knot values
// y_base .. y_base+5.  The adjoint kernels use them to differentiate the Akima
// interpolation exactly (its slope weights |m_{i+1} - m_i| included).
#pragma once

#include "spline.cuh"

struct D6 {
    double v, g[6];
};
__device__ __forceinline__ D6 d6_const(double v)
{
    D6 r;
    r.v = v;
    for (int k = 0; k < 6; ++k) r.g[k] = 0.0;
    return r;
}
__device__ __forceinline__ D6 operator+(const D6 &a, const D6 &b)
{
    D6 r;
    r.v = a.v + b.v;
    for (int k = 0; k < 6; ++k) r.g[k] = a.g[k] + b.g[k];
    return r;
}
__device__ __forceinline__ D6 operator-(const D6 &a, const D6 &b)
{
    D6 r;
    r.v = a.v - b.v;
    for (int k = 0; k < 6; ++k) r.g[k] = a.g[k] - b.g[k];
    return r;
}
__device__ __forceinline__ D6 operator*(const D6 &a, const D6 &b)
{
    D6 r;
    r.v = a.v * b.v;
    for (int k = 0; k < 6; ++k) r.g[k] = a.g[k] * b.v + a.v * b.g[k];
    return r;
}
__device__ __forceinline__ D6 operator*(double s, const D6 &a)
{
    D6 r;
    r.v = s * a.v;
    for (int k = 0; k < 6; ++k) r.g[k] = s * a.g[k];
    return r;
}
__device__ __forceinline__ D6 operator/(const D6 &a, const D6 &b)
{
    D6 r;
    r.v = a.v / b.v;
    for (int k = 0; k < 6; ++k) r.g[k] = (a.g[k] - r.v * b.g[k]) / b.v;
    return r;
}
__device__ __forceinline__ D6 d6_abs(const D6 &a) { return a.v < 0 ? -1.0 * a : a; }

// knot value y[k] seeded at position k - base
__device__ __forceinline__ D6 d6_knot(const double *y, int k, int base)
{
    D6 r = d6_const(y[k]);
    r.g[k - base] = 1.0;
    return r;
}

// Akima secant m_k with the non-periodic end rule of spline.cuh's akima_secant,
// seeded relative to base (every knot it reads lies in [base, base + 5] for
// k in [i - 2, i + 2] and base = i - 2, clamped into the table)
__device__ __forceinline__ D6 d6_secant(const double *x, const double *y, int n, int k, int base)
{
    auto sec = [&](int j) {
        return (d6_knot(y, j + 1, base) - d6_knot(y, j, base)) / d6_const(x[j + 1] - x[j]);
    };
    if (k >= 0 && k <= n - 2) return sec(k);
    if (k < 0) {
        const D6 m0 = sec(0), m1 = sec(1);
        return k == -1 ? 2.0 * m0 - m1 : 3.0 * m0 - 2.0 * m1;
    }
    const D6 ma = sec(n - 2), mb = sec(n - 3);
    return k == n - 1 ? 2.0 * ma - mb : 3.0 * ma - 2.0 * mb;
}

__device__ __forceinline__ D6 d6_node_slope(const D6 &mm2, const D6 &mm1, const D6 &m0,
                                            const D6 &mp1)
{
    const D6 w1 = d6_abs(mp1 - m0), w2 = d6_abs(mm1 - mm2);
    const D6 ne = w1 + w2;
    if (ne.v == 0.0) return 0.5 * (mm1 + m0);
    return (w1 * mm1 + w2 * m0) / ne;
}

// First knot of the six whose values an Akima record of interval i reads
// (n >= 6 knots)
__device__ __forceinline__ int d6_base(int n, int i)
{
    int base = i - 2;
    if (base < 0) base = 0;
    if (base > n - 6) base = n - 6;
    return base;
}

// The Akima record {y_i, b, c, d} of interval i (0 <= i <= n - 2, the same
// coefficients as akima_interval) with partials with respect to the knot
// values y_base .. y_base+5, base = d6_base(n, i)
__device__ __forceinline__ void akima_record_d6(const double *x, const double *y, int n, int i,
                                                D6 (&rec)[4])
{
    const int base = d6_base(n, i);
    D6 m[5];
    for (int k = 0; k < 5; ++k) m[k] = d6_secant(x, y, n, i - 2 + k, base);
    const D6 t0 = d6_node_slope(m[0], m[1], m[2], m[3]);
    const D6 t1 = d6_node_slope(m[1], m[2], m[3], m[4]);
    const double h = x[i + 1] - x[i];
    rec[0] = d6_knot(y, i, base);
    rec[1] = t0;
    rec[2] = (3.0 * m[2] - 2.0 * t0 - t1) / d6_const(h);
    rec[3] = (t0 + t1 - 2.0 * m[2]) / d6_const(h * h);
}

// Akima value at v in interval i (x_i <= v < x_{i+1}) with its partials with
// respect to y_base .. y_base+5, base = d6_base(n, i) (the operation order of
// akima_eval_at for the value)
__device__ __forceinline__ D6 akima_eval_d6(const double *x, const double *y, int n, int i,
                                            double v)
{
    D6 rec[4];
    akima_record_d6(x, y, n, i, rec);
    const D6 dx = d6_const(v - x[i]);
    return rec[0] + dx * (rec[1] + dx * (rec[2] + rec[3] * dx));
}
