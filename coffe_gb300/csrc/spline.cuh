// Device cubic splines with GSL interp semantics (the evaluator behind
// coffe_interp_spline, common.c:704-710): the interval is the one a binary
// search over the knots returns (x_i <= v < x_{i+1}, last interval for
// v == x_{n-1}), values outside [x_0, x_{n-1}] are NaN, and the cubic is
// y_i + dx (b_i + dx (c_i + d_i dx)).
//
// The binary search is replaced by a uniform "hint" table over [x_0, x_{n-1}]
// (hint[j] = interval of the bin's left edge) plus a short forward scan, which
// returns the same interval in O(1) loads for any strictly increasing knots.
#pragma once

#include "common.cuh"

struct Spl64 {
    const double *x;    // n knots
    const double4_32a *c;   // n-1 records (y_i, b_i, c_i, d_i)
    const int *hint;    // nh entries
    double x0, xn, inv_dh;
    int n, nh;
};

struct Spl32 {
    const float *x;
    const float4 *c;
    const int *hint;
    float x0, xn, inv_dh;
    int n, nh;
};

template <typename S> struct SplTraits;
template <> struct SplTraits<Spl64> { typedef double T; typedef double4_32a C4; };
template <> struct SplTraits<Spl32> { typedef float T; typedef float4 C4; };

__device__ __forceinline__ double4_32a ldg_c4(const double4_32a *p)
{
    const double2 *q = reinterpret_cast<const double2 *>(p);
    const double2 a = __ldg(q), b = __ldg(q + 1);
    return make_double4_32a(a.x, a.y, b.x, b.y);
}
__device__ __forceinline__ float4 ldg_c4(const float4 *p) { return __ldg(p); }

template <typename S>
__device__ __forceinline__ int spl_interval(const S &s, typename SplTraits<S>::T v)
{
    int j = (int)((v - s.x0) * s.inv_dh);
    j = j < 0 ? 0 : (j >= s.nh ? s.nh - 1 : j);
    int i = __ldg(s.hint + j);
    while (i > 0 && __ldg(s.x + i) > v) --i;
    while (i < s.n - 2 && __ldg(s.x + i + 1) <= v) ++i;
    return i;
}

template <typename S>
__device__ __forceinline__ typename SplTraits<S>::T spl_eval(const S &s, typename SplTraits<S>::T v)
{
    typedef typename SplTraits<S>::T T;
    if (!(v >= s.x0 && v <= s.xn)) return cg_nan<T>();
    const int i = spl_interval(s, v);
    const T dx = v - __ldg(s.x + i);
    const typename SplTraits<S>::C4 c = ldg_c4(s.c + i);
    return c.x + dx * (c.y + dx * (c.z + c.w * dx));
}

// ---------------------------------------------------------------------------
// Akima (1970) coefficients of one interval from the raw knots, with the
// non-periodic end rule (secant slopes extrapolated linearly past both ends:
// m_{-1} = 2 m_0 - m_1, m_{-2} = 3 m_0 - 2 m_1, and symmetrically), as
// gsl_interp_akima.  Used both to build coefficient records and to evaluate
// tables on the fly (the I_l^n tables are evaluated a few times per output,
// so their records are never stored).
// a / b: IEEE division, or (FAST, float) the approximate __fdividef (2 ulp;
// positive knot spacings and |b| < 2^126 here)
template <typename T, bool FAST> __device__ __forceinline__ T akima_div(T a, T b) { return a / b; }
template <> __device__ __forceinline__ float akima_div<float, true>(float a, float b)
{
    return __fdividef(a, b);
}

template <typename T, bool FAST = false>
__device__ __forceinline__ T akima_secant(const T *x, const T *y, int n, int k)
{
    if (k >= 0 && k <= n - 2) return akima_div<T, FAST>(y[k + 1] - y[k], x[k + 1] - x[k]);
    const T m0 = akima_div<T, FAST>(y[1] - y[0], x[1] - x[0]);
    const T m1 = akima_div<T, FAST>(y[2] - y[1], x[2] - x[1]);
    const T ma = akima_div<T, FAST>(y[n - 1] - y[n - 2], x[n - 1] - x[n - 2]);
    const T mb = akima_div<T, FAST>(y[n - 2] - y[n - 3], x[n - 2] - x[n - 3]);
    if (k == -1) return T(2) * m0 - m1;
    if (k == -2) return T(3) * m0 - T(2) * m1;
    if (k == n - 1) return T(2) * ma - mb;
    return T(3) * ma - T(2) * mb; // k == n
}

template <typename T, bool FAST = false>
__device__ __forceinline__ T akima_node_slope(T mm2, T mm1, T m0, T mp1)
{
    // slope at knot i from m_{i-2}, m_{i-1}, m_i, m_{i+1}
    const T w1 = fabs(mp1 - m0);
    const T w2 = fabs(mm1 - mm2);
    const T ne = w1 + w2;
    if (ne == T(0)) return T(0.5) * (mm1 + m0);
    return akima_div<T, FAST>(w1 * mm1 + w2 * m0, ne);
}

// Coefficients (b, c, d) of interval i, 0 <= i <= n-2.
template <typename T, bool FAST = false>
__device__ __forceinline__ void akima_interval(const T *x, const T *y, int n, int i, T &b, T &c,
                                               T &d)
{
    const T mm2 = akima_secant<T, FAST>(x, y, n, i - 2);
    const T mm1 = akima_secant<T, FAST>(x, y, n, i - 1);
    const T m0 = akima_secant<T, FAST>(x, y, n, i);
    const T mp1 = akima_secant<T, FAST>(x, y, n, i + 1);
    const T mp2 = akima_secant<T, FAST>(x, y, n, i + 2);
    const T t0 = akima_node_slope<T, FAST>(mm2, mm1, m0, mp1);
    const T t1 = akima_node_slope<T, FAST>(mm1, m0, mp1, mp2);
    const T h = x[i + 1] - x[i];
    b = t0;
    c = akima_div<T, FAST>(T(3) * m0 - T(2) * t0 - t1, h);
    d = akima_div<T, FAST>(t0 + t1 - T(2) * m0, h * h);
}

// Akima evaluation straight from knots (x, y), interval found by the caller.
template <typename T, bool FAST = false>
__device__ __forceinline__ T akima_eval_at(const T *x, const T *y, int n, int i, T v)
{
    T b, c, d;
    akima_interval<T, FAST>(x, y, n, i, b, c, d);
    const T dx = v - x[i];
    return y[i] + dx * (b + dx * (c + d * dx));
}

// Host-side owner of one spline's device arrays (FP64 and FP32 records).
struct SplineBuf {
    int n = 0, nh = 0;
    double x0 = 0, xn = 0;
    double *x = nullptr;
    double4_32a *c64 = nullptr;
    float *x32 = nullptr;
    float4 *c32 = nullptr;
    int *hint = nullptr;

    Spl64 v64() const { return Spl64{x, c64, hint, x0, xn, (double)nh / (xn - x0), n, nh}; }
    Spl32 v32() const
    {
        return Spl32{x32, c32, hint, (float)x0, (float)xn, (float)((double)nh / (xn - x0)), n, nh};
    }
};

struct coffe_gpu_ctx;
// Builds an Akima spline from device arrays x, y (n knots, strictly increasing x).
int spline_build(coffe_gpu_ctx *ctx, SplineBuf &s, const double *d_x, const double *d_y, int n);
void spline_free(SplineBuf &s);
