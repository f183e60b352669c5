// Warp-cooperative QUADPACK QAG with the 61-point Gauss-Kronrod rule: the
// integrator behind coffe_integrate_1d_prec_gsl (common.c:1004-1040, which
// calls gsl_integration_qag with epsabs = 0, key GSL_INTEG_GAUSS61).
//
// One warp integrates one function.  A panel's 61 nodes are spread over the
// lanes (lane t < 30 takes the pair +-XGK[t], lane 30 the centre) and the
// Kronrod, Gauss, |f| and |f - mean| sums are warp reductions.  The adaptive
// loop is QUADPACK's: bisect the interval with the largest error estimate
// until the summed error is within max(epsabs, epsrel |area|), with the same
// round-off detection; intervals live in the caller's shared memory.
#pragma once

#include "common.cuh"
#include "gk61_table.h"

static __device__ const double cg_gk_xgk[31] = CG_GK61_XGK_INIT;
static __device__ const double cg_gk_wgk[31] = CG_GK61_WGK_INIT;
static __device__ const double cg_gk_wg[15] = CG_GK61_WG_INIT;

// per-lane node data of the GK61 rule, loaded once per kernel
template <typename T> struct GkLane {
    T x;   // abscissa (0 for the centre lane, unused for lane 31)
    T wk;  // Kronrod weight
    T wg;  // Gauss weight (0 for Kronrod-only nodes)
    bool active, centre;
};

template <typename T> __device__ __forceinline__ GkLane<T> gk_lane()
{
    const int lane = threadIdx.x & 31;
    GkLane<T> g;
    g.active = lane <= 30;
    g.centre = lane == 30;
    const int k = lane < 31 ? lane : 30;
    g.x = (T)cg_gk_xgk[k];
    g.wk = lane < 31 ? (T)cg_gk_wgk[k] : T(0);
    g.wg = (lane < 30 && (lane & 1)) ? (T)cg_gk_wg[lane >> 1] : T(0);
    return g;
}

// smallest |integral| for which QUADPACK applies its round-off floor
template <typename T> __device__ __forceinline__ T qk_tiny();
template <> __device__ __forceinline__ double qk_tiny<double>() { return CG_DBL_MIN / (50 * CG_DBL_EPS); }
template <> __device__ __forceinline__ float qk_tiny<float>() { return 0.0f; }

// unit round-off of the working precision: QUADPACK's round-off floor
// (50 eps |f|) and its round-off exit use it, so the float path stops where
// float arithmetic stops resolving the error, as the double path does at DBL_EPSILON
template <typename T> __device__ __forceinline__ T qk_eps();
template <> __device__ __forceinline__ double qk_eps<double>() { return CG_DBL_EPS; }
template <> __device__ __forceinline__ float qk_eps<float>() { return 1.1920928955078125e-07f; }

// x^1.5: pow as QUADPACK writes it in FP64; x sqrt(x) in FP32 (the same
// function to an ulp, a fraction of powf's instructions)
__device__ __forceinline__ double qk_pow15(double x) { return pow(x, 1.5); }
__device__ __forceinline__ float qk_pow15(float x) { return x * sqrtf(x); }

template <typename T> __device__ __forceinline__ T qk_rescale_error(T err, T result_abs, T result_asc)
{
    err = fabs(err);
    if (result_asc != T(0) && err != T(0)) {
        const T scale = qk_pow15(T(200) * err / result_asc);
        err = scale < T(1) ? result_asc * scale : result_asc;
    }
    if (result_abs > qk_tiny<T>()) {
        const T min_err = T(50) * qk_eps<T>() * result_abs;
        if (min_err > err) err = min_err;
    }
    return err;
}

template <typename T> struct QkOut {
    T result, abserr, resabs, resasc;
};

// Panel reduction from this lane's two function values (f1 at c - x, f2 at
// c + x; the centre lane passes f2 = 0).  All lanes receive the result.
template <typename T>
__device__ __forceinline__ QkOut<T> qk61_reduce(const GkLane<T> &g, T f1, T f2, T half_length)
{
    const T fs = f1 + f2;
    const T K = warp_sum(g.wk * fs);
    const T G = warp_sum(g.wg * fs);
    const T A = warp_sum(g.wk * (fabs(f1) + fabs(f2)));
    const T mean = K * T(0.5);
    T asc = T(0);
    if (g.active) asc = g.wk * (g.centre ? fabs(f1 - mean) : fabs(f1 - mean) + fabs(f2 - mean));
    asc = warp_sum(asc);
    const T ahl = fabs(half_length);
    QkOut<T> o;
    o.result = K * half_length;
    o.resabs = A * ahl;
    o.resasc = asc * ahl;
    o.abserr = qk_rescale_error((K - G) * half_length, o.resabs, o.resasc);
    return o;
}

// One GK61 panel of a scalar functor f over [a, b].
template <typename T, class F>
__device__ __forceinline__ QkOut<T> qk61_warp(const F &f, const GkLane<T> &g, T a, T b)
{
    const T center = T(0.5) * (a + b);
    const T half_length = T(0.5) * (b - a);
    T f1 = T(0), f2 = T(0);
    if (g.centre) {
        f1 = f(center);
    } else if (g.active) {
        const T absc = half_length * g.x;
        f1 = f(center - absc);
        f2 = f(center + absc);
    }
    return qk61_reduce(g, f1, f2, half_length);
}

// Interval store of one warp in shared memory.
template <typename T> struct QagStore {
    T *a, *b, *r, *e;
    int cap;
};

// Warp argmax of e[0..size) with the lowest index winning ties (the first
// maximum a linear scan finds).
template <typename T> __device__ __forceinline__ int qag_argmax(const QagStore<T> &s, int size)
{
    const int lane = threadIdx.x & 31;
    T best = T(-1);
    int bi = 0x7fffffff;
    for (int i = lane; i < size; i += 32) {
        const T v = s.e[i];
        if (v > best) {
            best = v;
            bi = i;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const T ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) {
            best = ob;
            bi = oi;
        }
    }
    return bi;
}

__device__ __forceinline__ bool qag_too_small(double a1, double a2, double b2)
{
    const double tmp = (1 + 100 * CG_DBL_EPS) * (fabs(a2) + 1000 * CG_DBL_MIN);
    return fabs(a1) <= tmp && fabs(b2) <= tmp;
}

// Adaptive continuation after a first panel `p0` over [a, b] (gsl qag.c
// semantics).  Returns the integral; *status: 0 ok, 1 limit reached,
// 2 round-off, 3 bad integrand behaviour.  `F` evaluates one point.  When
// n_final is given it receives the number of intervals of the final
// partition: 1 when the first panel is the result ([a, b]; the store is not
// written), else the intervals s.a[0..n) / s.b[0..n) whose results sum up to
// the returned integral.
template <typename T, class F>
__device__ T qag_continue(const F &f, const GkLane<T> &g, T a, T b, QkOut<T> p0, T epsabs,
                          T epsrel, const QagStore<T> &s, int limit, int *status,
                          int *n_final = nullptr)
{
    const int lane = threadIdx.x & 31;
    T tolerance = fmax(epsabs, epsrel * fabs(p0.result));
    const T round_off = T(50) * qk_eps<T>() * p0.resabs;
    *status = 0;
    if (n_final) *n_final = 1;
    if (p0.abserr <= round_off && p0.abserr > tolerance) {
        *status = 2;
        return p0.result;
    }
    if ((p0.abserr <= tolerance && p0.abserr != p0.resasc) || p0.abserr == T(0)) return p0.result;
    if (limit <= 1 || s.cap < 2) {
        *status = 1;
        return p0.result;
    }
    if (lane == 0) {
        s.a[0] = a;
        s.b[0] = b;
        s.r[0] = p0.result;
        s.e[0] = p0.abserr;
    }
    __syncwarp();
    int size = 1;
    T area = p0.result, errsum = p0.abserr;
    int rt1 = 0, rt2 = 0, error_type = 0;
    int iteration = 1;
    const int lim = limit < s.cap ? limit : s.cap;
    do {
        const int im = qag_argmax(s, size);
        const T a_i = s.a[im], b_i = s.b[im], r_i = s.r[im], e_i = s.e[im];
        const T a1 = a_i, b1 = T(0.5) * (a_i + b_i), a2 = b1, b2 = b_i;
        const QkOut<T> p1 = qk61_warp(f, g, a1, b1);
        const QkOut<T> p2 = qk61_warp(f, g, a2, b2);
        const T area12 = p1.result + p2.result;
        const T error12 = p1.abserr + p2.abserr;
        errsum += (error12 - e_i);
        area += area12 - r_i;
        if (p1.resasc != p1.abserr && p2.resasc != p2.abserr) {
            const T delta = r_i - area12;
            if (fabs(delta) <= T(1.0e-5) * fabs(area12) && error12 >= T(0.99) * e_i) rt1++;
            if (iteration >= 10 && error12 > e_i) rt2++;
        }
        tolerance = fmax(epsabs, epsrel * fabs(area));
        if (errsum > tolerance) {
            if (rt1 >= 6 || rt2 >= 20) error_type = 2;
            if (qag_too_small((double)a1, (double)a2, (double)b2)) error_type = 3;
        }
        __syncwarp();
        if (lane == 0) {
            s.a[im] = a1;
            s.b[im] = b1;
            s.r[im] = p1.result;
            s.e[im] = p1.abserr;
            s.a[size] = a2;
            s.b[size] = b2;
            s.r[size] = p2.result;
            s.e[size] = p2.abserr;
        }
        __syncwarp();
        size++;
        iteration++;
    } while (iteration < lim && !error_type && errsum > tolerance);
    if (n_final) *n_final = size;
    if (error_type)
        *status = error_type;
    else if (errsum > tolerance)
        *status = 1;
    // sum of the interval results in index order (gsl sum_results)
    T result = T(0);
    if (lane == 0)
        for (int i = 0; i < size; ++i) result += s.r[i];
    return __shfl_sync(0xffffffffu, result, 0);
}

// Full QAG: first panel then the adaptive loop.
template <typename T, class F>
__device__ __forceinline__ T qag61_warp(const F &f, T a, T b, T epsabs, T epsrel,
                                        const QagStore<T> &s, int limit, int *status,
                                        int *n_final = nullptr)
{
    const GkLane<T> g = gk_lane<T>();
    const QkOut<T> p0 = qk61_warp(f, g, a, b);
    return qag_continue(f, g, a, b, p0, epsabs, epsrel, s, limit, status, n_final);
}
