// Lensing contributions to the multipoles of a ragged batch of
// (spectrum, mean redshift, separation list) requests: the single-integrated
// density/RSD x lensing terms and the double-integrated lensing-lensing term
// of the full-sky correlation function, projected on Legendre multipoles.
//
// Restates coffe_integrate(SINGLE_INTEGRATED / DOUBLE_INTEGRATED, MULTIPOLES)
// (signal.c:607-671, 704-754) with the integrands of signal.c:141-237,
// functions_single_integrated (functions.c:1486-2483) and
// functions_double_integrated (functions.c:3460-3836): linear P(k), full sky,
// no renormalisation.  The reference integrates the unit cube (v, x) or
// (v, x1, x2), mu = 2v - 1, with Cuhre (common.c:1096-1110); here the cube is
// integrated with fixed Gauss-Legendre product rules: n_mu nodes in v and,
// per x line, n_x nodes split into two panels of n_x / 2 at the point of the
// line where the integrand's separation argument is smallest (its narrow
// peak): x* = lambda1 / chi2 on an x2 line of len-len, x* = min(chi1, chi2)
// cos(theta) / max(chi1, chi2) on the single-integrated line.
//
// Work split (one launch each, per chunk of pairs):
//   lens_double_kernel  one CTA per (pair, mu node): threads own x1 lines and
//                       sweep their x2 line; one partial per (pair, mu);
//   lens_single_kernel  one warp per (pair, mu node), FP64 (lens_single_fast_kernel
//                       on the mixed path: FP32 with the RSD-lensing
//                       coefficients expanded so that they cancel nothing);
//   lens_reduce_kernel  per (pair, l): the mu weights and P_l(mu), summed in a
//                       fixed order, added to the nonintegrated multipole.
// The six I_l^n tables the integrands read are evaluated through Akima
// records {y, b, c, d} built once per call and interleaved per interval, so a
// node's six lookups share one interval search and one 192-byte (FP64) or
// 96-byte (float) block.
#include <math.h>

#include <algorithm>
#include <vector>

#include "ctx.cuh"
#include "dual6.cuh"
#include "qag.cuh"

namespace {

#define LENS_THREADS 128
#define LENS_NT 6
enum { L00 = 0, L02, L04, L11, L13, L20 };

struct LensArgs {
    int n_req, n_l, n_mu, n_x, nh, contrib;
    // mu nodes evaluated: mu0 .. mu0 + n_mu_run - 1 of the rule, weighted by
    // mu_w (the upper half twice when the terms are even in mu)
    int mu0, n_mu_run;
    double mu_w;
    // the terms are even in mu: an even multipole of a run over every node
    // sums the mu > 0 half twice, as it does when only that half is evaluated
    int sym;
    int tab_len, n_terms;
    int term[LENS_NT];
    double inv_dlog; // N / ln(kmax/kmin), r0 = 1
    double Om, pref2, pref4;
    int has_b1, has_b2, has_s1, has_s2;
    long long pair0, n_items;
    int ls[8];
};

struct LensBg64 {
    Spl64 chi_of_z, z_of_chi, D1, f, a, b1, b2, s1, s2;
};
template <typename S> struct LensBgT {
    S z_of_chi, D1, a;
};

template <typename TT> struct Rec4;
template <> struct Rec4<double> { typedef double4_32a type; };
template <> struct Rec4<float> { typedef float4 type; };

__device__ __forceinline__ int lens_find_request(const int64_t *__restrict__ req_offset, int n_req,
                                                 long long item)
{
    int lo = 0, hi = n_req;
    while (hi > lo + 1) {
        const int mid = (lo + hi) >> 1;
        if (req_offset[mid] <= item)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// rec[(s * (len - 1) + i) * 6 + t]: Akima record of interval i of table
// (spectrum s, lensing term t), from the raw table knots (spline.cuh's
// akima_interval: the coefficients the reference's Akima spline holds)
template <typename TT>
__global__ void lens_records_kernel(LensArgs a, const TT *__restrict__ tab_x,
                                    const TT *__restrict__ tab_y, int n_spectra,
                                    typename Rec4<TT>::type *__restrict__ rec)
{
    const int len = a.tab_len, ni = len - 1;
    const long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= (long long)n_spectra * ni * LENS_NT) return;
    const int t = (int)(item % LENS_NT);
    const long long si = item / LENS_NT;
    const int i = (int)(si % ni);
    const int s = (int)(si / ni);
    const TT *y = tab_y + ((size_t)s * a.n_terms + a.term[t]) * len;
    TT b, c, d;
    akima_interval<TT>(tab_x, y, len, i, b, c, d);
    typename Rec4<TT>::type r;
    r.x = y[i];
    r.y = b;
    r.z = c;
    r.w = d;
    rec[item] = r;
}

// interval of r in the table knots as a binary search returns it (an O(1)
// guess on the log-spaced part, then a local correction); -1 outside
template <typename TT>
__device__ __forceinline__ int lens_interval(const TT *__restrict__ x, int n, TT inv_dlog, TT r)
{
    if (!(r >= x[0] && r <= x[n - 1])) return -1;
    const int first = CG_N_SMALL_R + 1;
    int i;
    if (r >= __ldg(x + first)) {
        i = first + (int)(log(r) * inv_dlog);
        if (i > n - 2) i = n - 2;
        if (i < first) i = first;
        while (i > 0 && __ldg(x + i) > r) --i;
        while (i < n - 2 && __ldg(x + i + 1) <= r) ++i;
    } else {
        int lo = 0, hi = first;
        while (hi > lo + 1) {
            const int mid = (lo + hi) / 2;
            if (__ldg(x + mid) > r)
                hi = mid;
            else
                lo = mid;
        }
        i = lo;
    }
    return i;
}

// the six lensing tables at r (NaN outside the tables)
template <typename T, typename TT>
__device__ __forceinline__ void lens_tables(const typename Rec4<TT>::type *__restrict__ recs,
                                            const TT *__restrict__ x, int n, TT inv_dlog, T r,
                                            T (&v)[LENS_NT])
{
    const int i = lens_interval<TT>(x, n, inv_dlog, (TT)r);
    if (i < 0) {
#pragma unroll
        for (int t = 0; t < LENS_NT; ++t) v[t] = cg_nan<T>();
        return;
    }
    const T dx = r - (T)__ldg(x + i);
    const typename Rec4<TT>::type *p = recs + (size_t)i * LENS_NT;
#pragma unroll
    for (int t = 0; t < LENS_NT; ++t) {
        const typename Rec4<TT>::type c = ldg_c4(p + t);
        v[t] = (T)c.x + dx * ((T)c.y + dx * ((T)c.z + (T)c.w * dx));
    }
}

// the value at r = 0 (first knot) of table t
template <typename TT>
__device__ __forceinline__ TT lens_at_zero(const typename Rec4<TT>::type *__restrict__ recs, int t)
{
    return ldg_c4(recs + t).x;
}

// Mixed lensing-lensing integrand regrouped by powers of ll = lambda1 lambda2
// (functions.c:3695-3775, checked equal symbolically):
//   v = ct A + ll (c2m B + ct^2 C) + ll^2 c2m ct D / r^2 + ll^3 c2m^2 E / r^4,
//   A = 4/3 I20 + 4/15 r^2 S, C = 8/5 S, S = I11 + I13,
//   B = 2/5 I00 + 4/7 I02 + 6/35 I04, D = 6/7 (I02 + I04) + 2 I13, E = I04:
// five functions of r, whose Akima records are the same combinations of the
// six tables' records (the interpolant is linear in the records), stored
// rec5[(s * (len - 1) + i) * 5 + u] for u = I20, S, B, D, E.
#define LENS_NC 5
template <typename R>
__global__ void lens_combine_kernel(const R *__restrict__ rec, long long n_int,
                                    R *__restrict__ rec5)
{
    typedef decltype(R::x) E;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_int) return;
    const R *p = rec + i * LENS_NT;
    const R i00 = p[L00], i02 = p[L02], i04 = p[L04], i11 = p[L11], i13 = p[L13], i20 = p[L20];
    auto lin = [](E a, R x, E b, R y, E c, R z) {
        R o;
        o.x = a * x.x + b * y.x + c * z.x;
        o.y = a * x.y + b * y.y + c * z.y;
        o.z = a * x.z + b * y.z + c * z.z;
        o.w = a * x.w + b * y.w + c * z.w;
        return o;
    };
    R *q = rec5 + i * LENS_NC;
    q[0] = i20;
    q[1] = lin(E(1), i11, E(1), i13, E(0), i13);
    q[2] = lin(E(0.4), i00, E(4) / E(7), i02, E(6) / E(35), i04);
    q[3] = lin(E(6) / E(7), i02, E(6) / E(7), i04, E(2), i13);
    q[4] = i04;
}

// the five combined functions at r (NaN outside the tables)
template <typename T, typename TT>
__device__ __forceinline__ void lens_tables5(const typename Rec4<TT>::type *__restrict__ recs5,
                                             const TT *__restrict__ x, int n, TT inv_dlog, T r,
                                             T (&v)[LENS_NC])
{
    const int i = lens_interval<TT>(x, n, inv_dlog, (TT)r);
    if (i < 0) {
#pragma unroll
        for (int u = 0; u < LENS_NC; ++u) v[u] = cg_nan<T>();
        return;
    }
    const T dx = r - (T)__ldg(x + i);
    const typename Rec4<TT>::type *p = recs5 + (size_t)i * LENS_NC;
#pragma unroll
    for (int u = 0; u < LENS_NC; ++u) {
        const typename Rec4<TT>::type c = ldg_c4(p + u);
        v[u] = (T)c.x + dx * ((T)c.y + dx * ((T)c.z + (T)c.w * dx));
    }
}

// a b + c with one rounding, in the working precision
__device__ __forceinline__ float lens_fma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double lens_fma(double a, double b, double c) { return fma(a, b, c); }

// Geometry of one (pair, mu node), functions.c:1498-1509 / 3473-3481, with
// cos(theta) = 1 - s, s = sep^2 (1 - mu^2) / (2 chi1 chi2) (no cancellation)
struct LensGeom {
    double chi1, chi2, s, ct, omc2, z1c, z2c;
};
__device__ __forceinline__ LensGeom lens_geom(const LensBg64 &g, double z_mean, double mu,
                                              double sep)
{
    LensGeom o;
    const double chi_mean = spl_eval(g.chi_of_z, z_mean);
    o.chi1 = chi_mean - sep * mu / 2.;
    o.chi2 = chi_mean + sep * mu / 2.;
    o.s = sep * sep * (1 - mu * mu) / (2. * chi_mean * chi_mean - mu * mu * sep * sep / 2.);
    o.ct = 1 - o.s;
    o.omc2 = o.s * (2 - o.s);
    o.z1c = spl_eval(g.z_of_chi, o.chi1);
    o.z2c = spl_eval(g.z_of_chi, o.chi2);
    return o;
}

// float sums with Kahan compensation, double sums plain
template <typename T> struct Acc {
    T s = T(0), c = T(0);
    __device__ __forceinline__ void add(T v)
    {
        if (sizeof(T) == 4) {
            const T y = v - c;
            const T t = s + y;
            c = (t - s) - y;
            s = t;
        } else {
            s += v;
        }
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// Mixed path: the lensing kernel D1(z(lambda)) / a(z(lambda)) along each side's
// line of sight, lambda = chi_i x, x in [0, 1], as a degree-9 polynomial in
// t = 2x - 1, interpolated at ten Chebyshev points (float background splines;
// the function's Chebyshev tail is at the splines' 5e-9 noise from degree 9
// for z <= 2.5).  The monomial coefficients are formed in FP64 from the inverse
// Vandermonde matrix of the points (host, FP64), so their cancellation is
// exact before they are rounded to float.
#define LENS_PDEG 9
struct LensPoly {
    float t[LENS_PDEG + 1];
    double td[LENS_PDEG + 1];
    double vinv[LENS_PDEG + 1][LENS_PDEG + 1];
};

LensPoly lens_poly_tables()
{
    const int n = LENS_PDEG + 1;
    LensPoly r;
    double V[LENS_PDEG + 1][2 * (LENS_PDEG + 1)];
    for (int j = 0; j < n; ++j) {
        const double t = cos((2 * j + 1) * CG_PI / (2.0 * n));
        r.t[j] = (float)t;
        r.td[j] = t;
        double p = 1.0;
        for (int c = 0; c < n; ++c, p *= t) V[j][c] = p;
        for (int c = 0; c < n; ++c) V[j][n + c] = c == j ? 1.0 : 0.0;
    }
    for (int c = 0; c < n; ++c) { // Gauss-Jordan with partial pivoting
        int piv = c;
        for (int r2 = c + 1; r2 < n; ++r2)
            if (fabs(V[r2][c]) > fabs(V[piv][c])) piv = r2;
        for (int k = 0; k < 2 * n; ++k) std::swap(V[c][k], V[piv][k]);
        const double d = V[c][c];
        for (int k = 0; k < 2 * n; ++k) V[c][k] /= d;
        for (int r2 = 0; r2 < n; ++r2)
            if (r2 != c) {
                const double m = V[r2][c];
                for (int k = 0; k < 2 * n; ++k) V[r2][k] -= m * V[c][k];
            }
    }
    for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k) r.vinv[j][k] = V[j][n + k];
    return r;
}

template <typename T> __device__ __forceinline__ T lens_horner(const T *c, T t)
{
    T v = c[LENS_PDEG];
#pragma unroll
    for (int k = LENS_PDEG - 1; k >= 0; --k) v = lens_fma(v, t, c[k]);
    return v;
}
// the Chebyshev point t_j of the polynomial fits in the working precision
template <typename T> __device__ __forceinline__ T lens_cheb(const LensPoly &p, int j);
template <> __device__ __forceinline__ float lens_cheb<float>(const LensPoly &p, int j)
{
    return p.t[j];
}
template <> __device__ __forceinline__ double lens_cheb<double>(const LensPoly &p, int j)
{
    return p.td[j];
}

// FAST selects the algorithm of the mixed path (D1 / a along both lines of
// sight as degree-9 polynomials, the integrand regrouped over the five
// combined records); with T = double it is that algorithm in FP64, the
// matched-algorithm baseline of the mixed path.  FAST = false: the reference's
// six-table form with spline lookups per node (the FP64 parity path).
template <typename T, typename S, typename TT, bool FAST>
__global__ void __launch_bounds__(LENS_THREADS)
    lens_double_kernel(LensArgs a, LensBg64 g64, LensBgT<S> gT, LensPoly poly,
                       const TT *__restrict__ tab_x,
                       const typename Rec4<TT>::type *__restrict__ rec,
                       const typename Rec4<TT>::type *__restrict__ rec5,
                       const int *__restrict__ req_spectrum, const double *__restrict__ req_z_mean,
                       const int64_t *__restrict__ req_offset, const double *__restrict__ sep,
                       const double *__restrict__ rule, double *__restrict__ part, int *err)
{
    static_assert(FAST || sizeof(T) == 8, "the FP32 plane kernel has only the fast algorithm");
    __shared__ double red[LENS_THREADS / 32];
    __shared__ T gval[2][LENS_PDEG + 1];
    __shared__ T gcoef[2][LENS_PDEG + 1];
    const long long item = blockIdx.x;
    const long long pair = a.pair0 + item / a.n_mu_run;
    const int im = a.mu0 + (int)(item % a.n_mu_run);
    const int q = lens_find_request(req_offset, a.n_req, pair);
    const int s = req_spectrum[q];
    const double *xf = rule + 2 * a.n_mu, *wf = xf + a.n_x, *xh = wf + a.n_x, *wh = xh + a.nh;
    const double mu = rule[im];
    const LensGeom G = lens_geom(g64, req_z_mean[q], mu, sep[pair]);
    const double s1 = a.has_s1 ? spl_eval(g64.s1, G.z1c) : 0.0;
    const double s2 = a.has_s2 ? spl_eval(g64.s2, G.z2c) : 0.0;
    const double pre = 9. * a.Om * a.Om * (2 - 5 * s1) * (2 - 5 * s2) / 4. * G.chi1 * G.chi2 * a.pref4;
    const typename Rec4<TT>::type *recs = rec + (size_t)s * (a.tab_len - 1) * LENS_NT;
    const typename Rec4<TT>::type *recs5 =
        FAST ? rec5 + (size_t)s * (a.tab_len - 1) * LENS_NC : nullptr;
    const T chi1 = (T)G.chi1, chi2 = (T)G.chi2, ss = (T)G.s, ct = (T)G.ct, c2m = (T)(-G.omc2);
    const T i11_0 = (T)lens_at_zero<TT>(recs, L11);
    const TT inv_dlog = (TT)a.inv_dlog;
    constexpr bool F32 = sizeof(T) == 4;
    // mixed path: float copies of the line rules follow the FP64 rule
    const float *xf32 = reinterpret_cast<const float *>(xh + 2 * a.nh);
    const float *wf32 = xf32 + a.n_x, *xh32 = wf32 + a.n_x, *wh32 = xh32 + a.nh;
    if (FAST) { // D1 / a along both lines of sight as polynomials in 2x - 1
        if (threadIdx.x < 2 * (LENS_PDEG + 1)) {
            const int side = threadIdx.x / (LENS_PDEG + 1), j = threadIdx.x % (LENS_PDEG + 1);
            const T lam = (T)(side ? G.chi2 : G.chi1) * T(0.5) * (lens_cheb<T>(poly, j) + T(1));
            const T zz = spl_eval(gT.z_of_chi, lam);
            gval[side][j] = (T)(spl_eval(gT.D1, zz) / spl_eval(gT.a, zz));
        }
        __syncthreads();
        if (threadIdx.x < 2 * (LENS_PDEG + 1)) {
            const int side = threadIdx.x / (LENS_PDEG + 1), j = threadIdx.x % (LENS_PDEG + 1);
            double c = 0.0;
            for (int k = 0; k <= LENS_PDEG; ++k) c += poly.vinv[j][k] * (double)gval[side][k];
            gcoef[side][j] = (T)c;
        }
        __syncthreads();
    }
    Acc<T> acc;
    for (int ia = threadIdx.x; ia < a.n_x; ia += blockDim.x) {
        const double x1d = 0.5 * (xf[ia] + 1.0);
        const T x1 = (T)x1d;
        const T l1 = chi1 * x1;
        T g1;
        if (FAST) {
            g1 = lens_horner(gcoef[0], (T)(2 * x1 - 1)) * (T(1) - x1);
        } else {
            const T z1 = spl_eval(gT.z_of_chi, l1);
            g1 = spl_eval(gT.D1, z1) / spl_eval(gT.a, z1) * (T(1) - x1);
        }
        const double xs = x1d * G.chi1 / G.chi2;
        const bool split = a.nh > 0 && xs > 0 && xs < 1;
        T line = T(0);
        for (int p = 0; p < (split ? 2 : 1); ++p) {
            const double lo = (split && p) ? xs : 0.0, hi = (split && !p) ? xs : 1.0;
            const double c = 0.5 * (lo + hi), hw = 0.5 * (hi - lo);
            const int np = split ? a.nh : a.n_x;
            const double *gx = split ? xh : xf, *gw = split ? wh : wf;
            const float *gx32 = split ? xh32 : xf32, *gw32 = split ? wh32 : wf32;
            const float cf = (float)c, hwf = (float)hw;
            Acc<T> pa;
            for (int k = 0; k < np; ++k) {
                T x2, wk;
                if (F32) {
                    x2 = (T)fmaf(hwf, gx32[k], cf);
                    wk = (T)gw32[k];
                } else {
                    x2 = (T)(c + hw * gx[k]);
                    wk = (T)gw[k];
                }
                T g2;
                if (FAST) {
                    g2 = lens_horner(gcoef[1], (T)(2 * x2 - 1)) * (T(1) - x2);
                } else {
                    const T z2 = spl_eval(gT.z_of_chi, chi2 * x2);
                    g2 = spl_eval(gT.D1, z2) / spl_eval(gT.a, z2) * (T(1) - x2);
                }
                const T l2 = chi2 * x2;
                const T ll = l1 * l2;
                const T dl = l1 - l2;
                const T r2 = dl * dl + T(2) * ll * ss;
                T v;
                if (r2 > T(1e-20)) {
                    // functions.c:3695-3775
                    if (FAST) { // regrouped in powers of ll over the five combined tables
                        T Q[LENS_NC];
                        lens_tables5<T, TT>(recs5, tab_x, a.tab_len, inv_dlog, (T)sqrt(r2), Q);
                        const T ir2 = T(1) / r2;
                        const T lc = ll * c2m * ir2;
                        const T vA =
                            ct * lens_fma(T(4.0 / 15.0) * r2, Q[1], T(4.0 / 3.0) * Q[0]);
                        const T vB = lens_fma(c2m, Q[2], ct * ct * T(8.0 / 5.0) * Q[1]);
                        const T vD = lens_fma(lc, Q[4], ct * Q[3]); // ll c2m E / r^2 + ct D
                        v = vA + ll * lens_fma(lc, vD, vB);
                    } else {
                        T I[LENS_NT];
                        lens_tables<T, TT>(recs, tab_x, a.tab_len, inv_dlog, sqrt(r2), I);
                        v = T(2) * c2m * ll * I[L00] / T(5) + T(4) * ct * I[L20] / T(3) +
                            T(4) * ct * (r2 + T(6) * ct * ll) * I[L11] / T(15) +
                            T(2) * c2m * ll * (T(2) * r2 + T(3) * ct * ll) * I[L02] / T(7) / r2 +
                            T(2) * ct *
                                (T(2) * r2 * r2 + T(12) * ct * r2 * ll + T(15) * c2m * ll * ll) *
                                I[L13] / T(15) / r2 +
                            c2m * ll *
                                (T(6) * r2 * r2 + T(30) * ct * r2 * ll + T(35) * c2m * ll * ll) *
                                I[L04] / T(35) / r2 / r2;
                    }
                } else {
                    // functions.c:3801-3833
                    v = T(4) + T(24) * ll * i11_0 / T(15);
                }
                pa.add(wk * g2 * v);
            }
            line += (T)hw * (T)pa.value();
        }
        acc.add((T)(0.5 * wf[ia]) * g1 * line);
    }
    double tot = warp_sum(acc.value());
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = tot;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        const double res = pre * t;
        if (!isfinite(res)) cg_flag(err, CG_ERR_NONFINITE);
        part[item] = res;
    }
}

// den-len + rsd-len at (mu, x) in FP64 (functions.c:1557-2483), per side:
// "2" = lensing to chi2 correlated with the local term at chi1, "1" = mirror
template <typename TT>
__device__ double lens_single_xi(const LensArgs &a, const LensBg64 &g,
                                 const typename Rec4<TT>::type *__restrict__ recs,
                                 const TT *__restrict__ tab_x, const LensGeom &G, double x,
                                 double b1, double b2, double s1, double s2, double f1c,
                                 double f2c, double D1z1c, double D1z2c, double mu)
{
    const double chi1 = G.chi1, chi2 = G.chi2, ct = G.ct, omc2 = G.omc2;
    const double lambda1 = chi1 * x, lambda2 = chi2 * x;
    double r21 = (lambda2 - chi1) * (lambda2 - chi1) + 2 * chi1 * lambda2 * G.s;
    double r22 = (lambda1 - chi2) * (lambda1 - chi2) + 2 * chi2 * lambda1 * G.s;
    if (r21 < 0) r21 = 0;
    if (r22 < 0) r22 = 0;
    const double z1 = spl_eval(g.z_of_chi, lambda1), z2 = spl_eval(g.z_of_chi, lambda2);
    const double D1z1 = spl_eval(g.D1, z1), D1z2 = spl_eval(g.D1, z2);
    const double az1 = spl_eval(g.a, z1), az2 = spl_eval(g.a, z2);
    const TT inv_dlog = (TT)a.inv_dlog;
    double I1[LENS_NT], I2[LENS_NT];
    lens_tables<double, TT>(recs, tab_x, a.tab_len, inv_dlog, sqrt(r21), I1);
    lens_tables<double, TT>(recs, tab_x, a.tab_len, inv_dlog, sqrt(r22), I2);
    const double I00_0 = (double)lens_at_zero<TT>(recs, L00);
    const double I11_0 = (double)lens_at_zero<TT>(recs, L11);
    double result = 0;
    if (a.contrib & COFFE_GPU_DEN) {
        double t1, t2;
        if (r21 != 0.0)
            t1 = chi2 * (2 * chi1 * ct * I1[L11] - chi1 * chi1 * lambda2 * omc2 * I1[L02] / r21);
        else
            t1 = chi2 * 2 * chi1 * I11_0;
        if (r22 != 0.0)
            t2 = chi1 * (2 * chi2 * ct * I2[L11] - chi2 * chi2 * lambda1 * omc2 * I2[L02] / r22);
        else
            t2 = chi1 * 2 * chi2 * I11_0;
        result += a.pref2 * (-3 * a.Om / 2. *
                             (b1 * (2 - 5 * s2) * D1z1c * (1 - x) * D1z2 / az2 * t1 +
                              b2 * (2 - 5 * s1) * D1z2c * (1 - x) * D1z1 / az1 * t2));
    }
    if (a.contrib & COFFE_GPU_RSD) {
        const double c2m1 = 2 * ct * ct - 1;
        // I00/I02 part (functions.c:2174-2183) and I04 part (2298-2306) of one
        // side.  The polynomials multiplying I02 / r^2 and I04 / r^4 vanish like
        // r^2 and r^4; written, as in the reference, in chi, lambda and
        // cos(theta) they cancel up to ~10 digits, so they are expanded in
        // d = chi - lambda and s = 1 - cos(theta) (the same polynomials), where
        // every term has the size of the result.
        const double ss = G.s;
        auto Q = [&](double ch, double d) {
            return d * d * d * (8 - 24 * ss + 12 * ss * ss) +
                   ch * d * d * (-2 + 38 * ss - 18 * ss * ss - 6 * ss * ss * ss) +
                   ch * ch * d * ss * (-22 + 9 * ss + 12 * ss * ss) +
                   ch * ch * ch * ss * (2 - 3 * ss - 6 * ss * ss);
        };
        auto P = [&](double ch, double d) {
            const double d2 = d * d, d3 = d2 * d, d4 = d2 * d2, d5 = d4 * d;
            const double ch2 = ch * ch, ch3 = ch2 * ch, ch4 = ch2 * ch2, ch5 = ch4 * ch;
            const double s2 = ss * ss, s3 = s2 * ss;
            return d5 * (4 - 12 * ss + 6 * s2) + ch * d4 * (-8 + 60 * ss - 48 * s2 + 6 * s3) +
                   ch2 * d3 * ss * (-92 + 114 * ss - 20 * s2 - s3) +
                   ch3 * d2 * ss * (48 - 120 * ss + 26 * s2 + 3 * s3) +
                   ch4 * d * s2 * (60 - 16 * ss - 3 * s2) + ch5 * s2 * (-12 + 4 * ss + s2);
        };
        auto A = [&](double ch, double la, const double *I, double r2) {
            return (la - 6 * ch * ct + 3 * la * c2m1) * I[L00] / 15. -
                   Q(ch, ch - la) * I[L02] / r2 / 21.;
        };
        auto B = [&](double ch, double la, const double *I, double r2) {
            return -P(ch, ch - la) * I[L04] / r2 / r2 / 35.;
        };
        const double w2 = chi2 * f1c * (2 - 5 * s2) * D1z1c * D1z2 / az2;
        const double w1 = chi1 * f2c * (2 - 5 * s1) * D1z2c * D1z1 / az1;
        const double c = a.pref2 * 3 * a.Om / 2.;
        if (r21 != 0 && r22 != 0) {
            result += c * (w2 * (1 - x) * A(chi1, lambda2, I1, r21) +
                           w1 * (1 - x) * A(chi2, lambda1, I2, r22));
            if (fabs(mu) < 0.999)
                result += c * (w2 * (1 - x) * B(chi1, lambda2, I1, r21) +
                               w1 * (1 - x) * B(chi2, lambda1, I2, r22));
            else
                result += c * (w2 * (1 - x) * 4. * (lambda2 + chi1) * I1[L04] / 35. +
                               w1 * (1 - x) * 4. * (lambda1 + chi2) * I2[L04] / 35.);
        } else if (r21 == 0 && r22 != 0) {
            result += c * (w2 * (1 - chi1 / chi2) * (-2 * chi1 * I00_0 / 15.) +
                           w1 * (1 - x) * (A(chi2, lambda1, I2, r22) + B(chi2, lambda1, I2, r22)));
        } else if (r21 != 0 && r22 == 0) {
            result += c * (w2 * (1 - x) * (A(chi1, lambda2, I1, r21) + B(chi1, lambda2, I1, r21)) +
                           w1 * (1 - chi2 / chi1) * (-2 * chi2 * I00_0 / 15.));
        } else {
            result += c * (w2 * (1 - chi1 / chi2) * (-2 * chi1 * I00_0 / 15.) +
                           w1 * (1 - chi2 / chi1) * (-2 * chi2 * I00_0 / 15.));
        }
    }
    return result;
}

template <typename TT>
__global__ void __launch_bounds__(LENS_THREADS)
    lens_single_kernel(LensArgs a, LensBg64 g, const TT *__restrict__ tab_x,
                       const typename Rec4<TT>::type *__restrict__ rec,
                       const int *__restrict__ req_spectrum, const double *__restrict__ req_z_mean,
                       const int64_t *__restrict__ req_offset, const double *__restrict__ sep,
                       const double *__restrict__ rule, double *__restrict__ part, int *err)
{
    const long long item = (long long)blockIdx.x * (LENS_THREADS / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (item >= a.n_items) return;
    const long long pair = a.pair0 + item / a.n_mu_run;
    const int im = a.mu0 + (int)(item % a.n_mu_run);
    const int q = lens_find_request(req_offset, a.n_req, pair);
    const int s = req_spectrum[q];
    const double *xf = rule + 2 * a.n_mu, *wf = xf + a.n_x, *xh = wf + a.n_x, *wh = xh + a.nh;
    const double mu = rule[im];
    const LensGeom G = lens_geom(g, req_z_mean[q], mu, sep[pair]);
    const double b1 = a.has_b1 ? spl_eval(g.b1, G.z1c) : 1.0;
    const double b2 = a.has_b2 ? spl_eval(g.b2, G.z2c) : 1.0;
    const double s1 = a.has_s1 ? spl_eval(g.s1, G.z1c) : 0.0;
    const double s2 = a.has_s2 ? spl_eval(g.s2, G.z2c) : 0.0;
    const double f1c = spl_eval(g.f, G.z1c), f2c = spl_eval(g.f, G.z2c);
    const double D1z1c = spl_eval(g.D1, G.z1c), D1z2c = spl_eval(g.D1, G.z2c);
    const typename Rec4<TT>::type *recs = rec + (size_t)s * (a.tab_len - 1) * LENS_NT;
    const double xs = fmin(G.chi1, G.chi2) * G.ct / fmax(G.chi1, G.chi2);
    const bool split = a.nh > 0 && xs > 0 && xs < 1;
    double sum = 0;
    for (int p = 0; p < (split ? 2 : 1); ++p) {
        const double lo = (split && p) ? xs : 0.0, hi = (split && !p) ? xs : 1.0;
        const double c = 0.5 * (lo + hi), hw = 0.5 * (hi - lo);
        const int np = split ? a.nh : a.n_x;
        const double *gx = split ? xh : xf, *gw = split ? wh : wf;
        double ps = 0;
        for (int k = lane; k < np; k += 32)
            ps += gw[k] * lens_single_xi<TT>(a, g, recs, tab_x, G, c + hw * gx[k], b1, b2, s1, s2,
                                             f1c, f2c, D1z1c, D1z2c, mu);
        sum += hw * warp_sum(ps);
    }
    if (lane == 0) {
        if (!isfinite(sum)) cg_flag(err, CG_ERR_NONFINITE);
        part[item] = sum;
    }
}

// Mixed path of lens_single_kernel: the same integrand in FP32, Kahan sums per
// lane.  The RSD-lensing polynomials Q and P are written in d = chi_i -
// lambda_j and s, where every term has the size of the result, so they need no
// FP64; d itself is formed from 1 - x and chi2 - chi1 = sep mu (d21 = chi2 (1 -
// x) - sep mu, d12 = chi1 (1 - x) + sep mu), which keeps its relative precision
// where lambda_j approaches chi_i.  D1 / a along both lines of sight is the
// per-item degree-9 polynomial of lens_double_kernel.  The per-item background
// values are FP64 lookups spread over the lanes (one per lane).  With T =
// double (tables and line rules in FP64) it is the same algorithm in FP64, the
// matched-algorithm baseline of the mixed path.
template <typename T, typename S, typename TT>
__global__ void __launch_bounds__(LENS_THREADS)
    lens_single_fast_kernel(LensArgs a, LensBg64 g, LensBgT<S> gT, LensPoly poly,
                            const TT *__restrict__ tab_x,
                            const typename Rec4<TT>::type *__restrict__ rec,
                            const int *__restrict__ req_spectrum,
                            const double *__restrict__ req_z_mean,
                            const int64_t *__restrict__ req_offset,
                            const double *__restrict__ sep, const double *__restrict__ rule,
                            double *__restrict__ part, int *err)
{
    const long long item = (long long)blockIdx.x * (LENS_THREADS / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (item >= a.n_items) return; // whole warps leave together
    const unsigned full = 0xffffffffu;
    const long long pair = a.pair0 + item / a.n_mu_run;
    const int im = a.mu0 + (int)(item % a.n_mu_run);
    const int q = lens_find_request(req_offset, a.n_req, pair);
    const int s = req_spectrum[q];
    const double mu = rule[im], r = sep[pair];
    // geometry as lens_geom, with z(chi1) on even and z(chi2) on odd lanes
    const double chi_mean = spl_eval(g.chi_of_z, req_z_mean[q]);
    const double chi1 = chi_mean - r * mu / 2., chi2 = chi_mean + r * mu / 2.;
    const double sd = r * r * (1 - mu * mu) / (2. * chi_mean * chi_mean - mu * mu * r * r / 2.);
    const double zl = spl_eval(g.z_of_chi, (lane & 1) ? chi2 : chi1);
    const double z1c = __shfl_sync(full, zl, 0), z2c = __shfl_sync(full, zl, 1);
    // lanes 0-7: b1, b2, s1, s2, f(z1), f(z2), D1(z1), D1(z2)
    const int k8 = lane & 7;
    const bool set = k8 == 0 ? a.has_b1 : k8 == 1 ? a.has_b2 : k8 == 2 ? a.has_s1 :
                     k8 == 3 ? a.has_s2 : true;
    const Spl64 sp = k8 == 0 ? g.b1 : k8 == 1 ? g.b2 : k8 == 2 ? g.s1 : k8 == 3 ? g.s2 :
                     k8 < 6 ? g.f : g.D1;
    double bv = k8 < 2 ? 1.0 : 0.0;
    if (set) bv = spl_eval(sp, (k8 & 1) ? z2c : z1c);
    const double b1 = __shfl_sync(full, bv, 0), b2 = __shfl_sync(full, bv, 1);
    const double s1 = __shfl_sync(full, bv, 2), s2 = __shfl_sync(full, bv, 3);
    const double f1c = __shfl_sync(full, bv, 4), f2c = __shfl_sync(full, bv, 5);
    const double D1z1c = __shfl_sync(full, bv, 6), D1z2c = __shfl_sync(full, bv, 7);
    // D1 / a along both lines of sight: lanes 0-9 side 1 (chi1), 10-19 side 2
    T gc1[LENS_PDEG + 1], gc2[LENS_PDEG + 1];
    {
        const int side = lane >= LENS_PDEG + 1, j = lane % (LENS_PDEG + 1);
        T gv = T(0);
        if (lane < 2 * (LENS_PDEG + 1)) {
            const T lam = (T)(side ? chi2 : chi1) * T(0.5) * (lens_cheb<T>(poly, j) + T(1));
            const T zz = spl_eval(gT.z_of_chi, lam);
            gv = spl_eval(gT.D1, zz) / spl_eval(gT.a, zz);
        }
        double c = 0.0;
#pragma unroll
        for (int k = 0; k <= LENS_PDEG; ++k)
            c += poly.vinv[j][k] * (double)__shfl_sync(full, gv, side * (LENS_PDEG + 1) + k);
        const T cf = (T)c;
#pragma unroll
        for (int k = 0; k <= LENS_PDEG; ++k) {
            gc1[k] = __shfl_sync(full, cf, k);
            gc2[k] = __shfl_sync(full, cf, LENS_PDEG + 1 + k);
        }
    }
    const typename Rec4<TT>::type *recs = rec + (size_t)s * (a.tab_len - 1) * LENS_NT;
    const TT inv_dlog = (TT)a.inv_dlog;
    const T I00_0 = (T)lens_at_zero<TT>(recs, L00), I11_0 = (T)lens_at_zero<TT>(recs, L11);
    const T c1 = (T)chi1, c2 = (T)chi2, dchi = (T)(r * mu), ss = (T)sd;
    const T ct = (T)(1 - sd), omc2 = (T)(sd * (2 - sd));
    const T c2m1 = (T)(1 - 2 * sd * (2 - sd));
    const bool den = a.contrib & COFFE_GPU_DEN, rsd = a.contrib & COFFE_GPU_RSD;
    const bool wide = fabs(mu) < 0.999;
    // functions.c:1708-1780 and 2174-2306 with the background factors folded
    const double kc = a.pref2 * 1.5 * a.Om;
    const T kd2 = (T)(-kc * b1 * (2 - 5 * s2) * D1z1c * chi1 * chi2);
    const T kd1 = (T)(-kc * b2 * (2 - 5 * s1) * D1z2c * chi1 * chi2);
    const T kr2 = (T)(kc * chi2 * f1c * (2 - 5 * s2) * D1z1c);
    const T kr1 = (T)(kc * chi1 * f2c * (2 - 5 * s1) * D1z2c);
    auto Q = [&](T ch, T d) {
        return d * d * d * (T(8) - T(24) * ss + T(12) * ss * ss) +
               ch * d * d * (T(-2) + T(38) * ss - T(18) * ss * ss - T(6) * ss * ss * ss) +
               ch * ch * d * ss * (T(-22) + T(9) * ss + T(12) * ss * ss) +
               ch * ch * ch * ss * (T(2) - T(3) * ss - T(6) * ss * ss);
    };
    auto P = [&](T ch, T d) {
        const T d2 = d * d, d3 = d2 * d, d4 = d2 * d2, d5 = d4 * d;
        const T ch2 = ch * ch, ch3 = ch2 * ch, ch4 = ch2 * ch2, ch5 = ch4 * ch;
        const T s2 = ss * ss, s3 = s2 * ss;
        return d5 * (T(4) - T(12) * ss + T(6) * s2) +
               ch * d4 * (T(-8) + T(60) * ss - T(48) * s2 + T(6) * s3) +
               ch2 * d3 * ss * (T(-92) + T(114) * ss - T(20) * s2 - s3) +
               ch3 * d2 * ss * (T(48) - T(120) * ss + T(26) * s2 + T(3) * s3) +
               ch4 * d * s2 * (T(60) - T(16) * ss - T(3) * s2) +
               ch5 * s2 * (T(-12) + T(4) * ss + s2);
    };
    // one side: density and RSD parts times D1 / a, without the (1 - x) factor
    auto side_val = [&](T ch, T la, T d, T r2, const T *I, T kd, T kr, T gl) {
        T v = T(0);
        if (r2 != T(0)) {
            const T ir2 = T(1) / r2;
            if (den) v += kd * (T(2) * ct * I[L11] - ch * la * omc2 * I[L02] * ir2);
            if (rsd) {
                v += kr * ((la - T(6) * ch * ct + T(3) * la * c2m1) * I[L00] * (T(1) / T(15)) -
                           Q(ch, d) * I[L02] * ir2 * (T(1) / T(21)));
                v += kr * (wide ? -P(ch, d) * I[L04] * ir2 * ir2 * (T(1) / T(35))
                                : T(4) * (la + ch) * I[L04] * (T(1) / T(35)));
            }
        } else {
            if (den) v += kd * T(2) * I11_0;
            if (rsd) v += kr * (T(-2) * ch * I00_0 * (T(1) / T(15)));
        }
        return v * gl;
    };
    constexpr bool F32 = sizeof(T) == 4;
    const double *xf = rule + 2 * a.n_mu, *wf = xf + a.n_x, *xh = wf + a.n_x, *wh = xh + a.nh;
    const float *xf32 = reinterpret_cast<const float *>(rule + 2 * a.n_mu + 2 * a.n_x + 2 * a.nh);
    const float *wf32 = xf32 + a.n_x, *xh32 = wf32 + a.n_x, *wh32 = xh32 + a.nh;
    const double xs = fmin(chi1, chi2) * (1 - sd) / fmax(chi1, chi2);
    const bool split = a.nh > 0 && xs > 0 && xs < 1;
    double sum = 0;
    for (int p = 0; p < (split ? 2 : 1); ++p) {
        const double lo = (split && p) ? xs : 0.0, hi = (split && !p) ? xs : 1.0;
        const T cf = (T)(0.5 * (lo + hi)), omcf = (T)(1 - 0.5 * (lo + hi));
        const T hwf = (T)(0.5 * (hi - lo));
        const int np = split ? a.nh : a.n_x;
        const float *gx32 = split ? xh32 : xf32, *gw32 = split ? wh32 : wf32;
        const double *gx64 = split ? xh : xf, *gw64 = split ? wh : wf;
        Acc<T> ps;
        for (int k = lane; k < np; k += 32) {
            const T gxk = F32 ? (T)gx32[k] : (T)gx64[k];
            const T gwk = F32 ? (T)gw32[k] : (T)gw64[k];
            const T x = lens_fma(hwf, gxk, cf), omx = lens_fma(-hwf, gxk, omcf);
            const T t = T(2) * x - T(1);
            const T la1 = c1 * x, la2 = c2 * x;
            const T d21 = lens_fma(c2, omx, -dchi), d12 = lens_fma(c1, omx, dchi);
            const T r21 = d21 * d21 + T(2) * c1 * la2 * ss;
            const T r22 = d12 * d12 + T(2) * c2 * la1 * ss;
            T I1[LENS_NT], I2[LENS_NT];
            lens_tables<T, TT>(recs, tab_x, a.tab_len, inv_dlog, sqrt(r21), I1);
            lens_tables<T, TT>(recs, tab_x, a.tab_len, inv_dlog, sqrt(r22), I2);
            const T v = side_val(c1, la2, d21, r21, I1, kd2, kr2, lens_horner(gc2, t)) +
                        side_val(c2, la1, d12, r22, I2, kd1, kr1, lens_horner(gc1, t));
            ps.add(gwk * omx * v);
        }
        sum += (double)hwf * warp_sum(ps.value());
    }
    if (lane == 0) {
        if (!isfinite(sum)) cg_flag(err, CG_ERR_NONFINITE);
        part[item] = sum;
    }
}

__device__ __forceinline__ double lens_legendre(int l, double x)
{
    if (l == 0) return 1.0;
    if (l == 1) return x;
    double p0 = 1.0, p1 = x;
    for (int k = 2; k <= l; ++k) {
        const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / (double)k;
        p0 = p1;
        p1 = p2;
    }
    return p1;
}

// out[pair][j] += (2l+1) sum_mu (w_mu / 2) P_l(mu) (single + double partials)
__global__ void lens_reduce_kernel(LensArgs a, const double *__restrict__ rule,
                                   const double *__restrict__ part_d,
                                   const double *__restrict__ part_s, long long n_pairs,
                                   double *__restrict__ out, int *err)
{
    // one warp per (pair, l); lanes take the mu nodes from the first one the
    // multipole sums (so a multipole's terms meet in the same lanes and order
    // whether or not the mu < 0 half was evaluated)
    const long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= n_pairs * a.n_l) return; // whole warps leave together
    const long long pl = t / a.n_l;
    const int j = (int)(t % a.n_l);
    const int l = a.ls[j];
    const bool half = a.sym && l % 2 == 0 && a.n_mu_run == a.n_mu;
    const int first = half ? a.n_mu / 2 : a.mu0, end = a.mu0 + a.n_mu_run;
    const double w = (half ? 2.0 : a.mu_w) * 0.5;
    double sum = 0;
    for (int im = first + lane; im < end; im += 32) {
        const int k = im - a.mu0;
        double v = 0;
        if (part_d) v += part_d[pl * a.n_mu_run + k];
        if (part_s) v += part_s[pl * a.n_mu_run + k];
        sum += w * rule[a.n_mu + im] * v * lens_legendre(l, rule[im]);
    }
    sum = warp_sum(sum);
    if (lane == 0) {
        const double res = (2 * l + 1) * sum;
        if (!isfinite(res)) cg_flag(err, CG_ERR_NONFINITE);
        out[(a.pair0 + pl) * a.n_l + j] += res;
    }
}

// correlation function: out[pair][m] += single + double partials at mu_m
__global__ void lens_cf_reduce_kernel(LensArgs a, const double *__restrict__ part_d,
                                      const double *__restrict__ part_s, long long n_pairs,
                                      double *__restrict__ out, int *err)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_pairs * a.n_mu_run) return;
    double v = 0;
    if (part_d) v += part_d[t];
    if (part_s) v += part_s[t];
    if (!isfinite(v)) cg_flag(err, CG_ERR_NONFINITE);
    out[a.pair0 * a.n_mu_run + t] += v;
}

// n-point Gauss-Legendre nodes and weights on [-1, 1] (Newton on P_n from the
// Tricomi initial guesses), nodes ascending
void gauss_legendre(int n, double *x, double *w)
{
    for (int i = 0; i < (n + 1) / 2; ++i) {
        double z = cos(CG_PI * (i + 0.75) / (n + 0.5));
        double dp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1.0, p2 = 0.0;
            for (int j = 1; j <= n; ++j) {
                const double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
            }
            dp = n * (z * p1 - p2) / (z * z - 1.0);
            const double z1 = z;
            z = z1 - p1 / dp;
            if (fabs(z - z1) <= 1e-15) break;
        }
        x[i] = -z;
        x[n - 1 - i] = z;
        w[i] = w[n - 1 - i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}


// ------------------------------------------------------------------ flat sky
#define FLAT_MAX_L 8
#define FLAT_WARPS 4
#define FLAT_CAP 128

struct FlatArgs {
    int n_req, n_l, tab_len, n_terms;
    double inv_dlog, Om, pref2, pref4, epsrel;
    int has_b1, has_b2, has_s1, has_s2;
    int ls[FLAT_MAX_L];
    int dl_term[FLAT_MAX_L][5];   // half-integer table of each k in the den-lensing sum
    double dl_coef[FLAT_MAX_L][5]; // (-1)^k 2^-k C(l,k) C(2l-2k,l) (l/2-k)!
    int ll_term[FLAT_MAX_L];      // integer table (1, l) of lensing-lensing
    double ll_coef[FLAT_MAX_L];   // (2l+1) l! / 2^l / ((l/2)!)^2
};

// Akima value of table t of spectrum s at r (NaN outside)
template <typename TT>
__device__ __forceinline__ double flat_table(const FlatArgs &a, const TT *__restrict__ tab_x,
                                             const TT *__restrict__ tab_y, int s, int t, double r)
{
    const TT *y = tab_y + ((size_t)s * a.n_terms + t) * a.tab_len;
    const int i = lens_interval<TT>(tab_x, a.tab_len, (TT)a.inv_dlog, (TT)r);
    if (i < 0) return cg_nan<double>();
    return (double)akima_eval_at<TT>(tab_x, y, a.tab_len, i, (TT)r);
}

// flat-sky density-lensing multipole (functions.c:4136-4253) times 2 pi^2
// (signal.c:619-630), added to out; one thread per (pair, l)
template <typename TT>
__global__ void flat_denlen_kernel(FlatArgs a, LensBg64 g, const TT *__restrict__ tab_x,
                                   const TT *__restrict__ tab_y, const int *__restrict__ req_spectrum,
                                   const double *__restrict__ req_z_mean,
                                   const int64_t *__restrict__ req_offset,
                                   const double *__restrict__ sep, long long total,
                                   double *__restrict__ out, int *err)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total * a.n_l) return;
    const long long item = t / a.n_l;
    const int j = (int)(t % a.n_l), l = a.ls[j];
    if (l % 2) return; // odd multipoles are zero (functions.c:4244-4247)
    const int q = lens_find_request(req_offset, a.n_req, item);
    const int s = req_spectrum[q];
    const double z = req_z_mean[q], r = sep[item];
    const double s1 = a.has_s1 ? spl_eval(g.s1, z) : 0.0, s2 = a.has_s2 ? spl_eval(g.s2, z) : 0.0;
    const double b1 = a.has_b1 ? spl_eval(g.b1, z) : 1.0, b2 = a.has_b2 ? spl_eval(g.b2, z) : 1.0;
    double result = 0;
    for (int k = 0; k <= l / 2; ++k)
        result += a.dl_coef[j][k] * flat_table<TT>(a, tab_x, tab_y, s, a.dl_term[j][k], r);
    const double D1 = spl_eval(g.D1, z);
    result *= -3 * a.Om / CG_PI / 8 * (2 * l + 1) * D1 * D1 * (1 + z) * r *
              ((2 - 5 * s1) * b2 + (2 - 5 * s2) * b1) * pow(2.0, 1 - l / 2);
    const double v = 2 * CG_PI * CG_PI * result / sqrt(2 * CG_PI) * a.pref2;
    if (!isfinite(v)) cg_flag(err, CG_ERR_NONFINITE);
    out[item * a.n_l + j] += v;
}

// functions_flatsky_lensing_lensing_multipoles (functions.c:4020-4132) at x
template <typename TT> struct FlatLL {
    const FlatArgs *a;
    const LensBg64 *g;
    const TT *tab_x, *tab_y;
    int s, j, l;
    double z, r, chi_mean, pre;
    __device__ __forceinline__ double operator()(double x) const
    {
        const double lambda = chi_mean * x;
        const double zl = spl_eval(g->z_of_chi, lambda);
        const double D1 = spl_eval(g->D1, zl);
        const double v = pre * flat_table<TT>(*a, tab_x, tab_y, s, a->ll_term[j], x * r) * D1 * D1 *
                         (1 + zl) * (1 + zl) * (x * (1 - x)) * (x * (1 - x));
        return l > 0 ? v * x * r * a->pref4 : v * a->pref4;
    }
};

// flat-sky lensing-lensing multipole: 2 pi^2 times the QAG integral over x in
// [0, 1] (signal.c:708-734), added to out; one warp per (pair, even l)
template <typename TT>
__global__ void __launch_bounds__(32 * FLAT_WARPS)
    flat_lenlen_kernel(FlatArgs a, LensBg64 g, const TT *__restrict__ tab_x,
                       const TT *__restrict__ tab_y, const int *__restrict__ req_spectrum,
                       const double *__restrict__ req_z_mean, const int64_t *__restrict__ req_offset,
                       const double *__restrict__ sep, long long total, double *__restrict__ out,
                       int *err)
{
    __shared__ double sa[FLAT_WARPS][FLAT_CAP], sb[FLAT_WARPS][FLAT_CAP], sr[FLAT_WARPS][FLAT_CAP],
        se[FLAT_WARPS][FLAT_CAP];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long t = (long long)blockIdx.x * FLAT_WARPS + w;
    if (t >= total * a.n_l) return;
    const long long item = t / a.n_l;
    const int j = (int)(t % a.n_l), l = a.ls[j];
    if (l % 2) return;
    const int q = lens_find_request(req_offset, a.n_req, item);
    FlatLL<TT> f;
    f.a = &a;
    f.g = &g;
    f.tab_x = tab_x;
    f.tab_y = tab_y;
    f.s = req_spectrum[q];
    f.j = j;
    f.l = l;
    f.z = req_z_mean[q];
    f.r = sep[item];
    f.chi_mean = spl_eval(g.chi_of_z, f.z);
    const double s1 = a.has_s1 ? spl_eval(g.s1, f.z) : 0.0, s2 = a.has_s2 ? spl_eval(g.s2, f.z) : 0.0;
    f.pre = a.ll_coef[j] * 9 * a.Om * a.Om * (2 - 5 * s1) * (2 - 5 * s2) * pow(f.chi_mean, 3) / 8. /
            CG_PI;
    QagStore<double> store{sa[w], sb[w], sr[w], se[w], FLAT_CAP};
    int status = 0;
    const double v = qag61_warp<double>(f, 0.0, 1.0, 0.0, a.epsrel, store, 50000, &status);
    if (lane == 0) {
        if (status == 1) cg_flag(err, CG_ERR_QAG_LIMIT);
        const double res = 2 * CG_PI * CG_PI * v;
        if (!isfinite(res)) cg_flag(err, CG_ERR_NONFINITE);
        out[item * a.n_l + j] += res;
    }
}

double host_fact(int n)
{
    double r = 1;
    for (int i = 2; i <= n; ++i) r *= i;
    return r;
}

template <typename T, typename S, typename TT, bool FAST>
int lensing_launch(coffe_gpu_ctx *ctx, LensArgs a, const LensBg64 &g64, const LensBgT<S> &gT,
                   const int *req_spectrum, const double *req_z_mean, const int64_t *req_offset,
                   const double *sep, double *out, long long total, bool do_single,
                   bool do_double, const double *rule, bool per_node)
{
    typedef typename Rec4<TT>::type R;
    int st;
    const TT *tab_x = (const TT *)(sizeof(TT) == 8 ? ctx->tab_x.p : ctx->tab_x32.p);
    const long long n_int = (long long)ctx->n_spectra * (a.tab_len - 1);
    const long long n_rec = n_int * LENS_NT;
    // fast algorithm: the five combined records follow the six tables' records
    const size_t rec_bytes = sizeof(R) * (size_t)(n_rec + (FAST ? n_int * LENS_NC : 0));
    if ((st = cg_ensure(ctx, ctx->lens_rec, rec_bytes))) return st;
    R *rec = (R *)ctx->lens_rec.p;
    R *rec5 = FAST ? rec + n_rec : nullptr;
    lens_records_kernel<TT><<<(unsigned)((n_rec + 255) / 256), 256, 0, ctx->stream>>>(
        a, tab_x, (const TT *)ctx->tab_y.p, ctx->n_spectra, rec);
    if ((st = cg_after_launch(ctx, "lens_records_kernel"))) return st;
    if (FAST && do_double) {
        lens_combine_kernel<R><<<(unsigned)((n_int + 255) / 256), 256, 0, ctx->stream>>>(
            rec, n_int, rec5);
        if ((st = cg_after_launch(ctx, "lens_combine_kernel"))) return st;
    }
    const bool single = do_single;
    // pairs per chunk: partials of at most 2^22 (pair, mu) items per kind
    const long long chunk = std::max(1LL, std::min(total, (1LL << 22) / a.n_mu_run));
    if ((st = cg_ensure(ctx, ctx->lens_part, sizeof(double) * 2 * (size_t)(chunk * a.n_mu_run))))
        return st;
    double *part_d = (double *)ctx->lens_part.p;
    double *part_s = part_d + chunk * a.n_mu_run;
    static const LensPoly poly = lens_poly_tables();
    for (long long p0 = 0; p0 < total; p0 += chunk) {
        const long long np = std::min(chunk, total - p0);
        a.pair0 = p0;
        a.n_items = np * a.n_mu_run;
        if (do_double) {
            lens_double_kernel<T, S, TT, FAST>
                <<<(unsigned)a.n_items, LENS_THREADS, 0, ctx->stream>>>(
                a, g64, gT, poly, tab_x, rec, rec5, req_spectrum, req_z_mean, req_offset, sep,
                rule, part_d, ctx->d_err);
            if ((st = cg_after_launch(ctx, "lens_double_kernel"))) return st;
        }
        if (single) {
            const long long blocks = (a.n_items + LENS_THREADS / 32 - 1) / (LENS_THREADS / 32);
            if constexpr (FAST)
                lens_single_fast_kernel<T, S, TT>
                    <<<(unsigned)blocks, LENS_THREADS, 0, ctx->stream>>>(
                        a, g64, gT, poly, tab_x, rec, req_spectrum, req_z_mean, req_offset, sep,
                        rule, part_s, ctx->d_err);
            else
                lens_single_kernel<TT><<<(unsigned)blocks, LENS_THREADS, 0, ctx->stream>>>(
                    a, g64, tab_x, rec, req_spectrum, req_z_mean, req_offset, sep, rule, part_s,
                    ctx->d_err);
            if ((st = cg_after_launch(ctx, "lens_single_kernel"))) return st;
        }
        if (per_node) {
            const long long nt = np * a.n_mu_run;
            lens_cf_reduce_kernel<<<(unsigned)((nt + 127) / 128), 128, 0, ctx->stream>>>(
                a, do_double ? part_d : nullptr, single ? part_s : nullptr, np, out, ctx->d_err);
            if ((st = cg_after_launch(ctx, "lens_cf_reduce_kernel"))) return st;
        } else {
            const long long nt = np * a.n_l;
            lens_reduce_kernel<<<(unsigned)((nt + 3) / 4), 128, 0, ctx->stream>>>(
                a, rule, do_double ? part_d : nullptr, single ? part_s : nullptr, np, out,
                ctx->d_err);
            if ((st = cg_after_launch(ctx, "lens_reduce_kernel"))) return st;
        }
    }
    return COFFE_GPU_OK;
}

// ----------------------------------------------------------------- adjoint
// Reverse mode of the full-sky lensing multipoles in FP64 (the parity path's
// six-table integrands, the same rules, mu symmetry and weights).  The
// integrands are linear in the table values; a table value at r in interval i
// is y_i + b dx + c dx^2 + d dx^3 of that interval's Akima record, so the
// cotangent of the records is accumulated as the four moments
// gR[((s * LENS_NT + t) * (len - 1) + i) * 4 + p] = sum g dx^p over the
// lookups, and adj_lens_records_kernel carries it to the table knots.

// cotangent of each (pair, mu node) partial of this chunk: the weight with
// which lens_reduce_kernel adds the partial to each multipole, times grad_out
__global__ void adj_lens_gpm_kernel(LensArgs a, const double *__restrict__ rule,
                                    const double *__restrict__ grad_out, long long n_pairs,
                                    double *__restrict__ gpm)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_pairs * a.n_mu_run) return;
    const long long pl = t / a.n_mu_run;
    const int im = a.mu0 + (int)(t % a.n_mu_run);
    double g = 0.0;
    for (int j = 0; j < a.n_l; ++j) {
        const int l = a.ls[j];
        const bool half = a.sym && l % 2 == 0 && a.n_mu_run == a.n_mu;
        const int first = half ? a.n_mu / 2 : a.mu0;
        if (im < first) continue;
        const double w = (half ? 2.0 : a.mu_w) * 0.5;
        g += grad_out[(a.pair0 + pl) * a.n_l + j] * (2 * l + 1) * w * rule[a.n_mu + im] *
             lens_legendre(l, rule[im]);
    }
    gpm[t] = g;
}

__device__ __forceinline__ void adj_rec_add(double *gR, long long at, double g, double dx)
{
    if (g == 0.0) return;
    const double g1 = g * dx, g2 = g1 * dx;
    atomicAdd(gR + at, g);
    atomicAdd(gR + at + 1, g1);
    atomicAdd(gR + at + 2, g2);
    atomicAdd(gR + at + 3, g2 * dx);
}

// table value at r from the FP64 records; interval and offset for the moments
__device__ __forceinline__ double adj_table_at(const double4_32a *__restrict__ recs, int i, int t,
                                               double dx)
{
    const double4_32a c = ldg_c4(recs + (size_t)i * LENS_NT + t);
    return c.x + dx * (c.y + dx * (c.z + c.w * dx));
}

// lensing-lensing partial of one (pair, mu node) (lens_double_kernel's FP64
// form) and, with gpm, the record cotangents of its lookups
__global__ void __launch_bounds__(LENS_THREADS)
    adj_lens_double_kernel(LensArgs a, LensBg64 g64, LensBgT<Spl64> gT,
                           const double *__restrict__ tab_x, const double4_32a *__restrict__ rec,
                           const int *__restrict__ req_spectrum,
                           const double *__restrict__ req_z_mean,
                           const int64_t *__restrict__ req_offset, const double *__restrict__ sep,
                           const double *__restrict__ rule, const double *__restrict__ gpm,
                           double *__restrict__ part, double *__restrict__ gR, int *err)
{
    __shared__ double red[LENS_THREADS / 32];
    const long long item = blockIdx.x;
    const long long pair = a.pair0 + item / a.n_mu_run;
    const int im = a.mu0 + (int)(item % a.n_mu_run);
    const int q = lens_find_request(req_offset, a.n_req, pair);
    const int s = req_spectrum[q];
    const double *xf = rule + 2 * a.n_mu, *wf = xf + a.n_x, *xh = wf + a.n_x, *wh = xh + a.nh;
    const LensGeom G = lens_geom(g64, req_z_mean[q], rule[im], sep[pair]);
    const double s1 = a.has_s1 ? spl_eval(g64.s1, G.z1c) : 0.0;
    const double s2 = a.has_s2 ? spl_eval(g64.s2, G.z2c) : 0.0;
    const double pre = 9. * a.Om * a.Om * (2 - 5 * s1) * (2 - 5 * s2) / 4. * G.chi1 * G.chi2 * a.pref4;
    const int ni = a.tab_len - 1;
    const double4_32a *recs = rec + (size_t)s * ni * LENS_NT;
    double *gRs = gR ? gR + (size_t)s * LENS_NT * ni * 4 : nullptr;
    const double chi1 = G.chi1, chi2 = G.chi2, ss = G.s, ct = G.ct, c2m = -G.omc2;
    const double i11_0 = lens_at_zero<double>(recs, L11);
    const double gp = gpm ? gpm[item] * pre : 0.0;
    Acc<double> acc;
    for (int ia = threadIdx.x; ia < a.n_x; ia += blockDim.x) {
        const double x1 = 0.5 * (xf[ia] + 1.0);
        const double l1 = chi1 * x1;
        const double z1 = spl_eval(gT.z_of_chi, l1);
        const double g1 = spl_eval(gT.D1, z1) / spl_eval(gT.a, z1) * (1 - x1);
        const double xs = x1 * G.chi1 / G.chi2;
        const bool split = a.nh > 0 && xs > 0 && xs < 1;
        double line = 0.0;
        for (int p = 0; p < (split ? 2 : 1); ++p) {
            const double lo = (split && p) ? xs : 0.0, hi = (split && !p) ? xs : 1.0;
            const double c = 0.5 * (lo + hi), hw = 0.5 * (hi - lo);
            const int np = split ? a.nh : a.n_x;
            const double *gx = split ? xh : xf, *gw = split ? wh : wf;
            const double gl = gp * 0.5 * wf[ia] * g1 * hw;
            Acc<double> pa;
            for (int k = 0; k < np; ++k) {
                const double x2 = c + hw * gx[k], wk = gw[k];
                const double z2 = spl_eval(gT.z_of_chi, chi2 * x2);
                const double g2 = spl_eval(gT.D1, z2) / spl_eval(gT.a, z2) * (1 - x2);
                const double l2 = chi2 * x2;
                const double ll = l1 * l2;
                const double dl = l1 - l2;
                const double r2 = dl * dl + 2 * ll * ss;
                const double gn = gl * wk * g2; // cotangent of v at this node
                double v;
                if (r2 > 1e-20) {
                    // functions.c:3695-3775 as a linear form in the six tables
                    double cof[LENS_NT];
                    cof[L00] = 2 * c2m * ll / 5;
                    cof[L20] = 4 * ct / 3;
                    cof[L11] = 4 * ct * (r2 + 6 * ct * ll) / 15;
                    cof[L02] = 2 * c2m * ll * (2 * r2 + 3 * ct * ll) / 7 / r2;
                    cof[L13] = 2 * ct * (2 * r2 * r2 + 12 * ct * r2 * ll + 15 * c2m * ll * ll) / 15 / r2;
                    cof[L04] = c2m * ll * (6 * r2 * r2 + 30 * ct * r2 * ll + 35 * c2m * ll * ll) / 35 /
                               r2 / r2;
                    const double r = sqrt(r2);
                    const int i = lens_interval<double>(tab_x, a.tab_len, a.inv_dlog, r);
                    if (i < 0) {
                        v = cg_nan<double>();
                    } else {
                        const double dx = r - tab_x[i];
                        v = 0.0;
#pragma unroll
                        for (int t = 0; t < LENS_NT; ++t) v += cof[t] * adj_table_at(recs, i, t, dx);
                        if (gRs)
#pragma unroll
                            for (int t = 0; t < LENS_NT; ++t)
                                adj_rec_add(gRs, ((long long)t * ni + i) * 4, gn * cof[t], dx);
                    }
                } else {
                    // functions.c:3801-3833
                    v = 4 + 24 * ll * i11_0 / 15;
                    if (gRs && gn != 0.0)
                        atomicAdd(gRs + (long long)L11 * ni * 4, gn * 24 * ll / 15);
                }
                pa.add(wk * g2 * v);
            }
            line += hw * pa.value();
        }
        acc.add(0.5 * wf[ia] * g1 * line);
    }
    double tot = warp_sum(acc.value());
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = tot;
    __syncthreads();
    if (threadIdx.x == 0 && part) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        const double res = pre * t;
        if (!isfinite(res)) cg_flag(err, CG_ERR_NONFINITE);
        part[item] = res;
    }
}

// The single-integrated den and RSD parts at (mu, x) (lens_single_xi) as
// linear forms in the six tables at r21 (c1), at r22 (c2) and in I11(0),
// I00(0)
struct AdjSingleCoef {
    double den1[LENS_NT], den2[LENS_NT], rsd1[LENS_NT], rsd2[LENS_NT];
    double den_i11_0, rsd_i00_0;
};

__device__ void adj_single_coef(const LensArgs &a, const LensGeom &G, double x, double lambda1,
                                double lambda2, double r21, double r22, double b1, double b2,
                                double s1, double s2, double f1c, double f2c, double D1z1c,
                                double D1z2c, double ga1, double ga2, double mu,
                                AdjSingleCoef &k)
{
    // ga1 = D1 / a at lambda1, ga2 at lambda2
    for (int t = 0; t < LENS_NT; ++t) k.den1[t] = k.den2[t] = k.rsd1[t] = k.rsd2[t] = 0.0;
    k.den_i11_0 = k.rsd_i00_0 = 0.0;
    const double chi1 = G.chi1, chi2 = G.chi2, ct = G.ct, omc2 = G.omc2;
    if (a.contrib & COFFE_GPU_DEN) {
        const double K1 = a.pref2 * (-3 * a.Om / 2.) * b1 * (2 - 5 * s2) * D1z1c * (1 - x) * ga2;
        const double K2 = a.pref2 * (-3 * a.Om / 2.) * b2 * (2 - 5 * s1) * D1z2c * (1 - x) * ga1;
        if (r21 != 0.0) {
            k.den1[L11] = K1 * chi2 * 2 * chi1 * ct;
            k.den1[L02] = -K1 * chi2 * chi1 * chi1 * lambda2 * omc2 / r21;
        } else {
            k.den_i11_0 += K1 * chi2 * 2 * chi1;
        }
        if (r22 != 0.0) {
            k.den2[L11] = K2 * chi1 * 2 * chi2 * ct;
            k.den2[L02] = -K2 * chi1 * chi2 * chi2 * lambda1 * omc2 / r22;
        } else {
            k.den_i11_0 += K2 * chi1 * 2 * chi2;
        }
    }
    if (a.contrib & COFFE_GPU_RSD) {
        const double c2m1 = 2 * ct * ct - 1;
        const double ss = G.s;
        auto Q = [&](double ch, double d) {
            return d * d * d * (8 - 24 * ss + 12 * ss * ss) +
                   ch * d * d * (-2 + 38 * ss - 18 * ss * ss - 6 * ss * ss * ss) +
                   ch * ch * d * ss * (-22 + 9 * ss + 12 * ss * ss) +
                   ch * ch * ch * ss * (2 - 3 * ss - 6 * ss * ss);
        };
        auto P = [&](double ch, double d) {
            const double d2 = d * d, d3 = d2 * d, d4 = d2 * d2, d5 = d4 * d;
            const double ch2 = ch * ch, ch3 = ch2 * ch, ch4 = ch2 * ch2, ch5 = ch4 * ch;
            const double sq = ss * ss, s3 = sq * ss;
            return d5 * (4 - 12 * ss + 6 * sq) + ch * d4 * (-8 + 60 * ss - 48 * sq + 6 * s3) +
                   ch2 * d3 * ss * (-92 + 114 * ss - 20 * sq - s3) +
                   ch3 * d2 * ss * (48 - 120 * ss + 26 * sq + 3 * s3) +
                   ch4 * d * sq * (60 - 16 * ss - 3 * sq) + ch5 * sq * (-12 + 4 * ss + sq);
        };
        // A: I00 and I02 parts, B: I04 part of one side (functions.c:2174-2183, 2298-2306)
        auto addA = [&](double *co, double w, double ch, double la, double r2) {
            co[L00] += w * (la - 6 * ch * ct + 3 * la * c2m1) / 15.;
            co[L02] += -w * Q(ch, ch - la) / r2 / 21.;
        };
        auto addB = [&](double *co, double w, double ch, double la, double r2) {
            co[L04] += -w * P(ch, ch - la) / r2 / r2 / 35.;
        };
        const double w2 = chi2 * f1c * (2 - 5 * s2) * D1z1c * ga2;
        const double w1 = chi1 * f2c * (2 - 5 * s1) * D1z2c * ga1;
        const double c = a.pref2 * 3 * a.Om / 2.;
        const double e2 = c * w2 * (1 - x), e1 = c * w1 * (1 - x);
        if (r21 != 0 && r22 != 0) {
            addA(k.rsd1, e2, chi1, lambda2, r21);
            addA(k.rsd2, e1, chi2, lambda1, r22);
            if (fabs(mu) < 0.999) {
                addB(k.rsd1, e2, chi1, lambda2, r21);
                addB(k.rsd2, e1, chi2, lambda1, r22);
            } else {
                k.rsd1[L04] += e2 * 4. * (lambda2 + chi1) / 35.;
                k.rsd2[L04] += e1 * 4. * (lambda1 + chi2) / 35.;
            }
        } else if (r21 == 0 && r22 != 0) {
            k.rsd_i00_0 += c * w2 * (1 - chi1 / chi2) * (-2 * chi1 / 15.);
            addA(k.rsd2, e1, chi2, lambda1, r22);
            addB(k.rsd2, e1, chi2, lambda1, r22);
        } else if (r21 != 0 && r22 == 0) {
            addA(k.rsd1, e2, chi1, lambda2, r21);
            addB(k.rsd1, e2, chi1, lambda2, r21);
            k.rsd_i00_0 += c * w1 * (1 - chi2 / chi1) * (-2 * chi2 / 15.);
        } else {
            k.rsd_i00_0 += c * w2 * (1 - chi1 / chi2) * (-2 * chi1 / 15.) +
                           c * w1 * (1 - chi2 / chi1) * (-2 * chi2 / 15.);
        }
    }
}

// single-integrated partial of one (pair, mu node) with the per-request bias
// (den) and growth (RSD) scales, one warp (lens_single_kernel); with gpm the
// record cotangents and the bias / growth-scale cotangents
__global__ void __launch_bounds__(LENS_THREADS)
    adj_lens_single_kernel(LensArgs a, LensBg64 g, const double *__restrict__ tab_x,
                           const double4_32a *__restrict__ rec,
                           const int *__restrict__ req_spectrum,
                           const double *__restrict__ req_z_mean,
                           const int64_t *__restrict__ req_offset, const double *__restrict__ sep,
                           const double *__restrict__ rule, const double *__restrict__ bias_scale,
                           const double *__restrict__ growth_scale,
                           const double *__restrict__ gpm, double *__restrict__ part,
                           double *__restrict__ gR, double *__restrict__ g_bias,
                           double *__restrict__ g_growth, int *err)
{
    const long long item = (long long)blockIdx.x * (LENS_THREADS / 32) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (item >= a.n_items) return;
    const long long pair = a.pair0 + item / a.n_mu_run;
    const int im = a.mu0 + (int)(item % a.n_mu_run);
    const int q = lens_find_request(req_offset, a.n_req, pair);
    const int s = req_spectrum[q];
    const double beta = bias_scale ? bias_scale[q] : 1.0;
    const double alpha = growth_scale ? growth_scale[q] : 1.0;
    const double *xf = rule + 2 * a.n_mu, *wf = xf + a.n_x, *xh = wf + a.n_x, *wh = xh + a.nh;
    const double mu = rule[im];
    const LensGeom G = lens_geom(g, req_z_mean[q], mu, sep[pair]);
    const double b1 = a.has_b1 ? spl_eval(g.b1, G.z1c) : 1.0;
    const double b2 = a.has_b2 ? spl_eval(g.b2, G.z2c) : 1.0;
    const double s1 = a.has_s1 ? spl_eval(g.s1, G.z1c) : 0.0;
    const double s2 = a.has_s2 ? spl_eval(g.s2, G.z2c) : 0.0;
    const double f1c = spl_eval(g.f, G.z1c), f2c = spl_eval(g.f, G.z2c);
    const double D1z1c = spl_eval(g.D1, G.z1c), D1z2c = spl_eval(g.D1, G.z2c);
    const int ni = a.tab_len - 1;
    const double4_32a *recs = rec + (size_t)s * ni * LENS_NT;
    double *gRs = gR ? gR + (size_t)s * LENS_NT * ni * 4 : nullptr;
    const double I00_0 = lens_at_zero<double>(recs, L00), I11_0 = lens_at_zero<double>(recs, L11);
    const double gi = gpm ? gpm[item] : 0.0;
    const double xs = fmin(G.chi1, G.chi2) * G.ct / fmax(G.chi1, G.chi2);
    const bool split = a.nh > 0 && xs > 0 && xs < 1;
    double den_sum = 0, rsd_sum = 0;
    for (int p = 0; p < (split ? 2 : 1); ++p) {
        const double lo = (split && p) ? xs : 0.0, hi = (split && !p) ? xs : 1.0;
        const double c = 0.5 * (lo + hi), hw = 0.5 * (hi - lo);
        const int np = split ? a.nh : a.n_x;
        const double *gx = split ? xh : xf, *gw = split ? wh : wf;
        double pd = 0, pr = 0;
        for (int k = lane; k < np; k += 32) {
            const double x = c + hw * gx[k];
            const double lambda1 = G.chi1 * x, lambda2 = G.chi2 * x;
            double r21 = (lambda2 - G.chi1) * (lambda2 - G.chi1) + 2 * G.chi1 * lambda2 * G.s;
            double r22 = (lambda1 - G.chi2) * (lambda1 - G.chi2) + 2 * G.chi2 * lambda1 * G.s;
            if (r21 < 0) r21 = 0;
            if (r22 < 0) r22 = 0;
            const double z1 = spl_eval(g.z_of_chi, lambda1), z2 = spl_eval(g.z_of_chi, lambda2);
            const double ga1 = spl_eval(g.D1, z1) / spl_eval(g.a, z1);
            const double ga2 = spl_eval(g.D1, z2) / spl_eval(g.a, z2);
            AdjSingleCoef K;
            adj_single_coef(a, G, x, lambda1, lambda2, r21, r22, b1, b2, s1, s2, f1c, f2c, D1z1c,
                            D1z2c, ga1, ga2, mu, K);
            const double ra = sqrt(r21), rb = sqrt(r22);
            const int ia = lens_interval<double>(tab_x, a.tab_len, a.inv_dlog, ra);
            const int ib = lens_interval<double>(tab_x, a.tab_len, a.inv_dlog, rb);
            double vd = K.den_i11_0 * I11_0, vr = K.rsd_i00_0 * I00_0;
            if (ia < 0 || ib < 0) {
                vd = vr = cg_nan<double>();
            } else {
                const double dxa = ra - tab_x[ia], dxb = rb - tab_x[ib];
#pragma unroll
                for (int t = 0; t < LENS_NT; ++t) {
                    const double Ia = adj_table_at(recs, ia, t, dxa);
                    const double Ib = adj_table_at(recs, ib, t, dxb);
                    vd += K.den1[t] * Ia + K.den2[t] * Ib;
                    vr += K.rsd1[t] * Ia + K.rsd2[t] * Ib;
                }
                if (gRs) {
                    const double gn = gi * hw * gw[k];
#pragma unroll
                    for (int t = 0; t < LENS_NT; ++t) {
                        adj_rec_add(gRs, ((long long)t * ni + ia) * 4,
                                    gn * (beta * K.den1[t] + alpha * K.rsd1[t]), dxa);
                        adj_rec_add(gRs, ((long long)t * ni + ib) * 4,
                                    gn * (beta * K.den2[t] + alpha * K.rsd2[t]), dxb);
                    }
                    if (K.den_i11_0 != 0.0)
                        atomicAdd(gRs + (long long)L11 * ni * 4, gn * beta * K.den_i11_0);
                    if (K.rsd_i00_0 != 0.0)
                        atomicAdd(gRs + (long long)L00 * ni * 4, gn * alpha * K.rsd_i00_0);
                }
            }
            pd += gw[k] * vd;
            pr += gw[k] * vr;
        }
        den_sum += hw * warp_sum(pd);
        rsd_sum += hw * warp_sum(pr);
    }
    if (lane == 0) {
        const double v = beta * den_sum + alpha * rsd_sum;
        if (!isfinite(v)) cg_flag(err, CG_ERR_NONFINITE);
        if (part) part[item] = v;
        if (gpm) {
            if (g_bias && den_sum != 0.0) atomicAdd(g_bias + q, gi * den_sum);
            if (g_growth && rsd_sum != 0.0) atomicAdd(g_growth + q, gi * rsd_sum);
        }
    }
}

// record cotangents -> table-knot cotangents gY[(s * n_at + t) * len + j]
// through the Akima coefficients of each interval (lens_records_kernel)
__global__ void adj_lens_records_kernel(LensArgs a, const double *__restrict__ tab_x,
                                        const double *__restrict__ tab_y, int n_spectra,
                                        const double *__restrict__ gR, double *__restrict__ gY,
                                        int n_at)
{
    const int len = a.tab_len, ni = len - 1;
    const long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= (long long)n_spectra * LENS_NT * ni) return;
    const double *g = gR + item * 4;
    if (g[0] == 0.0 && g[1] == 0.0 && g[2] == 0.0 && g[3] == 0.0) return;
    const int i = (int)(item % ni);
    const long long st = item / ni;
    const int t = (int)(st % LENS_NT);
    const int s = (int)(st / LENS_NT);
    const double *y = tab_y + ((size_t)s * a.n_terms + a.term[t]) * len;
    D6 r[4];
    akima_record_d6(tab_x, y, len, i, r);
    double *dst = gY + ((size_t)s * n_at + t) * len + d6_base(len, i);
    for (int k = 0; k < 6; ++k) {
        const double v = g[0] * r[0].g[k] + g[1] * r[1].g[k] + g[2] * r[2].g[k] + g[3] * r[3].g[k];
        if (v != 0.0) atomicAdd(dst + k, v);
    }
}

} // namespace

// Adds the lensing terms (contrib & COFFE_GPU_LEN) to out; the arguments are
// those multipoles_run has validated, all arrays on the device.
// flat-sky lensing terms (ctx->flat_local_nonlocal / flat_nonlocal)
static int flatsky_run(coffe_gpu_ctx *ctx, bool denlen, bool lenlen, double epsrel, int n_req,
                       const int *req_spectrum, const double *req_z_mean,
                       const int64_t *req_offset, const double *sep, int n_l, const int *l,
                       double *out, long long total)
{
    FlatArgs f;
    f.n_req = n_req;
    f.n_l = n_l;
    f.tab_len = (int)(ctx->N + CG_N_SMALL_R + 1);
    f.n_terms = ctx->n_terms;
    f.inv_dlog = (double)ctx->N / log(ctx->kmax / ctx->kmin);
    f.Om = ctx->Omega0_m;
    f.pref2 = pow(CG_H0 * ctx->h, 2);
    f.pref4 = pow(CG_H0 * ctx->h, 4);
    f.epsrel = epsrel;
    f.has_b1 = ctx->bias_set[0];
    f.has_b2 = ctx->bias_set[1];
    f.has_s1 = ctx->bias_set[2];
    f.has_s2 = ctx->bias_set[3];
    for (int j = 0; j < FLAT_MAX_L; ++j) {
        f.ls[j] = j < n_l ? l[j] : 1;
        f.ll_term[j] = -1;
        f.ll_coef[j] = 0;
        for (int k = 0; k < 5; ++k) {
            f.dl_term[j][k] = -1;
            f.dl_coef[j][k] = 0;
        }
    }
    for (int j = 0; j < n_l; ++j) {
        const int L = l[j];
        if (L % 2) continue;
        if (denlen) {
            if (L / 2 + 1 > 5) {
                cg_set_error(ctx, "multipoles: flat-sky density-lensing supports l <= 8");
                return COFFE_GPU_EINVAL;
            }
            for (int k = 0; k <= L / 2; ++k) {
                const int t = cg_find_term(ctx, L - 2 * k + 3, L - 2 * k + 1, 1);
                if (t < 0) {
                    cg_set_error(ctx, "multipoles: flat-sky density-lensing needs the half-integer "
                                      "integral (%d/2, %d/2)", L - 2 * k + 3, L - 2 * k + 1);
                    return COFFE_GPU_ESTATE;
                }
                f.dl_term[j][k] = t;
                f.dl_coef[j][k] = pow(-1, k) / pow(2, k) * host_fact(L) / host_fact(k) /
                                  host_fact(L - k) * host_fact(2 * L - 2 * k) / host_fact(L) /
                                  host_fact(L - 2 * k) * host_fact(L / 2 - k);
            }
        }
        if (lenlen) {
            const int t = cg_find_term(ctx, 1, L);
            if (t < 0 || !ctx->int_small_r) {
                cg_set_error(ctx, "multipoles: flat-sky lensing-lensing needs the integral (1, %d) "
                                  "with its r = 0 and sub-Mpc entries (COFFE_GPU_SMALL_R)", L);
                return COFFE_GPU_ESTATE;
            }
            f.ll_term[j] = t;
            f.ll_coef[j] = (2 * L + 1) * host_fact(L) / pow(2, L) / pow(host_fact(L / 2), 2);
        }
    }
    LensBg64 g;
    g.chi_of_z = ctx->bg[BG_CHI_OF_Z].v64();
    g.z_of_chi = ctx->bg[BG_Z_OF_CHI].v64();
    g.D1 = ctx->bg[BG_D1].v64();
    g.f = ctx->bg[BG_F].v64();
    g.a = ctx->bg[BG_A].v64();
    g.b1 = ctx->bias[0].v64();
    g.b2 = ctx->bias[1].v64();
    g.s1 = ctx->bias[2].v64();
    g.s2 = ctx->bias[3].v64();
    const long long items = total * n_l;
    int st;
    const bool mixed = ctx->int_precision == COFFE_GPU_MIXED;
    if (denlen) {
        const unsigned blocks = (unsigned)((items + 127) / 128);
        if (mixed)
            flat_denlen_kernel<float><<<blocks, 128, 0, ctx->stream>>>(
                f, g, (const float *)ctx->tab_x32.p, (const float *)ctx->tab_y.p, req_spectrum,
                req_z_mean, req_offset, sep, total, out, ctx->d_err);
        else
            flat_denlen_kernel<double><<<blocks, 128, 0, ctx->stream>>>(
                f, g, (const double *)ctx->tab_x.p, (const double *)ctx->tab_y.p, req_spectrum,
                req_z_mean, req_offset, sep, total, out, ctx->d_err);
        if ((st = cg_after_launch(ctx, "flat_denlen_kernel"))) return st;
    }
    if (lenlen) {
        const unsigned blocks = (unsigned)((items + FLAT_WARPS - 1) / FLAT_WARPS);
        if (mixed)
            flat_lenlen_kernel<float><<<blocks, 32 * FLAT_WARPS, 0, ctx->stream>>>(
                f, g, (const float *)ctx->tab_x32.p, (const float *)ctx->tab_y.p, req_spectrum,
                req_z_mean, req_offset, sep, total, out, ctx->d_err);
        else
            flat_lenlen_kernel<double><<<blocks, 32 * FLAT_WARPS, 0, ctx->stream>>>(
                f, g, (const double *)ctx->tab_x.p, (const double *)ctx->tab_y.p, req_spectrum,
                req_z_mean, req_offset, sep, total, out, ctx->d_err);
        if ((st = cg_after_launch(ctx, "flat_lenlen_kernel"))) return st;
    }
    return COFFE_GPU_OK;
}

// float copies of the line rules (x, w_x, x_h, w_h) after the FP64 rule
// mu[n_mu], w_mu[n_mu], x[n_x], w_x[n_x], x_h[nh], w_h[nh] (r has room)
static void lens_rule_floats(const LensArgs &a, std::vector<double> &r)
{
    const size_t off = 2 * (size_t)a.n_mu + 2 * (size_t)a.n_x + 2 * (size_t)a.nh;
    float *f = reinterpret_cast<float *>(r.data() + off);
    for (size_t i = 0; i < 2 * (size_t)a.n_x + 2 * (size_t)a.nh; ++i)
        f[i] = (float)r[2 * (size_t)a.n_mu + i];
}

// arguments of the lensing kernels for a validated call (n_mu mu nodes)
static int lens_args(coffe_gpu_ctx *ctx, int contrib, int n_req, int n_l, const int *l, int n_mu,
                     LensArgs *out)
{
    LensArgs a;
    const int want[LENS_NT][2] = {{0, 0}, {0, 2}, {0, 4}, {1, 1}, {1, 3}, {2, 0}};
    for (int t = 0; t < LENS_NT; ++t) {
        a.term[t] = cg_find_term(ctx, want[t][0], want[t][1]);
        if (a.term[t] < 0) {
            cg_set_error(ctx, "lensing needs the integral (n=%d, l=%d)", want[t][0], want[t][1]);
            return COFFE_GPU_ESTATE;
        }
    }
    a.n_req = n_req;
    a.n_l = n_l;
    a.n_mu = n_mu;
    a.mu0 = 0;
    a.n_mu_run = n_mu;
    a.mu_w = 1.0;
    a.sym = 0;
    a.n_x = ctx->lens_n_x;
    a.nh = (a.n_x % 2 == 0) ? a.n_x / 2 : 0;
    a.contrib = contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD | COFFE_GPU_LEN);
    a.tab_len = (int)(ctx->N + CG_N_SMALL_R + 1);
    a.n_terms = ctx->n_terms;
    a.inv_dlog = (double)ctx->N / log(ctx->kmax / ctx->kmin);
    a.Om = ctx->Omega0_m;
    a.pref2 = pow(CG_H0 * ctx->h, 2);
    a.pref4 = pow(CG_H0 * ctx->h, 4);
    a.has_b1 = ctx->bias_set[0];
    a.has_b2 = ctx->bias_set[1];
    a.has_s1 = ctx->bias_set[2];
    a.has_s2 = ctx->bias_set[3];
    a.pair0 = 0;
    a.n_items = 0;
    for (int i = 0; i < 8; ++i) a.ls[i] = i < n_l ? l[i] : 0;
    *out = a;
    return COFFE_GPU_OK;
}

static LensBg64 lens_bg64(const coffe_gpu_ctx *ctx)
{
    LensBg64 g64;
    g64.chi_of_z = ctx->bg[BG_CHI_OF_Z].v64();
    g64.z_of_chi = ctx->bg[BG_Z_OF_CHI].v64();
    g64.D1 = ctx->bg[BG_D1].v64();
    g64.f = ctx->bg[BG_F].v64();
    g64.a = ctx->bg[BG_A].v64();
    g64.b1 = ctx->bias[0].v64();
    g64.b2 = ctx->bias[1].v64();
    g64.s1 = ctx->bias[2].v64();
    g64.s2 = ctx->bias[3].v64();
    return g64;
}

// Adds the lensing terms of the correlation function (corrfunc.c:55-141:
// signal.c:584-605 single-integrated, 695-702 double-integrated, always the
// full-sky forms) at the n_mu values mu_host to out[item * n_mu + m], with the
// x line rules of coffe_gpu_set_lensing_rule.
int corrfunc_lensing_run(coffe_gpu_ctx *ctx, int contrib, int precision, int n_req,
                         const int *req_spectrum, const double *req_z_mean,
                         const int64_t *req_offset, const double *sep, int n_mu,
                         const double *mu_host, double *out, long long total)
{
    if (!(contrib & COFFE_GPU_LEN) || total <= 0) return COFFE_GPU_OK;
    if (!ctx->int_small_r) {
        cg_set_error(ctx, "corrfunc: lensing needs the r = 0 and sub-Mpc table entries "
                          "(integrals_init with COFFE_GPU_SMALL_R)");
        return COFFE_GPU_ESTATE;
    }
    const bool only_cross = (contrib & COFFE_GPU_ONLY_CROSS) != 0;
    const bool single = (contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD)) != 0;
    const bool dbl = !only_cross;
    if (!single && !dbl) return COFFE_GPU_OK;
    int st;
    LensArgs a;
    const int l0 = 0;
    if ((st = lens_args(ctx, contrib, n_req, 1, &l0, n_mu, &a))) return st;
    // rule: mu[n_mu], (unused weights)[n_mu], x[n_x], w_x[n_x], x_h[nh], w_h[nh]
    std::vector<double> r(2 * (size_t)a.n_mu + 3 * (size_t)a.n_x + 3 * (size_t)a.nh, 0.0);
    for (int m = 0; m < n_mu; ++m) r[m] = mu_host[m];
    gauss_legendre(a.n_x, r.data() + 2 * a.n_mu, r.data() + 2 * a.n_mu + a.n_x);
    if (a.nh)
        gauss_legendre(a.nh, r.data() + 2 * a.n_mu + 2 * a.n_x,
                       r.data() + 2 * a.n_mu + 2 * a.n_x + a.nh);
    lens_rule_floats(a, r);
    if ((st = cg_ensure(ctx, ctx->cf_rule, sizeof(double) * r.size()))) return st;
    CG_CUDA(ctx, cudaMemcpyAsync(ctx->cf_rule.p, r.data(), sizeof(double) * r.size(),
                                 cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream)); // r is a host temporary
    const double *rule = (const double *)ctx->cf_rule.p;
    const LensBg64 g64 = lens_bg64(ctx);
    if (precision == COFFE_GPU_MIXED) {
        LensBgT<Spl32> gT{ctx->bg[BG_Z_OF_CHI].v32(), ctx->bg[BG_D1].v32(), ctx->bg[BG_A].v32()};
        return lensing_launch<float, Spl32, float, true>(ctx, a, g64, gT, req_spectrum,
                                                         req_z_mean, req_offset, sep, out, total,
                                                         single, dbl, rule, true);
    }
    LensBgT<Spl64> gT{ctx->bg[BG_Z_OF_CHI].v64(), ctx->bg[BG_D1].v64(), ctx->bg[BG_A].v64()};
    return lensing_launch<double, Spl64, double, false>(ctx, a, g64, gT, req_spectrum,
                                                        req_z_mean, req_offset, sep, out, total,
                                                        single, dbl, rule, true);
}

void gauss_legendre_nodes(int n, double *x, double *w) { gauss_legendre(n, x, w); }

// LensArgs of a validated multipole call with the full-sky single-integrated
// term (single_full) or not, the mu symmetry applied, and the Gauss-Legendre
// rule on the device (ctx->lens_rule)
static int lens_prepare(coffe_gpu_ctx *ctx, int contrib, int n_req, int n_l, const int *l,
                        bool single_full, LensArgs *out)
{
    int st;
    LensArgs a;
    if ((st = lens_args(ctx, contrib, n_req, n_l, l, ctx->lens_n_mu, &a))) return st;
    // mu -> -mu swaps chi1 and chi2, i.e. the roles of the two tracers: when
    // they share their magnification bias (and, for density-lensing, their
    // galaxy bias) both lensing terms are even in mu, so each even multipole
    // is summed over the rule's nodes with mu > 0 (the rule is symmetric),
    // counted twice; odd multipoles over every node, which are then evaluated
    auto same_tracer = [&](int i, int j) {
        return (!ctx->bias_set[i] && !ctx->bias_set[j]) ||
               (ctx->bias_set[i] && ctx->bias_set[j] && ctx->bias_host[i] == ctx->bias_host[j]);
    };
    a.sym = a.n_mu % 2 == 0 && same_tracer(2, 3) &&
            (!(single_full && (contrib & COFFE_GPU_DEN)) || same_tracer(0, 1));
    bool mirror = a.sym;
    for (int j = 0; j < n_l; ++j) mirror = mirror && l[j] % 2 == 0;
    if (mirror) {
        a.mu0 = a.n_mu / 2;
        a.n_mu_run = a.n_mu / 2;
        a.mu_w = 2.0;
    }
    // the Gauss-Legendre rule: mu[n_mu], w_mu[n_mu], x[n_x], w_x[n_x], x_h[nh], w_h[nh]
    if (ctx->lens_rule_mu != a.n_mu || ctx->lens_rule_x != a.n_x) {
        std::vector<double> r(2 * (size_t)a.n_mu + 3 * (size_t)a.n_x + 3 * (size_t)a.nh);
        gauss_legendre(a.n_mu, r.data(), r.data() + a.n_mu);
        gauss_legendre(a.n_x, r.data() + 2 * a.n_mu, r.data() + 2 * a.n_mu + a.n_x);
        if (a.nh)
            gauss_legendre(a.nh, r.data() + 2 * a.n_mu + 2 * a.n_x,
                           r.data() + 2 * a.n_mu + 2 * a.n_x + a.nh);
        lens_rule_floats(a, r);
        if ((st = cg_ensure(ctx, ctx->lens_rule, sizeof(double) * r.size()))) return st;
        CG_CUDA(ctx, cudaMemcpyAsync(ctx->lens_rule.p, r.data(), sizeof(double) * r.size(),
                                     cudaMemcpyHostToDevice, ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream)); // r is a host temporary
        ctx->lens_rule_mu = a.n_mu;
        ctx->lens_rule_x = a.n_x;
    }
    *out = a;
    return COFFE_GPU_OK;
}

int lensing_run(coffe_gpu_ctx *ctx, int contrib, int precision, double epsrel, int n_req,
                const int *req_spectrum, const double *req_z_mean, const int64_t *req_offset,
                const double *sep, int n_l, const int *l, double *out, long long total)
{
    if (!(contrib & COFFE_GPU_LEN) || total <= 0) return COFFE_GPU_OK;
    // which forms of the single- and double-integrated terms (signal.c:607-754)
    const bool only_cross = (contrib & COFFE_GPU_ONLY_CROSS) != 0;
    const bool want_single = (contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD)) != 0;
    const bool single_full = want_single && !ctx->flat_local_nonlocal;
    const bool single_flat = want_single && ctx->flat_local_nonlocal && (contrib & COFFE_GPU_DEN);
    const bool double_full = !only_cross && !ctx->flat_nonlocal;
    const bool double_flat = !only_cross && ctx->flat_nonlocal;
    int st;
    if (single_flat || double_flat)
        if ((st = flatsky_run(ctx, single_flat, double_flat, epsrel, n_req, req_spectrum,
                              req_z_mean, req_offset, sep, n_l, l, out, total)))
            return st;
    if (!single_full && !double_full) return COFFE_GPU_OK;
    if (!ctx->int_small_r) {
        cg_set_error(ctx, "multipoles: lensing needs the r = 0 and sub-Mpc table entries "
                          "(integrals_init with COFFE_GPU_SMALL_R)");
        return COFFE_GPU_ESTATE;
    }
    LensArgs a;
    if ((st = lens_prepare(ctx, contrib, n_req, n_l, l, single_full, &a))) return st;
    const LensBg64 g64 = lens_bg64(ctx);
    if (precision == COFFE_GPU_MIXED) {
        LensBgT<Spl32> gT{ctx->bg[BG_Z_OF_CHI].v32(), ctx->bg[BG_D1].v32(), ctx->bg[BG_A].v32()};
        return lensing_launch<float, Spl32, float, true>(
            ctx, a, g64, gT, req_spectrum, req_z_mean, req_offset, sep, out, total, single_full,
            double_full, (const double *)ctx->lens_rule.p, false);
    }
    LensBgT<Spl64> gT{ctx->bg[BG_Z_OF_CHI].v64(), ctx->bg[BG_D1].v64(), ctx->bg[BG_A].v64()};
    // COFFE_GPU_FP64_FASTALG: the mixed path's lensing algorithm in FP64
    if (precision == COFFE_GPU_FP64_FASTALG)
        return lensing_launch<double, Spl64, double, true>(
            ctx, a, g64, gT, req_spectrum, req_z_mean, req_offset, sep, out, total, single_full,
            double_full, (const double *)ctx->lens_rule.p, false);
    return lensing_launch<double, Spl64, double, false>(
        ctx, a, g64, gT, req_spectrum, req_z_mean, req_offset, sep, out, total, single_full,
        double_full, (const double *)ctx->lens_rule.p, false);
}

// Reverse mode of the full-sky lensing terms of coffe_gpu_multipoles (FP64
// tables with the sub-Mpc entries): value_out (when not NULL) += the lensing
// multipoles with the den-lensing part scaled by bias_scale[q] and the
// RSD-lensing part by growth_scale[q]; with grad_out, the table cotangents
// are added to gY[(s * n_at + t) * tab_len + j] for t in the order of the six
// lensing tables (I00, I02, I04, I11, I13, I20) and the scale cotangents to
// grad_bias / grad_growth.
int lensing_adjoint_run(coffe_gpu_ctx *ctx, int contrib, int n_req, const int *req_spectrum,
                        const double *req_z_mean, const int64_t *req_offset, const double *sep,
                        long long total, int n_l, const int *l, const double *bias_scale,
                        const double *growth_scale, const double *grad_out, double *value_out,
                        double *gY, int n_at, double *grad_bias, double *grad_growth)
{
    if (!(contrib & COFFE_GPU_LEN) || total <= 0) return COFFE_GPU_OK;
    if (ctx->flat_local_nonlocal || ctx->flat_nonlocal) {
        cg_set_error(ctx, "multipoles adjoint: the lensing terms are differentiated in their "
                          "full-sky form only (coffe_gpu_set_flatsky(ctx, 0, 0))");
        return COFFE_GPU_EINVAL;
    }
    if (!ctx->int_small_r) {
        cg_set_error(ctx, "multipoles adjoint: lensing needs the r = 0 and sub-Mpc table "
                          "entries (integrals_init with COFFE_GPU_SMALL_R)");
        return COFFE_GPU_ESTATE;
    }
    const bool single = (contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD)) != 0;
    int st;
    LensArgs a;
    if ((st = lens_prepare(ctx, contrib, n_req, n_l, l, single, &a))) return st;
    const double *rule = (const double *)ctx->lens_rule.p;
    const LensBg64 g64 = lens_bg64(ctx);
    LensBgT<Spl64> gT{ctx->bg[BG_Z_OF_CHI].v64(), ctx->bg[BG_D1].v64(), ctx->bg[BG_A].v64()};
    const double *tab_x = (const double *)ctx->tab_x.p;
    const int ni = a.tab_len - 1;
    const long long n_int = (long long)ctx->n_spectra * ni;
    const long long n_rec = n_int * LENS_NT;
    // the FP64 records, then (with grad_out) the record cotangents
    const size_t b_rec = (sizeof(double4_32a) * (size_t)n_rec + 255) & ~(size_t)255;
    const size_t b_gR = grad_out ? sizeof(double) * 4 * (size_t)n_rec : 0;
    if ((st = cg_ensure(ctx, ctx->lens_rec, b_rec + b_gR))) return st;
    double4_32a *rec = (double4_32a *)ctx->lens_rec.p;
    double *gR = grad_out ? (double *)((char *)ctx->lens_rec.p + b_rec) : nullptr;
    lens_records_kernel<double><<<(unsigned)((n_rec + 255) / 256), 256, 0, ctx->stream>>>(
        a, tab_x, (const double *)ctx->tab_y.p, ctx->n_spectra, rec);
    if ((st = cg_after_launch(ctx, "lens_records_kernel"))) return st;
    if (gR) CG_CUDA(ctx, cudaMemsetAsync(gR, 0, b_gR, ctx->stream));
    // pairs per chunk: at most 2^22 (pair, mu) items
    const long long chunk = std::max(1LL, std::min(total, (1LL << 22) / a.n_mu_run));
    const size_t per = (size_t)(chunk * a.n_mu_run);
    if ((st = cg_ensure(ctx, ctx->lens_part, sizeof(double) * 3 * per))) return st;
    double *part_d = (double *)ctx->lens_part.p;
    double *part_s = part_d + per;
    double *gpm = grad_out ? part_s + per : nullptr;
    for (long long p0 = 0; p0 < total; p0 += chunk) {
        const long long np = std::min(chunk, total - p0);
        a.pair0 = p0;
        a.n_items = np * a.n_mu_run;
        if (gpm) {
            adj_lens_gpm_kernel<<<(unsigned)((a.n_items + 127) / 128), 128, 0, ctx->stream>>>(
                a, rule, grad_out, np, gpm);
            if ((st = cg_after_launch(ctx, "adj_lens_gpm_kernel"))) return st;
        }
        adj_lens_double_kernel<<<(unsigned)a.n_items, LENS_THREADS, 0, ctx->stream>>>(
            a, g64, gT, tab_x, rec, req_spectrum, req_z_mean, req_offset, sep, rule, gpm,
            value_out ? part_d : nullptr, gR, ctx->d_err);
        if ((st = cg_after_launch(ctx, "adj_lens_double_kernel"))) return st;
        if (single) {
            const long long blocks = (a.n_items + LENS_THREADS / 32 - 1) / (LENS_THREADS / 32);
            adj_lens_single_kernel<<<(unsigned)blocks, LENS_THREADS, 0, ctx->stream>>>(
                a, g64, tab_x, rec, req_spectrum, req_z_mean, req_offset, sep, rule, bias_scale,
                growth_scale, gpm, value_out ? part_s : nullptr, gR, grad_bias, grad_growth,
                ctx->d_err);
            if ((st = cg_after_launch(ctx, "adj_lens_single_kernel"))) return st;
        }
        if (value_out) {
            const long long nt = np * a.n_l;
            lens_reduce_kernel<<<(unsigned)((nt + 3) / 4), 128, 0, ctx->stream>>>(
                a, rule, part_d, single ? part_s : nullptr, np, value_out, ctx->d_err);
            if ((st = cg_after_launch(ctx, "lens_reduce_kernel"))) return st;
        }
    }
    if (!gR) return COFFE_GPU_OK;
    adj_lens_records_kernel<<<(unsigned)((n_rec + 255) / 256), 256, 0, ctx->stream>>>(
        a, tab_x, (const double *)ctx->tab_y.p, ctx->n_spectra, gR, gY, n_at);
    return cg_after_launch(ctx, "adj_lens_records_kernel");
}
