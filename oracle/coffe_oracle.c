/*
 * coffe_oracle.c -- FP64 CPU restatement of COFFE's correlation-function hot
 * path.  TEST INFRASTRUCTURE ONLY: the oracle the tests compare the GPU product
 * against, never part of it.  See coffe_oracle.h for the contract and the reference citations.
 *
 * Build: make -C oracle  (gcc -O2 -fopenmp -ffp-contract=off, shared library)
 */
#include "coffe_oracle.h"

#include <complex.h>
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* the 61-point Gauss-Kronrod rule, generated from its definition at 60 digits
   by coffe_gb300/csrc/gen_gk61.py (one table for the library and the oracle;
   the oracle is pinned against the reference's golden vectors independently) */
#include "../coffe_gb300/csrc/gk61_table.h"
static const double OR_GK61_XGK[31] = CG_GK61_XGK_INIT;
static const double OR_GK61_WGK[31] = CG_GK61_WGK_INIT;
static const double OR_GK61_WG[15] = CG_GK61_WG_INIT;

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#define OR_SQRT_PI 1.7724538509055160272981674833411451827975494561224
#define OR_H0 (1. / 2997.92458) /* H0 in h/Mpc, common.h:76 */
#define OR_QAG_LIMIT 50000      /* COFFE_MAX_INTSPACE, common.h:72 */

/* ======================================================================
 * splines (GSL interp semantics: binary search, NaN outside [x0, x_{n-1}])
 * ====================================================================== */

static size_t or_bsearch(const double *x, size_t n, double v)
{
    size_t lo = 0, hi = n - 1;
    while (hi > lo + 1) {
        size_t mid = (lo + hi) / 2;
        if (x[mid] > v)
            hi = mid;
        else
            lo = mid;
    }
    return lo;
}

/* natural cubic spline: tridiagonal system for c_i = y''_i / 2, c_0 = c_{n-1} = 0 */
static int cspline_coeffs(const double *x, const double *y, size_t n, double *b,
                          double *c_int, double *d)
{
    double *c = (double *)calloc(n, sizeof(double));
    size_t m = n - 2;
    if (!c)
        return -1;
    if (m > 0) {
        double *diag = (double *)malloc(sizeof(double) * m);
        double *off = (double *)malloc(sizeof(double) * m);
        double *rhs = (double *)malloc(sizeof(double) * m);
        for (size_t i = 0; i < m; ++i) {
            const double h_i = x[i + 1] - x[i];
            const double h_ip1 = x[i + 2] - x[i + 1];
            const double g_i = 1.0 / h_i, g_ip1 = 1.0 / h_ip1;
            off[i] = h_ip1;
            diag[i] = 2.0 * (h_ip1 + h_i);
            rhs[i] = 3.0 * ((y[i + 2] - y[i + 1]) * g_ip1 - (y[i + 1] - y[i]) * g_i);
        }
        /* Thomas algorithm for the symmetric tridiagonal system */
        for (size_t i = 1; i < m; ++i) {
            const double w = off[i - 1] / diag[i - 1];
            diag[i] -= w * off[i - 1];
            rhs[i] -= w * rhs[i - 1];
        }
        c[m] = rhs[m - 1] / diag[m - 1];
        for (size_t i = m - 1; i-- > 0;)
            c[i + 1] = (rhs[i] - off[i] * c[i + 2]) / diag[i];
        free(diag);
        free(off);
        free(rhs);
    }
    for (size_t i = 0; i + 1 < n; ++i) {
        const double h = x[i + 1] - x[i];
        const double dy = y[i + 1] - y[i];
        b[i] = dy / h - h * (c[i + 1] + 2.0 * c[i]) / 3.0;
        c_int[i] = c[i];
        d[i] = (c[i + 1] - c[i]) / (3.0 * h);
    }
    free(c);
    return 0;
}

/* Akima (1970) with linearly extrapolated end slopes (the non-periodic rule) */
static int akima_coeffs(const double *x, const double *y, size_t n, double *b,
                        double *c, double *d)
{
    /* m[k + 2] holds the secant slope m_k, k = -2 .. n */
    double *mm = (double *)malloc(sizeof(double) * (n + 3));
    double *t = (double *)malloc(sizeof(double) * n);
    if (!mm || !t) {
        free(mm);
        free(t);
        return -1;
    }
    double *m = mm + 2;
    for (size_t i = 0; i + 1 < n; ++i)
        m[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]);
    m[-1] = 2.0 * m[0] - m[1];
    m[-2] = 3.0 * m[0] - 2.0 * m[1];
    m[n - 1] = 2.0 * m[n - 2] - m[n - 3];
    m[n] = 3.0 * m[n - 2] - 2.0 * m[n - 3];
    for (size_t i = 0; i < n; ++i) {
        const long k = (long)i;
        const double w1 = fabs(m[k + 1] - m[k]);
        const double w2 = fabs(m[k - 1] - m[k - 2]);
        const double ne = w1 + w2;
        if (ne == 0.0)
            t[i] = 0.5 * (m[k - 1] + m[k]);
        else
            t[i] = (w1 * m[k - 1] + w2 * m[k]) / ne;
    }
    for (size_t i = 0; i + 1 < n; ++i) {
        const double h = x[i + 1] - x[i];
        b[i] = t[i];
        c[i] = (3.0 * m[i] - 2.0 * t[i] - t[i + 1]) / h;
        d[i] = (t[i] + t[i + 1] - 2.0 * m[i]) / (h * h);
    }
    free(mm);
    free(t);
    return 0;
}

int or_spline_coeffs(int type, const double *x, const double *y, size_t n, double *b,
                     double *c, double *d)
{
    if (type == OR_CSPLINE) {
        if (n < 3)
            return -1;
        return cspline_coeffs(x, y, n, b, c, d);
    }
    if (type == OR_AKIMA) {
        if (n < 5)
            return -1;
        return akima_coeffs(x, y, n, b, c, d);
    }
    if (type == OR_LINEAR) {
        if (n < 2)
            return -1;
        for (size_t i = 0; i + 1 < n; ++i) {
            b[i] = (y[i + 1] - y[i]) / (x[i + 1] - x[i]);
            c[i] = 0.0;
            d[i] = 0.0;
        }
        return 0;
    }
    return -1;
}

int or_spline_init(or_spline_t *s, const double *x, const double *y, size_t n, int type)
{
    memset(s, 0, sizeof(*s));
    if (n < 2)
        return -1;
    s->n = n;
    s->type = type;
    s->x = (double *)malloc(sizeof(double) * n);
    s->y = (double *)malloc(sizeof(double) * n);
    s->b = (double *)malloc(sizeof(double) * n);
    s->c = (double *)malloc(sizeof(double) * n);
    s->d = (double *)malloc(sizeof(double) * n);
    if (!s->x || !s->y || !s->b || !s->c || !s->d) {
        or_spline_free(s);
        return -1;
    }
    memcpy(s->x, x, sizeof(double) * n);
    memcpy(s->y, y, sizeof(double) * n);
    if (or_spline_coeffs(type, x, y, n, s->b, s->c, s->d) != 0) {
        or_spline_free(s);
        return -1;
    }
    return 0;
}

double or_spline_eval(const or_spline_t *s, double v)
{
    if (!(v >= s->x[0] && v <= s->x[s->n - 1]))
        return NAN;
    const size_t i = or_bsearch(s->x, s->n, v);
    const double dx = v - s->x[i];
    return s->y[i] + dx * (s->b[i] + dx * (s->c[i] + s->d[i] * dx));
}

void or_spline_free(or_spline_t *s)
{
    free(s->x);
    free(s->y);
    free(s->b);
    free(s->c);
    free(s->d);
    memset(s, 0, sizeof(*s));
}

int or_spline_eval_array(int type, const double *x, const double *y, size_t n,
                         const double *xq, double *yq, size_t nq)
{
    or_spline_t s;
    if (or_spline_init(&s, x, y, n, type) != 0)
        return -1;
    for (size_t i = 0; i < nq; ++i)
        yq[i] = or_spline_eval(&s, xq[i]);
    or_spline_free(&s);
    return 0;
}

/* ======================================================================
 * QUADPACK QAG with the 61-point Gauss-Kronrod rule
 * ====================================================================== */

static double rescale_error(double err, double result_abs, double result_asc)
{
    err = fabs(err);
    if (result_asc != 0 && err != 0) {
        const double scale = pow((200 * err / result_asc), 1.5);
        if (scale < 1)
            err = result_asc * scale;
        else
            err = result_asc;
    }
    if (result_abs > DBL_MIN / (50 * DBL_EPSILON)) {
        const double min_err = 50 * DBL_EPSILON * result_abs;
        if (min_err > err)
            err = min_err;
    }
    return err;
}

double or_qk61(or_fn f, void *p, double a, double b, double *abserr, double *resabs,
               double *resasc)
{
    double fv1[30], fv2[30];
    const double center = 0.5 * (a + b);
    const double half_length = 0.5 * (b - a);
    const double abs_half_length = fabs(half_length);
    const double f_center = f(center, p);
    double result_gauss = 0;
    double result_kronrod = f_center * OR_GK61_WGK[30];
    double result_abs = fabs(result_kronrod);
    for (int j = 0; j < 15; ++j) {
        const int jtw = 2 * j + 1;
        const double abscissa = half_length * OR_GK61_XGK[jtw];
        const double fval1 = f(center - abscissa, p);
        const double fval2 = f(center + abscissa, p);
        const double fsum = fval1 + fval2;
        fv1[jtw] = fval1;
        fv2[jtw] = fval2;
        result_gauss += OR_GK61_WG[j] * fsum;
        result_kronrod += OR_GK61_WGK[jtw] * fsum;
        result_abs += OR_GK61_WGK[jtw] * (fabs(fval1) + fabs(fval2));
    }
    for (int j = 0; j < 15; ++j) {
        const int jtwm1 = 2 * j;
        const double abscissa = half_length * OR_GK61_XGK[jtwm1];
        const double fval1 = f(center - abscissa, p);
        const double fval2 = f(center + abscissa, p);
        fv1[jtwm1] = fval1;
        fv2[jtwm1] = fval2;
        result_kronrod += OR_GK61_WGK[jtwm1] * (fval1 + fval2);
        result_abs += OR_GK61_WGK[jtwm1] * (fabs(fval1) + fabs(fval2));
    }
    const double mean = result_kronrod * 0.5;
    double result_asc = OR_GK61_WGK[30] * fabs(f_center - mean);
    for (int j = 0; j < 30; ++j)
        result_asc += OR_GK61_WGK[j] * (fabs(fv1[j] - mean) + fabs(fv2[j] - mean));
    const double err = (result_kronrod - result_gauss) * half_length;
    result_kronrod *= half_length;
    result_abs *= abs_half_length;
    result_asc *= abs_half_length;
    *resabs = result_abs;
    *resasc = result_asc;
    *abserr = rescale_error(err, result_abs, result_asc);
    return result_kronrod;
}

static int subinterval_too_small(double a1, double a2, double b2)
{
    const double e = DBL_EPSILON, u = DBL_MIN;
    const double tmp = (1 + 100 * e) * (fabs(a2) + 1000 * u);
    return fabs(a1) <= tmp && fabs(b2) <= tmp;
}

static _Thread_local int or_tl_intervals = 0;

int or_last_qag_intervals(void) { return or_tl_intervals; }

double or_qag61(or_fn f, void *p, double a, double b, double epsabs, double epsrel,
                size_t limit, double *abserr_out, int *status)
{
    double result0, abserr0, resabs0, resasc0;
    int st = 0;
    result0 = or_qk61(f, p, a, b, &abserr0, &resabs0, &resasc0);
    double tolerance = fmax(epsabs, epsrel * fabs(result0));
    const double round_off = 50 * DBL_EPSILON * resabs0;
    or_tl_intervals = 1;
    if (abserr0 <= round_off && abserr0 > tolerance) {
        if (abserr_out)
            *abserr_out = abserr0;
        if (status)
            *status = 2;
        return result0;
    } else if ((abserr0 <= tolerance && abserr0 != resasc0) || abserr0 == 0.0) {
        if (abserr_out)
            *abserr_out = abserr0;
        if (status)
            *status = 0;
        return result0;
    } else if (limit == 1) {
        if (abserr_out)
            *abserr_out = abserr0;
        if (status)
            *status = 1;
        return result0;
    }
    size_t cap = 64;
    double *al = (double *)malloc(sizeof(double) * cap);
    double *bl = (double *)malloc(sizeof(double) * cap);
    double *rl = (double *)malloc(sizeof(double) * cap);
    double *el = (double *)malloc(sizeof(double) * cap);
    size_t size = 1;
    al[0] = a;
    bl[0] = b;
    rl[0] = result0;
    el[0] = abserr0;
    double area = result0, errsum = abserr0;
    int roundoff_type1 = 0, roundoff_type2 = 0, error_type = 0;
    size_t iteration = 1;
    do {
        size_t imax = 0;
        for (size_t i = 1; i < size; ++i)
            if (el[i] > el[imax])
                imax = i;
        const double a_i = al[imax], b_i = bl[imax], r_i = rl[imax], e_i = el[imax];
        const double a1 = a_i, b1 = 0.5 * (a_i + b_i), a2 = b1, b2 = b_i;
        double error1, error2, resabs1, resabs2, resasc1, resasc2;
        const double area1 = or_qk61(f, p, a1, b1, &error1, &resabs1, &resasc1);
        const double area2 = or_qk61(f, p, a2, b2, &error2, &resabs2, &resasc2);
        const double area12 = area1 + area2;
        const double error12 = error1 + error2;
        errsum += (error12 - e_i);
        area += area12 - r_i;
        if (resasc1 != error1 && resasc2 != error2) {
            const double delta = r_i - area12;
            if (fabs(delta) <= 1.0e-5 * fabs(area12) && error12 >= 0.99 * e_i)
                roundoff_type1++;
            if (iteration >= 10 && error12 > e_i)
                roundoff_type2++;
        }
        tolerance = fmax(epsabs, epsrel * fabs(area));
        if (errsum > tolerance) {
            if (roundoff_type1 >= 6 || roundoff_type2 >= 20)
                error_type = 2;
            if (subinterval_too_small(a1, a2, b2))
                error_type = 3;
        }
        if (size == cap) {
            cap *= 2;
            al = (double *)realloc(al, sizeof(double) * cap);
            bl = (double *)realloc(bl, sizeof(double) * cap);
            rl = (double *)realloc(rl, sizeof(double) * cap);
            el = (double *)realloc(el, sizeof(double) * cap);
        }
        al[imax] = a1;
        bl[imax] = b1;
        rl[imax] = area1;
        el[imax] = error1;
        al[size] = a2;
        bl[size] = b2;
        rl[size] = area2;
        el[size] = error2;
        size++;
        iteration++;
    } while (iteration < limit && !error_type && errsum > tolerance);
    double result = 0;
    for (size_t i = 0; i < size; ++i)
        result += rl[i];
    if (error_type)
        st = error_type;
    else if (iteration >= limit && errsum > tolerance)
        st = 1;
    or_tl_intervals = (int)size;
    free(al);
    free(bl);
    free(rl);
    free(el);
    if (abserr_out)
        *abserr_out = errsum;
    if (status)
        *status = st;
    return result;
}

int or_gauss_legendre(size_t n, double *x, double *w)
{
    if (n == 0)
        return -1;
    for (size_t i = 0; i < (n + 1) / 2; ++i) {
        double z = cos(M_PI * ((double)i + 0.75) / ((double)n + 0.5));
        double pp = 0.0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1.0, p2 = 0.0;
            for (size_t j = 1; j <= n; ++j) {
                const double p3 = p2;
                p2 = p1;
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / (double)j;
            }
            pp = (double)n * (z * p1 - p2) / (z * z - 1.0);
            const double z1 = z;
            z = z1 - p1 / pp;
            if (fabs(z - z1) <= 1e-16)
                break;
        }
        x[i] = -z;
        x[n - 1 - i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * pp * pp);
        w[n - 1 - i] = w[i];
    }
    return 0;
}

/* ======================================================================
 * special functions
 * ====================================================================== */

/* Lanczos approximation, g = 7, 9 terms, as twofast_lgamma (twofast.c:97-144) */
static const double or_lanczos_coeff[8] = {
    676.5203681218851,     -1259.1392167224028,  771.32342877765313,
    -176.61502916214059,   12.507343278686905,   -0.13857109526572012,
    9.9843695780195716e-6, 1.5056327351493116e-7};

static double complex or_lgamma_cplx(double complex z)
{
    if (creal(z) < 0.5)
        return log(M_PI) - clog(csin(M_PI * z)) - or_lgamma_cplx(1. - z);
    double complex x = 0.99999999999980993;
    z -= 1;
    for (int i = 0; i < 8; ++i)
        x += or_lanczos_coeff[i] / (z + (double)i + 1.);
    const double complex t = z + 8 - 0.5;
    return log(2 * M_PI) / 2. + (z + 0.5) * clog(t) - t + clog(x);
}

void or_lgamma_c(double zr, double zi, double *rr, double *ri)
{
    const double complex r = or_lgamma_cplx(zr + I * zi);
    *rr = creal(r);
    *ri = cimag(r);
}

double or_legendre(int l, double x)
{
    if (l == 0)
        return 1.0;
    if (l == 1)
        return x;
    double p0 = 1.0, p1 = x;
    for (int k = 2; k <= l; ++k) {
        const double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / (double)k;
        p0 = p1;
        p1 = p2;
    }
    return p1;
}

/* j_l(x): ascending series for x below l + 1 (and below 1), else upward
   recurrence from the closed forms of j_0 and j_1 (stable for x > l). */
double or_sph_bessel(int l, double x)
{
    if (x < 0)
        return (l % 2 ? -1.0 : 1.0) * or_sph_bessel(l, -x);
    const double thr = (l < 1 ? 1.0 : (double)l + 1.0);
    if (x < thr) {
        /* x^l / (2l+1)!! * sum_k (-x^2/2)^k / (k! (2l+3)(2l+5)...(2l+2k+1)) */
        double pref = 1.0;
        for (int k = 1; k <= l; ++k)
            pref *= x / (2.0 * k + 1.0);
        const double y = -0.5 * x * x;
        double term = 1.0, sum = 1.0;
        for (int k = 1; k < 200; ++k) {
            term *= y / ((double)k * (2.0 * l + 2.0 * k + 1.0));
            sum += term;
            if (fabs(term) < 1e-17 * fabs(sum))
                break;
        }
        return pref * sum;
    }
    const double s = sin(x), c = cos(x);
    double j0 = s / x;
    if (l == 0)
        return j0;
    double j1 = (s / x - c) / x;
    for (int k = 1; k < l; ++k) {
        const double j2 = (2.0 * k + 1.0) / x * j1 - j0;
        j0 = j1;
        j1 = j2;
    }
    return j1;
}

/* ======================================================================
 * FFT: recursive mixed-radix decimation in time, any length
 * ====================================================================== */

static void fft_rec(const double *xr, const double *xi, size_t stride, size_t n,
                    double *yr, double *yi, const double *wr, const double *wi,
                    size_t N)
{
    if (n == 1) {
        yr[0] = xr[0];
        yi[0] = xi[0];
        return;
    }
    size_t p = 0;
    for (size_t f = 2; f * f <= n; ++f)
        if (n % f == 0) {
            p = f;
            break;
        }
    if (p == 0)
        p = n;
    const size_t m = n / p;
    for (size_t r = 0; r < p; ++r)
        fft_rec(xr + r * stride, xi + r * stride, stride * p, m, yr + r * m, yi + r * m,
                wr, wi, N);
    double *tr = (double *)malloc(sizeof(double) * n);
    double *ti = (double *)malloc(sizeof(double) * n);
    const size_t step = N / n;
    for (size_t k = 0; k < m; ++k) {
        for (size_t q = 0; q < p; ++q) {
            const size_t kk = k + q * m;
            double sr = 0, si = 0;
            for (size_t r = 0; r < p; ++r) {
                const size_t e = ((r * kk) % n) * step;
                const double ar = yr[r * m + k], ai = yi[r * m + k];
                sr += ar * wr[e] - ai * wi[e];
                si += ar * wi[e] + ai * wr[e];
            }
            tr[kk] = sr;
            ti[kk] = si;
        }
    }
    memcpy(yr, tr, sizeof(double) * n);
    memcpy(yi, ti, sizeof(double) * n);
    free(tr);
    free(ti);
}

int or_fft(double *re, double *im, size_t n, int sign)
{
    if (n == 0)
        return -1;
    double *wr = (double *)malloc(sizeof(double) * n);
    double *wi = (double *)malloc(sizeof(double) * n);
    double *yr = (double *)malloc(sizeof(double) * n);
    double *yi = (double *)malloc(sizeof(double) * n);
    for (size_t j = 0; j < n; ++j) {
        const double ang = 2.0 * M_PI * (double)j / (double)n;
        wr[j] = cos(ang);
        wi[j] = (sign < 0 ? -1.0 : 1.0) * sin(ang);
    }
    fft_rec(re, im, 1, n, yr, yi, wr, wi, n);
    memcpy(re, yr, sizeof(double) * n);
    memcpy(im, yi, sizeof(double) * n);
    free(wr);
    free(wi);
    free(yr);
    free(yi);
    return 0;
}

/* ======================================================================
 * FFTLog (twofast.c)
 * ====================================================================== */

static double twofast_window(double value, double xmin, double xmax, double xleft,
                             double xright)
{
    /* twofast.c:54-90 */
    double result;
    if (value > xleft && value < xright && value > xmin && value < xmax)
        result = 1.0;
    else if (value <= xmin || value >= xmax)
        result = 0.0;
    else {
        if (value <= xleft)
            result = (value - xmin) / (xleft - xmin);
        else
            result = (xmax - value) / (xmax - xright);
        result = result - sin(2 * M_PI * result) / 2. / M_PI;
    }
    return result;
}

double or_twofast_selectqnu(double l, double nu)
{
    const double n1 = 0.9, n2 = 0.9999;
    const double qmin = fmax(n2 - 1.0 - nu, -l);
    const double qmax = fmin(n1 + 3.0 - nu, 2.0);
    const double qbest = (2. + n1 + n2) / 2. - nu;
    double q = qbest;
    if (!(qmin < q && q < qmax))
        q = (qmin + 2. * qmax) / 3.;
    return q;
}

/* twofast_mql (twofast.c:196-224).  The reflection branch of the Lanczos
   log-Gamma overflows csin for |Im(pi z)| above ~710; the reference then gets
   lnGamma = -inf and the mode's coefficient becomes exactly zero.  That
   behaviour is kept. */
static double complex twofast_mql(double t, double q, double l, double alpha)
{
    const double complex n = q - 1. - t * I;
    const double complex unl =
        cpow(2, n - 1.) * OR_SQRT_PI *
        cexp(or_lgamma_cplx((1. + l + n) / 2.) - or_lgamma_cplx((2. + l - n) / 2.));
    if (isfinite(creal(unl)) && isfinite(cimag(unl)))
        return cpow(alpha, t * I - q) * unl;
    return NAN;
}

int or_twofast_1bessel(double *out_x, double *out_y, size_t N, const double *in_x,
                       const double *in_y, size_t in_len, double l, double nu,
                       double r0, double k0, double kmin, double kmax)
{
    if (N < 4 || in_len < 3)
        return -1;
    const size_t N2 = N / 2 + 1;
    const double qnu = or_twofast_selectqnu(l, nu);
    const double G = log(kmax / kmin);
    const double q = qnu + nu;
    or_spline_t sp;
    if (or_spline_init(&sp, in_x, in_y, in_len, OR_CSPLINE) != 0)
        return -1;
    /* twofast_fft_input (twofast.c:252-360) */
    const double L = 2 * M_PI * N / log(kmax / kmin);
    double *xmod = (double *)malloc(sizeof(double) * N);
    double *re = (double *)malloc(sizeof(double) * N);
    double *im = (double *)malloc(sizeof(double) * N);
    const double xmax_w = k0 * pow(kmax / kmin, (double)(N - 1) / N);
    const double xleft_w = exp(0.46) * kmin;
    const double xright_w = exp(-0.46) * k0 * pow(kmax / kmin, (double)(N - 1) / N);
    for (size_t i = 0; i < N; ++i)
        xmod[i] = k0 * pow(kmax / kmin, (double)i / N);
    for (size_t i = 0; i < N; ++i) {
        const double ki = k0 * pow(kmax / kmin, (double)i / N);
        re[i] = pow(kmax / kmin, (3. - q) * i / N) * or_spline_eval(&sp, ki) *
                twofast_window(ki, kmin, xmax_w, xleft_w, xright_w);
        im[i] = 0.0;
    }
    or_spline_free(&sp);
    or_fft(re, im, N, -1);
    double complex *c = (double complex *)malloc(sizeof(double complex) * N2);
    for (size_t i = 0; i < N2; ++i) {
        const double w = twofast_window(xmod[N2 - 2 + i], kmin, xmax_w, xleft_w, xright_w);
        c[i] = w * conj(re[i] + I * im[i]) / L;
    }
    /* multiply by the Gamma-ratio kernel (twofast.c:426-446) */
    for (size_t i = 0; i < N2; ++i)
        c[i] = c[i] * twofast_mql(2 * M_PI * i / G, qnu, l, k0 * r0);
    /* c2r (FFTW semantics: Hermitian extension, imaginary parts of DC and
       Nyquist ignored), twofast.c:448-465 */
    for (size_t i = 0; i < N2; ++i) {
        re[i] = creal(c[i]);
        im[i] = cimag(c[i]);
    }
    im[0] = 0.0;
    if (N % 2 == 0)
        im[N / 2] = 0.0;
    for (size_t i = N2; i < N; ++i) {
        re[i] = re[N - i];
        im[i] = -im[N - i];
    }
    or_fft(re, im, N, +1);
    for (size_t i = 0; i < N; ++i) {
        out_x[i] = r0 * pow(kmax / kmin, (double)i / N);
        const double pref =
            k0 * k0 * k0 * pow(kmax / kmin, -((qnu + nu) * i / N)) / M_PI / pow(r0 * k0, nu) / G;
        out_y[i] = re[i] * pref;
    }
    free(c);
    free(xmod);
    free(re);
    free(im);
    return 0;
}

/* ======================================================================
 * I_l^n tables (integrals.c)
 * ====================================================================== */

static const double or_min_sep[OR_N_SMALL_R] = {
    /* integrals.c:111-126: the sub-Mpc separations evaluated by direct quadrature */
    1E-6,   1E-5,   1E-4,  1E-3,    2E-3,  5E-3,   7E-3,   8E-3,  9E-3,   1E-2,   1.1E-2,
    1.2E-2, 1.25E-2, 1.3E-2, 1.35E-2, 1.5E-2, 2E-2, 2.5E-2, 3E-2,  3.5E-2, 5E-2,   7E-2,
    8E-2,   9E-2,   1E-1,  1.1E-1,  1.2E-1, 1.25E-1, 1.3E-1, 1.35E-1, 1.5E-1, 1.75E-1, 2E-1,
    2.5E-1, 3E-1,   3.5E-1, 4E-1,   5E-1,  6E-1,   7E-1,   8E-1,  9E-1};

typedef struct {
    const or_spline_t *pk;
    double r;
    int n, l;
} or_bessel_par_t;

static double bessel_integrand(double k, void *vp)
{
    /* integrals.c:280-325 (integer n, l) */
    const or_bessel_par_t *p = (const or_bessel_par_t *)vp;
    const double bf = or_sph_bessel(p->l, k * p->r) / pow(k * p->r, (double)p->n);
    return k * k * or_spline_eval(p->pk, k) * bf;
}

static double prefactor_integrand(double k, void *vp)
{
    /* integrals.c:238-269 */
    const or_bessel_par_t *p = (const or_bessel_par_t *)vp;
    return pow(k, 2.0 + p->l - p->n) * or_spline_eval(p->pk, k);
}

static double integrate_function(or_fn func, const or_spline_t *pk, int n, int l,
                                 double sep, double kmin, double kmax)
{
    /* integrals.c:333-383 */
    or_bessel_par_t p = {pk, sep, n, l};
    const double result = or_qag61(func, &p, kmin, kmax, 0, 1e-5, OR_QAG_LIMIT, NULL, NULL);
    double output;
    if (n >= l && sep > 0)
        output = result * pow(sep, (double)(n - l));
    else
        output = result;
    return output / 2. / M_PI / M_PI;
}

double or_integral_direct(const double *k, const double *pk, size_t nk, int n, int l,
                          double r, double kmin, double kmax)
{
    or_spline_t sp;
    if (or_spline_init(&sp, k, pk, nk, OR_AKIMA) != 0)
        return NAN;
    const double v = integrate_function(bessel_integrand, &sp, n, l, r, kmin, kmax);
    or_spline_free(&sp);
    return v;
}

/* ------------------------------------------- divergent I^4_0 (integrals.c:773-914) */

typedef struct {
    const or_spline_t *pk;
    double r1, r2;
} or_renorm_par_t;

static double renorm0_integrand(double k, void *vp)
{
    /* integrals.c:390-404: P (1 - j0(kr)^2) / k^2 */
    const or_renorm_par_t *p = (const or_renorm_par_t *)vp;
    const double j = or_sph_bessel(0, k * p->r1);
    return or_spline_eval(p->pk, k) * (1. - j * j) / k / k;
}

static double renorm_integrand(double k, void *vp)
{
    /* integrals.c:406-422: P j0(k chi1) j0(k chi2) / k^2 */
    const or_renorm_par_t *p = (const or_renorm_par_t *)vp;
    return or_spline_eval(p->pk, k) * or_sph_bessel(0, k * p->r1) * or_sph_bessel(0, k * p->r2) /
           k / k;
}

/* The fixed separations (Mpc) of the divergent integral's spline, independent of
   the user's separations (integrals.c:76-103) */
static const double or_div_sep[] = {
    1e-06, 5e-06, 0.0001, 0.005, 0.01, 0.02, 0.05, 0.1, 0.2, 0.4,
    0.8, 1., 1.5, 2., 3., 4., 5., 6., 7., 8.,
    9., 10., 11., 12., 13., 14., 15., 16., 17., 18.,
    19., 20., 21., 22., 23., 24., 25., 26., 27., 28.,
    29., 30., 32., 34., 36., 38., 40., 42., 44., 46.,
    48., 50., 52., 54., 56., 58., 60., 62., 64., 66.,
    68., 70., 72., 74., 76., 78., 80., 81., 82., 83.,
    84., 85., 86., 87., 88., 89., 90., 91., 92., 93.,
    94., 95., 95.5, 96., 96.5, 97., 97.5, 98., 98.5, 99.,
    99.5, 100., 100.5, 101., 101.5, 102., 102.5, 103., 103.5, 104.,
    104.5, 105., 106., 107., 108., 109., 110., 112., 114., 116.,
    118., 120., 124., 128., 132., 136., 140., 144., 148., 152.,
    156., 160., 164., 168., 172., 176., 180., 185., 190., 195.,
    200., 205., 210., 215., 220., 225., 230., 235., 240., 250.,
    260., 270., 280., 290., 300., 320., 340., 360., 380., 400.,
    420., 440., 460., 480., 500., 520., 540., 560., 580., 600.,
    620., 640., 660., 680., 700., 750., 800., 850., 900., 950.,
    1000., 1050., 1100., 1150., 1200., 1250., 1300., 1350., 1400., 1450.,
    1500., 1550., 1600., 1650., 1700., 1750., 1800., 1850., 1900., 1950.,
    2000., 2050., 2100., 2150., 2200., 2250., 2300., 2350., 2400., 2450.,
    2500., 2550., 2600., 2650., 2700., 2750., 2800., 2850., 2900., 2950.,
    3000., 3050., 3100., 3150., 3200., 3250., 3300., 3350., 3400., 3450.,
    3500., 3550., 3600., 3650., 3700., 3750., 3800., 3850., 3900., 3950.,
    4000., 4050., 4100., 4150., 4200., 4250., 4300., 4350., 4400., 4450.,
    4500., 4550., 4600., 4650., 4700., 4750., 4800., 4850., 4900., 4950.,
    5000., 5050., 5100., 5150., 5200., 5250., 5300., 5350., 5400., 5450.,
    5500., 5550., 5600., 5650., 5700., 5750., 5800., 5850., 5900., 5950.,
    6000., 6050., 6100., 6150., 6200., 6250., 6300., 6350., 6400., 6450.,
    6500., 6550., 6600., 7000., 8000., 9000., 10000., 11000., 12000., 13000.,
    14000., 15000., 16000., 17000., 18000., 19000., 20000.,
};

size_t or_divergent_separations(double *out, size_t cap)
{
    const size_t n = sizeof(or_div_sep) / sizeof(or_div_sep[0]);
    for (size_t i = 0; i < n && i < cap; ++i)
        out[i] = or_div_sep[i];
    return n;
}

/* At each separation r_i: result = r^4 I^4_0(r) = (1/2pi^2) int k^2 P j0(kr)/(kr)^4 dk
   r^4 (integrals_integrate_function with n = 4, l = 0, integrals.c:333-383), and
   result0 = (1/2pi^2) r^4 int P (1 - j0(kr)^2)/k^2 dk (the same function applies its
   r^(n - l) factor to the r = 0 renormalisation integrand, integrals.c:812-826);
   GK61 QAG at relative 1e-5 over [kmin, kmax], Akima P(k).  status: or of the
   QAG statuses. */
int or_divergent_i40(const double *k, const double *pk, size_t nk, double kmin, double kmax,
                     const double *r, size_t nr, double *result, double *result0, int nthreads)
{
    or_spline_t sp;
    if (or_spline_init(&sp, k, pk, nk, OR_AKIMA) != 0)
        return -1;
#ifdef _OPENMP
    if (nthreads <= 0)
        nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (long i = 0; i < (long)nr; ++i) {
        result[i] = integrate_function(bessel_integrand, &sp, 4, 0, r[i], kmin, kmax);
        or_renorm_par_t p = {&sp, r[i], 0.};
        double v = or_qag61(renorm0_integrand, &p, kmin, kmax, 0, 1e-5, OR_QAG_LIMIT, NULL, NULL);
        if (r[i] > 0)
            v *= pow(r[i], 4.0);
        result0[i] = v / 2. / M_PI / M_PI;
    }
    (void)nthreads;
    or_spline_free(&sp);
    return 0;
}

/* out[b * n1 + a] = (1/2pi^2) int P j0(k chi1[a]) j0(k chi2[b]) / k^2 dk, GK61 QAG
   at relative 1e-5 (integrals_renormalization, integrals.c:424-444; the
   reference fills result2d[k * (nbins + 1) + j] for chi_j, chi_k,
   integrals.c:880-893) */
int or_renormalization_grid(const double *k, const double *pk, size_t nk, double kmin,
                            double kmax, const double *chi1, size_t n1, const double *chi2,
                            size_t n2, double *out, int nthreads)
{
    or_spline_t sp;
    if (or_spline_init(&sp, k, pk, nk, OR_AKIMA) != 0)
        return -1;
#ifdef _OPENMP
    if (nthreads <= 0)
        nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
#endif
    for (long t = 0; t < (long)(n1 * n2); ++t) {
        const size_t a = (size_t)t % n1, b = (size_t)t / n1;
        or_renorm_par_t p = {&sp, chi1[a], chi2[b]};
        out[t] = or_qag61(renorm_integrand, &p, kmin, kmax, 0, 1e-5, OR_QAG_LIMIT, NULL, NULL) /
                 2. / M_PI / M_PI;
    }
    (void)nthreads;
    or_spline_free(&sp);
    return 0;
}

int or_integral_table(const double *k, const double *pk, size_t nk, int n, int l,
                      size_t N, double kmin, double kmax, int with_small_r,
                      double *out_x, double *out_y)
{
    /* integrals.c:459-573 */
    const size_t off = OR_N_SMALL_R + 1;
    double *fx = out_x + off, *fy = out_y + off;
    if (or_twofast_1bessel(fx, fy, N, k, pk, nk, (double)l, (double)n, 1.0, kmin, kmin,
                           kmax) != 0)
        return -1;
    if (n >= l)
        for (size_t i = 0; i < N; ++i)
            fy[i] = fy[i] * pow(fx[i], (double)(n - l));
    out_x[0] = 0.0;
    for (size_t i = 1; i <= OR_N_SMALL_R; ++i)
        out_x[i] = or_min_sep[i - 1];
    if (!with_small_r) {
        for (size_t i = 0; i < off; ++i)
            out_y[i] = NAN;
        return 0;
    }
    or_spline_t sp;
    if (or_spline_init(&sp, k, pk, nk, OR_AKIMA) != 0)
        return -1;
    if (n >= l) {
        const double coeff = sqrt(M_PI / 2.) / pow(2, l + 0.5) / tgamma(l + 1.5);
        out_y[0] = integrate_function(prefactor_integrand, &sp, n, l, 0, kmin, kmax) * coeff;
    } else {
        out_y[0] = 0.0;
    }
    for (size_t i = 1; i <= OR_N_SMALL_R; ++i)
        out_y[i] = integrate_function(bessel_integrand, &sp, n, l, out_x[i], kmin, kmax);
    or_spline_free(&sp);
    return 0;
}

/* ======================================================================
 * background (background.c:301-696), flat LCDM: w = -1, wint = 1
 * ====================================================================== */

#define OR_XINT_BINS 16384
#define OR_XINT_ZMAX 100.0

typedef struct {
    double om; /* Omega0_cdm + Omega0_baryon */
    double og, ode;
} or_bgpar_t;

/* x(z) = Om/(1-Om) (1+z)^3 through the linear spline on the 16385-point grid
   of background.c:337-412 */
static double xint_lin(const or_bgpar_t *p, double z)
{
    const double dz = OR_XINT_ZMAX / OR_XINT_BINS;
    const double ratio = p->om / (1.0 - p->om);
    double u = z / dz;
    size_t i = (size_t)u;
    if (i >= OR_XINT_BINS)
        i = OR_XINT_BINS - 1;
    const double z0 = OR_XINT_ZMAX * (double)i / OR_XINT_BINS;
    const double z1 = OR_XINT_ZMAX * (double)(i + 1) / OR_XINT_BINS;
    const double x0 = ratio * (1 + z0) * (1 + z0) * (1 + z0);
    const double x1 = ratio * (1 + z1) * (1 + z1) * (1 + z1);
    return x0 + (z - z0) * ((x1 - x0) / (z1 - z0));
}

static void growth_rhs(const or_bgpar_t *p, double a, const double y[2], double f[2])
{
    /* growth_rate_ode, background.c:190-211, with w = -1 */
    const double z = 1. / a - 1;
    const double w = -1.0;
    const double x = xint_lin(p, z);
    f[0] = y[1];
    f[1] = -3. / 2 * (1 - w / (1 + x)) * y[1] / a + 3. / 2 * x / (1 + x) * y[0] / (a * a);
}

/* The growth ODE from a = 0.05, (D, D') = (0.05, 1) (background.c:430-481):
   one trajectory of OR_ODE_STEPS classical RK4 steps of 1e-3 in a up to a = 1,
   stored as (D, D', dD/da, dD'/da) per step point, and read at each node by
   cubic Hermite interpolation between the two steps around it.  (The
   reference integrates every node separately with GSL's adaptive rk2; this
   restatement agrees with it to that solver's tolerance.) */
#define OR_ODE_A0 0.05
#define OR_ODE_STEPS 950

static void growth_trajectory(const or_bgpar_t *p, double (*tr)[4])
{
    const double h = (1.0 - OR_ODE_A0) / OR_ODE_STEPS;
    double y[2] = {0.05, 1.0};
    for (int s = 0; s <= OR_ODE_STEPS; ++s) {
        const double a = OR_ODE_A0 + h * (double)s;
        double k1[2], k2[2], k3[2], k4[2], t[2];
        growth_rhs(p, a, y, k1);
        tr[s][0] = y[0];
        tr[s][1] = y[1];
        tr[s][2] = k1[0];
        tr[s][3] = k1[1];
        if (s == OR_ODE_STEPS)
            break;
        t[0] = y[0] + 0.5 * h * k1[0];
        t[1] = y[1] + 0.5 * h * k1[1];
        growth_rhs(p, a + 0.5 * h, t, k2);
        t[0] = y[0] + 0.5 * h * k2[0];
        t[1] = y[1] + 0.5 * h * k2[1];
        growth_rhs(p, a + 0.5 * h, t, k3);
        t[0] = y[0] + h * k3[0];
        t[1] = y[1] + h * k3[1];
        growth_rhs(p, a + h, t, k4);
        y[0] += h / 6.0 * (k1[0] + 2.0 * k2[0] + 2.0 * k3[0] + k4[0]);
        y[1] += h / 6.0 * (k1[1] + 2.0 * k2[1] + 2.0 * k3[1] + k4[1]);
    }
}

static void growth_at(double (*tr)[4], double ai, double y[2])
{
    const double h = (1.0 - OR_ODE_A0) / OR_ODE_STEPS;
    int s = (int)floor((ai - OR_ODE_A0) / h);
    if (s < 0)
        s = 0;
    if (s > OR_ODE_STEPS - 1)
        s = OR_ODE_STEPS - 1;
    const double t = (ai - (OR_ODE_A0 + h * (double)s)) / h;
    const double t2 = t * t, t3 = t2 * t;
    const double h00 = 2 * t3 - 3 * t2 + 1, h10 = t3 - 2 * t2 + t, h01 = -2 * t3 + 3 * t2,
                 h11 = t3 - t2;
    for (int c = 0; c < 2; ++c)
        y[c] = h00 * tr[s][c] + h10 * h * tr[s][2 + c] + h01 * tr[s + 1][c] +
               h11 * h * tr[s + 1][2 + c];
}

static double comoving_integrand(double z, void *vp)
{
    /* integrand_comoving, background.c:281-296 */
    const or_bgpar_t *p = (const or_bgpar_t *)vp;
    return 1. / sqrt(p->om * pow(1 + z, 3) + p->og * pow(1 + z, 4) + p->ode * 1.0);
}

int or_background_nodes(const or_cosmo_t *c, size_t bins, double *z, double *a,
                        double *Hz, double *confH, double *confHp, double *D1,
                        double *f, double *chi, double *D1_unnormalised)
{
    if (bins < 5)
        return -1;
    or_bgpar_t p;
    p.om = c->Omega0_cdm + c->Omega0_baryon;
    p.og = c->Omega0_gamma;
    p.ode = c->Omega0_de;
    double *Dtmp = (double *)malloc(sizeof(double) * bins);
    double *ftmp = (double *)malloc(sizeof(double) * bins);
    double(*tr)[4] = (double(*)[4])malloc(sizeof(double) * 4 * (OR_ODE_STEPS + 1));
    growth_trajectory(&p, tr);
#pragma omp parallel for schedule(dynamic, 16)
    for (long li = 0; li < (long)bins; ++li) {
        const size_t i = (size_t)li;
        const double zi = 15. * i / (double)(bins - 1);
        const double ai = 1. / (1. + zi);
        double y[2];
        growth_at(tr, ai, y);
        Dtmp[i] = y[0];
        ftmp[i] = y[1] * ai / y[0];
        const double Hi =
            sqrt(p.om * pow(1 + zi, 3) + p.og * pow(1 + zi, 4) + p.ode * 1.0) * c->h * OR_H0;
        if (z)
            z[i] = zi;
        if (a)
            a[i] = ai;
        if (Hz)
            Hz[i] = Hi;
        if (confH)
            confH[i] = ai * Hi;
        if (confHp)
            confHp[i] = -(pow(1 + zi, 3) * (2 * (1 + zi) * p.og + p.om) +
                          (1 + 3 * (-1.0)) * p.ode * 1.0) /
                        pow(1 + zi, 2) / 2. * pow(c->h * OR_H0, 2);
        if (chi)
            chi[i] = or_qag61(comoving_integrand, &p, 0., zi, 0, 1e-5, OR_QAG_LIMIT, NULL,
                              NULL) /
                     (c->h * OR_H0);
    }
    for (size_t i = 0; i < bins; ++i) {
        if (D1_unnormalised)
            D1_unnormalised[i] = Dtmp[i];
        if (D1)
            D1[i] = Dtmp[i] / Dtmp[0];
        if (f)
            f[i] = ftmp[i];
    }
    free(Dtmp);
    free(ftmp);
    free(tr);
    return 0;
}

/* ======================================================================
 * multipoles of the nonintegrated den+RSD terms
 * ====================================================================== */

#define OR_MAX_INTEGRALS 32

struct or_model {
    or_spline_t chi_of_z, z_of_chi, D1, f, a, confH;
    or_spline_t bias[4];
    int have_bias[4];
    int nint;
    int int_n[OR_MAX_INTEGRALS], int_l[OR_MAX_INTEGRALS];
    or_spline_t integral[OR_MAX_INTEGRALS];
    double h, Omega0_m;
    int have_bg;
};

or_model_t *or_model_new(void)
{
    or_model_t *m = (or_model_t *)calloc(1, sizeof(or_model_t));
    return m;
}

void or_model_free(or_model_t *m)
{
    if (!m)
        return;
    if (m->have_bg) {
        or_spline_free(&m->chi_of_z);
        or_spline_free(&m->z_of_chi);
        or_spline_free(&m->D1);
        or_spline_free(&m->f);
        or_spline_free(&m->a);
        or_spline_free(&m->confH);
    }
    for (int i = 0; i < 4; ++i)
        if (m->have_bias[i])
            or_spline_free(&m->bias[i]);
    for (int i = 0; i < m->nint; ++i)
        or_spline_free(&m->integral[i]);
    free(m);
}

int or_model_set_background(or_model_t *m, const double *z, const double *chi,
                            const double *D1, const double *f, const double *a,
                            const double *confH, size_t bins, double h, double Omega0_m)
{
    if (m->have_bg) {
        or_spline_free(&m->chi_of_z);
        or_spline_free(&m->z_of_chi);
        or_spline_free(&m->D1);
        or_spline_free(&m->f);
        or_spline_free(&m->a);
        or_spline_free(&m->confH);
    }
    int e = 0;
    e |= or_spline_init(&m->chi_of_z, z, chi, bins, OR_AKIMA);
    e |= or_spline_init(&m->z_of_chi, chi, z, bins, OR_AKIMA);
    e |= or_spline_init(&m->D1, z, D1, bins, OR_AKIMA);
    e |= or_spline_init(&m->f, z, f, bins, OR_AKIMA);
    e |= or_spline_init(&m->a, z, a, bins, OR_AKIMA);
    e |= or_spline_init(&m->confH, z, confH, bins, OR_AKIMA);
    m->h = h;
    m->Omega0_m = Omega0_m;
    m->have_bg = 1;
    return e ? -1 : 0;
}

int or_model_set_bias(or_model_t *m, int which, const double *z, const double *v, size_t n)
{
    if (which < 0 || which > 3)
        return -1;
    if (m->have_bias[which])
        or_spline_free(&m->bias[which]);
    m->have_bias[which] = 0;
    if (or_spline_init(&m->bias[which], z, v, n, OR_AKIMA) != 0)
        return -1;
    m->have_bias[which] = 1;
    return 0;
}

int or_model_set_integral(or_model_t *m, int n, int l, const double *x, const double *y,
                          size_t len)
{
    for (int i = 0; i < m->nint; ++i)
        if (m->int_n[i] == n && m->int_l[i] == l) {
            or_spline_free(&m->integral[i]);
            return or_spline_init(&m->integral[i], x, y, len, OR_AKIMA);
        }
    if (m->nint >= OR_MAX_INTEGRALS)
        return -1;
    const int i = m->nint;
    if (or_spline_init(&m->integral[i], x, y, len, OR_AKIMA) != 0)
        return -1;
    m->int_n[i] = n;
    m->int_l[i] = l;
    m->nint++;
    return 0;
}

static const or_spline_t *find_integral(const or_model_t *m, int n, int l)
{
    for (int i = 0; i < m->nint; ++i)
        if (m->int_n[i] == n && m->int_l[i] == l)
            return &m->integral[i];
    return NULL;
}

static double bias_eval(const or_model_t *m, int which, double z, double dflt)
{
    return m->have_bias[which] ? or_spline_eval(&m->bias[which], z) : dflt;
}

/*
 * xi(z_mean, mu, r) of the nonintegrated den-den, rsd-rsd and den-rsd terms
 * (functions.c:89-1484; den-den 129-229, rsd-rsd 230-362, den-rsd 670-771,
 * D1(z1) D1(z2) factor 1463-1466), full-sky branch.
 *
 * The coefficients are written in terms of s = 1 - cos(theta) =
 * r^2 (1 - mu^2) / D with D = 2 chi^2 - mu^2 r^2 / 2 = 2 chi1 chi2.  This is
 * algebraically identical to the reference's expressions in cos(theta) and
 * chi1/r, chi2/r, but avoids their cancellation: e.g. the I04 coefficient of
 * rsd-rsd subtracts two terms of size (chi/r)^4 ~ 1e10 to leave O(1), losing up
 * to six digits in FP64.  The expanded I04 polynomial is
 *   (1-mu^2)^2 (3c^2 - 10c + 19) / 4 + 4 mu^2 (1-mu^2)(c^2 - 5c - 2)
 *   + 4 (3c^2 - 1) mu^4          (= 8 P_4(mu) at c = 1).
 */
double or_xi_nonintegrated(const or_model_t *m, int contrib, double z_mean, double mu,
                           double sep)
{
    const double chi_mean = or_spline_eval(&m->chi_of_z, z_mean);
    const double chi1 = chi_mean - sep * mu / 2.;
    const double chi2 = chi_mean + sep * mu / 2.;
    const double mu2 = mu * mu;
    const double omm = 1.0 - mu2;
    const double D = 2. * chi_mean * chi_mean - mu2 * sep * sep / 2.;
    const double s = sep * sep * omm / D;
    const double c = 1.0 - s;
    const double z1 = or_spline_eval(&m->z_of_chi, chi1);
    const double z2 = or_spline_eval(&m->z_of_chi, chi2);
    const double f1 = or_spline_eval(&m->f, z1);
    const double f2 = or_spline_eval(&m->f, z2);
    const double b1 = bias_eval(m, 0, z1, 1.0);
    const double b2 = bias_eval(m, 1, z2, 1.0);
    const or_spline_t *i00 = find_integral(m, 0, 0);
    const or_spline_t *i02 = find_integral(m, 0, 2);
    const or_spline_t *i04 = find_integral(m, 0, 4);
    const double I00 = or_spline_eval(i00, sep);
    double result = 0;
    if (contrib & OR_CONTRIB_DEN)
        result += b1 * b2 * I00;
    if (contrib & OR_CONTRIB_RSD) {
        const double I02 = or_spline_eval(i02, sep);
        const double I04 = or_spline_eval(i04, sep);
        const double c2 = c * c;
        const double q4 = omm * omm * (3 * c2 - 10 * c + 19) / 4. +
                          4 * mu2 * omm * (c2 - 5 * c - 2) + 4 * (3 * c2 - 1) * mu2 * mu2;
        result += f1 * f2 * (1 + 2 * c2) / 15 * I00 -
                  f1 * f2 / 21. * ((1 + 11. * c2) - 9 * c * (2 - s) * omm) * I02 +
                  f1 * f2 * q4 / 35. * I04;
    }
    if ((contrib & OR_CONTRIB_DEN) && (contrib & OR_CONTRIB_RSD)) {
        const double I02 = or_spline_eval(i02, sep);
        const double g = (2 - s) * omm / D;
        result += (b1 * f2 / 3. + b2 * f1 / 3.) * I00 -
                  (b1 * f2 * (2. / 3. - g * chi1 * chi1) + b2 * f1 * (2. / 3. - g * chi2 * chi2)) *
                      I02;
    }
    return result * or_spline_eval(&m->D1, z1) * or_spline_eval(&m->D1, z2);
}

typedef struct {
    const or_model_t *m;
    int contrib, l;
    double z_mean, sep;
} or_mp_par_t;

static double mp_integrand(double x, void *vp)
{
    /* multipoles_nonintegrated_integrand, signal.c:83-111 */
    const or_mp_par_t *p = (const or_mp_par_t *)vp;
    const double mu = 2 * x - 1;
    const double xi = or_xi_nonintegrated(p->m, p->contrib, p->z_mean, mu, p->sep);
    if (p->l == 0)
        return xi;
    return xi * or_legendre(p->l, mu);
}

double or_multipole_nonintegrated(const or_model_t *m, int contrib, double z_mean,
                                  double sep, int l, double epsrel)
{
    /* coffe_integrate(NONINTEGRATED, MULTIPOLES), signal.c:521-542 */
    if (!(contrib & (OR_CONTRIB_DEN | OR_CONTRIB_RSD)))
        return 0.0;
    or_mp_par_t p = {m, contrib, l, z_mean, sep};
    const double r = or_qag61(mp_integrand, &p, 0, 1, 0, epsrel, OR_QAG_LIMIT, NULL, NULL);
    return (2 * l + 1) * r;
}

double or_multipole_nonintegrated_gl(const or_model_t *m, int contrib, double z_mean,
                                     double sep, int l, size_t n_mu)
{
    double *x = (double *)malloc(sizeof(double) * n_mu);
    double *w = (double *)malloc(sizeof(double) * n_mu);
    or_gauss_legendre(n_mu, x, w);
    double s = 0;
    for (size_t i = 0; i < n_mu; ++i)
        s += w[i] * or_xi_nonintegrated(m, contrib, z_mean, x[i], sep) * or_legendre(l, x[i]);
    free(x);
    free(w);
    return (2 * l + 1) * 0.5 * s;
}

int or_multipoles_batch(const or_model_t *m, int contrib, const double *z_mean,
                        const double *sep, const int *l, size_t count, double epsrel,
                        double *out, int nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0)
        nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
#endif
    for (long i = 0; i < (long)count; ++i)
        out[i] = or_multipole_nonintegrated(m, contrib, z_mean[i], sep[i], l[i], epsrel);
    (void)nthreads;
    return 0;
}

/* ------------------------------------------------------------------ lensing
 * Full-sky lensing terms of the linear-P(k), non-divergent path
 * (flatsky_local_nonlocal = flatsky_nonlocal = only_cross_correlations = 0,
 * the reference's defaults, parser.c:801, 1018-1022).
 *
 * Geometry as functions.c:1498-1509 and 3473-3481: chi_{1,2} = chi(z_mean) -+
 * sep mu / 2, lambda_i = chi_i x_i.  cos(theta) is formed as 1 - s with
 * s = sep^2 (1 - mu^2) / (2 chi1 chi2) (the same quantity as the reference's
 * ratio, without its cancellation), 1 - cos^2 = s (2 - s), and the squared
 * distances as r21 = (lambda2 - chi1)^2 + 2 chi1 lambda2 s etc., which equal
 * the reference's lambda2^2 + chi1^2 - 2 chi1 lambda2 cos(theta).
 */
typedef struct {
    double chi_mean, chi1, chi2, s, ct, one_m_ct2;
} or_lens_geom_t;

static or_lens_geom_t lens_geom(const or_model_t *m, double z_mean, double mu, double sep)
{
    or_lens_geom_t g;
    g.chi_mean = or_spline_eval(&m->chi_of_z, z_mean);
    g.chi1 = g.chi_mean - sep * mu / 2.;
    g.chi2 = g.chi_mean + sep * mu / 2.;
    g.s = sep * sep * (1 - mu * mu) / (2. * g.chi_mean * g.chi_mean - mu * mu * sep * sep / 2.);
    g.ct = 1 - g.s;
    g.one_m_ct2 = g.s * (2 - g.s);
    return g;
}

/* den-len + len-den (functions.c:1557-2052) and rsd-len + len-rsd
   (functions.c:2053-2483) single-integrated xi at (mu, x), without the
   (2l+1) P_l(mu) of the multipole integrand (signal.c:141-186) */
double or_xi_single_integrated(const or_model_t *m, int contrib, double z_mean, double mu,
                               double sep, double x)
{
    if (!(contrib & OR_CONTRIB_LEN) || !(contrib & (OR_CONTRIB_DEN | OR_CONTRIB_RSD)))
        return 0.0;
    const or_lens_geom_t g = lens_geom(m, z_mean, mu, sep);
    const double chi1 = g.chi1, chi2 = g.chi2, ct = g.ct, omc2 = g.one_m_ct2;
    const double lambda1 = chi1 * x, lambda2 = chi2 * x;
    double r21 = (lambda2 - chi1) * (lambda2 - chi1) + 2 * chi1 * lambda2 * g.s;
    double r22 = (lambda1 - chi2) * (lambda1 - chi2) + 2 * chi2 * lambda1 * g.s;
    if (r21 < 0) r21 = 0;
    if (r22 < 0) r22 = 0;
    const double z1c = or_spline_eval(&m->z_of_chi, chi1);
    const double z2c = or_spline_eval(&m->z_of_chi, chi2);
    const double z1 = or_spline_eval(&m->z_of_chi, lambda1);
    const double z2 = or_spline_eval(&m->z_of_chi, lambda2);
    const double s1 = bias_eval(m, 2, z1c, 0.0), s2 = bias_eval(m, 3, z2c, 0.0);
    const double pref = pow(OR_H0 * m->h, 2);
    const double Om = m->Omega0_m;
    /* the "2" side: the lensing convergence along the line of sight to chi2,
       correlated with the local term at chi1 (and the mirror "1" side) */
    const double D1z1 = or_spline_eval(&m->D1, z1), D1z2 = or_spline_eval(&m->D1, z2);
    const double az1 = or_spline_eval(&m->a, z1), az2 = or_spline_eval(&m->a, z2);
    const double D1z1c = or_spline_eval(&m->D1, z1c), D1z2c = or_spline_eval(&m->D1, z2c);
    const double sr21 = sqrt(r21), sr22 = sqrt(r22);
    const or_spline_t *i00 = find_integral(m, 0, 0), *i02 = find_integral(m, 0, 2),
                      *i04 = find_integral(m, 0, 4), *i11 = find_integral(m, 1, 1);
    double result = 0;
    if (contrib & OR_CONTRIB_DEN) {
        const double b1 = bias_eval(m, 0, z1c, 1.0), b2 = bias_eval(m, 1, z2c, 1.0);
        /* functions.c:1620-1719 (both nonzero), 1720-1876, 1877-1974, 1975-2050 */
        double t1, t2;
        if (r21 != 0.0)
            t1 = chi2 * (2 * chi1 * ct * or_spline_eval(i11, sr21) -
                         chi1 * chi1 * lambda2 * omc2 * or_spline_eval(i02, sr21) / r21);
        else
            t1 = chi2 * 2 * chi1 * or_spline_eval(i11, 0.0);
        if (r22 != 0.0)
            t2 = chi1 * (2 * chi2 * ct * or_spline_eval(i11, sr22) -
                         chi2 * chi2 * lambda1 * omc2 * or_spline_eval(i02, sr22) / r22);
        else
            t2 = chi1 * 2 * chi2 * or_spline_eval(i11, 0.0);
        result += pref * (-3 * Om / 2. *
                          (b1 * (2 - 5 * s2) * D1z1c * (1 - x) * D1z2 / az2 * t1 +
                           b2 * (2 - 5 * s1) * D1z2c * (1 - x) * D1z1 / az1 * t2));
    }
    if (contrib & OR_CONTRIB_RSD) {
        const double f1c = or_spline_eval(&m->f, z1c), f2c = or_spline_eval(&m->f, z2c);
        const double c2m1 = 2 * ct * ct - 1; /* cos(2 theta) */
        /* I00/I02 part (functions.c:2174-2183) and I04 part (2298-2306) of one
           side.  The reference's polynomials in (chi, lambda, cos theta) that
           multiply I02 / r^2 and I04 / r^4 vanish like r^2 and r^4 and lose up
           to ~10 digits to cancellation; they are expanded here in d = chi -
           lambda and s = 1 - cos(theta) (identical polynomials), where every
           term is of the size of the result. */
#define OR_RL_Q(ch, d, ss)                                                                     \
    ((d) * (d) * (d) * (8 - 24 * (ss) + 12 * (ss) * (ss)) +                                    \
     (ch) * (d) * (d) * (-2 + 38 * (ss) - 18 * (ss) * (ss) - 6 * (ss) * (ss) * (ss)) +         \
     (ch) * (ch) * (d) * (ss) * (-22 + 9 * (ss) + 12 * (ss) * (ss)) +                          \
     (ch) * (ch) * (ch) * (ss) * (2 - 3 * (ss) - 6 * (ss) * (ss)))
#define OR_RL_P(ch, d, ss)                                                                     \
    (pow(d, 5) * (4 - 12 * (ss) + 6 * (ss) * (ss)) +                                           \
     (ch) * pow(d, 4) * (-8 + 60 * (ss) - 48 * (ss) * (ss) + 6 * pow(ss, 3)) +                 \
     pow(ch, 2) * pow(d, 3) * (ss) * (-92 + 114 * (ss) - 20 * (ss) * (ss) - pow(ss, 3)) +     \
     pow(ch, 3) * pow(d, 2) * (ss) * (48 - 120 * (ss) + 26 * (ss) * (ss) + 3 * pow(ss, 3)) +  \
     pow(ch, 4) * (d) * (ss) * (ss) * (60 - 16 * (ss) - 3 * (ss) * (ss)) +                     \
     pow(ch, 5) * (ss) * (ss) * (-12 + 4 * (ss) + (ss) * (ss)))
#define OR_RL_A(ch, la, sr, r2)                                                                \
    ((la - 6 * ch * ct + 3 * la * c2m1) * or_spline_eval(i00, sr) / 15. -                     \
     OR_RL_Q(ch, (ch) - (la), g.s) * or_spline_eval(i02, sr) / (r2) / 21.)
#define OR_RL_B(ch, la, sr, r2)                                                                \
    (-OR_RL_P(ch, (ch) - (la), g.s) * or_spline_eval(i04, sr) / (r2) / (r2) / 35.)
        const double w2 = chi2 * f1c * (2 - 5 * s2) * D1z1c * D1z2 / az2; /* side at chi2 */
        const double w1 = chi1 * f2c * (2 - 5 * s1) * D1z2c * D1z1 / az1; /* side at chi1 */
        const double c = pref * 3 * Om / 2.;
        if (r21 != 0 && r22 != 0) {
            /* functions.c:2060-2391 */
            result += c * (w2 * (1 - x) * OR_RL_A(chi1, lambda2, sr21, r21) +
                           w1 * (1 - x) * OR_RL_A(chi2, lambda1, sr22, r22));
            if (fabs(mu) < 0.999)
                result += c * (w2 * (1 - x) * OR_RL_B(chi1, lambda2, sr21, r21) +
                               w1 * (1 - x) * OR_RL_B(chi2, lambda1, sr22, r22));
            else
                result += c * (w2 * (1 - x) * 4. * (lambda2 + chi1) * or_spline_eval(i04, sr21) / 35. +
                               w1 * (1 - x) * 4. * (lambda1 + chi2) * or_spline_eval(i04, sr22) / 35.);
        } else if (r21 == 0 && r22 != 0) {
            /* functions.c:2392-2426 */
            result += c * (w2 * (1 - chi1 / chi2) * (-2 * chi1 * or_spline_eval(i00, 0.0) / 15.) +
                           w1 * (1 - x) *
                               (OR_RL_A(chi2, lambda1, sr22, r22) + OR_RL_B(chi2, lambda1, sr22, r22)));
        } else if (r21 != 0 && r22 == 0) {
            /* functions.c:2427-2462 */
            result += c * (w2 * (1 - x) *
                               (OR_RL_A(chi1, lambda2, sr21, r21) + OR_RL_B(chi1, lambda2, sr21, r21)) +
                           w1 * (1 - chi2 / chi1) * (-2 * chi2 * or_spline_eval(i00, 0.0) / 15.));
        } else {
            /* functions.c:2463-2481 */
            result += c * (w2 * (1 - chi1 / chi2) * (-2 * chi1 * or_spline_eval(i00, 0.0) / 15.) +
                           w1 * (1 - chi2 / chi1) * (-2 * chi2 * or_spline_eval(i00, 0.0) / 15.));
        }
#undef OR_RL_A
#undef OR_RL_B
#undef OR_RL_P
#undef OR_RL_Q
    }
    return result;
}

/* len-len double-integrated xi at (mu, x1, x2) (functions.c:3460-3836 and the
   (H0 h)^4 factor of 3988-3990) */
double or_xi_double_integrated(const or_model_t *m, int contrib, double z_mean, double mu,
                               double sep, double x1, double x2)
{
    if (!(contrib & OR_CONTRIB_LEN))
        return 0.0;
    const or_lens_geom_t g = lens_geom(m, z_mean, mu, sep);
    const double chi1 = g.chi1, chi2 = g.chi2, ct = g.ct, omc2 = g.one_m_ct2;
    const double lambda1 = chi1 * x1, lambda2 = chi2 * x2;
    double r2 = (lambda1 - lambda2) * (lambda1 - lambda2) + 2 * lambda1 * lambda2 * g.s;
    if (r2 < 0) r2 = 0;
    const double z1c = or_spline_eval(&m->z_of_chi, chi1);
    const double z2c = or_spline_eval(&m->z_of_chi, chi2);
    const double z1 = or_spline_eval(&m->z_of_chi, lambda1);
    const double z2 = or_spline_eval(&m->z_of_chi, lambda2);
    const double s1 = bias_eval(m, 2, z1c, 0.0), s2 = bias_eval(m, 3, z2c, 0.0);
    const double Om = m->Omega0_m;
    const double pre = 9. * Om * Om * (2 - 5 * s1) * (2 - 5 * s2) / 4. * chi1 * chi2 *
                       or_spline_eval(&m->D1, z1) * or_spline_eval(&m->D1, z2) /
                       or_spline_eval(&m->a, z1) / or_spline_eval(&m->a, z2) * (1 - x1) * (1 - x2);
    const double ll = lambda1 * lambda2;
    double result;
    if (r2 > 1e-20) {
        const double r = sqrt(r2);
        const double c2m = -omc2; /* cos^2 - 1 */
        result = pre * (2 * c2m * ll * or_spline_eval(find_integral(m, 0, 0), r) / 5. +
                        4 * ct * or_spline_eval(find_integral(m, 2, 0), r) / 3. +
                        4 * ct * (r2 + 6 * ct * ll) * or_spline_eval(find_integral(m, 1, 1), r) / 15. +
                        2 * c2m * ll * (2 * r2 + 3 * ct * ll) *
                            or_spline_eval(find_integral(m, 0, 2), r) / 7. / r2 +
                        2 * ct * (2 * r2 * r2 + 12 * ct * r2 * ll + 15 * c2m * ll * ll) *
                            or_spline_eval(find_integral(m, 1, 3), r) / 15. / r2 +
                        c2m * ll * (6 * r2 * r2 + 30 * ct * r2 * ll + 35 * c2m * ll * ll) *
                            or_spline_eval(find_integral(m, 0, 4), r) / 35. / r2 / r2);
    } else {
        /* functions.c:3801-3833 */
        result = pre * (4. + 24. * ll * or_spline_eval(find_integral(m, 1, 1), 0.0) / 15.);
    }
    return result * pow(OR_H0 * m->h, 4);
}

/* Lensing multipoles with Gauss-Legendre product rules on the unit cube of
   signal.c:141-237 (mu = 2 v - 1): n_mu nodes in v and, per x line, n_x nodes
   split into two panels of n_x / 2 at the point where the integrand's
   separation argument is smallest (x* = lambda1 / chi2 for the inner len-len
   line, x* = min(chi1, chi2) cos(theta) / max(chi1, chi2) for the single
   integral), where its narrow peak sits; GL nodes cluster at panel ends, so
   the peak is resolved at no extra cost.  n_x odd or 0 panels fall back to
   one panel.  out[j] = (2 l_j + 1) * integral (signal.c:659-668, 742-751);
   nothing is added for the nonintegrated terms. */
typedef struct {
    size_t n;
    const double *xf, *wf; /* n-point rule on [-1, 1] */
    const double *xh, *wh; /* n/2-point rule on [-1, 1] */
} or_line_rule_t;

static double lens_line(double x0, double x1_, double xs, const or_line_rule_t *R, int which,
                        const or_model_t *m, int contrib, double z_mean, double mu, double sep,
                        double xa)
{
    /* integrates over [x0, x1_]: two panels [x0, xs], [xs, x1_] of n/2 GL nodes
       when xs is inside and n even, else one panel of n nodes */
    double acc = 0.0;
    const size_t n = R->n;
    const int split = (n % 2 == 0) && xs > x0 && xs < x1_;
    const size_t np = split ? n / 2 : n;
    const double *gx = split ? R->xh : R->xf, *gw = split ? R->wh : R->wf;
    const double lo[2] = {x0, xs}, hi[2] = {xs, x1_};
    for (int p = 0; p < (split ? 2 : 1); ++p) {
        const double a = split ? lo[p] : x0, b = split ? hi[p] : x1_;
        const double c = 0.5 * (a + b), h = 0.5 * (b - a);
        double part = 0.0;
        for (size_t i = 0; i < np; ++i) {
            const double x = c + h * gx[i];
            part += gw[i] * (which == 1 ? or_xi_single_integrated(m, contrib, z_mean, mu, sep, x)
                                        : or_xi_double_integrated(m, contrib, z_mean, mu, sep, xa, x));
        }
        acc += h * part;
    }
    return acc;
}

/* tracers i and j (0/1 galaxy, 2/3 magnification bias) are the same function:
   both unset, or both set from equal samples */
static int same_tracer(const or_model_t *m, int i, int j)
{
    if (!m->have_bias[i] || !m->have_bias[j])
        return !m->have_bias[i] && !m->have_bias[j];
    const or_spline_t *a = &m->bias[i], *b = &m->bias[j];
    return a->n == b->n && a->type == b->type &&
           memcmp(a->x, b->x, sizeof(double) * a->n) == 0 &&
           memcmp(a->y, b->y, sizeof(double) * a->n) == 0;
}

/* The lensing multipoles on the product rule.  mu -> -mu swaps chi1 and chi2,
   i.e. the roles of the two tracers; when they share their magnification bias
   (and, with density-lensing, their galaxy bias) both lensing terms are even
   in mu, and each even multipole is summed over the rule's nodes with mu > 0
   (the Gauss-Legendre rule is symmetric), each counted twice, whatever else
   the list holds; odd multipoles over every node (nodes mu < 0 are evaluated
   only when an odd one is asked for).  Quadrature choice of this restatement
   (the reference uses Cuhre): the plane rule at a node -mu is the one at mu
   with x1 and x2 exchanged, equal to it up to the rule's own error. */
int or_multipoles_lensing_gl(const or_model_t *m, int contrib, double z_mean, double sep,
                             int n_l, const int *ls, size_t n_mu, size_t n_x, double *out)
{
    double *xm = (double *)malloc(sizeof(double) * n_mu), *wm = (double *)malloc(sizeof(double) * n_mu);
    double *xf = (double *)malloc(sizeof(double) * n_x), *wf = (double *)malloc(sizeof(double) * n_x);
    double *xh = (double *)malloc(sizeof(double) * n_x), *wh = (double *)malloc(sizeof(double) * n_x);
    if (!xm || !wm || !xf || !wf || !xh || !wh) {
        free(xm); free(wm); free(xf); free(wf); free(xh); free(wh);
        return -1;
    }
    or_gauss_legendre(n_mu, xm, wm);
    or_gauss_legendre(n_x, xf, wf);
    if (n_x >= 2) or_gauss_legendre(n_x / 2, xh, wh);
    for (int j = 0; j < n_l; ++j) out[j] = 0.0;
    const int single = (contrib & OR_CONTRIB_LEN) && (contrib & (OR_CONTRIB_DEN | OR_CONTRIB_RSD));
    const int dbl = (contrib & OR_CONTRIB_LEN) != 0;
    const or_line_rule_t R = {n_x, xf, wf, xh, wh};
    const int sym = n_mu % 2 == 0 && same_tracer(m, 2, 3) &&
                    (!(single && (contrib & OR_CONTRIB_DEN)) || same_tracer(m, 0, 1));
    int all_even = 1;
    for (int j = 0; j < n_l; ++j)
        all_even = all_even && ls[j] % 2 == 0;
    for (size_t i = (sym && all_even) ? n_mu / 2 : 0; i < n_mu; ++i) {
        const double mu = xm[i], wmu = 0.5 * wm[i]; /* dv = dmu / 2 */
        const or_lens_geom_t g = lens_geom(m, z_mean, mu, sep);
        double acc = 0.0;
        if (single) {
            const double xs = fmin(g.chi1, g.chi2) * g.ct / fmax(g.chi1, g.chi2);
            acc += lens_line(0, 1, xs, &R, 1, m, contrib, z_mean, mu, sep, 0);
        }
        if (dbl)
            for (size_t a = 0; a < n_x; ++a) {
                const double x1 = 0.5 * (xf[a] + 1.0);
                const double xs = x1 * g.chi1 / g.chi2;
                acc += 0.5 * wf[a] * lens_line(0, 1, xs, &R, 2, m, contrib, z_mean, mu, sep, x1);
            }
        for (int j = 0; j < n_l; ++j) {
            /* even l of equal tracers: the mu > 0 half, twice; else every node */
            const int half = sym && ls[j] % 2 == 0;
            if (half && i < n_mu / 2)
                continue;
            out[j] += (half ? 2.0 : 1.0) * wmu * acc * or_legendre(ls[j], mu);
        }
    }
    for (int j = 0; j < n_l; ++j) out[j] *= (2 * ls[j] + 1);
    free(xm); free(wm); free(xf); free(wf); free(xh); free(wh);
    return 0;
}

/* many (z_mean, sep) points, OpenMP over points; out[p * n_l + j] */
int or_multipoles_lensing_batch(const or_model_t *m, int contrib, const double *z_mean,
                                const double *sep, size_t count, int n_l, const int *ls,
                                size_t n_mu, size_t n_x, double *out, int nthreads)
{
    int bad = 0;
#ifdef _OPENMP
    if (nthreads <= 0)
        nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads) reduction(| : bad)
#endif
    for (long p = 0; p < (long)count; ++p)
        bad |= or_multipoles_lensing_gl(m, contrib, z_mean[p], sep[p], n_l, ls, n_mu, n_x,
                                        out + (size_t)p * n_l) != 0;
    (void)nthreads;
    return bad ? -1 : 0;
}

/* The correlation function at (z_mean, mu, sep) as coffe_corrfunc_init sums it
   (corrfunc.c:55-141 with coffe_integrate's CORRFUNC branches, signal.c:511-518,
   584-605, 695-702): the nonintegrated den/rsd terms at mu, plus with len the
   single-integrated den/rsd x lensing line integral over x and the
   double-integrated lensing-lensing integral over (x1, x2), both at mu.  The
   reference integrates the two lensing parts with GSL QAG and Cuhre; here the
   split Gauss-Legendre rules of or_multipoles_lensing_gl (n_x nodes per line).
   The CORRFUNC branches have no flat-sky forms. */
double or_corrfunc_gl(const or_model_t *m, int contrib, double z_mean, double mu, double sep,
                      size_t n_x)
{
    double *xf = (double *)malloc(sizeof(double) * n_x), *wf = (double *)malloc(sizeof(double) * n_x);
    double *xh = (double *)malloc(sizeof(double) * n_x), *wh = (double *)malloc(sizeof(double) * n_x);
    if (!xf || !wf || !xh || !wh) {
        free(xf); free(wf); free(xh); free(wh);
        return NAN;
    }
    or_gauss_legendre(n_x, xf, wf);
    if (n_x >= 2) or_gauss_legendre(n_x / 2, xh, wh);
    double acc = 0.0;
    if (contrib & (OR_CONTRIB_DEN | OR_CONTRIB_RSD))
        acc += or_xi_nonintegrated(m, contrib, z_mean, mu, sep);
    if (contrib & OR_CONTRIB_LEN) {
        const or_line_rule_t R = {n_x, xf, wf, xh, wh};
        const or_lens_geom_t g = lens_geom(m, z_mean, mu, sep);
        if (contrib & (OR_CONTRIB_DEN | OR_CONTRIB_RSD)) {
            const double xs = fmin(g.chi1, g.chi2) * g.ct / fmax(g.chi1, g.chi2);
            acc += lens_line(0, 1, xs, &R, 1, m, contrib, z_mean, mu, sep, 0);
        }
        for (size_t a = 0; a < n_x; ++a) {
            const double x1 = 0.5 * (xf[a] + 1.0);
            const double xs = x1 * g.chi1 / g.chi2;
            acc += 0.5 * wf[a] * lens_line(0, 1, xs, &R, 2, m, contrib, z_mean, mu, sep, x1);
        }
    }
    free(xf); free(wf); free(xh); free(wh);
    return acc;
}

/* many (z_mean, mu, sep) points, OpenMP over points */
int or_corrfunc_batch(const or_model_t *m, int contrib, const double *z_mean, const double *mu,
                      const double *sep, size_t count, size_t n_x, double *out, int nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0)
        nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (long p = 0; p < (long)count; ++p)
        out[p] = or_corrfunc_gl(m, contrib, z_mean[p], mu[p], sep[p], n_x);
    (void)nthreads;
    return 0;
}

/* Redshift-averaged multipole (average_multipoles.c:69-156 with coffe_integrate's
   AVERAGE_MULTIPOLES branches, signal.c:241-310, 543-551, 672-680, 755-763):
     (2l+1) int_0^1 dv0 int_0^1 dv1 xi(z(v0), mu = 2 v1 - 1, r) P_l(mu) H0 h / (confH(z) (1 + z))
   with z(v0) = z1 + (z2 - z1) v0, z1 = z(chi(z_min) + r/2), z2 = z(chi(z_max) - r/2),
   the unit-cube measure as the reference writes it.  The reference integrates the
   cube with Cuhre (2D; 3D and 4D with the lensing terms); here n_z Gauss-Legendre
   nodes in v0 and, per node, the multipole at z_mean = z(v0) as or_multipole_nonintegrated
   computes it (QAG GK61 in mu), plus with len the lensing multipoles of
   or_multipoles_lensing_gl (n_mu x n_x rules). */
double or_average_multipole(const or_model_t *m, int contrib, double z_min, double z_max,
                            double sep, int l, size_t n_z, size_t n_mu, size_t n_x)
{
    double *xz = (double *)malloc(sizeof(double) * n_z), *wz = (double *)malloc(sizeof(double) * n_z);
    if (!xz || !wz) {
        free(xz); free(wz);
        return NAN;
    }
    or_gauss_legendre(n_z, xz, wz);
    const double z1 = or_spline_eval(&m->z_of_chi, or_spline_eval(&m->chi_of_z, z_min) + sep / 2.);
    const double z2 = or_spline_eval(&m->z_of_chi, or_spline_eval(&m->chi_of_z, z_max) - sep / 2.);
    double acc = 0.0;
    for (size_t k = 0; k < n_z; ++k) {
        const double v = 0.5 * (xz[k] + 1.0);
        const double z = (z2 - z1) * v + z1;
        double mp = 0.0;
        if (contrib & (OR_CONTRIB_DEN | OR_CONTRIB_RSD))
            mp += or_multipole_nonintegrated(m, contrib, z, sep, l, 1e-5);
        if (contrib & OR_CONTRIB_LEN) {
            double lv = 0.0;
            or_multipoles_lensing_gl(m, contrib, z, sep, 1, &l, n_mu, n_x, &lv);
            mp += lv;
        }
        acc += 0.5 * wz[k] * mp * OR_H0 * m->h / (or_spline_eval(&m->confH, z) * (1.0 + z));
    }
    free(xz); free(wz);
    return acc;
}

int or_average_multipoles_batch(const or_model_t *m, int contrib, const double *z_min,
                                const double *z_max, const double *sep, const int *l,
                                size_t count, size_t n_z, size_t n_mu, size_t n_x, double *out,
                                int nthreads)
{
#ifdef _OPENMP
    if (nthreads <= 0)
        nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (long p = 0; p < (long)count; ++p)
        out[p] = or_average_multipole(m, contrib, z_min[p], z_max[p], sep[p], l[p], n_z, n_mu, n_x);
    (void)nthreads;
    return 0;
}

/* --------------------------------------------------------------- covariance
 * Flat-sky Gaussian covariance of the multipoles (covariance.c:477-1103) with
 * the double-Bessel integrals by 2D FFTLog (covariance.c:357-470,
 * twobessel.c:16-122, utils.c:179-258) or by direct quadrature
 * (covariance.c:305-341).
 */

/* (l1 l2 l3; 0 0 0)^2 by the closed form for even J = l1 + l2 + l3 (zero for
   odd J or when the triangle condition fails) */
static double w3j0_sq(int l1, int l2, int l3)
{
    const int J = l1 + l2 + l3;
    if (J % 2 || l3 < abs(l1 - l2) || l3 > l1 + l2)
        return 0.0;
    const int g = J / 2;
    /* log of [(J-2l1)! (J-2l2)! (J-2l3)! / (J+1)!] [g! / ((g-l1)! (g-l2)! (g-l3)!)]^2 */
    const double lr = lgamma(J - 2. * l1 + 1) + lgamma(J - 2. * l2 + 1) + lgamma(J - 2. * l3 + 1) -
                      lgamma(J + 2.) +
                      2 * (lgamma(g + 1.) - lgamma(g - l1 + 1.) - lgamma(g - l2 + 1.) -
                           lgamma(g - l3 + 1.));
    return exp(lr);
}

/* int_{-1}^{1} P_n P_m P_a P_b dmu = 2 sum_L (2L+1) (n m L;000)^2 (a b L;000)^2
   (coffe_legendre_integral, common.c:1370-1394) */
double or_legendre_integral(int n, int m, int a, int b)
{
    if ((n + m + a + b) % 2 != 0)
        return 0;
    const int lo = abs(n - m) > abs(a - b) ? abs(n - m) : abs(a - b);
    const int hi = n + m < a + b ? n + m : a + b;
    double r = 0;
    for (int L = lo; L <= hi; ++L)
        r += (2. * L + 1) * w3j0_sq(n, m, L) * w3j0_sq(a, b, L);
    return 2 * r;
}

/* g_l(eta) = exp(z ln 2 + lnGamma((l + z)/2) - lnGamma((3 + l - z)/2)),
   z = nu + i eta (utils.c:212-221) */
static void twob_gl(double l, double nu, double eta, double *gr, double *gi)
{
    double a_r, a_i, b_r, b_i;
    or_lgamma_c((l + nu) / 2., eta / 2., &a_r, &a_i);
    or_lgamma_c((3. + l - nu) / 2., -eta / 2., &b_r, &b_i);
    const double er = nu * log(2.) + a_r - b_r, ei = eta * log(2.) + a_i - b_i;
    *gr = exp(er) * cos(ei);
    *gi = exp(er) * sin(ei);
}

static double twob_window(long t, long ncut)
{
    return (double)t / ncut - 1. / (2. * M_PI) * sin(2. * t * M_PI / ncut);
}

/* 2D FFTLog (two_sph_bessel, twobessel.c:16-122; C branch) of a kernel that
   is diagonal in (k1, k2): fk1k2[i][j] = diag[i] delta_ij on the log grid k.
   out[a * N + b] = result(r1[a], r2[b]), r[i] = 1 / k[N - 1 - i]. */
int or_twobessel_diag(const double *k, const double *diag, size_t N, double l1, double l2,
                      double nu1, double nu2, double c_window_width, double *r, double *out)
{
    if (N % 2)
        return -1;
    const long hN = (long)N / 2;
    const double dlnk = log(k[1] / k[0]);
    for (size_t i = 0; i < N; ++i)
        r[i] = 1. / k[N - 1 - i];
    const double kr = k[0] * r[0];
    /* forward r2c 2D of the diagonal: out[m][n] = F[(m + n) mod N] */
    double *Fr = (double *)malloc(sizeof(double) * N), *Fi = (double *)malloc(sizeof(double) * N);
    double *Xr = (double *)malloc(sizeof(double) * N * (hN + 1));
    double *Xi = (double *)malloc(sizeof(double) * N * (hN + 1));
    if (!Fr || !Fi || !Xr || !Xi) {
        free(Fr); free(Fi); free(Xr); free(Xi);
        return -1;
    }
    for (size_t i = 0; i < N; ++i) {
        Fr[i] = diag[i] / pow(k[i], nu1) / pow(k[i], nu2);
        Fi[i] = 0;
    }
    or_fft(Fr, Fi, N, -1);
    /* windows (c_window_2d, utils.c:235-258) */
    const long nc1 = (long)(hN * c_window_width), nc2 = (long)(hN * c_window_width);
    /* per-row and per-column factors (k0 r0)^(-+ i eta) g_l */
    for (long m = 0; m < (long)N; ++m) {
        const long mm = m <= hN ? m : (long)N - m;
        const double eta_m = 2 * M_PI / dlnk / N * mm;
        double g1r, g1i;
        twob_gl(l1, nu1, eta_m, &g1r, &g1i);
        /* (kr)^(-i eta) = exp(-i eta ln kr) */
        double pr = cos(-eta_m * log(kr)), pi_ = sin(-eta_m * log(kr));
        if (m > hN) { /* conj of the m <= N/2 factor */
            pi_ = -pi_;
            g1i = -g1i;
        }
        const double R_r = pr * g1r - pi_ * g1i, R_i = pr * g1i + pi_ * g1r;
        double wr = 1.0;
        if (m <= hN && hN - m <= nc1) wr = twob_window(hN - m, nc1);
        if (m >= hN + 1 && m - hN - 1 <= nc1) wr = twob_window(m - hN - 1, nc1);
        for (long n = 0; n <= hN; ++n) {
            const double eta_n = 2 * M_PI / dlnk / N * n;
            double g2r, g2i;
            twob_gl(l2, nu2, eta_n, &g2r, &g2i);
            const double qr = cos(-eta_n * log(kr)), qi = sin(-eta_n * log(kr));
            const double C_r = qr * g2r - qi * g2i, C_i = qr * g2i + qi * g2r;
            double wc = 1.0;
            if (hN - n <= nc2) wc = twob_window(hN - n, nc2);
            const long f = (m + n) % (long)N;
            double vr = Fr[f] * wc * wr, vi = Fi[f] * wc * wr;
            /* times C * R, then conjugated */
            const double fr = C_r * R_r - C_i * R_i, fi = C_r * R_i + C_i * R_r;
            const double tr = vr * fr - vi * fi, ti = vr * fi + vi * fr;
            Xr[m * (hN + 1) + n] = tr;
            Xi[m * (hN + 1) + n] = -ti;
        }
    }
    free(Fr);
    free(Fi);
    /* c2r 2D: inverse c2c along m for every n, then c2r along n per row */
    int bad = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : bad)
#endif
    for (long n = 0; n <= hN; ++n) {
        double *cr = (double *)malloc(sizeof(double) * N), *ci = (double *)malloc(sizeof(double) * N);
        if (!cr || !ci) { free(cr); free(ci); bad |= 1; continue; }
        for (size_t m = 0; m < N; ++m) {
            cr[m] = Xr[m * (hN + 1) + n];
            ci[m] = Xi[m * (hN + 1) + n];
        }
        or_fft(cr, ci, N, +1);
        for (size_t m = 0; m < N; ++m) {
            Xr[m * (hN + 1) + n] = cr[m];
            Xi[m * (hN + 1) + n] = ci[m];
        }
        free(cr);
        free(ci);
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : bad)
#endif
    for (long a = 0; a < (long)N; ++a) {
        double *cr = (double *)malloc(sizeof(double) * N), *ci = (double *)malloc(sizeof(double) * N);
        if (!cr || !ci) { free(cr); free(ci); bad |= 1; continue; }
        /* Hermitian completion along n; c2r ignores Im of the n = 0, N/2 terms */
        for (long n = 0; n <= hN; ++n) {
            cr[n] = Xr[a * (hN + 1) + n];
            ci[n] = (n == 0 || n == hN) ? 0.0 : Xi[a * (hN + 1) + n];
        }
        for (long n = hN + 1; n < (long)N; ++n) {
            cr[n] = cr[N - n];
            ci[n] = -ci[N - n];
        }
        or_fft(cr, ci, N, +1);
        for (size_t b = 0; b < N; ++b)
            out[a * N + b] = cr[b] * M_PI / (16. * N * N * pow(r[b], nu2) * pow(r[a], nu1));
        free(cr);
        free(ci);
    }
    free(Xr);
    free(Xi);
    return bad ? -1 : 0;
}

/* Bicubic interpolation on a rectilinear grid as gsl_interp2d_bicubic builds
   it (covariance.c:445-464 via coffe_init_spline2d, common.c:579-613): partial
   derivatives zx, zy, zxy at the knots from natural cubic splines (zx along x
   per y row, zy along y per x column, zxy along y of zx), then the bicubic
   Hermite patch of each cell.  z[j * nx + i] = f(x_i, y_j). */
typedef struct {
    size_t nx, ny;
    const double *x, *y, *z;
    double *zx, *zy, *zxy;
} or_bicubic_t;

static double cspline_node_deriv(const or_spline_t *s, size_t i)
{
    /* derivative of the natural cubic spline at knot i (gsl_spline_eval_deriv) */
    if (i + 1 < s->n)
        return s->b[i];
    const size_t j = s->n - 2;
    const double h = s->x[j + 1] - s->x[j];
    return s->b[j] + 2 * s->c[j] * h + 3 * s->d[j] * h * h;
}

static int bicubic_init(or_bicubic_t *B, const double *x, const double *y, const double *z,
                        size_t nx, size_t ny)
{
    B->nx = nx; B->ny = ny; B->x = x; B->y = y; B->z = z;
    B->zx = (double *)malloc(sizeof(double) * nx * ny);
    B->zy = (double *)malloc(sizeof(double) * nx * ny);
    B->zxy = (double *)malloc(sizeof(double) * nx * ny);
    if (!B->zx || !B->zy || !B->zxy)
        return -1;
    int bad = 0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : bad)
#endif
    for (long j = 0; j < (long)ny; ++j) {
        or_spline_t s;
        if (or_spline_init(&s, x, z + j * nx, nx, OR_CSPLINE)) { bad |= 1; continue; }
        for (size_t i = 0; i < nx; ++i) B->zx[j * nx + i] = cspline_node_deriv(&s, i);
        or_spline_free(&s);
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static) reduction(| : bad)
#endif
    for (long i = 0; i < (long)nx; ++i) {
        double *col = (double *)malloc(sizeof(double) * ny), *colx = (double *)malloc(sizeof(double) * ny);
        if (!col || !colx) { free(col); free(colx); bad |= 1; continue; }
        for (size_t j = 0; j < ny; ++j) {
            col[j] = z[j * nx + i];
            colx[j] = B->zx[j * nx + i];
        }
        or_spline_t s, sx;
        if (or_spline_init(&s, y, col, ny, OR_CSPLINE) || or_spline_init(&sx, y, colx, ny, OR_CSPLINE)) {
            bad |= 1;
        } else {
            for (size_t j = 0; j < ny; ++j) {
                B->zy[j * nx + i] = cspline_node_deriv(&s, j);
                B->zxy[j * nx + i] = cspline_node_deriv(&sx, j);
            }
            or_spline_free(&s);
            or_spline_free(&sx);
        }
        free(col);
        free(colx);
    }
    return bad ? -1 : 0;
}

static void bicubic_free(or_bicubic_t *B)
{
    free(B->zx); free(B->zy); free(B->zxy);
}

static size_t grid_index(const double *x, size_t n, double v)
{
    /* x_i <= v < x_{i+1} (last interval for v == x_{n-1}) */
    size_t lo = 0, hi = n - 1;
    while (hi > lo + 1) {
        const size_t mid = (lo + hi) / 2;
        if (x[mid] > v) hi = mid; else lo = mid;
    }
    return lo;
}

static double bicubic_eval(const or_bicubic_t *B, double xv, double yv)
{
    if (!(xv >= B->x[0] && xv <= B->x[B->nx - 1] && yv >= B->y[0] && yv <= B->y[B->ny - 1]))
        return NAN;
    const size_t i = grid_index(B->x, B->nx, xv), j = grid_index(B->y, B->ny, yv);
    const double dx = B->x[i + 1] - B->x[i], dy = B->y[j + 1] - B->y[j];
    const double t = (xv - B->x[i]) / dx, u = (yv - B->y[j]) / dy;
    /* cubic Hermite basis: value at 0 / 1, slope at 0 / 1 */
    const double ht[2] = {(2 * t - 3) * t * t + 1, (3 - 2 * t) * t * t};
    const double gt[2] = {((t - 2) * t + 1) * t, (t - 1) * t * t};
    const double hu[2] = {(2 * u - 3) * u * u + 1, (3 - 2 * u) * u * u};
    const double gu[2] = {((u - 2) * u + 1) * u, (u - 1) * u * u};
    double v = 0;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) {
            const size_t q = (j + b) * B->nx + (i + a);
            v += B->z[q] * ht[a] * hu[b] + B->zx[q] * dx * gt[a] * hu[b] +
                 B->zy[q] * dy * ht[a] * gu[b] + B->zxy[q] * dx * dy * gt[a] * gu[b];
        }
    return v;
}

/* covariance_integrate_fftlog (covariance.c:357-470): the 2D FFTLog of
   diag(k^3 P(k)^power / dlnk) on N log-spaced k in [kmin, kmax), resampled by
   bicubic interpolation at the separations: out[nsep * n + m] = value at
   (sep[m], sep[n]).  P(k) through the Akima spline of (k, pk). */
int or_covariance_fftlog(const double *k, const double *pk, size_t nk, int power, int l1, int l2,
                         size_t N, const double *sep, size_t nsep, double kmin, double kmax,
                         double *out)
{
    or_spline_t P;
    if (or_spline_init(&P, k, pk, nk, OR_AKIMA))
        return -1;
    const double step = log(kmax / kmin) / N;
    double *ks = (double *)malloc(sizeof(double) * N), *dg = (double *)malloc(sizeof(double) * N);
    double *r = (double *)malloc(sizeof(double) * N), *res = (double *)malloc(sizeof(double) * N * N);
    double *zt = (double *)malloc(sizeof(double) * N * N);
    int st = -1;
    if (ks && dg && r && res && zt) {
        for (size_t i = 0; i < N; ++i) {
            ks[i] = kmin * pow(kmax / kmin, (double)i / N);
            dg[i] = pow(ks[i], 3) * pow(or_spline_eval(&P, ks[i]), power) / step;
        }
        st = or_twobessel_diag(ks, dg, N, l1, l2, 1.01, 1.01, 0.25, r, res);
        if (!st) {
            /* z(x = r1[a], y = r2[b]) at zt[b * N + a] (covariance.c:432-437) */
            for (size_t a = 0; a < N; ++a)
                for (size_t b = 0; b < N; ++b) zt[b * N + a] = res[a * N + b];
            or_bicubic_t B;
            st = bicubic_init(&B, r, r, zt, N, N);
            if (!st)
                for (size_t m = 0; m < nsep; ++m)
                    for (size_t n = 0; n < nsep; ++n)
                        out[nsep * n + m] = bicubic_eval(&B, sep[m], sep[n]);
            bicubic_free(&B);
        }
    }
    free(ks); free(dg); free(r); free(res); free(zt);
    or_spline_free(&P);
    return st;
}

/* direct double-Bessel integral (covariance_integral, covariance.c:305-341,
   no window): 2/pi int_kmin^kmax k^2 P(k)^power j_l1(k r1) j_l2(k r2) dk */
typedef struct {
    const or_spline_t *P;
    int power, l1, l2;
    double r1, r2;
} or_cov_par_t;

static double cov_integrand(double kk, void *vp)
{
    const or_cov_par_t *p = (const or_cov_par_t *)vp;
    return kk * kk * pow(or_spline_eval(p->P, kk), p->power) * or_sph_bessel(p->l1, kk * p->r1) *
           or_sph_bessel(p->l2, kk * p->r2);
}

double or_covariance_integral(const double *k, const double *pk, size_t nk, int power, double r1,
                              double r2, int l1, int l2, double kmin, double kmax, double epsrel,
                              int power_of_spline)
{
    /* the reference's integrand reads an Akima spline of the node values
       P^power (temp_spectrum_pk2, covariance.c:609-628); power_of_spline != 0
       uses the power of the spline of P instead, as the FFTLog path samples it
       (covariance.c:397-402) */
    or_spline_t P;
    double *pp = (double *)malloc(sizeof(double) * nk);
    if (!pp)
        return NAN;
    for (size_t i = 0; i < nk; ++i) pp[i] = power_of_spline ? pk[i] : pow(pk[i], power);
    const int bad = or_spline_init(&P, k, pp, nk, OR_AKIMA);
    free(pp);
    if (bad)
        return NAN;
    or_cov_par_t p = {&P, power_of_spline ? power : 1, l1, l2, r1, r2};
    double err;
    int status;
    const double v = or_qag61(cov_integrand, &p, kmin, kmax, 0, epsrel, 50000, &err, &status);
    or_spline_free(&P);
    return 2 * v / M_PI;
}

static double cov_coeff(double b1, double b2, double f, int ell)
{
    /* covariance_coefficient, covariance.c:40-57 */
    switch (ell) {
    case 0: return b1 * b2 + (b1 + b2) * f / 3 + f * f / 5.;
    case 2: return 2 * (b1 + b2) * f / 3. + 4 * f * f / 7.;
    case 4: return 8 * f * f / 35.;
    default: return 0;
    }
}

static int isign(int m) { return abs(m) % 2 == 0 ? 1 : -1; }

/* Multipole covariance (covariance.c:786-1059) for one population (all four
   covariance_pop = 1, the defaults, parser.c:945-948), no window, linear P(k):
   ipk / ipk2 hold the double-Bessel integrals I[l1][l2](r1 = sep[m],
   r2 = sep[n]) at [(i * nl + j) * nsep * nsep + nsep * n + m] for ALL (i, j)
   already multiplied by (2l1+1)(2l2+1) 2/pi^2 and (2l1+1)(2l2+1)/pi^2
   (covariance.c:752-763, transposes 773-784).  out in (z, l1, r1, l2, r2)
   order (covariance.c:1046-1059). */
int or_covariance_multipoles(const or_model_t *mdl, int contrib, size_t nz, const double *z_mean,
                             const double *deltaz, const double *fsky, const double *density1,
                             const double *density2, const double *pixelsize, size_t nl, const int *ls, size_t nsep,
                             const double *sep, const double *ipk, const double *ipk2,
                             double *out)
{
    double *V = (double *)malloc(sizeof(double) * nz);
    if (!V)
        return -1;
    for (size_t zk = 0; zk < nz; ++zk) {
        const double c1 = or_spline_eval(&mdl->chi_of_z, z_mean[zk] - deltaz[zk]);
        const double c2 = or_spline_eval(&mdl->chi_of_z, z_mean[zk] + deltaz[zk]);
        V[zk] = 4 * M_PI * fsky[zk] * (pow(c2, 3) - pow(c1, 3)) / 3.;
    }
    const int e = or_covariance_multipoles_v(mdl, contrib, nz, z_mean, V, density1, density2,
                                             pixelsize, nl, ls, nsep, sep, ipk, ipk2, out);
    free(V);
    return e;
}

/* covariance_volume_integrand (covariance.c:150-162) */
static double avg_volume_integrand(double z, void *vp)
{
    const or_model_t *m = (const or_model_t *)vp;
    const double chi = or_spline_eval(&m->chi_of_z, z);
    return 1. / or_spline_eval(&m->confH, z) / (chi * chi) / (1 + z);
}

/* Effective volume of a redshift window for the covariance of the averaged
   multipoles (covariance.c:811-840): 4 pi fsky / int_{z_min}^{z_max} dz
   / (conformal_H chi^2 (1 + z)) / (H0 h)^2, the integral by QAG at relative
   tolerance 1e-5 (integration_1d_prec). */
double or_average_covariance_volume(const or_model_t *m, double z_min, double z_max, double fsky)
{
    const double vint = or_qag61(avg_volume_integrand, (void *)m, z_min, z_max, 0.0, 1e-5,
                                 OR_QAG_LIMIT, NULL, NULL);
    return 4 * M_PI * fsky / vint / pow(OR_H0 * m->h, 2);
}

/* the assembly of covariance.c:842-1059 for bins at redshifts z[] with volumes V[] */
int or_covariance_multipoles_v(const or_model_t *mdl, int contrib, size_t nz, const double *zbin,
                               const double *Vbin, const double *density1, const double *density2,
                               const double *pixelsize, size_t nl, const int *ls, size_t nsep,
                               const double *sep, const double *ipk, const double *ipk2,
                               double *out)
{
    size_t idx = 0;
    for (size_t zk = 0; zk < nz; ++zk) {
        const double z = zbin[zk];
        const double V = Vbin[zk];
        const double b = (contrib & OR_CONTRIB_DEN) ? bias_eval(mdl, 0, z, 1.0) : 0.0;
        const double f = (contrib & OR_CONTRIB_RSD) ? or_spline_eval(&mdl->f, z) : 0.0;
        const double D1 = or_spline_eval(&mdl->D1, z);
        const double n1 = density1[zk], n2 = density2[zk];
        for (size_t i = 0; i < nl; ++i)
            for (size_t m = 0; m < nsep; ++m)
                for (size_t j = 0; j < nl; ++j)
                    for (size_t n = 0; n < nsep; ++n) {
                        const int l1 = ls[i], l2 = ls[j];
                        double cosmic = 0;
                        for (int a = 0; a <= 4; a += 2)
                            for (int bb = 0; bb <= 4; bb += 2)
                                cosmic += (cov_coeff(b, b, f, a) * cov_coeff(b, b, f, bb) +
                                           isign(bb) * cov_coeff(b, b, f, a) * cov_coeff(b, b, f, bb)) *
                                          or_legendre_integral(l1, l2, a, bb);
                        cosmic /= 4.;
                        double mixed = 0;
                        for (int a = 0; a <= 4; a += 2)
                            mixed += (cov_coeff(b, b, f, a) / n2 + cov_coeff(b, b, f, a) / n1 +
                                      cov_coeff(b, b, f, a) / n2 + cov_coeff(b, b, f, a) / n1) *
                                     or_legendre_integral(l1, l2, a, 0);
                        mixed /= 8.;
                        const double pois = (l1 == l2 && m == n)
                                                ? (2 * l1 + 1) / 4. / M_PI * (1 + isign(l2)) /
                                                      sep[n] / sep[m] / pixelsize[zk] / n1 / n2 / V
                                                : 0.0;
                        const size_t q = (i * nl + j) * nsep * nsep + nsep * n + m;
                        const double cm = isign((l2 - l1) / 2) * isign(l1 + l2) * D1 * D1 * ipk[q] * mixed / V;
                        const double cc = isign((l2 - l1) / 2) * D1 * D1 * D1 * D1 * ipk2[q] * cosmic / V;
                        out[idx++] = pois + cm + cc;
                    }
    }
    return 0;
}

/* ---------------------------------------------------------------- flat sky
 * Half-integer tables I^{n/2}_{l/2} (integrals.c:189-207, the HALF_INTEGER
 * state) and the flat-sky lensing multipoles (functions.c:4020-4253 with the
 * 2 pi^2 of signal.c:619-630, 708-734).  Half-integer tables are stored in the
 * model under the keys (OR_HALF_KEY + n, OR_HALF_KEY + l).
 */
#define OR_HALF_KEY 10000

/* FFTLog table of I^{n_num/2}_{l_num/2} on N points, times r^(n-l) when
   n >= l (integrals.c:459-523); the r = 0 and sub-Mpc entries are NaN */
int or_integral_table_half(const double *k, const double *pk, size_t nk, int n_num, int l_num,
                           size_t N, double kmin, double kmax, double *out_x, double *out_y)
{
    const size_t off = OR_N_SMALL_R + 1;
    const double n = n_num / 2., l = l_num / 2.;
    double *fx = out_x + off, *fy = out_y + off;
    if (or_twofast_1bessel(fx, fy, N, k, pk, nk, l, n, 1.0, kmin, kmin, kmax) != 0)
        return -1;
    if (n >= l)
        for (size_t i = 0; i < N; ++i)
            fy[i] = fy[i] * pow(fx[i], n - l);
    out_x[0] = 0.0;
    for (size_t i = 1; i <= OR_N_SMALL_R; ++i)
        out_x[i] = or_min_sep[i - 1];
    for (size_t i = 0; i < off; ++i)
        out_y[i] = NAN;
    return 0;
}

static double or_fact(int n)
{
    double r = 1;
    for (int i = 2; i <= n; ++i) r *= i;
    return r;
}

static double or_choose(int n, int k)
{
    return or_fact(n) / or_fact(k) / or_fact(n - k);
}

/* flat-sky density-lensing multipole (functions.c:4136-4253), even l, times
   2 pi^2 (signal.c:619-630); needs the half-integer tables
   ((l - 2k + 3)/2, (l - 2k + 1)/2), k = 0..l/2 */
double or_flatsky_density_lensing(const or_model_t *m, double z_mean, double sep, int l)
{
    if (l % 2)
        return 0.0;
    const double s1 = bias_eval(m, 2, z_mean, 0.0), s2 = bias_eval(m, 3, z_mean, 0.0);
    const double b1 = bias_eval(m, 0, z_mean, 1.0), b2 = bias_eval(m, 1, z_mean, 1.0);
    double result = 0;
    for (int k = 0; k <= l / 2; ++k) {
        const or_spline_t *tab = find_integral(m, OR_HALF_KEY + l - 2 * k + 3, OR_HALF_KEY + l - 2 * k + 1);
        if (!tab)
            return NAN;
        result += pow(-1, k) / pow(2, k) * or_choose(l, k) * or_choose(2 * l - 2 * k, l) *
                  or_fact(l / 2 - k) * or_spline_eval(tab, sep);
    }
    const double D1 = or_spline_eval(&m->D1, z_mean);
    result *= -3 * m->Omega0_m / M_PI / 8 * (2 * l + 1) * D1 * D1 * (1 + z_mean) * sep *
              ((2 - 5 * s1) * b2 + (2 - 5 * s2) * b1) * pow(2, 1 - l / 2);
    return 2 * M_PI * M_PI * result / sqrt(2 * M_PI) * pow(OR_H0 * m->h, 2);
}

typedef struct {
    const or_model_t *m;
    double z_mean, sep;
    int l;
} or_flat_par_t;

/* functions_flatsky_lensing_lensing_multipoles (functions.c:4020-4132) */
static double flat_ll_integrand(double x, void *vp)
{
    const or_flat_par_t *p = (const or_flat_par_t *)vp;
    const or_model_t *m = p->m;
    const int l = p->l;
    const double chi_mean = or_spline_eval(&m->chi_of_z, p->z_mean);
    const double lambda = chi_mean * x;
    const double s1 = bias_eval(m, 2, p->z_mean, 0.0), s2 = bias_eval(m, 3, p->z_mean, 0.0);
    const double zl = or_spline_eval(&m->z_of_chi, lambda);
    const double D1 = or_spline_eval(&m->D1, zl);
    double result = (2 * l + 1) * or_fact(l) / pow(2, l) / pow(or_fact(l / 2), 2) * 9 *
                    m->Omega0_m * m->Omega0_m * (2 - 5 * s1) * (2 - 5 * s2) * pow(chi_mean, 3) /
                    8. / M_PI * or_spline_eval(find_integral(m, 1, l), x * p->sep) * D1 * D1 *
                    (1 + zl) * (1 + zl) * pow(x * (1 - x), 2);
    if (l > 0)
        return result * x * p->sep * pow(OR_H0 * m->h, 4);
    return result * pow(OR_H0 * m->h, 4);
}

/* flat-sky lensing-lensing multipole, even l: 2 pi^2 times the QAG integral
   over x in [0, 1] (signal.c:708-734); needs the integer tables I^1_l with
   their r = 0 and sub-Mpc entries */
double or_flatsky_lensing_lensing(const or_model_t *m, double z_mean, double sep, int l,
                                  double epsrel)
{
    if (l % 2 || !find_integral(m, 1, l))
        return l % 2 ? 0.0 : NAN;
    or_flat_par_t p = {m, z_mean, sep, l};
    double err;
    int status;
    const double v = or_qag61(flat_ll_integrand, &p, 0, 1, 0, epsrel, 50000, &err, &status);
    return 2 * M_PI * M_PI * v;
}
