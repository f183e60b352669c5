/*
 * coffe_oracle.h -- CPU restatement of the COFFE correlation-function hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the tests compare the
 * GPU product (coffe_gb300) against.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it; the product never links, imports or calls it.
 *
 * Every routine restates, in FP64 and in code written for this project, the
 * algorithm of the reference file:line cited beside it (paths relative to the
 * COFFE source tree).  Third-party arithmetic the reference delegates to GSL 2.7
 * (splines, QAG) and FFTW 3.3.9 (real FFTs) is restated from the published
 * algorithms: Akima (1970) / natural cubic splines, QUADPACK's QAG with the
 * 61-point Gauss-Kronrod rule (Piessens et al. 1983), and a mixed-radix
 * Cooley-Tukey DFT with FFTW's unnormalised sign conventions.
 */
#ifndef COFFE_ORACLE_H
#define COFFE_ORACLE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ splines */
/* type: 0 = natural cubic (gsl_interp_cspline), 1 = Akima (gsl_interp_akima),
   2 = linear.  Reference: common.c:524-576 (coffe_init_spline), 704-710. */
enum { OR_CSPLINE = 0, OR_AKIMA = 1, OR_LINEAR = 2 };

typedef struct {
    size_t n;
    int type;
    double *x, *y, *b, *c, *d; /* y_i + b_i dx + c_i dx^2 + d_i dx^3 */
} or_spline_t;

int or_spline_init(or_spline_t *s, const double *x, const double *y, size_t n, int type);
double or_spline_eval(const or_spline_t *s, double x);
void or_spline_free(or_spline_t *s);
/* convenience for ctypes: build a spline and evaluate it at nq points */
int or_spline_eval_array(int type, const double *x, const double *y, size_t n,
                         const double *xq, double *yq, size_t nq);
/* per-interval coefficients (b, c, d each n-1 long) for table comparisons */
int or_spline_coeffs(int type, const double *x, const double *y, size_t n,
                     double *b, double *c, double *d);

/* --------------------------------------------------------------- quadrature */
typedef double (*or_fn)(double, void *);
/* QUADPACK QAG with GK61; common.c:1004-1040 calls gsl_integration_qag with
   epsabs = 0, epsrel = precision, limit = 50000, key GSL_INTEG_GAUSS61. */
double or_qag61(or_fn f, void *p, double a, double b, double epsabs, double epsrel,
                size_t limit, double *abserr, int *status);
/* one GK61 panel; returns the Kronrod estimate and the QUADPACK error */
double or_qk61(or_fn f, void *p, double a, double b, double *abserr,
               double *resabs, double *resasc);
/* n-point Gauss-Legendre nodes/weights on [-1, 1] (Newton on P_n) */
int or_gauss_legendre(size_t n, double *x, double *w);

/* ------------------------------------------------------------- special fns */
/* complex log-Gamma, Lanczos g=7 (twofast.c:97-144) */
void or_lgamma_c(double zr, double zi, double *rr, double *ri);
/* spherical Bessel j_l(x), l >= 0 (replaces gsl_sf_bessel_jl, integrals.c:309) */
double or_sph_bessel(int l, double x);
/* Legendre P_l (replaces gsl_sf_legendre_Pl, signal.c:109) */
double or_legendre(int l, double x);

/* --------------------------------------------------------------------- FFT */
/* in-place complex DFT of any length; sign = -1 forward, +1 backward,
   unnormalised (FFTW convention). */
int or_fft(double *re, double *im, size_t n, int sign);

/* ------------------------------------------------------------------ FFTLog */
double or_twofast_selectqnu(double l, double nu);              /* twofast.c:240-250 */
int or_twofast_1bessel(double *out_x, double *out_y, size_t N, /* twofast.c:362-483 */
                       const double *in_x, const double *in_y, size_t in_len,
                       double l, double nu, double r0, double k0, double kmin,
                       double kmax);
/* Full I_l^n table as coffe_integrals_renormalizable (integrals.c:459-573):
   out has N + 43 points: r = 0, the 42 sub-Mpc separations (QAG), then the N
   FFTLog points, times r^(n-l) when n >= l.  with_small_r = 0 leaves the
   first 43 y values at NaN (x values are still filled).
   P(k) is read through an Akima spline of (k, pk) for the direct integrals
   and a natural cubic spline for the FFTLog resampling, as the reference does. */
#define OR_N_SMALL_R 42
int or_integral_table(const double *k, const double *pk, size_t nk, int n, int l,
                      size_t N, double kmin, double kmax, int with_small_r,
                      double *out_x, double *out_y);
/* one direct integral (1/2pi^2) int k^2 P(k) j_l(kr)/(kr)^n dk, times r^(n-l)
   when n >= l (integrals.c:333-383), P(k) through the Akima spline */
double or_integral_direct(const double *k, const double *pk, size_t nk, int n, int l,
                          double r, double kmin, double kmax);
/* The fixed separations of the divergent integral (integrals.c:76-103): writes at
   most cap of them to out, returns their count. */
size_t or_divergent_separations(double *out, size_t cap);
/* The divergent I^4_0 on separations r (integrals.c:773-845): result = r^4 I^4_0(r),
   result0 = its r = 0 renormalisation integral times r^4, both / 2 pi^2. */
int or_divergent_i40(const double *k, const double *pk, size_t nk, double kmin, double kmax,
                     const double *r, size_t nr, double *result, double *result0, int nthreads);
/* The renormalisation grid (integrals.c:424-444, 848-903):
   out[b * n1 + a] = (1/2pi^2) int P j0(k chi1[a]) j0(k chi2[b]) / k^2 dk. */
int or_renormalization_grid(const double *k, const double *pk, size_t nk, double kmin,
                            double kmax, const double *chi1, size_t n1, const double *chi2,
                            size_t n2, double *out, int nthreads);

/* -------------------------------------------------------------- background */
typedef struct {
    double Omega0_cdm, Omega0_baryon, Omega0_gamma, Omega0_de, h;
} or_cosmo_t;
/* Node values at z_i = 15 i / (bins - 1) (background.c:415-537, flat LCDM,
   w0 = -1, wa = 0).  Units: H, conformal H in 1/Mpc; chi in Mpc.  D1 is
   normalised to 1 at z = 0.  Any output pointer may be NULL. */
int or_background_nodes(const or_cosmo_t *c, size_t bins, double *z, double *a,
                        double *Hz, double *confH, double *confHp, double *D1,
                        double *f, double *chi, double *D1_unnormalised);

/* -------------------------------------------------------------- multipoles */
typedef struct or_model or_model_t;
enum { OR_CONTRIB_DEN = 1, OR_CONTRIB_RSD = 2, OR_CONTRIB_LEN = 4 };

or_model_t *or_model_new(void);
void or_model_free(or_model_t *m);
/* background splines (Akima, common.c:524) from node arrays on one z grid */
int or_model_set_background(or_model_t *m, const double *z, const double *chi,
                            const double *D1, const double *f, const double *a,
                            const double *confH, size_t bins, double h,
                            double Omega0_m);
/* which: 0 = galaxy_bias1, 1 = galaxy_bias2, 2 = magnification_bias1,
   3 = magnification_bias2; Akima over (z, value) */
int or_model_set_bias(or_model_t *m, int which, const double *z, const double *v,
                      size_t n);
/* an I_l^n table (x, y of length len) read through an Akima spline */
int or_model_set_integral(or_model_t *m, int n, int l, const double *x,
                          const double *y, size_t len);
/* den+RSD nonintegrated correlation function xi(z_mean, mu, r)
   (functions.c:89-1484, den 129-229, rsd 230-362, den-rsd 670-771) */
double or_xi_nonintegrated(const or_model_t *m, int contrib, double z_mean,
                           double mu, double sep);
/* one multipole by adaptive GK61 QAG (signal.c:83-111, 521-542) */
double or_multipole_nonintegrated(const or_model_t *m, int contrib, double z_mean,
                                  double sep, int l, double epsrel);
/* batch over count points, OpenMP-parallel like multipoles.c:88-99 */
int or_multipoles_batch(const or_model_t *m, int contrib, const double *z_mean,
                        const double *sep, const int *l, size_t count,
                        double epsrel, double *out, int nthreads);
/* same as or_multipole_nonintegrated but with a fixed n-point Gauss-Legendre
   rule in mu instead of QAG (comparator for fixed-rule paths) */
double or_multipole_nonintegrated_gl(const or_model_t *m, int contrib, double z_mean,
                                     double sep, int l, size_t n_mu);

/* ----------------------------------------------------------------- lensing */
/* den-len + rsd-len single-integrated xi at (mu, x) (functions.c:1486-2483,
   full sky, linear P(k), no renormalisation) */
double or_xi_single_integrated(const or_model_t *m, int contrib, double z_mean, double mu,
                               double sep, double x);
/* len-len double-integrated xi at (mu, x1, x2) (functions.c:3460-3836) */
double or_xi_double_integrated(const or_model_t *m, int contrib, double z_mean, double mu,
                               double sep, double x1, double x2);
/* lensing multipoles (single + double integrated terms selected by contrib)
   with product Gauss-Legendre rules: n_mu x n_x (single), n_mu x n_x x n_x
   (double); out[j] for l = ls[j] */
int or_multipoles_lensing_gl(const or_model_t *m, int contrib, double z_mean, double sep,
                             int n_l, const int *ls, size_t n_mu, size_t n_x, double *out);
/* redshift-averaged multipoles (average_multipoles.c:69-156) */
double or_average_multipole(const or_model_t *m, int contrib, double z_min, double z_max,
                            double sep, int l, size_t n_z, size_t n_mu, size_t n_x);
int or_average_multipoles_batch(const or_model_t *m, int contrib, const double *z_min,
                                const double *z_max, const double *sep, const int *l,
                                size_t count, size_t n_z, size_t n_mu, size_t n_x, double *out,
                                int nthreads);
/* correlation function (corrfunc.c:55-141): nonintegrated + lensing at fixed mu */
double or_corrfunc_gl(const or_model_t *m, int contrib, double z_mean, double mu, double sep,
                      size_t n_x);
int or_corrfunc_batch(const or_model_t *m, int contrib, const double *z_mean, const double *mu,
                      const double *sep, size_t count, size_t n_x, double *out, int nthreads);
int or_multipoles_lensing_batch(const or_model_t *m, int contrib, const double *z_mean,
                                const double *sep, size_t count, int n_l, const int *ls,
                                size_t n_mu, size_t n_x, double *out, int nthreads);

/* -------------------------------------------------------------- covariance */
/* int P_n P_m P_a P_b dmu over [-1, 1] (common.c:1370-1394) */
double or_legendre_integral(int n, int m, int a, int b);
/* 2D FFTLog (twobessel.c:16-122) of a kernel diagonal in (k1, k2);
   out[a * N + b] at (r[a], r[b]), r[i] = 1 / k[N - 1 - i] */
int or_twobessel_diag(const double *k, const double *diag, size_t N, double l1, double l2,
                      double nu1, double nu2, double c_window_width, double *r, double *out);
/* covariance_integrate_fftlog (covariance.c:357-470); out[nsep * n + m] */
int or_covariance_fftlog(const double *k, const double *pk, size_t nk, int power, int l1, int l2,
                         size_t N, const double *sep, size_t nsep, double kmin, double kmax,
                         double *out);
/* covariance_integral without window (covariance.c:305-341) */
double or_covariance_integral(const double *k, const double *pk, size_t nk, int power, double r1,
                              double r2, int l1, int l2, double kmin, double kmax, double epsrel,
                              int power_of_spline);
/* multipole covariance assembly (covariance.c:786-1059), one population */
/* the assembly for bins at redshifts zbin[] with volumes Vbin[] */
int or_covariance_multipoles_v(const or_model_t *mdl, int contrib, size_t nz, const double *zbin,
                               const double *Vbin, const double *density1, const double *density2,
                               const double *pixelsize, size_t nl, const int *ls, size_t nsep,
                               const double *sep, const double *ipk, const double *ipk2,
                               double *out);
/* effective volume of a redshift window, covariance of the averaged multipoles */
double or_average_covariance_volume(const or_model_t *m, double z_min, double z_max, double fsky);
int or_covariance_multipoles(const or_model_t *mdl, int contrib, size_t nz, const double *z_mean,
                             const double *deltaz, const double *fsky, const double *density1,
                             const double *density2, const double *pixelsize, size_t nl, const int *ls, size_t nsep,
                             const double *sep, const double *ipk, const double *ipk2,
                             double *out);

/* ---------------------------------------------------------------- flat sky */
/* half-integer table I^{n_num/2}_{l_num/2} (FFT part; small-r entries NaN);
   stored in a model with or_model_set_integral(m, 10000 + n_num, 10000 + l_num, ...) */
int or_integral_table_half(const double *k, const double *pk, size_t nk, int n_num, int l_num,
                           size_t N, double kmin, double kmax, double *out_x, double *out_y);
/* flat-sky density-lensing multipole (functions.c:4136-4253) x 2 pi^2 */
double or_flatsky_density_lensing(const or_model_t *m, double z_mean, double sep, int l);
/* flat-sky lensing-lensing multipole (functions.c:4020-4132) by QAG x 2 pi^2 */
double or_flatsky_lensing_lensing(const or_model_t *m, double z_mean, double sep, int l,
                                  double epsrel);

/* number of QAG subdivisions taken by the last or_multipole_nonintegrated call
   in this thread (diagnostic) */
int or_last_qag_intervals(void);

#ifdef __cplusplus
}
#endif
#endif
