/*
 * coffe_gpu.h -- C ABI of the GB300 (sm_103a) implementation of COFFE's
 * correlation-function hot path.
 *
 * Plain C types only (pointers, sizes, doubles, ints): no CUDA, C++ or torch
 * types cross this boundary, so the reference's C drivers (integrals.c,
 * multipoles.c, covariance.c), its Cython wrapper (python/coffe/coffe.pxd) or
 * any ctypes/cffi caller can bind it directly.
 *
 * Conventions shared by every entry point:
 *  - Return value: COFFE_GPU_OK (0) or a negative coffe_gpu_status.  Nothing
 *    here calls exit(); the reference's fatal exits (e.g. twofast.c:82-88,
 *    functions.c:1470-1483) become error returns.
 *  - Units follow the reference internals: k in 1/Mpc, P(k) in Mpc^3,
 *    separations and comoving distances in Mpc.
 *  - A context owns the device buffers and one CUDA stream; calls on one
 *    context are stream-ordered and must not be made from two host threads at
 *    once.  Separate contexts are independent.
 *  - Array arguments are host pointers unless a *_device flag says otherwise.
 */
#ifndef COFFE_GPU_H
#define COFFE_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct coffe_gpu_ctx coffe_gpu_ctx_t;

enum coffe_gpu_status {
    COFFE_GPU_OK = 0,
    COFFE_GPU_EINVAL = -1,     /* bad argument (size, range, NULL pointer) */
    COFFE_GPU_ECUDA = -2,      /* a CUDA runtime call failed */
    COFFE_GPU_ENOMEM = -3,     /* device allocation failed */
    COFFE_GPU_ENONFINITE = -4, /* a kernel produced NaN/Inf (reference would exit) */
    COFFE_GPU_ESTATE = -5,     /* a prerequisite (background, integrals) is missing */
    COFFE_GPU_ELIMIT = -6      /* adaptive quadrature ran out of subintervals */
};

/* Precision of a computation. */
enum coffe_gpu_precision {
    COFFE_GPU_FP64 = 0,        /* plain FP64 everywhere: the parity path */
    COFFE_GPU_MIXED = 1,       /* FP32 FFT/spline/integrand arithmetic with compensated
                                  sums; FP64 Gamma-ratio coefficients and background */
    COFFE_GPU_FP64_FASTALG = 2 /* coffe_gpu_multipoles only, on FP64 tables: FP64
                                  arithmetic through the mixed path's algorithm, the
                                  precision-only baseline of COFFE_GPU_MIXED (~1e-8
                                  from the parity path).  Den/RSD terms with unit
                                  biases and even multipoles: per-request background
                                  polynomials, regrouped integrand; lensing terms:
                                  D1/a polynomials along the lines of sight, the
                                  plane integrand over five combined table records.
                                  Other den/RSD cases and other calls take the FP64
                                  path. */
};

/* Contributions to the 2-point function (the den, rsd, len flags of
   coffe_parameters_t.correlation_contrib, common.h). */
enum coffe_gpu_contrib {
    COFFE_GPU_DEN = 1,
    COFFE_GPU_RSD = 2,
    COFFE_GPU_LEN = 4
};

/* ----------------------------------------------------------------- context */

/* Creates a context on CUDA device `device`.  No reference counterpart: the
   reference keeps its state in coffe_parameters_t / coffe_background_t. */
int coffe_gpu_ctx_create(int device, coffe_gpu_ctx_t **ctx);
int coffe_gpu_ctx_destroy(coffe_gpu_ctx_t *ctx);
/* Human-readable text of a status code (static storage). */
const char *coffe_gpu_strerror(int status);
/* Text of the last error recorded on this context (static to the context). */
const char *coffe_gpu_last_error(const coffe_gpu_ctx_t *ctx);
/* Blocks until all work queued on the context's stream has finished. */
int coffe_gpu_synchronize(coffe_gpu_ctx_t *ctx);
/* Makes the context enqueue on an external cudaStream_t (passed as void*);
   NULL restores the context's own stream. */
int coffe_gpu_set_stream(coffe_gpu_ctx_t *ctx, void *stream);

/* -------------------------------------------------------------- background */

/* Flat LCDM cosmology (w0 = -1, wa = 0), the fields of coffe_parameters_t that
   coffe_background_init reads (background.c:301-537). */
typedef struct {
    double Omega0_cdm;
    double Omega0_baryon;
    double Omega0_gamma;
    double Omega0_de;
    double h;
    int bins; /* background_bins; nodes at z_i = 15 i / (bins - 1) */
} coffe_gpu_cosmology_t;

/* Replaces coffe_background_init (background.c:301-696) for flat LCDM: the
   node values of chi(z) (GK61 QAG of 1/E, FP64), D1 and f (growth ODE, FP64)
   and a, H, conformal H, its derivative are computed on the device and splined
   (Akima, as interp_method's default, parser.c:807). */
int coffe_gpu_background_init(coffe_gpu_ctx_t *ctx, const coffe_gpu_cosmology_t *c);

/* Alternative to coffe_gpu_background_init for callers that already own a
   background (e.g. a coffe_background_t built by the reference): node arrays
   on one strictly increasing z grid; chi in Mpc, conformal H in 1/Mpc.
   `Omega0_m` and `h` are the cosmology's (lensing prefactors). */
int coffe_gpu_background_set(coffe_gpu_ctx_t *ctx, const double *z, const double *chi,
                             const double *D1, const double *f, const double *a,
                             const double *conformal_Hz, size_t bins, double Omega0_m,
                             double h);

/* Copies the background nodes to host arrays of length `bins` (any may be
   NULL).  Hz and conformal_Hz_prime are only available after _init. */
int coffe_gpu_background_get(coffe_gpu_ctx_t *ctx, double *z, double *chi, double *D1,
                             double *f, double *a, double *Hz, double *conformal_Hz,
                             double *conformal_Hz_prime);

/* Bias of a population as an Akima spline of (z, value) (galaxy_bias1/2,
   magnification_bias1/2 of coffe_parameters_t; parser.c:36-51 sets constant
   defaults b = 1, s = 0, which is also what an unset bias means here).
   which: 0 = galaxy_bias1, 1 = galaxy_bias2, 2 = magnification_bias1,
   3 = magnification_bias2.  n >= 5 (Akima's minimum). */
int coffe_gpu_set_bias(coffe_gpu_ctx_t *ctx, int which, const double *z,
                       const double *value, size_t n);

/* --------------------------------------------------------------- integrals */

/* Number of points of one I_l^n table for an FFT size N: r = 0, the 42
   sub-Mpc separations of integrals.c:111-126, then the N FFTLog points. */
size_t coffe_gpu_integral_table_len(size_t N);

/* Replaces coffe_integrals_init (integrals.c:580-770) for a batch of power
   spectra.  For each spectrum s (P(k) sampled at the shared grid k[0..nk-1],
   pk[s*nk + i]) and each term t (integer n[t], l[t]) builds the table of
   I_l^n(r) = 1/(2 pi^2) int dk k^2 P(k) j_l(kr)/(kr)^n (times r^(n-l) when
   n >= l) with the FFTLog of twofast_1bessel (twofast.c:362-483) on N points
   (N a power of two, 64 <= N <= 16384), kmin = k[0], kmax = k[nk-1]
   (set_power_spectrum_linear, coffe.pyx:2929-2996).
   flags: bit 0 (COFFE_GPU_SMALL_R) also fills the r = 0 value and the 42
   sub-Mpc points by GK61 QAG (integrals.c:524-562); without it those 43
   entries are NaN and tables serve lookups at r >= the third FFT node
   (1.01 Mpc at the default grids).
   precision: COFFE_GPU_FP64 or COFFE_GPU_MIXED (FP64 Gamma-ratio coefficients;
   the forward transform in double-float on the FP32 pipes, the inverse
   transforms in FP32, tables stored as float: ~1e-6 of a table's scale, 1e-4
   relative above 1e-3 of it).  Tables stay on the device for
   coffe_gpu_multipoles. */
#define COFFE_GPU_SMALL_R 1
/* flags bit 1: `pk` is a device pointer (n_spectra * nk doubles). */
#define COFFE_GPU_PK_DEVICE 2
/* flags bit 2: enqueue only -- no host synchronisation; device-side errors are
   reported by the next call that checks them (coffe_gpu_synchronize, or a
   host-array coffe_gpu_multipoles).  The grid arguments (k, n, l, N) must be
   those of the previous call so that no per-grid table is rebuilt (otherwise
   the call synchronises once to build them).  With host P(k) the call returns
   once P(k) has been copied (the array may then be reused); the table kernels
   may still be running, and a following host-array coffe_gpu_multipoles
   uploads its requests meanwhile. */
#define COFFE_GPU_ASYNC 4
/* flags bit 3, COFFE_GPU_MIXED only: the inverse transforms in double-float as
   well (tables to ~1e-7 of their scale, the float storage; about twice the
   time of the table stage). */
#define COFFE_GPU_TABLES_DF 8
int coffe_gpu_integrals_init(coffe_gpu_ctx_t *ctx, const double *k, const double *pk,
                             int n_spectra, size_t nk, const int *n, const int *l,
                             int n_terms, size_t N, int precision, unsigned flags);

/* coffe_gpu_integrals_init with half-integer terms (the HALF_INTEGER state of
   coffe_integral_t, integrals.c:189-207): where half[t] = 1, n[t] and l[t] are
   the numerators of n/2 and l/2 (e.g. (3, 1) is I^{3/2}_{1/2}, as the flat-sky
   density-lensing multipoles read them, functions.c:4209-4228).  Their r = 0
   and sub-Mpc entries are not computed (NaN) even with COFFE_GPU_SMALL_R; the
   FFTLog part serves r >= the third FFT node.  half may be NULL (all integer). */
int coffe_gpu_integrals_init_ex(coffe_gpu_ctx_t *ctx, const double *k, const double *pk,
                                int n_spectra, size_t nk, const int *n, const int *l,
                                const int *half, int n_terms, size_t N, int precision,
                                unsigned flags);

/* Copies table (spectrum, term) out: x and y of coffe_gpu_integral_table_len(N)
   points (the arrays coffe_integrals_init hands to coffe_init_spline,
   integrals.c:652-658). */
int coffe_gpu_integral_get(coffe_gpu_ctx_t *ctx, int spectrum, int term, double *x,
                           double *y);

/* Evaluates table (spectrum, term) at nq separations through the same Akima
   spline the reference builds (coffe_interp_spline, common.c:704-710; the
   lookup Coffe.integral does, coffe.pyx:1657-1713). */
int coffe_gpu_integral_eval(coffe_gpu_ctx_t *ctx, int spectrum, int term, const double *r,
                            size_t nq, double *out);

/* -------------------------------------------------------------- multipoles */

/* Replaces coffe_multipoles_init (multipoles.c:48-136) for many spectra,
   mean redshifts and uneven separation lists in one launch.
   Request q (0 <= q < n_req) uses spectrum req_spectrum[q] of the last
   coffe_gpu_integrals_init, mean redshift req_z_mean[q] and the separations
   sep[req_offset[q] .. req_offset[q+1]-1] (req_offset has n_req+1 entries,
   req_offset[0] = 0).  For every separation and every multipole l[0..n_l-1]
   the output is
     out[(req_offset[q] + j) * n_l + i] = (2l+1) int_0^1 dx xi(mu=2x-1) P_l(mu)
   of the nonintegrated den/rsd terms selected by `contrib` (signal.c:83-111,
   521-542; functions.c:89-771), by adaptive GK61 QAG with relative tolerance
   `epsrel` (integration_1d_prec, default 1e-5, parser.c:769).
   The integrals (0,0), (0,2) and (0,4) must be among the terms.
   With COFFE_GPU_LEN in `contrib` the full-sky lensing terms are added, as
   coffe_multipoles_init adds the single- and double-integrated parts
   (multipoles.c:100-130): den/rsd x lensing if den or rsd is selected
   (functions.c:1486-2483) and lensing-lensing (functions.c:3460-3836), by the
   Gauss-Legendre rule of coffe_gpu_set_lensing_rule.  They also need the
   integrals (1,1), (1,3), (2,0) and tables built with COFFE_GPU_SMALL_R.
   precision: COFFE_GPU_FP64 follows the reference in FP64; COFFE_GPU_MIXED
   evaluates the integrand in FP32 with compensated FP32 sums.
   All arrays are host pointers unless arrays_on_device != 0, in which case
   every array (including out) is a device pointer.  With host arrays and
   without lensing, an `out` in page-locked host memory mapped into the
   device's address space (cudaHostAlloc / cudaHostRegister) is written by the
   kernels directly, with no device copy and download.  With host arrays a
   non-positive separation returns COFFE_GPU_EINVAL after the work has run
   (the check runs on the device copy, in stream order with the work), so
   `out` is then unspecified. */
int coffe_gpu_multipoles(coffe_gpu_ctx_t *ctx, int contrib, int precision, double epsrel,
                         int n_req, const int *req_spectrum, const double *req_z_mean,
                         const int64_t *req_offset, const double *sep, int n_l,
                         const int *l, double *out, int arrays_on_device);

/* Contribution bit: only the cross-correlations of the selected terms
   (only_cross_correlations, functions.c:129-362, 3516-3519): den-den, rsd-rsd
   and lensing-lensing are dropped, den-rsd and the den/rsd-lensing terms kept. */
#define COFFE_GPU_ONLY_CROSS 8

/* Flat-sky forms of the lensing terms, as the flatsky_local_nonlocal and
   flatsky_nonlocal flags select them in coffe_integrate (signal.c:607-671,
   704-754): local_nonlocal != 0 replaces the single-integrated den/rsd-lensing
   terms by the flat-sky density-lensing multipoles (closed sums over the
   half-integer tables ((l-2k+3)/2, (l-2k+1)/2), functions.c:4136-4253; RSD-
   lensing vanishes in that limit); nonlocal != 0 replaces lensing-lensing by
   its flat-sky multipoles (even l; a QAG integral over the line of sight of the
   integer tables (1, l), functions.c:4020-4132).  Default: both off. */
int coffe_gpu_set_flatsky(coffe_gpu_ctx_t *ctx, int local_nonlocal, int nonlocal);

/* Quadrature rule of the lensing terms (contrib & COFFE_GPU_LEN), which
   replaces the reference's Cuhre cubature of the unit cube (common.c:1074-1110,
   integration_bins evaluations at most): n_mu Gauss-Legendre nodes in
   v (mu = 2v - 1) and n_x nodes per x line, split into two panels of n_x / 2 at
   the line's integrand peak (n_x even).  The single-integrated den/rsd-lensing
   terms (functions.c:1486-2483) use n_mu x n_x nodes, lensing-lensing
   (functions.c:3460-3836) n_mu x n_x x n_x.  When both tracers share their
   magnification bias (and, with density-lensing, their galaxy bias) and n_mu
   is even, the terms are even in mu (mu -> -mu exchanges the tracers): each
   even multipole sums the n_mu / 2 nodes with mu > 0, each counted twice, and
   only those nodes are evaluated unless an odd multipole (which sums every
   node) is requested too.  Defaults 128 and 256; 2 <= n_mu, n_x <= 4096. */
int coffe_gpu_set_lensing_rule(coffe_gpu_ctx_t *ctx, int n_mu, int n_x);

/* Stream-ordered variant of coffe_gpu_multipoles for device-resident
   requests: every array except `l` (host, n_l entries) is a device pointer,
   n_sep = req_offset[n_req] is passed by the caller, and nothing synchronises
   the host; device-side errors surface at the next coffe_gpu_synchronize.
   The host-side argument checks of coffe_gpu_multipoles are the caller's. */
int coffe_gpu_multipoles_async(coffe_gpu_ctx_t *ctx, int contrib, int precision,
                               double epsrel, int n_req, int64_t n_sep,
                               const int *req_spectrum, const double *req_z_mean,
                               const int64_t *req_offset, const double *sep, int n_l,
                               const int *l, double *out);

/* No counterpart in the reference (its multipoles allocate freely on the host).
   Same computation, arguments and results as coffe_gpu_multipoles_async, for
   callers that must not have the library allocate device memory during the call:
   a process whose device memory is all handed to a pool at start-up (PyTorch's
   caching allocator, a service that reserves its HBM up front) could see a
   growing scratch buffer fail halfway through a run, and cudaMalloc/cudaFree
   synchronise the whole device, stalling every other stream of a process that
   shares the GPU.  The other multipole entry points grow their scratch (retry
   list, node table) on demand; this one takes it from one fixed array in the
   library's own device memory (8 MiB + 20 KiB) and never calls cudaMalloc,
   cudaFree or any other allocating routine.
   - Limit: n_sep * n_l <= COFFE_GPU_NOALLOC_MAX_OUTPUTS per call; larger calls
     return COFFE_GPU_EINVAL with the reason in coffe_gpu_last_error (split the
     requests into several calls).
   - Set-up: coffe_gpu_ctx_create loads, on its device, the module that holds
     the array (which places the array in device memory) and every kernel this
     entry point launches, so once a context exists a call allocates nothing;
     each call looks the array's address up again (cudaGetSymbolAddress, with
     the context's device current), so no address outlives its context.
   - Concurrency: every call on one device uses the same array, so two calls on
     the same device whose work can overlap (different streams, contexts or host
     threads) race and corrupt each other's results; serialise them, e.g. on one
     stream.
   - Arrays as for coffe_gpu_multipoles_async (device pointers, `l` on the host);
     device-side errors surface at the next coffe_gpu_synchronize, and
     coffe_gpu_multipoles_retries does not count these calls. */
#define COFFE_GPU_NOALLOC_MAX_OUTPUTS 1048576
int coffe_gpu_multipoles_noalloc(coffe_gpu_ctx_t *ctx, int contrib, int precision,
                                 double epsrel, int n_req, int64_t n_sep,
                                 const int *req_spectrum, const double *req_z_mean,
                                 const int64_t *req_offset, const double *sep, int n_l,
                                 const int *l, double *out);

/* coffe_average_multipoles_init (average_multipoles.c:69-156) batched: window q
   (spectrum win_spectrum[q], redshifts z_min[q] < z_max[q]) with separations
   sep[win_offset[q] .. win_offset[q+1]-1]; for each separation r and multipole
   l[i],
     out[(win_offset[q] + j) * n_l + i] = (2l+1) int_0^1 dv0 int_0^1 dv1
         xi(z(v0), mu = 2 v1 - 1, r) P_l(mu) H0 h / (conformal_H(z) (1 + z)),
   z(v0) = z1 + (z2 - z1) v0, z1 = z(chi(z_min) + r/2), z2 = z(chi(z_max) - r/2)
   (signal.c:241-310 and the AVERAGE_MULTIPOLES branches 543-551, 672-680,
   755-763), with the contributions of `contrib` as coffe_gpu_multipoles.  The
   reference integrates the cube with Cuhre; here n_z (<= 256) Gauss-Legendre
   nodes in v0 and, per node, the multipole at z_mean = z(v0) as
   coffe_gpu_multipoles computes it (adaptive GK61 in mu, epsrel; the lensing
   rules of coffe_gpu_set_lensing_rule).  `l` is a host array; the others are
   host pointers unless arrays_on_device != 0. */
int coffe_gpu_average_multipoles(coffe_gpu_ctx_t *ctx, int contrib, int precision,
                                 double epsrel, int n_win, const int *win_spectrum,
                                 const double *z_min, const double *z_max,
                                 const int64_t *win_offset, const double *sep, int n_l,
                                 const int *l, int n_z, double *out, int arrays_on_device);

/* coffe_corrfunc_init (corrfunc.c:55-141) batched like coffe_gpu_multipoles:
   for request q, its separation j and mu[m] (n_mu <= 1024 values in [-1, 1]),
     out[(req_offset[q] + j) * n_mu + m] = xi(z_mean_q, mu_m, sep_j),
   the nonintegrated den/rsd terms at mu (functions.c:89-771; signal.c:511-518)
   plus, with COFFE_GPU_LEN, the single-integrated den/rsd x lensing line
   integral and the double-integrated lensing-lensing plane at mu
   (signal.c:584-605, 695-702: full-sky forms, the CORRFUNC branches have no
   flat-sky ones), by the Gauss-Legendre line rules of
   coffe_gpu_set_lensing_rule (n_x; the reference uses QAG and Cuhre).
   COFFE_GPU_ONLY_CROSS drops the auto-correlations as in coffe_gpu_multipoles.
   `mu` is a host array; the other arrays are host pointers unless
   arrays_on_device != 0 (then all of them, out included, are device
   pointers). */
int coffe_gpu_corrfunc(coffe_gpu_ctx_t *ctx, int contrib, int precision, int n_req,
                       const int *req_spectrum, const double *req_z_mean,
                       const int64_t *req_offset, const double *sep, int n_mu, const double *mu,
                       double *out, int arrays_on_device);

/* Number of (separation, multipole) outputs of the last multipoles call on
   this context whose first GK61 panel missed the tolerance and went through
   the adaptive bisection (after coffe_gpu_multipoles_scaled: whose first
   panel the test rejects; synchronises the context's stream); -1 if none ran.
   No counterpart in the reference (its QAG keeps this count internal). */
long long coffe_gpu_multipoles_retries(coffe_gpu_ctx_t *ctx);

/* ------------------------------------------------------------------ tuning */

/* No counterpart in the reference (FFTW plans its own transforms; the rest is
   plain C): launch shapes of the GPU kernels.  A configuration is used by the
   table stage of coffe_gpu_integrals_init (the per-spectrum spline pass and
   the FFTLog transforms) and by the mixed-precision multipole kernel for unit
   biases.  Every choice gives the same results except fft_radix, which changes
   the rounding of the double-float transforms (by ~1e-14 relative). */
typedef struct {
    int fft_threads;  /* threads per block of the FFTLog inverse transforms: 128, 256, 512, 1024 */
    int fft_radix;    /* 2 or 4: stages of the mixed-precision (double-float) transforms */
    int fft_swizzle;  /* 0 or 1: XOR-swizzled shared-memory layout of those transforms */
    int spline_group; /* 2, 4 or 8 spectra per block of the mixed-precision spline pass */
    int lane_threads; /* 64, 128 or 256 threads per block of the mixed multipole kernel */
    int lane_unroll;  /* 1 or 2 quadrature nodes per step of that kernel's node loop */
    int fft_threads_fwd; /* threads per block of the forward transforms: 128 .. 1024 */
    int lane_pack;    /* 1 or 2 separations per thread of that kernel (2: both evaluated
                         at once with packed FP32 pair instructions) */
    int fft_fused;    /* 1: the mixed table stage as one kernel per (spectrum, q), all in
                         shared memory (where it fits: FFT size <= 8192, the k grid no
                         shorter than N/2 + 1 and no longer than 8192); 0: three kernels */
    int lane_poly;    /* 1: that kernel forms each separation's integrand as a polynomial
                         in mu^2 once and takes the first-panel sums as its moments; 0:
                         the integrand evaluated at every node (same results to float
                         rounding) */
} coffe_gpu_tuning_t;

/* ---- the divergent integral I^4_0 and its renormalisation (integrals.c:773-914),
   which the reference builds when par->divergent is set (for the d2 and g1-g5
   terms).  P(k): Akima spline of the host arrays (k, pk) (nk >= 5, k > 0
   strictly increasing, P finite), integrated over [kmin, kmax] (inside the k
   range; the reference's defaults are 1e-5 and 300 h/Mpc), GK61 QAG at relative
   1e-5 per value, one warp per value on the device.  Units: k in 1/Mpc, P in
   Mpc^3, separations in Mpc. */

/* The fixed separations (Mpc) on which coffe_integrals_init splines I^4_0
   (integrals.c:76-103): writes min(cap, count) of them to out (out may be NULL)
   and returns their count (297). */
size_t coffe_gpu_divergent_separations(double *out, size_t cap);

/* At each separation sep[i] > 0 (integrals.c:797-826):
     result[i]  = r^4 I^4_0(r) = (1/2 pi^2) int k^2 P(k) j0(kr) / (kr)^4 dk r^4,
     result0[i] = (1/2 pi^2) r^4 int P(k) (1 - j0(kr)^2) / k^2 dk
   (the reference applies the r^(n-l) = r^4 factor of integrals_integrate_function
   to both; it then splines result0 with its first knot set to r = 0, value 0).
   Host arrays. */
int coffe_gpu_divergent_integral(coffe_gpu_ctx_t *ctx, const double *k, const double *pk,
                                 size_t nk, double kmin, double kmax, const double *sep,
                                 size_t n_sep, double *result, double *result0);

/* The renormalisation term on a grid (integrals.c:424-444, 848-903):
     out[b * n1 + a] = (1/2 pi^2) int P(k) j0(k chi1[a]) j0(k chi2[b]) / k^2 dk
   for chi >= 0 (the reference's grid is chi_j = j chi_max / 200, j = 0..200, in
   both directions, chi_max = chi(max z_mean + deltaz)).  Host arrays. */
int coffe_gpu_renormalization_grid(coffe_gpu_ctx_t *ctx, const double *k, const double *pk,
                                   size_t nk, double kmin, double kmax, const double *chi1,
                                   size_t n1, const double *chi2, size_t n2, double *out);

/* enable != 0 switches on benchmark mode: the first table build and the first
   mixed multipole call of each shape (FFT size, spectra, terms and precision;
   number of multipoles, contributions and batch size to the next power of
   two) time every candidate configuration on the call's own inputs, keep the
   fastest for that shape and finish with it; later calls of the shape reuse
   it.  Calls made while the stream is being captured never time: they use the
   shape's chosen configuration, else the default. */
int coffe_gpu_set_autotune(coffe_gpu_ctx_t *ctx, int enable);
/* the configuration the most recent table build and mixed multipole call used */
int coffe_gpu_get_tuning(const coffe_gpu_ctx_t *ctx, coffe_gpu_tuning_t *out);
/* sets the default configuration (validated) and forgets the chosen ones */
int coffe_gpu_set_tuning(coffe_gpu_ctx_t *ctx, const coffe_gpu_tuning_t *t);

/* ------------------------------------------------------------- derivatives */

/* No counterpart in the reference (which has no derivatives): the den/rsd
   multipoles as a differentiable function of the spectra and of a galaxy-bias
   and a growth-rate scale per request (b -> bias_scale[q] b, f ->
   growth_scale[q] f; NULL means 1), evaluated on the first GK61 panel of the
   multipole quadrature -- the value coffe_gpu_multipoles returns wherever that
   panel meets the tolerance, which on the benchmark batches is all but ~1 in
   10^6 outputs.  Tables from the last coffe_gpu_integrals_init (FP64, with the
   integrals (0,0), (0,2), (0,4)); separations >= the third FFTLog node above
   1 Mpc (the Akima stencil must stay on the FFTLog part of the tables).
   Every array is a device pointer except `l` (host, n_l entries); out as
   coffe_gpu_multipoles: out[(req_offset[q] + j) * n_l + i].  The call applies
   QUADPACK's acceptance test to each first panel (relative tolerance 1e-5,
   the reference's default integration_1d_prec) and counts the outputs it
   rejects -- there the adaptive result differs from this value -- in the
   counter coffe_gpu_multipoles_retries reads.
   contrib may add COFFE_GPU_LEN: the full-sky lensing terms on the
   Gauss-Legendre rule of coffe_gpu_set_lensing_rule, as coffe_gpu_multipoles
   computes them in FP64 (same mu symmetry and weights; the den-lensing part
   scaled by bias_scale, the RSD-lensing part by growth_scale); the tables
   then need (1,1), (1,3), (2,0) too and COFFE_GPU_SMALL_R, and the flat-sky
   switches of coffe_gpu_set_flatsky must be off. */
int coffe_gpu_multipoles_scaled(coffe_gpu_ctx_t *ctx, int contrib, int n_req, int64_t n_sep,
                                const int *req_spectrum, const double *req_z_mean,
                                const int64_t *req_offset, const double *sep, int n_l,
                                const int *l, const double *bias_scale,
                                const double *growth_scale, double *out);

/* Reverse-mode derivative of coffe_gpu_multipoles_scaled: given grad_out (same
   layout as out), writes grad_pk[s * nk + i] = sum grad_out * d out / d P_s(k_i)
   for every spectrum of the last coffe_gpu_integrals_init (through the
   natural-spline resampling, the FFTLog transform and the Akima interpolation
   of the tables, twofast.c:362-483; with COFFE_GPU_LEN also through the
   lensing integrands and the QAG integrals of the r = 0 and sub-Mpc table
   entries, integrals.c:524-562, on their final partition), and, when not
   NULL, grad_bias_scale[q] and grad_growth_scale[q].  Device pointers except
   `l`. */
int coffe_gpu_multipoles_adjoint(coffe_gpu_ctx_t *ctx, int contrib, int n_req, int64_t n_sep,
                                 const int *req_spectrum, const double *req_z_mean,
                                 const int64_t *req_offset, const double *sep, int n_l,
                                 const int *l, const double *bias_scale,
                                 const double *growth_scale, const double *grad_out,
                                 double *grad_pk, double *grad_bias_scale,
                                 double *grad_growth_scale);

/* -------------------------------------------------------------- covariance */

/* The double-Bessel integrals of the multipole covariance by 2D FFTLog, as
   covariance_integrate_fftlog computes them (covariance.c:357-470 with
   two_sph_bessel, twobessel.c:16-122; nu = 1.01, window 0.25): for each job q
   the 2D FFTLog of diag(k^3 P(k)^power[q] / dlnk) on N log-spaced k in
   [k[0], k[nk-1]) with multipoles l1[q], l2[q], resampled bicubically at the
   separations:
     out[q * n_sep^2 + n_sep * n + m] = value at (r1 = sep[m], r2 = sep[n])
   (unscaled; coffe_covariance_init multiplies by (2l1+1)(2l2+1) 2/pi^2 or
   /pi^2).  P(k) through the Akima spline of (k, pk); N a power of two in
   [64, 8192]; separations inside [1/k(N-1), 1/k[0]].  Host arrays. */
int coffe_gpu_covariance_integrals(coffe_gpu_ctx_t *ctx, const double *k, const double *pk,
                                   size_t nk, size_t N, int n_jobs, const int *power,
                                   const int *l1, const int *l2, const double *sep, int n_sep,
                                   double *out);

/* Replaces coffe_covariance_init (covariance.c:477-1103) for the multipole
   covariance with covariance_integration_method = fftlog, one population
   (covariance_pop1..4 = 1, the defaults), no window, linear P(k): the Poisson,
   mixed and cosmic-variance terms for every redshift bin (z_mean, deltaz, fsky,
   number densities density1/2, pixelsize), multipoles l[0..n_l-1] and
   separations, in the reference's output order
     out[(((z * n_l + i1) * n_sep + m) * n_l + i2) * n_sep + n]
   = cov(z, l1 = l[i1], r1 = sep[m], l2 = l[i2], r2 = sep[n]) (covariance.c:
   1046-1059).  Background from coffe_gpu_background_init/_set, galaxy bias 1
   from coffe_gpu_set_bias (default 1).  contrib: den and/or rsd (bias or
   growth rate zero otherwise, covariance.c:845-861).  Host arrays. */
int coffe_gpu_covariance_multipoles(coffe_gpu_ctx_t *ctx, int contrib, const double *k,
                                    const double *pk, size_t nk, size_t N, int n_z,
                                    const double *z_mean, const double *deltaz,
                                    const double *fsky, const double *density1,
                                    const double *density2, const double *pixelsize, int n_l,
                                    const int *l, int n_sep, const double *sep, double *out);

/* The covariance of the redshift-averaged multipoles (coffe_covariance_init's
   average branch, covariance.c:811-840): as coffe_gpu_covariance_multipoles
   with redshift windows 0 < z_min[w] < z_max[w] in place of (z_mean, deltaz):
   every window at z = (z_min + z_max)/2 with the effective volume
   4 pi fsky / int_{z_min}^{z_max} dz / (conformal_H chi^2 (1 + z)) / (H0 h)^2
   (covariance.c:150-162; the reference's QAG, here 16 Gauss-Legendre panels
   uniform in ln z).  Output order (window, l1, r1, l2, r2).  Host arrays. */
int coffe_gpu_average_covariance_multipoles(coffe_gpu_ctx_t *ctx, int contrib,
                                            const double *k, const double *pk, size_t nk,
                                            size_t N, int n_win, const double *z_min,
                                            const double *z_max, const double *fsky,
                                            const double *density1, const double *density2,
                                            const double *pixelsize, int n_l, const int *l,
                                            int n_sep, const double *sep, double *out);

/* No counterpart in the reference: the measured arithmetic rate of this
   context's device, the denominator of the compute-bound kernels' roofline
   fractions.  kind: COFFE_GPU_PEAK_FP64 (fma.rn.f64), COFFE_GPU_PEAK_FP32
   (fma.rn.f32) or COFFE_GPU_PEAK_FP32X2 (fma.rn.f32x2, two FP32 lanes per
   instruction).  Independent FMA chains on every SM, best of three ~10 ms
   launches timed with CUDA events; *flops_per_s counts an FMA as 2 FLOP. */
#define COFFE_GPU_PEAK_FP64 0
#define COFFE_GPU_PEAK_FP32 1
#define COFFE_GPU_PEAK_FP32X2 2
int coffe_gpu_measure_peak(coffe_gpu_ctx_t *ctx, int kind, double *flops_per_s);

/* No counterpart in the reference (its only timing is the clock() prints of
   its verbose mode): per-kernel device time.  enable != 0 records a CUDA event
   on the context's stream after every kernel launch, and one at the start of
   each table (coffe_gpu_integrals_init*) and multipole call; the interval
   between consecutive events of a call is charged to the kernel launched in
   it (a copy or memset enqueued before a kernel is charged to that kernel).
   Calls made while the stream is being captured record nothing.  Costs a few
   microseconds per launch; off by default. */
int coffe_gpu_set_kernel_timing(coffe_gpu_ctx_t *ctx, int enable);
/* Synchronises the stream and accumulates the recorded intervals, then writes
   up to `cap` entries: kernel name (valid until the next call of this
   function on the context or its destruction), launches and total
   milliseconds.  Returns the number of distinct kernels timed since the last
   reset (may exceed cap) or a negative status; reset != 0 clears the totals
   after writing them. */
int coffe_gpu_kernel_times(coffe_gpu_ctx_t *ctx, const char **names, long long *launches,
                           double *total_ms, int cap, int reset);

/* No counterpart in the reference: failure injection for tests.  The nth
   device allocation this context makes from now on fails as an exhausted
   device would make it fail (COFFE_GPU_ENOMEM from the call that needed it),
   without calling cudaMalloc; nth = 0 disarms.  Allocations are made on first
   use and when a call needs larger buffers than any before it. */
int coffe_gpu_debug_fail_alloc(coffe_gpu_ctx_t *ctx, int nth);

/* Kernel launches issued by this context since creation (for accounting). */
long long coffe_gpu_launch_count(const coffe_gpu_ctx_t *ctx);

#ifdef __cplusplus
}
#endif
#endif /* COFFE_GPU_H */
