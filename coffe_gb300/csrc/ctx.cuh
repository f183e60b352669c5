// Host-side context of the C ABI (include/coffe_gpu.h): device buffers, the
// stream, error state and the cached per-grid tables.
#pragma once

#include <stdarg.h>
#include <stdio.h>

#include <array>
#include <map>
#include <string>
#include <vector>

#include "spline.cuh"

#define CG_MAX_TERMS 64
#define CG_N_SMALL_R 42

// Device buffer that only grows.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

enum cg_bg_fn { BG_CHI_OF_Z = 0, BG_Z_OF_CHI, BG_D1, BG_F, BG_A, BG_CONFH, BG_NFN };

struct coffe_gpu_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    // uploads that overlap work on `stream` (created on first use) and the
    // events that order them
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_ev[3] = {nullptr, nullptr, nullptr};
    // set by the host-array multipole call for the duration of its run: the
    // stream its request uploads went to, for work that needs only them
    cudaStream_t prep_stream = nullptr;
    int *d_err = nullptr;   // device error bits (cg_err_bits)
    int *h_err = nullptr;   // pinned mirror
    long long launches = 0; // kernels launched through this context
    int fail_alloc_in = 0;  // > 0: that many allocations from now, the last fails
    // kernel timing mode: events after each launch, totals per kernel name
    bool timing = false;
    std::vector<cudaEvent_t> timing_events;
    std::vector<const char *> timing_marks; // nullptr: the start of a call
    std::map<std::string, std::pair<long long, double>> timing_totals;
    std::vector<std::string> timing_names; // names of the last coffe_gpu_kernel_times
    int sm_count = 0;
    char last_error[512] = {0};
    // the multipole output of the running call is page-locked host memory
    // (mapped): the den/rsd kernels stage each block's results in shared
    // memory and store them as whole lines
    bool out_host = false;

    // ---- background
    int bg_bins = 0;
    bool bg_ready = false, bg_has_H = false;
    double Omega0_m = 0.3, h = 0.67;
    DevBuf bg_nodes; // bins * 8 doubles: z, chi, D1, f, a, confH, H, confHp
    DevBuf bg_traj;  // growth ODE trajectory (D, D', and derivatives) per RK4 step
    std::vector<double4_32a> bg_traj_host;
    SplineBuf bg[BG_NFN];
    // fused f / D1 coefficient records on a uniform z grid (multipoles.cu)
    bool z_uniform = false;
    double z0 = 0, zn = 0, dz = 0;
    DevBuf zrec64, zrec32;
    // (D1, f D1) at CG_CHI_TAB uniform chi over the background's range, FP64
    // and float, for the per-request background fits (linear interpolation)
    DevBuf chi_tab64, chi_tab32;
    double chi_t0 = 0, chi_tn = 0;
    DevBuf cf_rule; // mu list + line rules of the last coffe_gpu_corrfunc call with lensing
    DevBuf avg_buf; // expanded requests of coffe_gpu_average_multipoles
    SplineBuf bias[4];
    bool bias_set[4] = {false, false, false, false};
    std::vector<double> bias_host[4]; // (z, value) samples as set, for symmetry checks
    DevBuf bias_nodes[4];

    // ---- integral tables
    bool int_ready = false;
    int n_spectra = 0, n_terms = 0, int_precision = 0;

    // ---- launch shapes (coffe_gpu_set_tuning / benchmark-mode autotuning)
    coffe_gpu_tuning_t tuning = {512, 4, 1, 8, 128, 2, 512, 1, 1, 1}; // default configuration
    coffe_gpu_tuning_t last_tuning = {512, 4, 1, 8, 128, 2, 512, 1, 1, 1};
    bool autotune = false;
    std::map<std::array<long long, 6>, coffe_gpu_tuning_t> tune_cache; // shape -> choice
    size_t N = 0, nk = 0;
    double kmin = 0, kmax = 0;
    bool int_small_r = false; // r = 0 and sub-Mpc entries filled
    int term_n[CG_MAX_TERMS], term_l[CG_MAX_TERMS], term_q[CG_MAX_TERMS];
    int term_half[CG_MAX_TERMS]; // 1: (n, l) are numerators of n/2, l/2
    int n_q = 0;
    double qvals[CG_MAX_TERMS];
    DevBuf tab_x;     // (N + 43) doubles, shared by all tables
    DevBuf tab_x32;   // same in float
    DevBuf tab_y;     // n_spectra * n_terms * (N + 43), double or float
    DevBuf pk;        // n_spectra * nk doubles (input spectra)
    DevBuf kgrid;     // nk doubles
    DevBuf csc;       // n_spectra * nk doubles: natural-spline c coefficients
    DevBuf csfac;     // 2 * nk doubles: Thomas factors of the shared k grid
    DevBuf samp_idx;  // N ints: input interval of each FFT node
    DevBuf samp_dx;   // N doubles: offset of each FFT node in its interval
    DevBuf samp_f32;  // N float4 (dx, h, 1/h, -) for the mixed path
    DevBuf csfac32;   // 4 * nk floats: spline factors for the mixed path
    DevBuf csband;    // 25 x (nk - 2) floats: band of the inverse spline matrix, by diagonal
    // host copies of the per-grid spline factors and band (sources of the uploads)
    std::vector<double> grid_fac_host;
    std::vector<float> grid_fac32_host, grid_band_host;
    int grid_band_ok = 0;         // the band factorises (geometric k grid)
    float grid_band_tau[25] = {}; // its 2 CS_BAND + 1 constants
    DevBuf samp_tdf;  // N float2: double-float dx / h of each FFT node (mixed path)
    DevBuf qfac_df;   // n_q * N float2: double-float windowed bias (mixed path)
    DevBuf pk_df;     // n_spectra * nk float2: double-float input spectra (mixed path)
    DevBuf qfac;      // n_q * N doubles: (kmax/kmin)^((3-q) i/N) W(k_i)
    DevBuf modec;     // n_terms * (N/2+1) double2: W_mode/L * M_{q,l}(t)
    DevBuf postf;     // n_terms * N doubles: prefactor * r^(n-l)
    DevBuf twid;      // N/2+1 double2 twiddles exp(-2 pi i j / N)
    DevBuf twid32;    // double-float (float4) copy
    DevBuf term_df;   // double-float copies of modec / modew / postf
    DevBuf spec;      // n_spectra * n_q * (N/2+1) double2 forward half spectra
    // cache key of the per-grid tables
    size_t grid_N = 0, grid_nk = 0;
    double grid_kmin = 0, grid_kmax = 0;
    std::vector<double> grid_k;
    std::vector<int> grid_terms;

    DevBuf term_meta; // per-term metadata of the integral tables

    // ---- multipole request staging (host-pointer calls) and retry list
    DevBuf req_buf;
    DevBuf mp_retry;
    DevBuf mp_bgfit; // per-request background polynomials of the mixed fast kernel
    // first-panel node tables, one per (multipole list, precision, layout):
    // each is written once and never overwritten while fewer than
    // CG_NODE_SLOTS distinct tables are in use, so a captured launch that
    // reads one stays valid when calls of another precision run in between
    struct NodeSlot {
        DevBuf buf;
        int nl = 0, prec = -1, mirror = -1;
        int ls[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    };
    static constexpr int CG_NODE_SLOTS = 8;
    NodeSlot mp_node_slots[CG_NODE_SLOTS];
    int mp_node_next = 0;

    // ---- flat-sky lensing and cross-correlation switches (lensing.cu)
    int flat_local_nonlocal = 0; // den-lensing in the flat-sky limit
    int flat_nonlocal = 0;       // lensing-lensing in the flat-sky limit

    // ---- lensing terms (lensing.cu)
    int lens_n_mu = 128, lens_n_x = 256; // Gauss-Legendre rule sizes
    DevBuf lens_rule;                    // the rule's nodes and weights
    int lens_rule_mu = 0, lens_rule_x = 0;
    DevBuf lens_rec;  // Akima records of the six lensing tables
    DevBuf lens_part; // per (pair, mu) partial integrals

    // ---- covariance (covariance.cu)
    SplineBuf cov_pk; // Akima spline of the covariance's P(k)
    DevBuf cov_buf;   // FFTLog work arrays
    DevBuf cov_out;   // integrals, assembly inputs and outputs

    // ---- multipole adjoint (adjoint.cu)
    DevBuf adj_buf; // table, spectrum and resampling cotangents
    DevBuf div_buf; // k, P(k), separations and results of the divergent integral
    DevBuf peak_buf; // per-thread outputs of the peak-rate kernels (peaks.cu)
};

void cg_set_error(coffe_gpu_ctx *ctx, const char *fmt, ...);
// index of the table I^n_l (half: numerators of half-integers) or -1
inline int cg_find_term(const coffe_gpu_ctx *ctx, int n, int l, int half = 0)
{
    for (int t = 0; t < ctx->n_terms; ++t)
        if (ctx->term_n[t] == n && ctx->term_l[t] == l && ctx->term_half[t] == half) return t;
    return -1;
}
int cg_ensure(coffe_gpu_ctx *ctx, DevBuf &b, size_t bytes);
void cg_release(DevBuf &b);
// Reads and clears the device error bits; maps them to a status.
int cg_check_device_errors(coffe_gpu_ctx *ctx, const char *where);
// Checks the last launch; counts it (and in timing mode records an event).
int cg_after_launch(coffe_gpu_ctx *ctx, const char *what);
// Timing mode: marks the start of a table or multipole call.
void cg_timing_begin(coffe_gpu_ctx *ctx);

// module entry points (host code)
int bg_init_device(coffe_gpu_ctx *ctx, const coffe_gpu_cosmology_t *c);
int bg_build_splines(coffe_gpu_ctx *ctx);
int integrals_build(coffe_gpu_ctx *ctx, const double *k, const double *pk, int n_spectra,
                    size_t nk, const int *n, const int *l, const int *half, int n_terms, size_t N,
                    int precision, unsigned flags);
int divergent_run(coffe_gpu_ctx *ctx, const double *k, const double *pk, size_t nk, double kmin,
                  double kmax, const double *r1, size_t n1, const double *r2, size_t n2,
                  double *out_a, double *out_b);
int integrals_eval(coffe_gpu_ctx *ctx, int spectrum, int term, const double *r, size_t nq,
                   double *out);
int multipoles_prepare_background(coffe_gpu_ctx *ctx);
// loads the module and kernels of coffe_gpu_multipoles_noalloc (ctx creation)
int multipoles_noalloc_prepare(coffe_gpu_ctx *ctx);

// Evicts the L2 cache on the context's stream: writes `bytes` (>= twice the L2)
// at buf, then reads them back, so that the lines left in L2 are clean and the
// work timed next neither finds its inputs there nor pays for writing the
// eviction's dirty lines back.
int cg_l2_evict(coffe_gpu_ctx *ctx, void *buf, size_t bytes, int value);
// creates ctx->copy_stream and ctx->copy_ev on first use
int cg_copy_stream(coffe_gpu_ctx *ctx);

// Configuration for one launch shape: the chosen one if the shape was tuned,
// else (benchmark mode, stream not capturing) the fastest of `cands` timed
// with `run` on the stream, else the default.  run(cfg) enqueues the work.
// cold: the work's inputs arrive from outside (new spectra): every timed run
// starts with the L2 cache evicted (cg_l2_evict), as it does in use, where the
// candidates rank differently than on L2-resident inputs.
template <typename Run>
int cg_tuned(coffe_gpu_ctx *ctx, const std::array<long long, 6> &key,
             const std::vector<coffe_gpu_tuning_t> &cands, Run run, coffe_gpu_tuning_t *out,
             bool cold = false)
{
    auto it = ctx->tune_cache.find(key);
    if (it != ctx->tune_cache.end()) {
        *out = it->second;
        return 0;
    }
    *out = ctx->tuning;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (!ctx->autotune || cands.size() < 2 ||
        cudaStreamIsCapturing(ctx->stream, &cap) != cudaSuccess ||
        cap != cudaStreamCaptureStatusNone)
        return 0;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return COFFE_GPU_ECUDA;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return COFFE_GPU_ECUDA;
    }
    void *flush = nullptr;
    size_t flush_bytes = 0;
    if (cold) {
        int l2 = 0;
        if (cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, ctx->device) == cudaSuccess &&
            l2 > 0 && cudaMalloc(&flush, 2 * (size_t)l2) == cudaSuccess)
            flush_bytes = 2 * (size_t)l2;
        else
            flush = nullptr; // no room: time on warm inputs
    }
    float best = 3.0e38f;
    int st = 0;
    for (const coffe_gpu_tuning_t &c : cands) {
        if ((st = run(c))) break; // warm-up of this configuration
        float t = 3.0e38f;
        for (int rep = 0; rep < 2 && !st; ++rep) {
            if (flush && (st = cg_l2_evict(ctx, flush, flush_bytes, rep))) break;
            cudaEventRecord(e0, ctx->stream);
            st = run(c);
            cudaEventRecord(e1, ctx->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess) st = COFFE_GPU_ECUDA;
            float ms = 0.f;
            if (!st && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms < t) t = ms;
        }
        if (st) break;
        if (t < best) {
            best = t;
            *out = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (flush) {
        cudaStreamSynchronize(ctx->stream);
        cudaFree(flush);
    }
    if (st) return st;
    ctx->tune_cache[key] = *out;
    return 0;
}
int multipoles_run(coffe_gpu_ctx *ctx, int contrib, int precision, double epsrel, int n_req,
                   const int *req_spectrum, const double *req_z_mean, const int64_t *req_offset,
                   const double *sep, int n_l, const int *l, double *out, long long total);
int multipoles_adjoint_run(coffe_gpu_ctx *ctx, int contrib, int n_req, const int *req_spectrum,
                           const double *req_z_mean, const int64_t *req_offset, const double *sep,
                           long long total, int n_l, const int *l, const double *bias_scale,
                           const double *growth_scale, const double *grad_out, double *value_out,
                           double *grad_pk, double *grad_bias, double *grad_growth);
int average_multipoles_run(coffe_gpu_ctx *ctx, int contrib, int precision, double epsrel,
                           int n_win, const int *win_spectrum, const double *z_min,
                           const double *z_max, const int64_t *win_offset, const double *sep,
                           int n_l, const int *l, int n_z, double *out, long long total);
int lensing_adjoint_run(coffe_gpu_ctx *ctx, int contrib, int n_req, const int *req_spectrum,
                        const double *req_z_mean, const int64_t *req_offset, const double *sep,
                        long long total, int n_l, const int *l, const double *bias_scale,
                        const double *growth_scale, const double *grad_out, double *value_out,
                        double *gY, int n_at, double *grad_bias, double *grad_growth);
// adjoint of the r = 0 and sub-Mpc table entries: gY's first CG_N_SMALL_R + 1
// entries of each of the n_at tables (term index term[t]) into grad_pk (added)
int small_r_adjoint_run(coffe_gpu_ctx *ctx, const double *gY, int n_at, const int *term,
                        double *grad_pk);
// n-point Gauss-Legendre nodes (ascending) and weights on [-1, 1]
void gauss_legendre_nodes(int n, double *x, double *w);
int corrfunc_run(coffe_gpu_ctx *ctx, int contrib, int precision, int n_req,
                 const int *req_spectrum, const double *req_z_mean, const int64_t *req_offset,
                 const double *sep, int n_mu, const double *mu, const double *mu_host,
                 double *out, long long total);
int corrfunc_lensing_run(coffe_gpu_ctx *ctx, int contrib, int precision, int n_req,
                         const int *req_spectrum, const double *req_z_mean,
                         const int64_t *req_offset, const double *sep, int n_mu,
                         const double *mu_host, double *out, long long total);
int lensing_run(coffe_gpu_ctx *ctx, int contrib, int precision, double epsrel, int n_req,
                const int *req_spectrum, const double *req_z_mean, const int64_t *req_offset,
                const double *sep, int n_l, const int *l, double *out, long long total);
