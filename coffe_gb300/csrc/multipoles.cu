// Multipoles of the nonintegrated density + RSD terms for a ragged batch of
// (spectrum, mean redshift, separation list) requests in one launch.
//
// Restates coffe_integrate(NONINTEGRATED, MULTIPOLES) (signal.c:521-542) with
// multipoles_nonintegrated_integrand (signal.c:83-111) and
// functions_nonintegrated (functions.c:89-1484; den-den 129-229, rsd-rsd
// 230-362, den-rsd 670-771, growth factors 1463-1466):
//     mp_l(z, r) = (2l+1) int_0^1 dx xi(z, mu = 2x - 1, r) P_l(mu)
// integrated by QUADPACK QAG with the 61-point Gauss-Kronrod rule.
//
// One warp owns one (request, separation) pair.  Each lane evaluates xi at two
// of the 61 nodes of the first panel; xi does not depend on l, so all
// requested multipoles share those evaluations (the reference recomputes the
// integrand once per l).  Each l then gets its own GK61 sums and error test;
// an l whose first panel misses the tolerance continues with the adaptive
// bisection of QAG for that l alone.
//
// FP64 path: the reference's arithmetic in double.  Mixed path: the same
// algorithm with float splines, integrand and Legendre polynomials, and
// compensated (two-sum) float reductions for the panel result.
#include "ctx.cuh"
#include "qag.cuh"

namespace {

#define MP_WARPS 4
#define MP_CAP 128
#define MP_MAX_L 8

template <typename S> struct SplPack {
    S z_of_chi, f, D1, b1, b2;
    int has_b1, has_b2;
};

// P_l(x) by the upward recurrence (gsl_sf_legendre_Pl), 1/k as a product
template <typename T> __device__ __forceinline__ T legendre_p(int l, T x)
{
    if (l == 0) return T(1);
    if (l == 1) return x;
    T p0 = T(1), p1 = x;
    for (int k = 2; k <= l; ++k) {
        const T p2 = ((T(2) * k - T(1)) * x * p1 - (T(k) - T(1)) * p0) * (T(1) / T(k));
        p0 = p1;
        p1 = p2;
    }
    return p1;
}

// xi(z_mean, mu, r) of the den/rsd terms in the cancellation-free form:
// with D = 2 chi^2 - mu^2 r^2 / 2 (= 2 chi1 chi2) and s = 1 - cos(theta) =
// r^2 (1 - mu^2) / D, the reference's cos(theta)- and chi/r-expressions
// become the polynomials below (identical algebra; the reference's I04
// coefficient cancels two terms of size (chi/r)^4).
template <typename T, typename S> struct Xi {
    SplPack<S> sp;
    T chi_mean, sep, I00, I02, I04;
    int contrib;

    __device__ __forceinline__ T operator()(T mu) const
    {
        const T chi1 = chi_mean - sep * mu * T(0.5);
        const T chi2 = chi_mean + sep * mu * T(0.5);
        const T mu2 = mu * mu;
        const T omm = T(1) - mu2;
        const T D = T(2) * chi_mean * chi_mean - mu2 * sep * sep * T(0.5);
        const T inv_D = T(1) / D;
        const T s = sep * sep * omm * inv_D;
        const T c = T(1) - s;
        const T z1 = spl_eval(sp.z_of_chi, chi1);
        const T z2 = spl_eval(sp.z_of_chi, chi2);
        const T f1 = spl_eval(sp.f, z1);
        const T f2 = spl_eval(sp.f, z2);
        const T b1 = sp.has_b1 ? spl_eval(sp.b1, z1) : T(1);
        const T b2 = sp.has_b2 ? spl_eval(sp.b2, z2) : T(1);
        T result = T(0);
        if (contrib & COFFE_GPU_DEN) result += b1 * b2 * I00;
        if (contrib & COFFE_GPU_RSD) {
            const T c2 = c * c;
            const T q4 = omm * omm * (T(3) * c2 - T(10) * c + T(19)) * T(0.25) +
                         T(4) * mu2 * omm * (c2 - T(5) * c - T(2)) +
                         T(4) * (T(3) * c2 - T(1)) * mu2 * mu2;
            const T ff = f1 * f2;
            result += ff * (T(1) + T(2) * c2) * T(1.0 / 15) * I00 -
                      ff * T(1.0 / 21) * ((T(1) + T(11) * c2) - T(9) * c * (T(2) - s) * omm) * I02 +
                      ff * q4 * T(1.0 / 35) * I04;
        }
        if ((contrib & COFFE_GPU_DEN) && (contrib & COFFE_GPU_RSD)) {
            const T g = (T(2) - s) * omm * inv_D;
            result += (b1 * f2 + b2 * f1) * T(1.0 / 3) * I00 -
                      (b1 * f2 * (T(2.0 / 3) - g * chi1 * chi1) +
                       b2 * f1 * (T(2.0 / 3) - g * chi2 * chi2)) *
                          I02;
        }
        return result * spl_eval(sp.D1, z1) * spl_eval(sp.D1, z2);
    }
};

// integrand of one multipole at x in [0, 1] (for the adaptive continuation)
template <typename T, typename S> struct MpIntegrand {
    Xi<T, S> xi;
    int l;
    __device__ __forceinline__ T operator()(T x) const
    {
        const T mu = T(2) * x - T(1);
        const T v = xi(mu);
        return l == 0 ? v : v * legendre_p<T>(l, mu);
    }
};

// Akima lookup of an I_l^n table: knots tab_x (r = 0, 42 sub-Mpc points, then
// r0 (kmax/kmin)^(i/N)), values y; the interval is found as a binary search
// would (an O(1) guess on the log grid, then a local correction).
template <typename T>
__device__ __forceinline__ T table_lookup(const T *__restrict__ x, const T *__restrict__ y, int n,
                                          T inv_dlog, T r)
{
    if (!(r >= x[0] && r <= x[n - 1])) return cg_nan<T>();
    int i;
    const int first = CG_N_SMALL_R + 1;
    if (r >= x[first]) {
        i = first + (int)(log(r) * inv_dlog);
        if (i > n - 2) i = n - 2;
        if (i < first) i = first;
        while (i > 0 && x[i] > r) --i;
        while (i < n - 2 && x[i + 1] <= r) ++i;
    } else {
        int lo = 0, hi = first;
        while (hi > lo + 1) {
            const int mid = (lo + hi) / 2;
            if (x[mid] > r)
                hi = mid;
            else
                lo = mid;
        }
        i = lo;
    }
    return akima_eval_at<T>(x, y, n, i, r);
}

struct MpArgs {
    int n_req, n_l, contrib;
    int t00, t02, t04;
    int n_terms, tab_len;
    double inv_dlog; // N / ln(kmax/kmin), r0 = 1
    long long per_warp; // contiguous separations per warp
    double epsrel;
    int ls[MP_MAX_L];
};

template <typename T, typename S, typename TT>
__global__ void __launch_bounds__(32 * MP_WARPS)
    multipoles_kernel(MpArgs a, SplPack<S> sp, S chi_of_z, const TT *__restrict__ tab_x,
                      const TT *__restrict__ tab_y, const int *__restrict__ req_spectrum,
                      const double *__restrict__ req_z_mean, const int64_t *__restrict__ req_offset,
                      const double *__restrict__ sep, long long total, double *__restrict__ out,
                      int *err)
{
    __shared__ T sa[MP_WARPS][MP_CAP], sb[MP_WARPS][MP_CAP], sr[MP_WARPS][MP_CAP],
        se[MP_WARPS][MP_CAP];
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const GkLane<T> g = gk_lane<T>();
    const long long warp_id = (long long)blockIdx.x * MP_WARPS + w;
    const long long begin = warp_id * a.per_warp;
    const long long end = begin + a.per_warp < total ? begin + a.per_warp : total;
    if (begin >= end) return;
    // request of the first separation: largest q with req_offset[q] <= begin
    int q;
    {
        int lo = 0, hi = a.n_req;
        while (hi > lo + 1) {
            const int mid = (lo + hi) >> 1;
            if (req_offset[mid] <= begin)
                lo = mid;
            else
                hi = mid;
        }
        q = lo;
    }
    long long q_end = req_offset[q + 1];
    for (long long item = begin; item < end; ++item) {
        while (item >= q_end) {
            ++q;
            q_end = req_offset[q + 1];
        }
        const int s = req_spectrum[q];
        const T r = (T)sep[item];
        const T zm = (T)req_z_mean[q];
        // the three I tables at r: lanes 0..2 look one up each
        T Iv = T(0);
        if (lane < 3) {
            const int t = lane == 0 ? a.t00 : (lane == 1 ? a.t02 : a.t04);
            const TT *y = tab_y + ((size_t)s * a.n_terms + t) * a.tab_len;
            Iv = (T)table_lookup<TT>(tab_x, y, a.tab_len, (TT)a.inv_dlog, (TT)r);
        }
        Xi<T, S> xi;
        xi.sp = sp;
        xi.sep = r;
        xi.contrib = a.contrib;
        xi.I00 = __shfl_sync(0xffffffffu, Iv, 0);
        xi.I02 = __shfl_sync(0xffffffffu, Iv, 1);
        xi.I04 = __shfl_sync(0xffffffffu, Iv, 2);
        xi.chi_mean = spl_eval(chi_of_z, zm);
        // first panel on [0, 1]: mu = 2x - 1 at x = 0.5 -+ 0.5 xgk
        T mu1 = T(0), mu2 = T(0), xi1 = T(0), xi2 = T(0);
        if (g.centre) {
            mu1 = T(0);
            xi1 = xi(mu1);
        } else if (g.active) {
            const T absc = T(0.5) * g.x;
            mu1 = T(2) * (T(0.5) - absc) - T(1);
            mu2 = T(2) * (T(0.5) + absc) - T(1);
            xi1 = xi(mu1);
            xi2 = xi(mu2);
        }
        for (int li = 0; li < a.n_l; ++li) {
            const int l = a.ls[li];
            T f1 = xi1, f2 = xi2;
            if (l != 0) {
                f1 = g.active ? xi1 * legendre_p<T>(l, mu1) : T(0);
                f2 = (g.active && !g.centre) ? xi2 * legendre_p<T>(l, mu2) : T(0);
            }
            QkOut<T> p0 = qk61_reduce<T>(g, f1, f2, T(0.5));
            if (sizeof(T) == 4) {
                // compensated sum of the Kronrod estimate
                const T fs = f1 + f2;
                const T prod = g.wk * fs;
                const T perr = fmaf((float)g.wk, (float)fs, -(float)prod);
                p0.result = (T)warp_sum_comp((float)prod, (float)perr) * T(0.5);
            }
            int status = 0;
            MpIntegrand<T, S> fn{xi, l};
            QagStore<T> store{sa[w], sb[w], sr[w], se[w], MP_CAP};
            const T v = qag_continue<T>(fn, g, T(0), T(1), p0, T(0), (T)a.epsrel, store, 50000,
                                        &status);
            if (lane == 0) {
                if (status == 1) cg_flag(err, CG_ERR_QAG_LIMIT);
                const double res = (double)(T(2 * l + 1) * v);
                if (!isfinite(res)) cg_flag(err, CG_ERR_NONFINITE);
                out[item * a.n_l + li] = res;
            }
        }
    }
}

} // namespace

int multipoles_run(coffe_gpu_ctx *ctx, int contrib, int precision, double epsrel, int n_req,
                   const int *req_spectrum, const double *req_z_mean, const int64_t *req_offset,
                   const double *sep, int n_l, const int *l, double *out, long long total)
{
    // all array pointers are device pointers here; total = req_offset[n_req]
    if (!ctx->bg_ready) {
        cg_set_error(ctx, "multipoles: background not initialised");
        return COFFE_GPU_ESTATE;
    }
    if (!ctx->int_ready) {
        cg_set_error(ctx, "multipoles: integrals not initialised");
        return COFFE_GPU_ESTATE;
    }
    if (n_l < 1 || n_l > MP_MAX_L || n_req < 1) {
        cg_set_error(ctx, "multipoles: need 1 <= n_l <= %d and n_req >= 1", MP_MAX_L);
        return COFFE_GPU_EINVAL;
    }
    if (precision != ctx->int_precision) {
        cg_set_error(ctx, "multipoles: precision %d differs from the integrals' (%d)", precision,
                     ctx->int_precision);
        return COFFE_GPU_EINVAL;
    }
    if (!(contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD)) || (contrib & ~7)) {
        cg_set_error(ctx, "multipoles: contrib must select den and/or rsd");
        return COFFE_GPU_EINVAL;
    }
    if (!(epsrel > 0)) {
        cg_set_error(ctx, "multipoles: epsrel must be positive");
        return COFFE_GPU_EINVAL;
    }
    MpArgs a;
    a.n_req = n_req;
    a.n_l = n_l;
    a.contrib = contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD);
    a.t00 = a.t02 = a.t04 = -1;
    for (int t = 0; t < ctx->n_terms; ++t) {
        if (ctx->term_n[t] == 0 && ctx->term_l[t] == 0) a.t00 = t;
        if (ctx->term_n[t] == 0 && ctx->term_l[t] == 2) a.t02 = t;
        if (ctx->term_n[t] == 0 && ctx->term_l[t] == 4) a.t04 = t;
    }
    if (a.t00 < 0 || a.t02 < 0 || a.t04 < 0) {
        cg_set_error(ctx, "multipoles: integrals (0,0), (0,2), (0,4) are required");
        return COFFE_GPU_ESTATE;
    }
    a.n_terms = ctx->n_terms;
    a.tab_len = (int)(ctx->N + CG_N_SMALL_R + 1);
    a.inv_dlog = (double)ctx->N / log(ctx->kmax / ctx->kmin);
    a.epsrel = epsrel;
    for (int i = 0; i < n_l; ++i) {
        if (l[i] < 0 || l[i] > 32) {
            cg_set_error(ctx, "multipoles: l = %d out of range", l[i]);
            return COFFE_GPU_EINVAL;
        }
        a.ls[i] = l[i];
    }
    if (total <= 0) return COFFE_GPU_OK;
    if (ctx->sm_count <= 0)
        CG_CUDA(ctx, cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount,
                                            ctx->device));
    const int sms = ctx->sm_count;
    // contiguous ranges of separations per warp (one request search per range)
    const long long max_warps = (long long)sms * 16 * MP_WARPS;
    long long nw = total < max_warps ? total : max_warps;
    a.per_warp = (total + nw - 1) / nw;
    nw = (total + a.per_warp - 1) / a.per_warp;
    const int blocks = (int)((nw + MP_WARPS - 1) / MP_WARPS);
    if (precision == COFFE_GPU_MIXED) {
        SplPack<Spl32> sp{ctx->bg[BG_Z_OF_CHI].v32(), ctx->bg[BG_F].v32(), ctx->bg[BG_D1].v32(),
                          ctx->bias[0].v32(), ctx->bias[1].v32(), ctx->bias_set[0],
                          ctx->bias_set[1]};
        multipoles_kernel<float, Spl32, float><<<blocks, 32 * MP_WARPS, 0, ctx->stream>>>(
            a, sp, ctx->bg[BG_CHI_OF_Z].v32(), (const float *)ctx->tab_x32.p,
            (const float *)ctx->tab_y.p, req_spectrum, req_z_mean, req_offset, sep, total, out,
            ctx->d_err);
    } else {
        SplPack<Spl64> sp{ctx->bg[BG_Z_OF_CHI].v64(), ctx->bg[BG_F].v64(), ctx->bg[BG_D1].v64(),
                          ctx->bias[0].v64(), ctx->bias[1].v64(), ctx->bias_set[0],
                          ctx->bias_set[1]};
        multipoles_kernel<double, Spl64, double><<<blocks, 32 * MP_WARPS, 0, ctx->stream>>>(
            a, sp, ctx->bg[BG_CHI_OF_Z].v64(), (const double *)ctx->tab_x.p,
            (const double *)ctx->tab_y.p, req_spectrum, req_z_mean, req_offset, sep, total, out,
            ctx->d_err);
    }
    return cg_after_launch(ctx, "multipoles_kernel");
}
