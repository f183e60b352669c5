// Reverse-mode derivatives of the den/RSD multipoles with respect to the input
// power spectra P(k), a per-request galaxy-bias scale and a per-request
// growth-rate scale (FP64).
//
// The multipole of one (request, separation, l) is, on the first GK61 panel
// that the forward quadrature accepts (signal.c:83-111, 521-542),
//   mp_l = sum_t I_t(r) sum_y m_y(beta, alpha) J_{t,y,l}(r, z),
// t in {I00, I02, I04} (the tables read at the separation, functions.c:
// 129-771), y in {bb, bf, ff} the bias/growth monomials beta^2, beta alpha,
// alpha^2 (b -> beta b, f -> alpha f), and J the GK61 integrals of the
// background-only coefficient functions times (2l+1) P_l(mu).  Everything
// between P(k) and the tables is linear: the natural-spline resampling of P(k)
// at the FFTLog nodes (twofast.c:399-401), the bias and window, the real FFT,
// the Gamma-ratio kernel and the c2r transform (twofast.c:362-483).  The only
// nonlinear step is the Akima interpolation of the tables at r, which is
// differentiated exactly (its slope weights |m_{i+1} - m_i| included).
//
// Kernels: adj_pair_kernel (per pair: J, table values and their Akima partials;
// scatters the table cotangents), adj_r2c_kernel (per spectrum and table: the
// adjoint of c2r, Gamma-ratio product and mode taper), adj_c2r_kernel (per
// spectrum and bias exponent q: the adjoint of the r2c transform), and
// adj_spline_kernel (per spectrum: the adjoint of the natural-spline
// resampling, one tridiagonal solve).
#include <math.h>

#include <vector>

#include "ctx.cuh"
#include "dual6.cuh"
#include "fft.cuh"
#include "qag.cuh"

namespace {

#define ADJ_MAX_L 8
#define ADJ_THREADS 128
enum { K00BB = 0, K00BF, K00FF, K02BF, K02FF, K04FF, NKIND };

#define ADJ_MAX_T 6
struct AdjArgs {
    int n_req, n_l, contrib, n_terms, tab_len, N, nk, n_q;
    int n_at;                // differentiated tables: 3 (den/RSD), 6 (with lensing)
    int t[ADJ_MAX_T];        // table index of I00, I02, I04 (and I11, I13, I20)
    int tq[ADJ_MAX_T];       // bias-exponent index of each table
    double inv_dlog; // N / ln(kmax/kmin)
    int has_b1, has_b2;
    int ls[ADJ_MAX_L];
};

struct AdjBg {
    Spl64 chi_of_z, z_of_chi, f, D1, b1, b2;
};

__device__ __forceinline__ int adj_find_request(const int64_t *__restrict__ off, int n, long long i)
{
    int lo = 0, hi = n;
    while (hi > lo + 1) {
        const int mid = (lo + hi) >> 1;
        if (off[mid] <= i)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

__device__ __forceinline__ double adj_legendre(int l, double x)
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

// per (request, separation): J integrals over the first GK61 panel, the three
// table values with their Akima partials; values and/or cotangents
__global__ void __launch_bounds__(ADJ_THREADS)
    adj_pair_kernel(AdjArgs a, AdjBg bg, const double *__restrict__ tab_x,
                    const double *__restrict__ tab_y, const int *__restrict__ req_spectrum,
                    const double *__restrict__ req_z_mean, const int64_t *__restrict__ req_offset,
                    const double *__restrict__ sep, long long total,
                    const double *__restrict__ bias_scale, const double *__restrict__ growth_scale,
                    const double *__restrict__ grad_out, double *__restrict__ value_out,
                    double *__restrict__ gY, double *__restrict__ g_bias,
                    double *__restrict__ g_growth, int *__restrict__ rejected, int *err)
{
    const long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= total) return;
    const int q = adj_find_request(req_offset, a.n_req, item);
    const int s = req_spectrum[q];
    const double r = sep[item], zm = req_z_mean[q];
    const double beta = bias_scale ? bias_scale[q] : 1.0;
    const double alpha = growth_scale ? growth_scale[q] : 1.0;
    // table interval at r (spline.cuh semantics) and the Akima stencil
    const int n = a.tab_len, first = CG_N_SMALL_R + 1;
    int i = -1;
    if (r >= tab_x[first] && r <= tab_x[n - 1]) {
        i = first + (int)(log(r) * a.inv_dlog);
        if (i > n - 2) i = n - 2;
        if (i < first) i = first;
        while (i > 0 && tab_x[i] > r) --i;
        while (i < n - 2 && tab_x[i + 1] <= r) ++i;
    }
    if (i < first + 2 || i + 3 > n - 1) {
        // the stencil would reach the sub-Mpc QAG entries or the table end
        cg_flag(err, CG_ERR_BOUNDS);
        if (value_out)
            for (int j = 0; j < a.n_l; ++j) value_out[item * a.n_l + j] = cg_nan<double>();
        return;
    }
    const double *y0 = tab_y + (size_t)s * a.n_terms * n;
    D6 I[3];
    for (int t = 0; t < 3; ++t) I[t] = akima_eval_d6(tab_x, y0 + (size_t)a.t[t] * n, n, i, r);
    // J integrals: first GK61 panel on [0, 1], mu = 2x - 1
    double J[NKIND][ADJ_MAX_L];
    for (int k = 0; k < NKIND; ++k)
        for (int j = 0; j < ADJ_MAX_L; ++j) J[k][j] = 0.0;
    const double chi_mean = spl_eval(bg.chi_of_z, zm);
    const bool den = a.contrib & COFFE_GPU_DEN, rsd = a.contrib & COFFE_GPU_RSD;
    const double bb = beta * beta, bf = beta * alpha, ff = alpha * alpha;
    // forward call: the integrand at each node for QUADPACK's acceptance test
    // of this first panel (sums per multipole: Kronrod, Gauss, |f|)
    double xiv[61], wkv[61], Kq[ADJ_MAX_L], Gq[ADJ_MAX_L], Aq[ADJ_MAX_L];
    for (int j = 0; j < ADJ_MAX_L; ++j) Kq[j] = Gq[j] = Aq[j] = 0.0;
    for (int node = 0; node < 61; ++node) {
        const int p = node >> 1;
        double x, wk, wg = 0.0;
        if (node == 60) {
            x = 0.5;
            wk = cg_gk_wgk[30];
        } else {
            const int g = p < 15 ? 2 * p + 1 : 2 * (p - 15);
            const double absc = 0.5 * cg_gk_xgk[g];
            x = (node & 1) ? 0.5 + absc : 0.5 - absc;
            wk = cg_gk_wgk[g];
            wg = p < 15 ? cg_gk_wg[p] : 0.0;
        }
        const double mu = 2 * x - 1;
        const double chi1 = chi_mean - r * mu * 0.5, chi2 = chi_mean + r * mu * 0.5;
        const double z1 = spl_eval(bg.z_of_chi, chi1), z2 = spl_eval(bg.z_of_chi, chi2);
        const double f1 = spl_eval(bg.f, z1), f2 = spl_eval(bg.f, z2);
        const double D = spl_eval(bg.D1, z1) * spl_eval(bg.D1, z2);
        const double b1 = a.has_b1 ? spl_eval(bg.b1, z1) : 1.0;
        const double b2 = a.has_b2 ? spl_eval(bg.b2, z2) : 1.0;
        const double mu2 = mu * mu, omm = 1 - mu2;
        const double Dd = 2 * chi_mean * chi_mean - mu2 * r * r * 0.5;
        const double ss = r * r * omm / Dd, c = 1 - ss, c2 = c * c;
        double co[NKIND] = {0, 0, 0, 0, 0, 0};
        if (den) co[K00BB] = b1 * b2;
        if (rsd) {
            const double ff = f1 * f2;
            const double q4 = omm * omm * (3 * c2 - 10 * c + 19) * 0.25 + 4 * mu2 * omm * (c2 - 5 * c - 2) +
                              4 * (3 * c2 - 1) * mu2 * mu2;
            co[K00FF] = ff * (1 + 2 * c2) / 15.;
            co[K02FF] = -ff / 21. * ((1 + 11 * c2) - 9 * c * (2 - ss) * omm);
            co[K04FF] = ff * q4 / 35.;
        }
        if (den && rsd) {
            const double g = (2 - ss) * omm / Dd;
            co[K00BF] = (b1 * f2 + b2 * f1) / 3.;
            co[K02BF] = -(b1 * f2 * (2. / 3. - g * chi1 * chi1) + b2 * f1 * (2. / 3. - g * chi2 * chi2));
        }
        for (int j = 0; j < a.n_l; ++j) {
            const double wp = wk * adj_legendre(a.ls[j], mu) * D;
            for (int k = 0; k < NKIND; ++k) J[k][j] += wp * co[k];
        }
        if (value_out) {
            const double xi = D * (I[0].v * (bb * co[K00BB] + bf * co[K00BF] + ff * co[K00FF]) +
                                   I[1].v * (bf * co[K02BF] + ff * co[K02FF]) +
                                   I[2].v * ff * co[K04FF]);
            xiv[node] = xi;
            wkv[node] = wk;
            for (int j = 0; j < a.n_l; ++j) {
                const double v = adj_legendre(a.ls[j], mu) * xi;
                Kq[j] += wk * v;
                Gq[j] += wg * v;
                Aq[j] += wk * fabs(v);
            }
        }
    }
    if (value_out && rejected) {
        // QUADPACK's test of the first panel (gsl qag.c) at the default
        // relative tolerance 1e-5: outputs it rejects would go through the
        // adaptive continuation in coffe_gpu_multipoles, so their first-panel
        // value is counted for the caller
        int nrej = 0;
        for (int j = 0; j < a.n_l; ++j) {
            double asc = 0.0;
            for (int node = 0; node < 61; ++node) {
                const int p = node >> 1;
                double mu = 0.0;
                if (node != 60) {
                    const int g = p < 15 ? 2 * p + 1 : 2 * (p - 15);
                    mu = (node & 1) ? cg_gk_xgk[g] : -cg_gk_xgk[g];
                }
                asc += wkv[node] * fabs(adj_legendre(a.ls[j], mu) * xiv[node] - 0.5 * Kq[j]);
            }
            const double result = 0.5 * Kq[j], resabs = 0.5 * Aq[j], resasc = 0.5 * asc;
            const double abserr = qk_rescale_error(0.5 * (Kq[j] - Gq[j]), resabs, resasc);
            const double tolerance = 1e-5 * fabs(result);
            const double round_off = 50 * qk_eps<double>() * resabs;
            const bool roundoff_fail = abserr <= round_off && abserr > tolerance;
            const bool ok = (abserr <= tolerance && abserr != resasc) || abserr == 0.0;
            if (!(ok || roundoff_fail)) ++nrej;
        }
        if (nrej) atomicAdd(rejected, nrej);
    }
    double gI[3] = {0, 0, 0}, gb = 0, gg = 0;
    for (int j = 0; j < a.n_l; ++j) {
        const double sc = (2 * a.ls[j] + 1) * 0.5;
        const double j00 = sc * (bb * J[K00BB][j] + bf * J[K00BF][j] + ff * J[K00FF][j]);
        const double j02 = sc * (bf * J[K02BF][j] + ff * J[K02FF][j]);
        const double j04 = sc * ff * J[K04FF][j];
        if (value_out) {
            const double v = I[0].v * j00 + I[1].v * j02 + I[2].v * j04;
            if (!isfinite(v)) cg_flag(err, CG_ERR_NONFINITE);
            value_out[item * a.n_l + j] = v;
        }
        if (grad_out) {
            const double G = grad_out[item * a.n_l + j];
            gI[0] += G * j00;
            gI[1] += G * j02;
            gI[2] += G * j04;
            gb += G * sc * (I[0].v * (2 * beta * J[K00BB][j] + alpha * J[K00BF][j]) +
                            I[1].v * alpha * J[K02BF][j]);
            gg += G * sc * (I[0].v * (beta * J[K00BF][j] + 2 * alpha * J[K00FF][j]) +
                            I[1].v * (beta * J[K02BF][j] + 2 * alpha * J[K02FF][j]) +
                            I[2].v * 2 * alpha * J[K04FF][j]);
        }
    }
    if (!grad_out) return;
    if (g_bias) atomicAdd(g_bias + q, gb);
    if (g_growth) atomicAdd(g_growth + q, gg);
    for (int t = 0; t < 3; ++t) {
        double *dst = gY + ((size_t)s * a.n_at + t) * n + (i - 2);
        for (int k = 0; k < 6; ++k) atomicAdd(dst + k, gI[t] * I[t].g[k]);
    }
}

// adjoint of [c2r, Gamma-ratio product, mode taper and conjugation] for one
// (spectrum, table): o = gY * postf; gX = w r2c(o) (w = 1 at k = 0, N/2,
// else 2); gA = gX conj(M); gU = modew conj(gA)
__global__ void adj_r2c_kernel(AdjArgs a, const double *__restrict__ gY,
                               const double *__restrict__ postf, const double2 *__restrict__ mcoef,
                               const double *__restrict__ modew, const double2 *__restrict__ tw,
                               double2 *__restrict__ gU)
{
    extern __shared__ __align__(16) unsigned char adj_smem[];
    double2 *buf = reinterpret_cast<double2 *>(adj_smem);
    const int s = blockIdx.x, t = blockIdx.y;
    const int N = a.N, M = N / 2;
    const int logM = 31 - __clz(M);
    const int term = a.t[t];
    const double *g = gY + ((size_t)s * a.n_at + t) * a.tab_len + CG_N_SMALL_R + 1;
    const double *pf = postf + (size_t)term * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double v = g[i] * pf[i];
        const int jj = __brev((unsigned)(i >> 1)) >> (32 - logM);
        if (i & 1)
            buf[jj].y = v;
        else
            buf[jj].x = v;
    }
    __syncthreads();
    smem_fft<double2>(buf, logM, tw, -1);
    const double2 *mc = mcoef + (size_t)term * (M + 1);
    double2 *out = gU + ((size_t)s * a.n_at + t) * (M + 1);
    for (int k = threadIdx.x; k <= M; k += blockDim.x) {
        const double2 zk = buf[k & (M - 1)];
        const double2 zm = buf[(M - k) & (M - 1)];
        const double ex = 0.5 * (zk.x + zm.x), ey = 0.5 * (zk.y - zm.y);
        const double ox = 0.5 * (zk.y + zm.y), oy = -0.5 * (zk.x - zm.x);
        const double2 w = tw[k];
        double yx = ex + (w.x * ox - w.y * oy);
        double yy = ey + (w.x * oy + w.y * ox);
        const double wt = (k == 0 || k == M) ? 1.0 : 2.0;
        yx *= wt;
        yy = (k == 0 || k == M) ? 0.0 : yy * wt;
        // gA = gX conj(M)
        const double2 m = mc[k];
        const double ar = yx * m.x + yy * m.y, ai = yy * m.x - yx * m.y;
        // gU = modew conj(gA)
        out[k] = make_double2(modew[k] * ar, -modew[k] * ai);
    }
}

// adjoint of the r2c transform for one (spectrum, q): u_bar_i =
// Re sum_{k <= N/2} H_k e^{2 pi i k i / N}, H = sum of gU over the tables with
// this q; evaluated as a c2r of H/2 (H_0, H_{N/2} real parts whole); times qfac
__global__ void adj_c2r_kernel(AdjArgs a, const double2 *__restrict__ gU,
                               const double *__restrict__ qfac, const double2 *__restrict__ tw,
                               double *__restrict__ Sbar)
{
    extern __shared__ __align__(16) unsigned char adj_smem[];
    double2 *buf = reinterpret_cast<double2 *>(adj_smem);
    const int s = blockIdx.x, qi = blockIdx.y;
    const int N = a.N, M = N / 2;
    const int logM = 31 - __clz(M);
    auto H = [&](int k) {
        double2 h = make_double2(0.0, 0.0);
        for (int t = 0; t < a.n_at; ++t)
            if (a.tq[t] == qi) {
                const double2 u = gU[((size_t)s * a.n_at + t) * (M + 1) + k];
                h.x += u.x;
                h.y += u.y;
            }
        if (k == 0 || k == M) return make_double2(h.x, 0.0);
        return make_double2(0.5 * h.x, 0.5 * h.y);
    };
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        const int km = M - k;
        const double2 xa = H(k), xb = H(km);
        const double fex = xa.x + xb.x, fey = xa.y - xb.y;
        const double dx = xa.x - xb.x, dy = xa.y + xb.y;
        const double2 w = tw[k];
        const double fox = dx * w.x + dy * w.y;
        const double foy = dy * w.x - dx * w.y;
        const int jj = __brev((unsigned)k) >> (32 - logM);
        buf[jj] = make_double2(fex - foy, fey + fox);
    }
    __syncthreads();
    smem_fft<double2>(buf, logM, tw, +1);
    const double *qf = qfac + (size_t)qi * N;
    double *o = Sbar + ((size_t)s * a.n_q + qi) * N;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double2 z = buf[i >> 1];
        o[i] = ((i & 1) ? z.y : z.x) * qf[i];
    }
}

// adjoint of the natural-spline resampling of P(k) at the FFTLog nodes
// (sample_input in fftlog.cu) for one spectrum; one thread, sequential in k
__global__ void adj_spline_kernel(AdjArgs a, const double *__restrict__ kx,
                                  const double *__restrict__ fac, const int *__restrict__ idx,
                                  const double *__restrict__ dxs, const double *__restrict__ Sbar,
                                  double *__restrict__ cbar, double *__restrict__ gpk,
                                  int n_spectra)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n_spectra) return;
    const int nk = a.nk, N = a.N, m = nk - 2;
    const double *invd = fac, *w = fac + nk, *gi = fac + 2 * nk;
    double *P = gpk + (size_t)s * nk;
    double *cb = cbar + (size_t)s * nk;
    for (int j = 0; j < nk; ++j) {
        P[j] = 0.0;
        cb[j] = 0.0;
    }
    for (int i = 0; i < N; ++i) {
        const int j = idx[i];
        if (j < 0) continue;
        double sb = 0.0;
        for (int q = 0; q < a.n_q; ++q) sb += Sbar[((size_t)s * a.n_q + q) * N + i];
        const double h = kx[j + 1] - kx[j], g = gi[j], dx = dxs[i];
        P[j] += sb * (1.0 - dx * g);
        P[j + 1] += sb * (dx * g);
        cb[j] += sb * (-2.0 * dx * h / 3.0 + dx * dx - dx * dx * dx * g / 3.0);
        cb[j + 1] += sb * (-dx * h / 3.0 + dx * dx * dx * g / 3.0);
    }
    // lambda = A^-1 cbar_interior (A symmetric): the forward elimination and
    // back substitution of the natural-spline system, in place in cb[1..m]
    for (int i = 0; i < m; ++i) {
        const double rhs = cb[i + 1];
        cb[i + 1] = i > 0 ? rhs - w[i] * cb[i] : rhs;
    }
    double ln = 0.0;
    for (int i = m - 1; i >= 0; --i) {
        ln = (cb[i + 1] - (kx[i + 2] - kx[i + 1]) * ln) * invd[i];
        cb[i + 1] = ln;
    }
    // rhs_i = 3 ((y_{i+2} - y_{i+1}) g_{i+1} - (y_{i+1} - y_i) g_i)
    for (int i = 0; i < m; ++i) {
        const double l = cb[i + 1];
        P[i] += 3.0 * gi[i] * l;
        P[i + 1] += -3.0 * (gi[i] + gi[i + 1]) * l;
        P[i + 2] += 3.0 * gi[i + 1] * l;
    }
}

} // namespace

// values (value_out) and/or cotangents (grad_out -> grad_pk, grad_bias,
// grad_growth); all arrays on the device; total = req_offset[n_req]
int multipoles_adjoint_run(coffe_gpu_ctx *ctx, int contrib, int n_req, const int *req_spectrum,
                           const double *req_z_mean, const int64_t *req_offset, const double *sep,
                           long long total, int n_l, const int *l, const double *bias_scale,
                           const double *growth_scale, const double *grad_out, double *value_out,
                           double *grad_pk, double *grad_bias, double *grad_growth)
{
    if (!ctx->bg_ready || !ctx->int_ready) {
        cg_set_error(ctx, "multipoles adjoint: %s not initialised",
                     ctx->bg_ready ? "integrals" : "background");
        return COFFE_GPU_ESTATE;
    }
    if (ctx->int_precision != COFFE_GPU_FP64) {
        cg_set_error(ctx, "multipoles adjoint: needs FP64 integral tables");
        return COFFE_GPU_EINVAL;
    }
    if (!(contrib & 7) || (contrib & ~7)) {
        cg_set_error(ctx, "multipoles adjoint: contrib must select den, rsd and/or len");
        return COFFE_GPU_EINVAL;
    }
    const bool len = (contrib & COFFE_GPU_LEN) != 0;
    const bool nonint = (contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD)) != 0;
    if (n_l < 1 || n_l > ADJ_MAX_L || n_req < 1) {
        cg_set_error(ctx, "multipoles adjoint: need 1 <= n_l <= %d, n_req >= 1", ADJ_MAX_L);
        return COFFE_GPU_EINVAL;
    }
    AdjArgs a;
    a.n_req = n_req;
    a.n_l = n_l;
    a.contrib = contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD);
    a.n_terms = ctx->n_terms;
    a.tab_len = (int)(ctx->N + CG_N_SMALL_R + 1);
    a.N = (int)ctx->N;
    a.nk = (int)ctx->nk;
    a.n_q = ctx->n_q;
    a.inv_dlog = (double)ctx->N / log(ctx->kmax / ctx->kmin);
    a.has_b1 = ctx->bias_set[0];
    a.has_b2 = ctx->bias_set[1];
    // the tables differentiated, in the lensing kernels' order (the den/RSD
    // integrand reads the first three)
    const int want[ADJ_MAX_T][2] = {{0, 0}, {0, 2}, {0, 4}, {1, 1}, {1, 3}, {2, 0}};
    a.n_at = len ? 6 : 3;
    for (int t = 0; t < a.n_at; ++t) {
        a.t[t] = cg_find_term(ctx, want[t][0], want[t][1]);
        if (a.t[t] < 0) {
            cg_set_error(ctx, "multipoles adjoint: the integral (n=%d, l=%d) is required",
                         want[t][0], want[t][1]);
            return COFFE_GPU_ESTATE;
        }
        a.tq[t] = ctx->term_q[a.t[t]];
    }
    for (int t = a.n_at; t < ADJ_MAX_T; ++t) a.t[t] = a.tq[t] = -1;
    for (int j = 0; j < ADJ_MAX_L; ++j) a.ls[j] = j < n_l ? l[j] : 0;
    for (int j = 0; j < n_l; ++j)
        if (l[j] < 0 || l[j] > 32) {
            cg_set_error(ctx, "multipoles adjoint: l = %d out of range", l[j]);
            return COFFE_GPU_EINVAL;
        }
    if (total <= 0) return COFFE_GPU_OK;
    const int N = a.N, M = N / 2, S = ctx->n_spectra;
    // each sub-buffer starts on a 256-byte boundary (gU holds 16-byte double2;
    // the table length N + 43 is odd, so gY's byte size is not a multiple of 16)
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t b_gY = al(sizeof(double) * (size_t)S * a.n_at * a.tab_len),
                 b_gU = al(sizeof(double2) * (size_t)S * a.n_at * (M + 1)),
                 b_Sb = al(sizeof(double) * (size_t)S * a.n_q * N),
                 b_cb = al(sizeof(double) * (size_t)S * a.nk);
    int st;
    if ((st = cg_ensure(ctx, ctx->adj_buf, b_gY + b_gU + b_Sb + b_cb))) return st;
    double *gY = (double *)ctx->adj_buf.p;
    double2 *gU = (double2 *)((char *)gY + b_gY);
    double *Sbar = (double *)((char *)gU + b_gU);
    double *cbar = (double *)((char *)Sbar + b_Sb);
    if (grad_out) {
        CG_CUDA(ctx, cudaMemsetAsync(gY, 0, b_gY, ctx->stream));
        if (grad_bias) CG_CUDA(ctx, cudaMemsetAsync(grad_bias, 0, sizeof(double) * n_req, ctx->stream));
        if (grad_growth) CG_CUDA(ctx, cudaMemsetAsync(grad_growth, 0, sizeof(double) * n_req, ctx->stream));
    }
    AdjBg bg{ctx->bg[BG_CHI_OF_Z].v64(), ctx->bg[BG_Z_OF_CHI].v64(), ctx->bg[BG_F].v64(),
             ctx->bg[BG_D1].v64(),       ctx->bias[0].v64(),        ctx->bias[1].v64()};
    // forward calls count the outputs whose first panel QUADPACK would reject
    // in the retry counter (coffe_gpu_multipoles_retries reads it)
    int *rejected = nullptr;
    if (value_out) {
        if ((st = cg_ensure(ctx, ctx->mp_retry, 256))) return st;
        rejected = (int *)ctx->mp_retry.p;
        CG_CUDA(ctx, cudaMemsetAsync(rejected, 0, sizeof(int), ctx->stream));
    }
    if (nonint) {
        adj_pair_kernel<<<(unsigned)((total + ADJ_THREADS - 1) / ADJ_THREADS), ADJ_THREADS, 0,
                          ctx->stream>>>(
            a, bg, (const double *)ctx->tab_x.p, (const double *)ctx->tab_y.p, req_spectrum,
            req_z_mean, req_offset, sep, total, bias_scale, growth_scale, grad_out, value_out, gY,
            grad_bias, grad_growth, rejected, ctx->d_err);
        if ((st = cg_after_launch(ctx, "adj_pair_kernel"))) return st;
    } else if (value_out) {
        CG_CUDA(ctx, cudaMemsetAsync(value_out, 0, sizeof(double) * (size_t)total * n_l,
                                     ctx->stream));
    }
    // the lensing terms: their values added to value_out, their table cotangents to gY
    if (len && (st = lensing_adjoint_run(ctx, contrib, n_req, req_spectrum, req_z_mean,
                                         req_offset, sep, total, n_l, l, bias_scale,
                                         growth_scale, grad_out, value_out, gY, a.n_at,
                                         grad_out ? grad_bias : nullptr,
                                         grad_out ? grad_growth : nullptr)))
        return st;
    if (!grad_out || !grad_pk) return COFFE_GPU_OK;
    const double2 *mcoef = (const double2 *)ctx->modec.p;
    const double *modew = (const double *)((const char *)ctx->modec.p + sizeof(double2) * (M + 1) * ctx->n_terms);
    const size_t smem = sizeof(double2) * M;
    CG_CUDA(ctx, cudaFuncSetAttribute(adj_r2c_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CG_CUDA(ctx, cudaFuncSetAttribute(adj_c2r_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    adj_r2c_kernel<<<dim3(S, a.n_at), 512, smem, ctx->stream>>>(a, gY, (const double *)ctx->postf.p, mcoef,
                                                           modew, (const double2 *)ctx->twid.p, gU);
    if ((st = cg_after_launch(ctx, "adj_r2c_kernel"))) return st;
    adj_c2r_kernel<<<dim3(S, a.n_q), 512, smem, ctx->stream>>>(a, gU, (const double *)ctx->qfac.p,
                                                               (const double2 *)ctx->twid.p, Sbar);
    if ((st = cg_after_launch(ctx, "adj_c2r_kernel"))) return st;
    adj_spline_kernel<<<(S + 63) / 64, 64, 0, ctx->stream>>>(
        a, (const double *)ctx->kgrid.p, (const double *)ctx->csfac.p, (const int *)ctx->samp_idx.p,
        (const double *)ctx->samp_dx.p, Sbar, cbar, grad_pk, S);
    if ((st = cg_after_launch(ctx, "adj_spline_kernel"))) return st;
    // the lensing lookups reach the r = 0 and sub-Mpc entries (their own QAG
    // integrals of P(k)); adj_spline_kernel has set grad_pk, these add to it
    if (len) return small_r_adjoint_run(ctx, gY, a.n_at, a.t, grad_pk);
    return COFFE_GPU_OK;
}
