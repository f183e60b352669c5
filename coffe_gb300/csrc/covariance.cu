// Flat-sky Gaussian covariance of the multipoles with the double-Bessel
// integrals by 2D FFTLog.
//
// Restates covariance_integrate_fftlog (covariance.c:357-470) with
// two_sph_bessel (twobessel.c:16-122, C branch), g_l / c_window_2d
// (utils.c:212-258) and the assembly of coffe_covariance_init
// (covariance.c:786-1059).  The FFTLog input is diagonal in (k1, k2) -- the
// reference fills an N x N matrix with k^3 P^p / dlnk on the diagonal -- so the
// forward 2D r2c transform is a 1D FFT F of the diagonal read at index
// (m + n) mod N; no N x N input is ever formed.  The inverse 2D c2r transform
// runs as one column FFT per retained frequency n (one CTA each, shared
// memory) followed by one row FFT per output row that the resampling needs.
//
// Resampling: the reference splines the whole N x N result with a bicubic
// interpolant whose knot derivatives come from natural cubic splines (GSL
// interp2d bicubic) and reads it at the separations.  A natural cubic spline's
// derivative at a knot depends on data d knots away with weight ~0.27^d, so
// the splines here are solved on the window of rows / columns around the
// separations plus CV_MARGIN = 64 knots on each side (0.27^64 ~ 1e-37): the
// same derivatives to rounding, without transforming rows nobody reads.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "cplx.cuh"
#include "ctx.cuh"

namespace {

#define CV_MARGIN 64
#define CV_THREADS 512
#define CV_NU 1.01
#define CV_WINDOW 0.25

__device__ __forceinline__ double2 dadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 dsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

// in-place radix-2 DIT FFT of N = 2^logN points held in bit-reversed order;
// tw[j] = exp(-2 pi i j / N), j < N/2; inverse: conjugate twiddles (unnormalised)
__device__ void cv_fft(double2 *buf, int logN, const double2 *__restrict__ tw, bool inverse)
{
    const int N = 1 << logN;
    for (int s = 1; s <= logN; ++s) {
        const int half = 1 << (s - 1);
        const int ts = N >> s;
        for (int b = threadIdx.x; b < N / 2; b += blockDim.x) {
            const int pos = b & (half - 1);
            const int i0 = ((b >> (s - 1)) << s) + pos;
            const int i1 = i0 + half;
            double2 w = __ldg(tw + pos * ts);
            if (inverse) w.y = -w.y;
            const double2 u = buf[i0], v = buf[i1];
            const double2 t = make_double2(w.x * v.x - w.y * v.y, w.x * v.y + w.y * v.x);
            buf[i0] = dadd(u, t);
            buf[i1] = dsub(u, t);
        }
        __syncthreads();
    }
}

__global__ void cv_twiddle_kernel(int N, double2 *tw)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N / 2) return;
    double s, c;
    sincospi(2.0 * j / N, &s, &c);
    tw[j] = make_double2(c, -s);
}

// sampled k_i, r_i = 1 / k_{N-1-i} (covariance.c:388-392, twobessel.c:43-45)
__global__ void cv_grid_kernel(int N, double kmin, double kmax, double *ks, double *r)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    ks[i] = kmin * pow(kmax / kmin, (double)i / N);
    r[N - 1 - i] = 1. / ks[i];
}

// F_p = FFT of diag(k^3 P(k)^p / dlnk) / k^(nu1 + nu2), one CTA per power
__global__ void cv_diag_fft_kernel(Spl64 P, int N, int logN, double step, const int *__restrict__ powers,
                                   const double *__restrict__ ks, const double2 *__restrict__ tw,
                                   double2 *__restrict__ F)
{
    extern __shared__ double2 cv_smem[];
    const int p = powers[blockIdx.x];
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double k = ks[i];
        const double d = pow(k, 3) * pow(spl_eval(P, k), p) / step;
        const int j = __brev((unsigned)i) >> (32 - logN);
        cv_smem[j] = make_double2(d / pow(k, CV_NU) / pow(k, CV_NU), 0.0);
    }
    __syncthreads();
    cv_fft(cv_smem, logN, tw, false);
    for (int i = threadIdx.x; i < N; i += blockDim.x) F[(size_t)blockIdx.x * N + i] = cv_smem[i];
}

// per-frequency factor (k0 r0)^(-i eta_m) g_l(eta_m) (twobessel.c:73-105):
// fac[m], m <= N/2, and its conjugate mirror for m > N/2
__global__ void cv_factor_kernel(const int *__restrict__ ls, int N, double dlnk, double kr,
                                 double2 *__restrict__ fac, int *err)
{
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= N) return;
    const double l = ls[blockIdx.y];
    const int hN = N / 2;
    const int mm = m <= hN ? m : N - m;
    const double eta = 2 * CG_PI / dlnk / N * mm;
    // g_l = exp(z ln 2 + lnGamma((l + z)/2) - lnGamma((3 + l - z)/2)), z = nu + i eta
    cplx a, b;
    const bool ok = cx_lgamma_lanczos(cx((l + CV_NU) / 2., eta / 2.), &a) &&
                    cx_lgamma_lanczos(cx((3. + l - CV_NU) / 2., -eta / 2.), &b);
    if (!ok) cg_flag(err, CG_ERR_NONFINITE);
    const double er = CV_NU * log(2.) + a.re - b.re, ei = eta * log(2.) + a.im - b.im;
    double gr = exp(er) * cos(ei), gi = exp(er) * sin(ei);
    double pr = cos(-eta * log(kr)), pi_ = sin(-eta * log(kr));
    if (m > hN) {
        pi_ = -pi_;
        gi = -gi;
    }
    fac[(size_t)blockIdx.y * N + m] = make_double2(pr * gr - pi_ * gi, pr * gi + pi_ * gr);
}

__device__ __forceinline__ double cv_window(long t, long ncut)
{
    return (double)t / ncut - 1. / (2. * CG_PI) * sin(2. * t * CG_PI / ncut);
}

struct CvJob {
    int fidx;  // index of F (power)
    int l1idx; // index of the row factor (l1)
    int l2idx; // index of the column factor (l2)
};

// column pass: CTA (n, job) builds X[m] = conj(F[(m+n) mod N] W_c(n) W_r(m)
// C(n) R(m)) for all m, inverse FFT along m, keeps rows [lo, lo + W)
__global__ void cv_column_kernel(int N, int logN, int lo, int W, const CvJob *__restrict__ jobs,
                                 const double2 *__restrict__ F, const double2 *__restrict__ fac,
                                 const double2 *__restrict__ tw, double2 *__restrict__ V)
{
    extern __shared__ double2 cv_smem[];
    const int n = blockIdx.x;
    const CvJob jb = jobs[blockIdx.y];
    const int hN = N / 2;
    const long nc = (long)(hN * CV_WINDOW);
    const double wc = (hN - n <= nc) ? cv_window(hN - n, nc) : 1.0;
    const double2 C = fac[(size_t)jb.l2idx * N + n];
    const double2 *Fp = F + (size_t)jb.fidx * N;
    const double2 *R1 = fac + (size_t)jb.l1idx * N;
    for (int m = threadIdx.x; m < N; m += blockDim.x) {
        double wr = 1.0;
        if (m <= hN && hN - m <= nc) wr = cv_window(hN - m, nc);
        if (m >= hN + 1 && m - hN - 1 <= nc) wr = cv_window(m - hN - 1, nc);
        const double2 f = Fp[(m + n) & (N - 1)];
        const double2 R = R1[m];
        const double vr = f.x * wc * wr, vi = f.y * wc * wr;
        const double fr = C.x * R.x - C.y * R.y, fi = C.x * R.y + C.y * R.x;
        const double tr = vr * fr - vi * fi, ti = vr * fi + vi * fr;
        const int j = __brev((unsigned)m) >> (32 - logN);
        cv_smem[j] = make_double2(tr, -ti);
    }
    __syncthreads();
    cv_fft(cv_smem, logN, tw, true);
    double2 *out = V + ((size_t)blockIdx.y * (hN + 1) + n) * W;
    for (int a = threadIdx.x; a < W; a += blockDim.x) out[a] = cv_smem[lo + a];
}

// row pass: CTA (a, job) completes row lo + a Hermitian-symmetrically along n
// (Im of n = 0, N/2 dropped, as a c2r transform does), inverse FFT, keeps
// columns [lo, lo + W) scaled by pi / (16 N^2 r_b^nu r_a^nu)
__global__ void cv_row_kernel(int N, int logN, int lo, int W, const double2 *__restrict__ V,
                              const double *__restrict__ r, const double2 *__restrict__ tw,
                              double *__restrict__ res)
{
    extern __shared__ double2 cv_smem[];
    const int a = blockIdx.x;
    const int hN = N / 2;
    const double2 *Vj = V + (size_t)blockIdx.y * (hN + 1) * W;
    for (int n = threadIdx.x; n < N; n += blockDim.x) {
        double2 c;
        if (n <= hN) {
            c = Vj[(size_t)n * W + a];
            if (n == 0 || n == hN) c.y = 0.0;
        } else {
            c = Vj[(size_t)(N - n) * W + a];
            c.y = -c.y;
        }
        const int j = __brev((unsigned)n) >> (32 - logN);
        cv_smem[j] = c;
    }
    __syncthreads();
    cv_fft(cv_smem, logN, tw, true);
    const double ra = r[lo + a];
    double *o = res + ((size_t)blockIdx.y * W + a) * W;
    for (int b = threadIdx.x; b < W; b += blockDim.x)
        o[b] = cv_smem[lo + b].x * CG_PI /
               (16. * (double)N * (double)N * pow(r[lo + b], CV_NU) * pow(ra, CV_NU));
}

// natural cubic spline (the oracle's / GSL's cspline) along one line of W
// knots x: values y[i * ys], derivative at every knot into d[i * ys];
// scratch: 2 W doubles
__device__ void cv_spline_deriv(const double *__restrict__ x, const double *y, long ys, double *d,
                                double *diag, double *rhs, int W)
{
    const int m = W - 2;
    for (int i = 0; i < m; ++i) {
        const double h_i = x[i + 1] - x[i], h_ip1 = x[i + 2] - x[i + 1];
        const double g_i = 1.0 / h_i, g_ip1 = 1.0 / h_ip1;
        diag[i] = 2.0 * (h_ip1 + h_i);
        rhs[i] = 3.0 * ((y[(i + 2) * ys] - y[(i + 1) * ys]) * g_ip1 - (y[(i + 1) * ys] - y[i * ys]) * g_i);
    }
    for (int i = 1; i < m; ++i) {
        const double off = x[i + 1] - x[i]; // off[i - 1] = h_i
        const double w = off / diag[i - 1];
        diag[i] -= w * off;
        rhs[i] -= w * rhs[i - 1];
    }
    // back substitution, c stored in rhs[] shifted: c[i + 1] -> rhs[i]; c[0] = c[W-1] = 0
    rhs[m - 1] = rhs[m - 1] / diag[m - 1];
    for (int i = m - 1; i-- > 0;) rhs[i] = (rhs[i] - (x[i + 2] - x[i + 1]) * rhs[i + 1]) / diag[i];
    auto c = [&](int i) { return (i == 0 || i == W - 1) ? 0.0 : rhs[i - 1]; };
    for (int i = 0; i + 1 < W; ++i) {
        const double h = x[i + 1] - x[i];
        d[i * ys] = (y[(i + 1) * ys] - y[i * ys]) / h - h * (c(i + 1) + 2.0 * c(i)) / 3.0;
    }
    {
        const int i = W - 2;
        const double h = x[i + 1] - x[i];
        const double b = (y[(i + 1) * ys] - y[i * ys]) / h - h * (c(i + 1) + 2.0 * c(i)) / 3.0;
        const double dd = (c(i + 1) - c(i)) / (3.0 * h);
        d[(W - 1) * ys] = b + 2 * c(i) * h + 3 * dd * h * h;
    }
}

// zx[a][b] = d/dx along a (r1) at fixed b; one thread per (job, b)
__global__ void cv_zx_kernel(int W, int n_jobs, const double *__restrict__ xr,
                             const double *__restrict__ res, double *__restrict__ zx,
                             double *__restrict__ scratch)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)n_jobs * W) return;
    const long job = t / W, b = t % W;
    const double *z = res + job * W * W + b;
    cv_spline_deriv(xr, z, W, zx + job * W * W + b, scratch + t * 2 * W, scratch + t * 2 * W + W, W);
}

// zy[a][b], zxy[a][b]: d/dy along b (r2) of z and zx at fixed a
__global__ void cv_zy_kernel(int W, int n_jobs, const double *__restrict__ xr,
                             const double *__restrict__ res, const double *__restrict__ zx,
                             double *__restrict__ zy, double *__restrict__ zxy,
                             double *__restrict__ scratch)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)n_jobs * W) return;
    const long job = t / W, a = t % W;
    const long off = job * W * W + a * W;
    double *s1 = scratch + t * 2 * W;
    cv_spline_deriv(xr, res + off, 1, zy + off, s1, s1 + W, W);
    cv_spline_deriv(xr, zx + off, 1, zxy + off, s1, s1 + W, W);
}

__device__ __forceinline__ int cv_cell(const double *__restrict__ x, int n, double v)
{
    int lo = 0, hi = n - 1;
    while (hi > lo + 1) {
        const int mid = (lo + hi) / 2;
        if (x[mid] > v)
            hi = mid;
        else
            lo = mid;
    }
    return lo;
}

// bicubic Hermite patch at (sep[m], sep[n]) (the oracle's bicubic_eval)
__global__ void cv_eval_kernel(int W, int n_jobs, int ns, const double *__restrict__ xr,
                               const double *__restrict__ sep, const double *__restrict__ res,
                               const double *__restrict__ zx, const double *__restrict__ zy,
                               const double *__restrict__ zxy, double *__restrict__ out, int *err)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)n_jobs * ns * ns) return;
    const long job = t / (ns * ns);
    const int n = (int)((t / ns) % ns), m = (int)(t % ns);
    const double xv = sep[m], yv = sep[n];
    const int i = cv_cell(xr, W, xv), j = cv_cell(xr, W, yv);
    const double dx = xr[i + 1] - xr[i], dy = xr[j + 1] - xr[j];
    const double tt = (xv - xr[i]) / dx, u = (yv - xr[j]) / dy;
    const double ht[2] = {(2 * tt - 3) * tt * tt + 1, (3 - 2 * tt) * tt * tt};
    const double gt[2] = {((tt - 2) * tt + 1) * tt, (tt - 1) * tt * tt};
    const double hu[2] = {(2 * u - 3) * u * u + 1, (3 - 2 * u) * u * u};
    const double gu[2] = {((u - 2) * u + 1) * u, (u - 1) * u * u};
    const long base = job * W * W;
    double v = 0;
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) {
            // z(x_{i+a}, y_{j+b}) = res[i+a][j+b]
            const long q = base + (long)(i + a) * W + (j + b);
            v += res[q] * ht[a] * hu[b] + zx[q] * dx * gt[a] * hu[b] + zy[q] * dy * ht[a] * gu[b] +
                 zxy[q] * dx * dy * gt[a] * gu[b];
        }
    if (!isfinite(v)) cg_flag(err, CG_ERR_NONFINITE);
    out[job * ns * ns + (long)ns * n + m] = v;
}

__device__ __forceinline__ double cv_coeff(double b1, double b2, double f, int ell)
{
    switch (ell) {
    case 0: return b1 * b2 + (b1 + b2) * f / 3 + f * f / 5.;
    case 2: return 2 * (b1 + b2) * f / 3. + 4 * f * f / 7.;
    case 4: return 8 * f * f / 35.;
    default: return 0;
    }
}
__device__ __forceinline__ int cv_sign(int m) { return abs(m) % 2 == 0 ? 1 : -1; }

struct CvZ {
    double V, b, f, D1, n1, n2, pix;
};

#define CV_VOL_PANELS 16
#define CV_VOL_NODES 16
// per-z scalars: volume, bias, growth rate, D1.  averaged = 0: bins (z_mean,
// deltaz) with the shell volume (covariance.c:796-810); averaged = 1: windows
// (z_min, z_max) at z = (z_min + z_max)/2 with the effective volume
// 4 pi fsky / int dz / (conformal_H chi^2 (1 + z)) / (H0 h)^2 (covariance.c:
// 811-840, 150-162), the integral by CV_VOL_PANELS Gauss-Legendre panels of
// CV_VOL_NODES nodes, uniform in ln z (the integrand rises as 1/chi^2).
__global__ void cv_zscalars_kernel(int nz, Spl64 chi_of_z, Spl64 f, Spl64 D1, Spl64 bias,
                                   Spl64 confH, double H0h, int has_bias, int contrib,
                                   int averaged, const double *__restrict__ zin,
                                   const double *__restrict__ gl, CvZ *__restrict__ zs)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nz) return;
    // zin per bin: (z_mean, deltaz) or (z_min, z_max), fsky, density1, density2, pixelsize
    const double za = zin[6 * k], zb = zin[6 * k + 1], fsky = zin[6 * k + 2];
    CvZ o;
    double z;
    if (averaged) {
        z = 0.5 * (za + zb);
        const double la = log(za), dl = (log(zb) - la) / CV_VOL_PANELS;
        double vint = 0;
        for (int p = 0; p < CV_VOL_PANELS; ++p) {
            const double a = exp(la + p * dl), b = exp(la + (p + 1) * dl);
            const double c = 0.5 * (a + b), h = 0.5 * (b - a);
            double part = 0;
            for (int i = 0; i < CV_VOL_NODES; ++i) {
                const double zz = c + h * gl[i];
                const double chi = spl_eval(chi_of_z, zz);
                part += gl[CV_VOL_NODES + i] / (spl_eval(confH, zz) * chi * chi * (1 + zz));
            }
            vint += h * part;
        }
        o.V = 4 * CG_PI * fsky / vint / (H0h * H0h);
    } else {
        z = za;
        const double c1 = spl_eval(chi_of_z, z - zb), c2 = spl_eval(chi_of_z, z + zb);
        o.V = 4 * CG_PI * fsky * (pow(c2, 3) - pow(c1, 3)) / 3.;
    }
    o.b = (contrib & COFFE_GPU_DEN) ? (has_bias ? spl_eval(bias, z) : 1.0) : 0.0;
    o.f = (contrib & COFFE_GPU_RSD) ? spl_eval(f, z) : 0.0;
    o.D1 = spl_eval(D1, z);
    o.n1 = zin[6 * k + 3];
    o.n2 = zin[6 * k + 4];
    o.pix = zin[6 * k + 5];
    zs[k] = o;
}

// covariance in (z, l1, r1, l2, r2) order (covariance.c:866-1059), one
// population: ipk / ipk2 [(i * nl + j) * ns * ns + ns * n + m], already scaled
__global__ void cv_assemble_kernel(int nz, int nl, int ns, const int *__restrict__ ls,
                                   const double *__restrict__ LI /* [nl][nl][3][3] */,
                                   const CvZ *__restrict__ zs, const double *__restrict__ sep,
                                   const double *__restrict__ ipk, const double *__restrict__ ipk2,
                                   double *__restrict__ out, int *err)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long per_z = (long)nl * ns * nl * ns;
    if (t >= nz * per_z) return;
    const int zk = (int)(t / per_z);
    long r_ = t % per_z;
    const int n = (int)(r_ % ns);
    r_ /= ns;
    const int j = (int)(r_ % nl);
    r_ /= nl;
    const int m = (int)(r_ % ns);
    const int i = (int)(r_ / ns);
    const CvZ Z = zs[zk];
    const int l1 = ls[i], l2 = ls[j];
    const double *L = LI + ((size_t)i * nl + j) * 9;
    double cosmic = 0;
    for (int a = 0; a <= 4; a += 2)
        for (int bb = 0; bb <= 4; bb += 2)
            cosmic += (cv_coeff(Z.b, Z.b, Z.f, a) * cv_coeff(Z.b, Z.b, Z.f, bb) +
                       cv_sign(bb) * cv_coeff(Z.b, Z.b, Z.f, a) * cv_coeff(Z.b, Z.b, Z.f, bb)) *
                      L[(a / 2) * 3 + bb / 2];
    cosmic /= 4.;
    double mixed = 0;
    for (int a = 0; a <= 4; a += 2)
        mixed += (cv_coeff(Z.b, Z.b, Z.f, a) / Z.n2 + cv_coeff(Z.b, Z.b, Z.f, a) / Z.n1 +
                  cv_coeff(Z.b, Z.b, Z.f, a) / Z.n2 + cv_coeff(Z.b, Z.b, Z.f, a) / Z.n1) *
                 L[(a / 2) * 3];
    mixed /= 8.;
    const double pois = (l1 == l2 && m == n) ? (2 * l1 + 1) / 4. / CG_PI * (1 + cv_sign(l2)) /
                                                   sep[n] / sep[m] / Z.pix / Z.n1 / Z.n2 / Z.V
                                             : 0.0;
    const size_t q = ((size_t)i * nl + j) * ns * ns + (size_t)ns * n + m;
    const double cm = cv_sign((l2 - l1) / 2) * cv_sign(l1 + l2) * Z.D1 * Z.D1 * ipk[q] * mixed / Z.V;
    const double cc = cv_sign((l2 - l1) / 2) * Z.D1 * Z.D1 * Z.D1 * Z.D1 * ipk2[q] * cosmic / Z.V;
    const double v = pois + cm + cc;
    if (!isfinite(v)) cg_flag(err, CG_ERR_NONFINITE);
    out[t] = v;
}

// scales the FFTLog integrals and fills the lower (l1 > l2) blocks by
// transposition (covariance.c:752-784)
__global__ void cv_scale_kernel(int nl, int ns, const int *__restrict__ ls,
                                const int *__restrict__ job_of, const double *__restrict__ raw,
                                double *__restrict__ ipk, double *__restrict__ ipk2)
{
    const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long)nl * nl * ns * ns) return;
    const int m = (int)(t % ns), n = (int)((t / ns) % ns);
    const int j = (int)((t / ((long)ns * ns)) % nl), i = (int)(t / ((long)ns * ns * nl));
    const int l1 = ls[i], l2 = ls[j];
    // the (min, max) block holds the computed values; the other is its transpose
    const int ii = i <= j ? i : j, jj = i <= j ? j : i;
    const int mm = i <= j ? m : n, nn = i <= j ? n : m;
    const int job1 = job_of[(ii * nl + jj) * 2], job2 = job_of[(ii * nl + jj) * 2 + 1];
    const int L1 = ls[ii], L2 = ls[jj];
    const double v1 = raw[(size_t)job1 * ns * ns + (size_t)ns * nn + mm] * (2 * L1 + 1) *
                      (2 * L2 + 1) * 2. / CG_PI / CG_PI;
    const double v2 = raw[(size_t)job2 * ns * ns + (size_t)ns * nn + mm] * (2 * L1 + 1) *
                      (2 * L2 + 1) / CG_PI / CG_PI;
    (void)l1;
    (void)l2;
    ipk[t] = v1;
    ipk2[t] = v2;
}

// w3j (l1 l2 l3; 0 0 0)^2 by the closed form, host side
double w3j0_sq(int l1, int l2, int l3)
{
    const int J = l1 + l2 + l3;
    if (J % 2 || l3 < abs(l1 - l2) || l3 > l1 + l2) return 0.0;
    const int g = J / 2;
    const double lr = lgamma(J - 2. * l1 + 1) + lgamma(J - 2. * l2 + 1) + lgamma(J - 2. * l3 + 1) -
                      lgamma(J + 2.) +
                      2 * (lgamma(g + 1.) - lgamma(g - l1 + 1.) - lgamma(g - l2 + 1.) -
                           lgamma(g - l3 + 1.));
    return exp(lr);
}

// int P_n P_m P_a P_b dmu (coffe_legendre_integral, common.c:1370-1394)
double legendre_integral(int n, int m, int a, int b)
{
    if ((n + m + a + b) % 2 != 0) return 0;
    const int lo = std::max(abs(n - m), abs(a - b));
    const int hi = std::min(n + m, a + b);
    double r = 0;
    for (int L = lo; L <= hi; ++L) r += (2. * L + 1) * w3j0_sq(n, m, L) * w3j0_sq(a, b, L);
    return 2 * r;
}

struct CvPlan {
    int N, logN, lo, W;
    double kmin, kmax, step, dlnk, kr;
};

// validates the grid, computes the row/column window of the separations
int cv_plan(coffe_gpu_ctx *ctx, const double *k, size_t nk, size_t N, const double *sep, int ns,
            CvPlan &P)
{
    if (N < 64 || N > 8192 || (N & (N - 1))) {
        cg_set_error(ctx, "covariance: N must be a power of two in [64, 8192] (got %zu)", N);
        return COFFE_GPU_EINVAL;
    }
    if (nk < 5 || !(k[0] > 0) || !(k[nk - 1] > k[0])) {
        cg_set_error(ctx, "covariance: need >= 5 increasing positive k");
        return COFFE_GPU_EINVAL;
    }
    if (ns < 1) {
        cg_set_error(ctx, "covariance: need at least one separation");
        return COFFE_GPU_EINVAL;
    }
    P.N = (int)N;
    P.logN = 0;
    while ((1 << P.logN) < P.N) ++P.logN;
    P.kmin = k[0];
    P.kmax = k[nk - 1];
    P.step = log(P.kmax / P.kmin) / N;
    // host copy of the r grid to find the window (same formulas as the device)
    std::vector<double> r(N);
    for (size_t i = 0; i < N; ++i) r[N - 1 - i] = 1. / (P.kmin * pow(P.kmax / P.kmin, (double)i / N));
    const double k1 = P.kmin * pow(P.kmax / P.kmin, 1.0 / N);
    P.dlnk = log(k1 / P.kmin);
    P.kr = P.kmin * r[0];
    int imin = (int)N, imax = -1;
    for (int q = 0; q < ns; ++q) {
        if (!(sep[q] >= r[0] && sep[q] <= r[N - 1])) {
            cg_set_error(ctx, "covariance: separation %g outside the FFTLog grid [%g, %g]", sep[q],
                         r[0], r[N - 1]);
            return COFFE_GPU_EINVAL;
        }
        const int i = (int)(std::upper_bound(r.begin(), r.end(), sep[q]) - r.begin()) - 1;
        imin = std::min(imin, std::max(i, 0));
        imax = std::max(imax, std::min(i + 1, (int)N - 1));
    }
    P.lo = std::max(0, imin - CV_MARGIN);
    const int hi = std::min((int)N, imax + 1 + CV_MARGIN);
    P.W = hi - P.lo;
    if (P.W < 4) {
        cg_set_error(ctx, "covariance: window of %d knots is too small", P.W);
        return COFFE_GPU_EINVAL;
    }
    return COFFE_GPU_OK;
}

// the FFTLog double-Bessel integrals for jobs (power, l1, l2): raw values
// [job][ns * n + m] at (sep[m], sep[n]); all pointers host
int cv_integrals(coffe_gpu_ctx *ctx, const double *k, const double *pk, size_t nk, size_t N,
                 int n_jobs, const int *power, const int *l1, const int *l2, const double *sep,
                 int ns, double *d_raw /* device, n_jobs * ns * ns */)
{
    CvPlan P;
    int st = cv_plan(ctx, k, nk, N, sep, ns, P);
    if (st) return st;
    // distinct powers and multipoles
    std::vector<int> pw, lv;
    std::vector<CvJob> jobs(n_jobs);
    for (int j = 0; j < n_jobs; ++j) {
        if (power[j] < 1 || power[j] > 4 || l1[j] < 0 || l2[j] < 0 || l1[j] > 64 || l2[j] > 64) {
            cg_set_error(ctx, "covariance: job %d has power %d, l1 %d, l2 %d", j, power[j], l1[j], l2[j]);
            return COFFE_GPU_EINVAL;
        }
        auto fi = std::find(pw.begin(), pw.end(), power[j]);
        if (fi == pw.end()) { pw.push_back(power[j]); fi = pw.end() - 1; }
        jobs[j].fidx = (int)(fi - pw.begin());
        auto a = std::find(lv.begin(), lv.end(), l1[j]);
        if (a == lv.end()) { lv.push_back(l1[j]); a = lv.end() - 1; }
        jobs[j].l1idx = (int)(a - lv.begin());
        auto b = std::find(lv.begin(), lv.end(), l2[j]);
        if (b == lv.end()) { lv.push_back(l2[j]); b = lv.end() - 1; }
        jobs[j].l2idx = (int)(b - lv.begin());
    }
    const int Nn = P.N, hN = Nn / 2, W = P.W;
    // device buffers in one allocation
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t b_k = al(sizeof(double) * (nk + nk)), b_grid = al(sizeof(double) * 2 * Nn),
                 b_tw = al(sizeof(double2) * (hN)), b_F = al(sizeof(double2) * pw.size() * Nn),
                 b_fac = al(sizeof(double2) * lv.size() * Nn), b_meta = al(sizeof(int) * (pw.size() + lv.size()) + sizeof(CvJob) * n_jobs),
                 b_V = al(sizeof(double2) * (size_t)n_jobs * (hN + 1) * W),
                 b_res = al(sizeof(double) * (size_t)n_jobs * W * W),
                 b_scr = al(sizeof(double) * (size_t)n_jobs * W * 2 * W),
                 b_sep = al(sizeof(double) * ns);
    const size_t total = b_k + b_grid + b_tw + b_F + b_fac + b_meta + b_V + 3 * b_res + b_res +
                         b_scr + b_sep;
    if ((st = cg_ensure(ctx, ctx->cov_buf, total))) return st;
    char *base = (char *)ctx->cov_buf.p;
    double *d_k = (double *)base; base += b_k;
    double *d_ks = (double *)base, *d_r = d_ks + Nn; base += b_grid;
    double2 *d_tw = (double2 *)base; base += b_tw;
    double2 *d_F = (double2 *)base; base += b_F;
    double2 *d_fac = (double2 *)base; base += b_fac;
    int *d_pw = (int *)base, *d_lv = d_pw + pw.size();
    CvJob *d_jobs = (CvJob *)(d_lv + lv.size()); base += b_meta;
    double2 *d_V = (double2 *)base; base += b_V;
    double *d_res = (double *)base; base += b_res;
    double *d_zx = (double *)base; base += b_res;
    double *d_zy = (double *)base; base += b_res;
    double *d_zxy = (double *)base; base += b_res;
    double *d_scr = (double *)base; base += b_scr;
    double *d_sep = (double *)base; base += b_sep;
    // inputs (host staging is synchronous below)
    std::vector<char> meta(sizeof(int) * (pw.size() + lv.size()) + sizeof(CvJob) * n_jobs);
    memcpy(meta.data(), pw.data(), sizeof(int) * pw.size());
    memcpy(meta.data() + sizeof(int) * pw.size(), lv.data(), sizeof(int) * lv.size());
    memcpy(meta.data() + sizeof(int) * (pw.size() + lv.size()), jobs.data(), sizeof(CvJob) * n_jobs);
    CG_CUDA(ctx, cudaMemcpyAsync(d_k, k, sizeof(double) * nk, cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(d_k + nk, pk, sizeof(double) * nk, cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(d_pw, meta.data(), meta.size(), cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(d_sep, sep, sizeof(double) * ns, cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // Akima spline of P(k) (the reference's power_spectrum_norm)
    if ((st = spline_build(ctx, ctx->cov_pk, d_k, d_k + nk, (int)nk))) return st;
    cv_twiddle_kernel<<<(hN + 255) / 256, 256, 0, ctx->stream>>>(Nn, d_tw);
    if ((st = cg_after_launch(ctx, "cv_twiddle_kernel"))) return st;
    cv_grid_kernel<<<(Nn + 255) / 256, 256, 0, ctx->stream>>>(Nn, P.kmin, P.kmax, d_ks, d_r);
    if ((st = cg_after_launch(ctx, "cv_grid_kernel"))) return st;
    const size_t smem = sizeof(double2) * Nn;
    CG_CUDA(ctx, cudaFuncSetAttribute(cv_diag_fft_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CG_CUDA(ctx, cudaFuncSetAttribute(cv_column_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CG_CUDA(ctx, cudaFuncSetAttribute(cv_row_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    cv_diag_fft_kernel<<<(unsigned)pw.size(), CV_THREADS, smem, ctx->stream>>>(
        ctx->cov_pk.v64(), Nn, P.logN, P.step, d_pw, d_ks, d_tw, d_F);
    if ((st = cg_after_launch(ctx, "cv_diag_fft_kernel"))) return st;
    cv_factor_kernel<<<dim3((Nn + 255) / 256, (unsigned)lv.size()), 256, 0, ctx->stream>>>(
        d_lv, Nn, P.dlnk, P.kr, d_fac, ctx->d_err);
    if ((st = cg_after_launch(ctx, "cv_factor_kernel"))) return st;
    cv_column_kernel<<<dim3(hN + 1, n_jobs), CV_THREADS, smem, ctx->stream>>>(
        Nn, P.logN, P.lo, W, d_jobs, d_F, d_fac, d_tw, d_V);
    if ((st = cg_after_launch(ctx, "cv_column_kernel"))) return st;
    cv_row_kernel<<<dim3(W, n_jobs), CV_THREADS, smem, ctx->stream>>>(Nn, P.logN, P.lo, W, d_V,
                                                                      d_r, d_tw, d_res);
    if ((st = cg_after_launch(ctx, "cv_row_kernel"))) return st;
    const long lines = (long)n_jobs * W;
    cv_zx_kernel<<<(unsigned)((lines + 127) / 128), 128, 0, ctx->stream>>>(W, n_jobs, d_r + P.lo,
                                                                          d_res, d_zx, d_scr);
    if ((st = cg_after_launch(ctx, "cv_zx_kernel"))) return st;
    cv_zy_kernel<<<(unsigned)((lines + 127) / 128), 128, 0, ctx->stream>>>(
        W, n_jobs, d_r + P.lo, d_res, d_zx, d_zy, d_zxy, d_scr);
    if ((st = cg_after_launch(ctx, "cv_zy_kernel"))) return st;
    const long nout = (long)n_jobs * ns * ns;
    cv_eval_kernel<<<(unsigned)((nout + 255) / 256), 256, 0, ctx->stream>>>(
        W, n_jobs, ns, d_r + P.lo, d_sep, d_res, d_zx, d_zy, d_zxy, d_raw, ctx->d_err);
    return cg_after_launch(ctx, "cv_eval_kernel");
}

} // namespace

extern "C" int coffe_gpu_covariance_integrals(coffe_gpu_ctx_t *ctx, const double *k,
                                              const double *pk, size_t nk, size_t N, int n_jobs,
                                              const int *power, const int *l1, const int *l2,
                                              const double *sep, int n_sep, double *out)
{
    if (!ctx || !k || !pk || !power || !l1 || !l2 || !sep || !out || n_jobs < 1 || n_sep < 1)
        return COFFE_GPU_EINVAL;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    int st;
    const size_t bytes = sizeof(double) * (size_t)n_jobs * n_sep * n_sep;
    if ((st = cg_ensure(ctx, ctx->cov_out, bytes))) return st;
    if ((st = cv_integrals(ctx, k, pk, nk, N, n_jobs, power, l1, l2, sep, n_sep,
                           (double *)ctx->cov_out.p)))
        return st;
    CG_CUDA(ctx, cudaMemcpyAsync(out, ctx->cov_out.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return cg_check_device_errors(ctx, "covariance_integrals");
}

// shared by coffe_gpu_covariance_multipoles (averaged = 0: za = z_mean,
// zb = deltaz) and coffe_gpu_average_covariance_multipoles (averaged = 1:
// za = z_min, zb = z_max)
static int covariance_impl(coffe_gpu_ctx_t *ctx, int contrib, const double *k, const double *pk,
                           size_t nk, size_t N, int n_z, int averaged, const double *za,
                           const double *zb, const double *fsky, const double *density1,
                           const double *density2, const double *pixelsize, int n_l, const int *l,
                           int n_sep, const double *sep, double *out)
{
    if (!ctx || !k || !pk || !za || !zb || !fsky || !density1 || !density2 || !pixelsize ||
        !l || !sep || !out || n_z < 1 || n_l < 1 || n_l > 16 || n_sep < 1)
        return COFFE_GPU_EINVAL;
    if (!ctx->bg_ready) {
        cg_set_error(ctx, "covariance: background not initialised");
        return COFFE_GPU_ESTATE;
    }
    if (!(contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD)) || (contrib & ~3)) {
        cg_set_error(ctx, "covariance: contrib must select den and/or rsd");
        return COFFE_GPU_EINVAL;
    }
    for (int q = 0; q < n_z; ++q) {
        const bool zok = averaged ? (za[q] > 0 && zb[q] > za[q]) : (zb[q] >= 0 && za[q] - zb[q] >= 0);
        if (!(density1[q] > 0 && density2[q] > 0 && fsky[q] > 0 && pixelsize[q] > 0 && zok)) {
            cg_set_error(ctx, "covariance: bad survey parameters in redshift bin %d", q);
            return COFFE_GPU_EINVAL;
        }
    }
    for (int i = 0; i < n_l; ++i)
        if (l[i] < 0 || l[i] > 64) {
            cg_set_error(ctx, "covariance: l = %d out of range", l[i]);
            return COFFE_GPU_EINVAL;
        }
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    // jobs: (p = 1, 2) for every l1 <= l2 (covariance.c:720-751)
    std::vector<int> pw, L1, L2, job_of((size_t)n_l * n_l * 2, 0);
    for (int i = 0; i < n_l; ++i)
        for (int j = i; j < n_l; ++j)
            for (int p = 1; p <= 2; ++p) {
                job_of[((size_t)i * n_l + j) * 2 + (p - 1)] = (int)pw.size();
                pw.push_back(p);
                L1.push_back(l[i]);
                L2.push_back(l[j]);
            }
    const int n_jobs = (int)pw.size();
    const size_t nss = (size_t)n_sep * n_sep;
    std::vector<double> LI((size_t)n_l * n_l * 9), zin((size_t)n_z * 6);
    for (int i = 0; i < n_l; ++i)
        for (int j = 0; j < n_l; ++j)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b)
                    LI[((size_t)i * n_l + j) * 9 + a * 3 + b] = legendre_integral(l[i], l[j], 2 * a, 2 * b);
    for (int q = 0; q < n_z; ++q) {
        zin[6 * q] = za[q];
        zin[6 * q + 1] = zb[q];
        zin[6 * q + 2] = fsky[q];
        zin[6 * q + 3] = density1[q];
        zin[6 * q + 4] = density2[q];
        zin[6 * q + 5] = pixelsize[q];
    }
    const size_t n_zin = zin.size();
    zin.resize(n_zin + 2 * CV_VOL_NODES);
    gauss_legendre_nodes(CV_VOL_NODES, zin.data() + n_zin, zin.data() + n_zin + CV_VOL_NODES);
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t b_raw = al(sizeof(double) * n_jobs * nss), b_ipk = al(sizeof(double) * n_l * n_l * nss),
                 b_li = al(sizeof(double) * LI.size()), b_zin = al(sizeof(double) * zin.size()),
                 b_zs = al(sizeof(CvZ) * n_z), b_meta = al(sizeof(int) * (n_l + job_of.size())),
                 b_out = al(sizeof(double) * n_z * n_l * n_l * nss), b_sep = al(sizeof(double) * n_sep);
    int st;
    if ((st = cg_ensure(ctx, ctx->cov_out, b_raw + 2 * b_ipk + b_li + b_zin + b_zs + b_meta + b_out + b_sep)))
        return st;
    char *base = (char *)ctx->cov_out.p;
    double *d_raw = (double *)base; base += b_raw;
    double *d_ipk = (double *)base; base += b_ipk;
    double *d_ipk2 = (double *)base; base += b_ipk;
    double *d_li = (double *)base; base += b_li;
    double *d_zin = (double *)base; base += b_zin;
    CvZ *d_zs = (CvZ *)base; base += b_zs;
    int *d_ls = (int *)base, *d_job = d_ls + n_l; base += b_meta;
    double *d_out = (double *)base; base += b_out;
    double *d_sep = (double *)base;
    if ((st = cv_integrals(ctx, k, pk, nk, N, n_jobs, pw.data(), L1.data(), L2.data(), sep, n_sep, d_raw)))
        return st;
    CG_CUDA(ctx, cudaMemcpyAsync(d_li, LI.data(), sizeof(double) * LI.size(), cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(d_zin, zin.data(), sizeof(double) * zin.size(), cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(d_ls, l, sizeof(int) * n_l, cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(d_job, job_of.data(), sizeof(int) * job_of.size(), cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(d_sep, sep, sizeof(double) * n_sep, cudaMemcpyHostToDevice, ctx->stream));
    const long nsc = (long)n_l * n_l * nss;
    cv_scale_kernel<<<(unsigned)((nsc + 255) / 256), 256, 0, ctx->stream>>>(n_l, n_sep, d_ls, d_job,
                                                                            d_raw, d_ipk, d_ipk2);
    if ((st = cg_after_launch(ctx, "cv_scale_kernel"))) return st;
    cv_zscalars_kernel<<<(n_z + 127) / 128, 128, 0, ctx->stream>>>(
        n_z, ctx->bg[BG_CHI_OF_Z].v64(), ctx->bg[BG_F].v64(), ctx->bg[BG_D1].v64(),
        ctx->bias[0].v64(), ctx->bg[BG_CONFH].v64(), CG_H0 * ctx->h, ctx->bias_set[0], contrib,
        averaged, d_zin, d_zin + n_zin, d_zs);
    if ((st = cg_after_launch(ctx, "cv_zscalars_kernel"))) return st;
    const long nout = (long)n_z * n_l * n_l * nss;
    cv_assemble_kernel<<<(unsigned)((nout + 255) / 256), 256, 0, ctx->stream>>>(
        n_z, n_l, n_sep, d_ls, d_li, d_zs, d_sep, d_ipk, d_ipk2, d_out, ctx->d_err);
    if ((st = cg_after_launch(ctx, "cv_assemble_kernel"))) return st;
    CG_CUDA(ctx, cudaMemcpyAsync(out, d_out, sizeof(double) * nout, cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return cg_check_device_errors(ctx, "covariance_multipoles");
}

extern "C" int coffe_gpu_covariance_multipoles(coffe_gpu_ctx_t *ctx, int contrib, const double *k,
                                               const double *pk, size_t nk, size_t N, int n_z,
                                               const double *z_mean, const double *deltaz,
                                               const double *fsky, const double *density1,
                                               const double *density2, const double *pixelsize,
                                               int n_l, const int *l, int n_sep, const double *sep,
                                               double *out)
{
    return covariance_impl(ctx, contrib, k, pk, nk, N, n_z, 0, z_mean, deltaz, fsky, density1,
                           density2, pixelsize, n_l, l, n_sep, sep, out);
}

extern "C" int coffe_gpu_average_covariance_multipoles(
    coffe_gpu_ctx_t *ctx, int contrib, const double *k, const double *pk, size_t nk, size_t N,
    int n_win, const double *z_min, const double *z_max, const double *fsky,
    const double *density1, const double *density2, const double *pixelsize, int n_l,
    const int *l, int n_sep, const double *sep, double *out)
{
    return covariance_impl(ctx, contrib, k, pk, nk, N, n_win, 1, z_min, z_max, fsky, density1,
                           density2, pixelsize, n_l, l, n_sep, sep, out);
}
