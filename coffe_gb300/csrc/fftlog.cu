// Batched FFTLog Bessel integrals I_l^n(r) on the device.
//
// Restates twofast_1bessel (twofast.c:362-483) and the table assembly of
// coffe_integrals_renormalizable (integrals.c:459-573) for many spectra:
//   1. P(k) is resampled on the FFT grid k_i = kmin (kmax/kmin)^(i/N) through
//      the natural cubic spline of the input table (twofast.c:399-401), biased
//      by (kmax/kmin)^((3-q) i/N) and tapered (twofast.c:275-290);
//   2. real FFT, conjugate, Fourier-mode taper / L (twofast.c:292-355);
//   3. per (n, l): multiply by the Gamma-ratio kernel M_{q,l}(t)
//      (twofast_mql, twofast.c:196-224), inverse real FFT (FFTW c2r,
//      unnormalised), times the prefactor (twofast.c:419-422) and r^(n-l).
// Everything that does not depend on the spectrum (sampling positions,
// biases, tapers, M_{q,l}, prefactors, twiddles) is a per-grid table built
// once; a spectrum costs one forward FFT per distinct q and one inverse FFT
// per term.  One CTA holds one transform in shared memory (radix-2, in place).
#include <cmath>
#include <algorithm>
#include <cstring>
#include <vector>

#include "bulk.cuh"
#include "cplx.cuh"
#include "ctx.cuh"
#include "dfloat.cuh"
#include "f32x2.cuh"
#include "dual6.cuh"
#include "fft.cuh"
#include "qag.cuh"

namespace {

// the 42 sub-Mpc separations evaluated by direct quadrature (integrals.c:111-126)
const double h_min_sep[CG_N_SMALL_R] = {
    1E-6,   1E-5,    1E-4,   1E-3,    2E-3,   5E-3,   7E-3,   8E-3,    9E-3,   1E-2,    1.1E-2,
    1.2E-2, 1.25E-2, 1.3E-2, 1.35E-2, 1.5E-2, 2E-2,   2.5E-2, 3E-2,    3.5E-2, 5E-2,    7E-2,
    8E-2,   9E-2,    1E-1,   1.1E-1,  1.2E-1, 1.25E-1, 1.3E-1, 1.35E-1, 1.5E-1, 1.75E-1, 2E-1,
    2.5E-1, 3E-1,    3.5E-1, 4E-1,    5E-1,   6E-1,   7E-1,   8E-1,    9E-1};

// twofast_selectqnu (twofast.c:240-250)
double select_qnu(double l, double nu)
{
    const double n1 = 0.9, n2 = 0.9999;
    const double qmin = std::max(n2 - 1.0 - nu, -l);
    const double qmax = std::min(n1 + 3.0 - nu, 2.0);
    const double qbest = (2. + n1 + n2) / 2. - nu;
    double q = qbest;
    if (!(qmin < q && q < qmax)) q = (qmin + 2. * qmax) / 3.;
    return q;
}

__device__ __forceinline__ double twofast_window(double value, double xmin, double xmax,
                                                 double xleft, double xright)
{
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
        result = result - sin(2 * CG_PI * result) / 2. / CG_PI;
    }
    return result;
}

struct GridPar {
    double kmin, kmax, k0, r0;
    int N, nk;
};

// --------------------------------------------------------------- per grid

// Factors of the natural-spline tridiagonal system on the shared k grid (host,
// once per grid; O(nk) sequential work that the host does in microseconds):
// fac = [1/diag'_i (eliminated diagonal), w_i (elimination multipliers),
// g_i = 1/h_i], each nk long; fac32 = their float copies and h_i for the
// mixed path: [1/diag', w, 1/h, h].
void csfac_host(const double *x, int nk, std::vector<double> &fac, std::vector<float> &fac32)
{
    const int m = nk - 2;
    fac.assign((size_t)3 * nk, 0.0);
    fac32.assign((size_t)4 * nk, 0.f);
    double *invd = fac.data(), *w = fac.data() + nk, *g = fac.data() + 2 * nk;
    for (int i = 0; i + 1 < nk; ++i) g[i] = 1.0 / (x[i + 1] - x[i]);
    double dprev = 0.0;
    w[0] = 0.0;
    for (int i = 0; i < m; ++i) {
        const double h_i = x[i + 1] - x[i];
        const double h_ip1 = x[i + 2] - x[i + 1];
        double d = 2.0 * (h_ip1 + h_i);
        if (i > 0) {
            w[i] = h_i / dprev;
            d -= w[i] * h_i;
        }
        invd[i] = 1.0 / d;
        dprev = d;
    }
    for (int i = 0; i < nk; ++i) {
        fac32[i] = i < m ? (float)invd[i] : 0.f;
        fac32[nk + i] = i < m ? (float)w[i] : 0.f;
        fac32[2 * nk + i] = i + 1 < nk ? (float)g[i] : 0.f;
        fac32[3 * nk + i] = i + 1 < nk ? (float)(x[i + 1] - x[i]) : 0.f;
    }
}

// FFT node -> (input interval, offset); windowed bias per distinct q
__global__ void sampling_kernel(GridPar g, const double *__restrict__ kx, int *__restrict__ idx,
                                double *__restrict__ dxs, float4 *__restrict__ sf32, int n_q,
                                const double *__restrict__ qv, double *__restrict__ qfac,
                                double *__restrict__ modew, double *__restrict__ tab_x,
                                float *__restrict__ tab_x32, float2 *__restrict__ tdf,
                                float2 *__restrict__ qfac_df)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int N = g.N;
    const double ratio = g.kmax / g.kmin;
    const double xmax_w = g.k0 * pow(ratio, (double)(N - 1) / N);
    const double xleft_w = exp(0.46) * g.kmin;
    const double xright_w = exp(-0.46) * g.k0 * pow(ratio, (double)(N - 1) / N);
    if (i < N) {
        const double ki = g.k0 * pow(ratio, (double)i / N);
        int lo = 0, hi = g.nk - 1;
        while (hi > lo + 1) {
            const int mid = (lo + hi) / 2;
            if (kx[mid] > ki)
                hi = mid;
            else
                lo = mid;
        }
        const bool inside = ki >= kx[0] && ki <= kx[g.nk - 1];
        idx[i] = inside ? lo : -1;
        dxs[i] = ki - kx[lo];
        const double hl = kx[lo + 1] - kx[lo];
        sf32[i] = make_float4((float)(ki - kx[lo]), (float)hl, (float)(1.0 / hl), 0.f);
        const dfl t = df_from_double((ki - kx[lo]) / hl); // mixed path: position in the interval
        tdf[i] = make_float2(t.hi, t.lo);
        const double w = twofast_window(ki, g.kmin, xmax_w, xleft_w, xright_w);
        for (int q = 0; q < n_q; ++q) {
            const double qf = pow(ratio, (3. - qv[q]) * i / N) * w;
            qfac[(size_t)q * N + i] = qf;
            const dfl qd = df_from_double(qf);
            qfac_df[(size_t)q * N + i] = make_float2(qd.hi, qd.lo);
        }
        const double ri = g.r0 * pow(ratio, (double)i / N);
        tab_x[CG_N_SMALL_R + 1 + i] = ri;
        tab_x32[CG_N_SMALL_R + 1 + i] = (float)ri;
    }
    const int M = N / 2;
    if (i <= M) {
        // Fourier-mode taper at x_mod[N2 - 2 + i] (twofast.c:298-355), over L
        const double L = 2 * CG_PI * N / log(ratio);
        const double xm = g.k0 * pow(ratio, (double)(M - 1 + i) / N);
        modew[i] = twofast_window(xm, g.kmin, xmax_w, xleft_w, xright_w) / L;
    }
}

// Gamma-ratio kernel M_{q,l}(t_m) of every term (FP64, twofast_mql) and the
// output prefactor times r^(n-l) (twofast.c:419-422, integrals.c:514-523)
__global__ void term_tables_kernel(GridPar g, int n_terms, const double *__restrict__ tq,
                                   const double *__restrict__ tl, const double *__restrict__ tn,
                                   double2 *__restrict__ mcoef, double *__restrict__ postf,
                                   int *err)
{
    const int N = g.N, M = N / 2;
    const int t = blockIdx.y;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_terms) return;
    const double qnu = tq[t], l = tl[t], nu = tn[t];
    const double G = log(g.kmax / g.kmin);
    if (i <= M) {
        const double tt = 2 * CG_PI * i / G;
        const cplx n = cx(qnu - 1., -tt);
        cplx lg1, lg2;
        const bool ok1 = cx_lgamma_lanczos(cx((1. + l + n.re) / 2., n.im / 2.), &lg1);
        const bool ok2 = cx_lgamma_lanczos(cx((2. + l - n.re) / 2., -n.im / 2.), &lg2);
        double2 out = make_double2(0.0, 0.0);
        if (!ok2) {
            cg_flag(err, CG_ERR_NONFINITE);
        } else if (ok1) {
            const cplx unl = cx_rpow(2.0, cx(n.re - 1., n.im)) * (CG_SQRT_PI * cx_exp(lg1 - lg2));
            if (!(isfinite(unl.re) && isfinite(unl.im))) {
                cg_flag(err, CG_ERR_NONFINITE);
            } else {
                const cplx m = cx_rpow(g.k0 * g.r0, cx(-qnu, tt)) * unl;
                out = make_double2(m.re, m.im);
            }
        }
        // ok1 == false: the reflection overflowed, lnGamma = -inf, M = 0
        mcoef[(size_t)t * (M + 1) + i] = out;
    }
    if (i < N) {
        const double ratio = g.kmax / g.kmin;
        double p = g.k0 * g.k0 * g.k0 * pow(ratio, -((qnu + nu) * i / N)) / CG_PI /
                   pow(g.r0 * g.k0, nu) / G;
        if (nu >= l) p *= pow(g.r0 * pow(ratio, (double)i / N), nu - l);
        postf[(size_t)t * N + i] = p;
    }
}

__global__ void twiddle_kernel(int N, double2 *__restrict__ tw, float4 *__restrict__ twdf)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j > N / 2) return;
    double s, c;
    sincospi(2.0 * (double)j / (double)N, &s, &c);
    tw[j] = make_double2(c, -s);
    twdf[j] = dfc_pack(dfc_from_double2(make_double2(c, -s)));
}

// Mixed-path copies of the per-grid tables: the mode taper in double-float
// (forward transform); the Gamma-ratio kernel M_{q,l}(t_m), the output
// prefactors and the twiddles rounded to float for the FP32 inverse transforms
// (each rounded once from its FP64 value), and the kernel and prefactors in
// double-float for the double-float inverse transforms (COFFE_GPU_TABLES_DF)
__global__ void term_tables_df_kernel(int M, int N, int n_terms, const double2 *__restrict__ mcoef,
                                      const double *__restrict__ postf,
                                      const double *__restrict__ modew,
                                      const double2 *__restrict__ tw, float2 *__restrict__ wdf,
                                      float2 *__restrict__ m32, float *__restrict__ p32,
                                      float2 *__restrict__ tw32, float4 *__restrict__ mdf,
                                      float2 *__restrict__ pdf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int t = blockIdx.y;
    if (i <= M) {
        const double2 m = mcoef[(size_t)t * (M + 1) + i];
        m32[(size_t)t * (M + 1) + i] = make_float2((float)m.x, (float)m.y);
        mdf[(size_t)t * (M + 1) + i] = dfc_pack(dfc_from_double2(m));
        if (t == 0) {
            const dfl v = df_from_double(modew[i]);
            wdf[i] = make_float2(v.hi, v.lo);
            tw32[i] = make_float2((float)tw[i].x, (float)tw[i].y);
        }
    }
    if (i < N) {
        const double pf = postf[(size_t)t * N + i];
        p32[(size_t)t * N + i] = (float)pf;
        const dfl v = df_from_double(pf);
        pdf[(size_t)t * N + i] = make_float2(v.hi, v.lo);
    }
}

// ------------------------------------------------------------ per spectrum

// Natural cubic spline coefficients c_i (= y''/2) of every spectrum on the
// shared k grid: one warp per spectrum.  The forward elimination
// r_i = rhs_i - w_i r_{i-1} and the back substitution
// c_{i+1} = (r_i - h_{i+1} c_{i+2}) / diag'_i are first-order linear
// recurrences; each lane owns a contiguous chunk, composes its chunk's affine
// map, a warp scan of the maps gives every chunk its incoming value, and each
// lane then replays its chunk.  Same algebra as the sequential Thomas sweep
// of the tridiagonal solve.
__device__ __forceinline__ void affine_scan(double &A, double &B, int lane)
{
    // inclusive scan of maps r -> A + B r, later lanes applied after earlier ones
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const double Ap = __shfl_up_sync(0xffffffffu, A, o);
        const double Bp = __shfl_up_sync(0xffffffffu, B, o);
        if (lane >= o) {
            A = A + B * Ap;
            B = B * Bp;
        }
    }
}

__global__ void cspline_c_kernel(const double *__restrict__ x, const double *__restrict__ pk,
                                 const double *__restrict__ fac, int nk, int n_spectra,
                                 double *__restrict__ cc)
{
    const int s = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int lane = threadIdx.x & 31;
    if (s >= n_spectra) return;
    const double *y = pk + (size_t)s * nk;
    double *c = cc + (size_t)s * nk;
    const double *invd = fac, *w = fac + nk, *g = fac + 2 * nk;
    const int m = nk - 2;
    const int chunk = (m + 31) / 32;
    const int lo = lane * chunk, hi = min(lo + chunk, m);
    // forward elimination, map r -> rhs_i - w_i r (w_0 = 0)
    double A = 0.0, B = 1.0;
    for (int i = lo; i < hi; ++i) {
        const double rhs = 3.0 * ((y[i + 2] - y[i + 1]) * g[i + 1] - (y[i + 1] - y[i]) * g[i]);
        const double b = i > 0 ? -w[i] : 0.0;
        A = rhs + b * A;
        B = b * B;
    }
    affine_scan(A, B, lane);
    double r = __shfl_up_sync(0xffffffffu, A, 1);
    if (lane == 0) r = 0.0;
    for (int i = lo; i < hi; ++i) {
        const double rhs = 3.0 * ((y[i + 2] - y[i + 1]) * g[i + 1] - (y[i + 1] - y[i]) * g[i]);
        r = i > 0 ? rhs - w[i] * r : rhs;
        c[i + 1] = r;
    }
    __syncwarp();
    // back substitution from the top: map c -> (r_i - h_{i+1} c) / diag'_i;
    // lane order reversed so the scan runs from i = m-1 down to 0
    const int rl = 31 - lane;
    const int blo = rl * chunk, bhi = min(blo + chunk, m);
    A = 0.0;
    B = 1.0;
    for (int i = bhi - 1; i >= blo; --i) {
        const double a_i = c[i + 1] * invd[i];
        const double b_i = -(x[i + 2] - x[i + 1]) * invd[i];
        A = a_i + b_i * A;
        B = b_i * B;
    }
    affine_scan(A, B, lane);
    double cn = __shfl_up_sync(0xffffffffu, A, 1);
    if (lane == 0) cn = 0.0; // c_{m+1} = c_{nk-1} = 0
    __syncwarp();
    for (int i = bhi - 1; i >= blo; --i) {
        cn = (c[i + 1] - (x[i + 2] - x[i + 1]) * cn) * invd[i];
        c[i + 1] = cn;
    }
    if (lane == 0) {
        c[0] = 0.0;
        c[nk - 1] = 0.0;
    }
}

// The mixed path's c: rows of the inverse of the natural-spline matrix decay
// like 0.27^|i - j| (2 - sqrt(3) on a uniform grid), so
//   c_{i+1} = sum_{|d| <= CS_BAND} Ainv[i][i + d] rhs_{i+d}
// with the band precomputed once per k grid (float; truncation 0.27^13 ~ 4e-8
// of the diagonal, the float resolution of c).  c enters the resampled P(k)
// only through the h (c1 + 2 c0)/3 and dx^2 terms, corrections of relative size
// ~(h/k)^2.  One thread per knot for CS_SPB spectra, rhs staged in shared
// memory, the band stored by diagonal so that its loads coalesce.
#define CS_BAND 12
// row stride of the band: m rounded up to a multiple of 8 (zeros past m), so
// that 8 consecutive coefficients of a row are two aligned float4
__host__ __device__ inline int cs_band_stride(int m) { return (m + 7) & ~7; }

#define CS_TILE 256
#define CS_HALO (CS_TILE + 2 * CS_BAND + 2)
// One pass per (tile of knots, group of CS_SPB spectra): reads the FP64
// spectra once, writes them as double-float pairs for the FFT input
// (integer split, no FP64 work) and the float spline coefficients.
template <int CS_SPB> // spectra per block: each thread keeps its band row in registers
__global__ void __launch_bounds__(CS_TILE)
    cspline_band_kernel(const double *__restrict__ pk, const float *__restrict__ band_t,
                        const float *__restrict__ fac32, int nk, int n_spectra,
                        float2 *__restrict__ pkdf, float *__restrict__ cc)
{
    __shared__ float y_s[CS_SPB][CS_HALO];
    __shared__ float rhs_s[CS_SPB][CS_TILE + 2 * CS_BAND];
    const int i0 = blockIdx.x * CS_TILE;
    const int s0 = blockIdx.y * CS_SPB;
    const int ns = min(CS_SPB, n_spectra - s0);
    const int m = nk - 2;
    const bool last_tile = blockIdx.x == gridDim.x - 1;
    const float *g = fac32 + 2 * nk;
    for (int t = threadIdx.x; t < CS_SPB * CS_HALO; t += blockDim.x) {
        const int q = t / CS_HALO, r = t - q * CS_HALO;
        const int i = i0 - CS_BAND + r;
        float h = 0.f;
        if (q < ns && i >= 0 && i < nk) {
            const size_t at = (size_t)(s0 + q) * nk + i;
            const dfl d = df_from_double_bits(pk[at]);
            h = d.hi;
            // each knot's pair is written by the tile that owns it (the last
            // tile also owns the two knots past the final spline row)
            if (i >= i0 && (i < i0 + CS_TILE || last_tile)) pkdf[at] = make_float2(d.hi, d.lo);
        }
        y_s[q][r] = h;
    }
    __syncthreads();
    for (int t = threadIdx.x; t < CS_SPB * (CS_TILE + 2 * CS_BAND); t += blockDim.x) {
        const int q = t / (CS_TILE + 2 * CS_BAND), r = t - q * (CS_TILE + 2 * CS_BAND);
        const int i = i0 - CS_BAND + r;
        float v = 0.f;
        if (i >= 0 && i < m) {
            const float ya = y_s[q][r], yb = y_s[q][r + 1], yc = y_s[q][r + 2];
            v = 3.f * ((yc - yb) * g[i + 1] - (yb - ya) * g[i]);
        }
        rhs_s[q][r] = v;
    }
    __syncthreads();
    const int i = i0 + threadIdx.x;
    if (i < m) {
        float bw[2 * CS_BAND + 1];
#pragma unroll
        for (int d = 0; d <= 2 * CS_BAND; ++d)
            bw[d] = __ldg(band_t + (size_t)d * cs_band_stride(m) + i);
        for (int q = 0; q < ns; ++q) {
            float acc = 0.f;
#pragma unroll
            for (int d = 0; d <= 2 * CS_BAND; ++d) acc = fmaf(bw[d], rhs_s[q][threadIdx.x + d], acc);
            cc[(size_t)(s0 + q) * nk + i + 1] = acc;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < ns) {
        cc[(size_t)(s0 + threadIdx.x) * nk] = 0.f;
        cc[(size_t)(s0 + threadIdx.x) * nk + nk - 1] = 0.f;
    }
}

// Band of the inverse natural-spline matrix (rows of A^-1 = columns, A
// symmetric), each from a tridiagonal solve on a window of 3 CS_BAND knots
// around the row (the window's edge changes the kept entries by 0.27^24 of
// the diagonal; windows touching the grid ends use the true boundary).
void cspline_band_host(const std::vector<double> &x, std::vector<float> &band)
{
    const int nk = (int)x.size(), m = nk - 2, W = 3 * CS_BAND, B = 2 * CS_BAND + 1;
    const int ms = cs_band_stride(m);
    band.assign((size_t)ms * B, 0.f);
    std::vector<double> dg(2 * W + 1), up(2 * W + 1), rhs(2 * W + 1);
    for (int j = 0; j < m; ++j) {
        const int lo = std::max(0, j - W), hi = std::min(m, j + W + 1), n = hi - lo;
        // rows i = lo..hi-1 (unknown c_{i+1}): diag 2 (h_i + h_{i+1}), coupling h_{i+1}
        for (int r = 0; r < n; ++r) {
            const int i = lo + r;
            dg[r] = 2.0 * ((x[i + 1] - x[i]) + (x[i + 2] - x[i + 1]));
            up[r] = x[i + 2] - x[i + 1];
            rhs[r] = i == j ? 1.0 : 0.0;
        }
        for (int r = 1; r < n; ++r) {
            const double w = up[r - 1] / dg[r - 1];
            dg[r] -= w * up[r - 1];
            rhs[r] -= w * rhs[r - 1];
        }
        rhs[n - 1] /= dg[n - 1];
        for (int r = n - 2; r >= 0; --r) rhs[r] = (rhs[r] - up[r] * rhs[r + 1]) / dg[r];
        for (int d = -CS_BAND; d <= CS_BAND; ++d) {
            const int i = j + d;
            if (i >= lo && i < hi) band[(size_t)(d + CS_BAND) * ms + j] = (float)rhs[i - lo];
        }
    }
}

// On a geometric k grid (h_j = h rho^j) the spline matrix is diag(h_i) times a
// Toeplitz matrix, so away from the ends (rows CS_BAND .. m - CS_BAND - 1) its
// inverse's band is tau_d g_{i+d}, g_j = 1 / h_j: 25 constants times one scale
// per knot.  BandFac holds the constants when the band has that form to float
// accuracy; the fused table kernel then multiplies the right-hand sides by g
// once and needs no band rows but the 2 CS_BAND end rows (their coefficients
// divided by g, appended to the band buffer).
struct BandFac {
    int ok;
    float tau[2 * CS_BAND + 1];
};
BandFac cspline_band_factor(const std::vector<double> &x, const std::vector<float> &band,
                            std::vector<float> &edge)
{
    BandFac f;
    f.ok = 0;
    const int nk = (int)x.size(), m = nk - 2, ms = cs_band_stride(m), B = 2 * CS_BAND + 1;
    edge.assign((size_t)2 * CS_BAND * B, 0.f);
    if (m < 4 * CS_BAND + 8) return f;
    auto g = [&](int j) { return 1.0 / (x[j + 1] - x[j]); };
    const int mid = m / 2;
    double tau[2 * CS_BAND + 1];
    for (int d = 0; d < B; ++d) tau[d] = band[(size_t)d * ms + mid] / g(mid + d - CS_BAND);
    for (int i = CS_BAND; i < m - CS_BAND; ++i) {
        double big = 0.0, err = 0.0;
        for (int d = 0; d < B; ++d) {
            const double b = band[(size_t)d * ms + i];
            big = std::max(big, std::fabs(b));
            err = std::max(err, std::fabs(b - tau[d] * g(i + d - CS_BAND)));
        }
        if (!(err <= 2e-7 * big)) return f;
    }
    for (int r = 0; r < 2 * CS_BAND; ++r) {
        const int i = r < CS_BAND ? r : m - 2 * CS_BAND + r;
        for (int d = 0; d < B; ++d) {
            const int j = i + d - CS_BAND;
            if (j >= 0 && j < m) edge[(size_t)r * B + d] = (float)(band[(size_t)d * ms + i] / g(j));
        }
    }
    for (int d = 0; d < B; ++d) f.tau[d] = (float)tau[d];
    f.ok = 1;
    return f;
}

template <typename T> struct V2;
template <> struct V2<double> { typedef double2 t; };
template <> struct V2<float> { typedef float2 t; };

// FP64 value of the biased, tapered FFT input at node i: the natural cubic
// spline of P(k) (twofast.c:399-401, gsl cspline with y + dx(b + dx(c + d dx)))
// times (kmax/kmin)^((3-q) i/N) W(k_i) (twofast.c:279-290)
__device__ __forceinline__ double sample_input(const double *__restrict__ kx,
                                               const double *__restrict__ y,
                                               const double *__restrict__ c,
                                               const double *__restrict__ gi,
                                               const int *__restrict__ idx,
                                               const double *__restrict__ dxs,
                                               const double *__restrict__ qf, int i)
{
    const int j = idx[i];
    if (j < 0) return cg_nan<double>();
    const double h = kx[j + 1] - kx[j];
    const double g = gi[j];
    const double y0 = y[j], y1 = y[j + 1], c0 = c[j], c1 = c[j + 1];
    const double b = (y1 - y0) * g - h * (c1 + 2.0 * c0) * (1.0 / 3.0);
    const double d = (c1 - c0) * g * (1.0 / 3.0);
    const double dx = dxs[i];
    return (y0 + dx * (b + dx * (c0 + d * dx))) * qf[i];
}

// ---- FP64 path

// Forward half: sample, bias, FFT, conjugate, mode taper.  Grid (spectrum, q).
__global__ void fftlog_forward_kernel(GridPar g, const double *__restrict__ kx,
                                      const double *__restrict__ pk,
                                      const double *__restrict__ cc, const double *__restrict__ fac,
                                      const int *__restrict__ idx,
                                      const double *__restrict__ dxs,
                                      const double *__restrict__ qfac,
                                      const double *__restrict__ modew,
                                      const double2 *__restrict__ tw, int n_q,
                                      double2 *__restrict__ spec, int *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *buf = reinterpret_cast<double2 *>(smem_raw);
    const int s = blockIdx.x, qi = blockIdx.y;
    const int N = g.N, M = N / 2;
    const int logM = 31 - __clz(M);
    const double *y = pk + (size_t)s * g.nk;
    const double *c = cc + (size_t)s * g.nk;
    const double *gi = fac + 2 * (size_t)g.nk;
    bool bad = false;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double v = sample_input(kx, y, c, gi, idx, dxs, qfac + (size_t)qi * N, i);
        if (!isfinite(v)) bad = true;
        const int jj = __brev((unsigned)(i >> 1)) >> (32 - logM);
        if (i & 1)
            buf[jj].y = v;
        else
            buf[jj].x = v;
    }
    if (bad) cg_flag(err, CG_ERR_NONFINITE);
    __syncthreads();
    smem_fft<double2>(buf, logM, tw, -1);
    // unpack the real FFT: Y_k = (Z_k + conj Z_{M-k})/2 - i w^k (Z_k - conj Z_{M-k})/2
    double2 *out = spec + ((size_t)s * n_q + qi) * (M + 1);
    for (int k = threadIdx.x; k <= M; k += blockDim.x) {
        const double2 zk = buf[k & (M - 1)];
        const double2 zm = buf[(M - k) & (M - 1)];
        const double ex = 0.5 * (zk.x + zm.x), ey = 0.5 * (zk.y - zm.y);
        const double ox = 0.5 * (zk.y + zm.y), oy = -0.5 * (zk.x - zm.x);
        const double2 w = tw[k];
        const double yx = ex + (w.x * ox - w.y * oy);
        const double yy = ey + (w.x * oy + w.y * ox);
        const double mw = modew[k];
        out[k] = make_double2(mw * yx, -mw * yy); // conjugate
    }
}

// Inverse half: multiply by M_{q,l}, c2r, prefactor.  Grid (spectrum, term).
__global__ void fftlog_inverse_kernel(GridPar g, const double2 *__restrict__ spec,
                                      const int *__restrict__ term_q, int n_q, int n_terms,
                                      const double2 *__restrict__ mcoef,
                                      const double *__restrict__ postf,
                                      const double2 *__restrict__ tw, double *__restrict__ tab,
                                      int *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    double2 *buf = reinterpret_cast<double2 *>(smem_raw);
    const int s = blockIdx.x, t = blockIdx.y;
    const int N = g.N, M = N / 2;
    const int logM = 31 - __clz(M);
    const double2 *in = spec + ((size_t)s * n_q + term_q[t]) * (M + 1);
    const double2 *mc = mcoef + (size_t)t * (M + 1);
    // X_k = S_k M_k with Im X_0 = Im X_M = 0 (FFTW c2r ignores them)
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        const int km = M - k;
        const double2 xa0 = cmul(in[k], mc[k]), xb0 = cmul(in[km], mc[km]);
        double2 xa = xa0, xb = xb0;
        if (k == 0) {
            xa.y = 0.0;
            xb.y = 0.0;
        }
        // Fe = X_k + conj X_{M-k};  Fo = (X_k - conj X_{M-k}) conj(w^k);  Z = Fe + i Fo
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
    const size_t len = (size_t)N + CG_N_SMALL_R + 1;
    double *o = tab + ((size_t)s * n_terms + t) * len + CG_N_SMALL_R + 1;
    const double *pf = postf + (size_t)t * N;
    bool bad = false;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double2 z = buf[i >> 1];
        const double r = ((i & 1) ? z.y : z.x) * pf[i];
        if (!isfinite(r)) bad = true;
        o[i] = r;
    }
    if (bad) cg_flag(err, CG_ERR_NONFINITE);
}

// ---- mixed path: the same transforms in double-float on the FP32 pipes

// Shared-memory layout of the double-float transforms: element i at
// i ^ f(i >> 3), f taking values below 8, so each aligned group of eight
// 16-byte elements (one 128-byte bank row) is permuted within itself.  f
// spreads the patterns that otherwise fall on one bank: the bit-reversed
// scatter (eight consecutive k differ in the three top index bits; the shift
// sh = logM - 6 brings them down), the stride-two radix-2 stage and the
// half = 2 radix-4 stage.  SWZ = false is the plain layout (needs M >= 8 for
// the swizzle).
template <bool SWZ> __device__ __forceinline__ int fft_slot(int i, int sh)
{
    if (!SWZ) return i;
    const int x = i >> 3;
    const int f = ((x & 1) * 3) | ((x & 2) << 1);
    return i ^ ((f ^ (x >> sh)) & 7);
}

// DIT FFT of M = 2^logM double-float complex points (bit-reversed input).
// RADIX 4: pairs of radix-2 stages fused into radix-4 butterflies in
// registers (three twiddle products per four points instead of four, half the
// shared-memory passes), after one twiddle-free radix-2 stage when logM is
// odd.  RADIX 2: one stage per pass.  tw[j] = exp(-2 pi i j / (2M)), j <= M;
// sign = -1 forward, +1 backward.
template <int RADIX, bool SWZ>
__device__ void smem_fft_df(float4 *buf, int logM, const float4 *__restrict__ tw, int sign,
                            bool first_done = false)
{
    const int M = 1 << logM;
    const int sh = logM > 6 ? logM - 6 : 0;
    if (RADIX == 2) {
        for (int st = 1; st <= logM; ++st) {
            const int half = 1 << (st - 1);
            const int stride = M >> (st - 1);
            for (int b = threadIdx.x; b < M / 2; b += blockDim.x) {
                const int pos = b & (half - 1);
                const int i0 = ((b >> (st - 1)) << st) + pos;
                const int p0 = fft_slot<SWZ>(i0, sh), p1 = fft_slot<SWZ>(i0 + half, sh);
                dfc w = dfc_load(tw[pos * stride]);
                if (sign > 0) w.im = df_neg(w.im);
                const dfc u = dfc_load(buf[p0]);
                const dfc t = dfc_mul(w, dfc_load(buf[p1]));
                buf[p0] = dfc_pack(dfc_add(u, t));
                buf[p1] = dfc_pack(dfc_sub(u, t));
            }
            __syncthreads();
        }
        return;
    }
    int st = 1;
    if (logM & 1) { // (first_done: the caller wrote the input with this stage applied)
        if (!first_done) {
            for (int b = threadIdx.x; b < M / 2; b += blockDim.x) {
                const int p0 = fft_slot<SWZ>(2 * b, sh), p1 = fft_slot<SWZ>(2 * b + 1, sh);
                const dfc u = dfc_load(buf[p0]), v = dfc_load(buf[p1]);
                buf[p0] = dfc_pack(dfc_add(u, v));
                buf[p1] = dfc_pack(dfc_sub(u, v));
            }
            __syncthreads();
        }
        st = 2;
    }
    for (; st < logM; st += 2) {
        // radix-2 stages st and st + 1: points i0 + {0, 1, 2, 3} half of a
        // block of 4 half; W = w_{4 half}^pos, twiddles W^2, W, W^3
        const int half = 1 << (st - 1);
        const int step = M >> st; // tw index of w_{4 half}
        for (int b = threadIdx.x; b < M / 4; b += blockDim.x) {
            const int pos = b & (half - 1);
            const int i0 = ((b >> (st - 1)) << (st + 1)) + pos;
            const int p0 = fft_slot<SWZ>(i0, sh), p1 = fft_slot<SWZ>(i0 + half, sh);
            const int p2 = fft_slot<SWZ>(i0 + 2 * half, sh), p3 = fft_slot<SWZ>(i0 + 3 * half, sh);
            const dfc x0 = dfc_load(buf[p0]);
            dfc x1 = dfc_load(buf[p1]);
            dfc x2 = dfc_load(buf[p2]);
            dfc x3 = dfc_load(buf[p3]);
            if (half > 1) { // pos = 0 when half = 1: all twiddles are one
                const int j = pos * step, j3 = 3 * j;
                dfc w1 = dfc_load(tw[2 * j]), w2 = dfc_load(tw[j]);
                dfc w3 = j3 <= M ? dfc_load(tw[j3]) : dfc_neg(dfc_load(tw[j3 - M]));
                if (sign > 0) {
                    w1 = dfc_conj(w1);
                    w2 = dfc_conj(w2);
                    w3 = dfc_conj(w3);
                }
                x1 = dfc_mul(x1, w1);
                x2 = dfc_mul(x2, w2);
                x3 = dfc_mul(x3, w3);
            }
            // t0..t3 stay unnormalised: each feeds only the normalising sums below
            const dfc t0 = dfc_add_raw(x0, x1), t1 = dfc_sub_raw(x0, x1);
            const dfc t2 = dfc_add_raw(x2, x3), t3 = dfc_sub_raw(x2, x3);
            // w_{4 half}^half = -i forward, +i backward
            const dfc r = sign < 0 ? dfc{t3.im, df_neg(t3.re)} : dfc{df_neg(t3.im), t3.re};
            buf[p0] = dfc_pack(dfc_add(t0, t2));
            buf[p1] = dfc_pack(dfc_add(t1, r));
            buf[p2] = dfc_pack(dfc_sub(t0, t2));
            buf[p3] = dfc_pack(dfc_sub(t1, r));
        }
        __syncthreads();
    }
}

// Mixed-path sampling in double-float: the secant part y0 + t (y1 - y0),
// t = dx / h, plus the spline-curvature correction dx (-h (c1 + 2 c0)/3 +
// dx (c0 + d dx)) in float (a relative correction of size ~(h/k)^2, so float
// is far below the target), times the windowed bias.
__device__ __forceinline__ dfl sample_input_df(const float2 *__restrict__ y,
                                               const float *__restrict__ c,
                                               const int *__restrict__ idx,
                                               const float2 *__restrict__ tdf,
                                               const float4 *__restrict__ sf,
                                               const float2 *__restrict__ qf, int i)
{
    const int j = idx[i];
    if (j < 0) return dfl{cg_nan<float>(), 0.f};
    const float2 a = y[j], b = y[j + 1], t = tdf[i], q = qf[i];
    const dfl y0{a.x, a.y};
    const dfl secant = df_add(y0, df_mul(dfl{t.x, t.y}, df_sub(dfl{b.x, b.y}, y0)));
    const float4 f = sf[i]; // (dx, h, 1/h, -)
    const float c0 = c[j], c1 = c[j + 1];
    const float d = (c1 - c0) * f.z * (1.f / 3.f);
    const float corr = f.x * (-f.y * (c1 + 2.f * c0) * (1.f / 3.f) + f.x * (c0 + d * f.x));
    return df_mul(df_add(secant, dfl{corr, 0.f}), dfl{q.x, q.y});
}

// The forward input written with the first (twiddle-free) radix-2 stage of
// smem_fft_df<4> applied, for odd logM: the complex points c and c + M/2
// (real samples 2c, 2c + 1, 2c + M, 2c + M + 1) occupy the neighbouring
// bit-reversed slots brev(c) and brev(c) + 1, so one thread samples both and
// stores their sum and difference, the stage's operations on the same values,
// without a pass over shared memory.  Returns whether a sample was not finite.
template <bool SWZ>
__device__ __forceinline__ bool fill_forward_r2(float4 *buf, int logM, const float2 *y,
                                                const float *c, const int *__restrict__ idx,
                                                const float2 *__restrict__ tdf,
                                                const float4 *__restrict__ sf,
                                                const float2 *__restrict__ qf)
{
    const int M = 1 << logM, sh = logM > 6 ? logM - 6 : 0;
    bool bad = false;
    for (int q = threadIdx.x; q < M / 2; q += blockDim.x) {
        const dfl a0 = sample_input_df(y, c, idx, tdf, sf, qf, 2 * q);
        const dfl a1 = sample_input_df(y, c, idx, tdf, sf, qf, 2 * q + 1);
        const dfl b0 = sample_input_df(y, c, idx, tdf, sf, qf, 2 * q + M);
        const dfl b1 = sample_input_df(y, c, idx, tdf, sf, qf, 2 * q + M + 1);
        if (!isfinite(a0.hi) || !isfinite(a1.hi) || !isfinite(b0.hi) || !isfinite(b1.hi))
            bad = true;
        const dfc u{a0, a1}, v{b0, b1};
        const int j0 = (int)(__brev((unsigned)q) >> (32 - logM)); // even
        buf[fft_slot<SWZ>(j0, sh)] = dfc_pack(dfc_add(u, v));
        buf[fft_slot<SWZ>(j0 + 1, sh)] = dfc_pack(dfc_sub(u, v));
    }
    return bad;
}

__device__ __forceinline__ void store_spec(float4 *p, dfc v) { *p = dfc_pack(v); }
__device__ __forceinline__ void store_spec(float2 *p, dfc v)
{
    *p = make_float2(v.re.hi + v.re.lo, v.im.hi + v.im.lo);
}

// OUT = float4: the double-float half spectrum (double-float inverse
// transforms); OUT = float2: rounded to float (FP32 inverse transforms)
template <int RADIX, bool SWZ, typename OUT>
__global__ void fftlog_forward_df_kernel(GridPar g, const float2 *__restrict__ pkdf,
                                         const float *__restrict__ cc32,
                                         const int *__restrict__ idx,
                                         const float2 *__restrict__ tdf,
                                         const float4 *__restrict__ sf32,
                                         const float2 *__restrict__ qfac_df,
                                         const float2 *__restrict__ modew_df,
                                         const float4 *__restrict__ twdf, int n_q,
                                         OUT *__restrict__ spec, int *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4 *buf = reinterpret_cast<float4 *>(smem_raw);
    float2 *buf2 = reinterpret_cast<float2 *>(smem_raw);
    const int s = blockIdx.x, qi = blockIdx.y;
    const int N = g.N, M = N / 2;
    const int logM = 31 - __clz(M);
    const int sh = logM > 6 ? logM - 6 : 0;
    const float2 *y = pkdf + (size_t)s * g.nk;
    const float *c = cc32 + (size_t)s * g.nk;
    const bool r2 = RADIX == 4 && (logM & 1);
    bool bad = false;
    if (r2) {
        bad = fill_forward_r2<SWZ>(buf, logM, y, c, idx, tdf, sf32, qfac_df + (size_t)qi * N);
    } else {
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            const dfl d = sample_input_df(y, c, idx, tdf, sf32, qfac_df + (size_t)qi * N, i);
            if (!isfinite(d.hi)) bad = true;
            const int jj = fft_slot<SWZ>(__brev((unsigned)(i >> 1)) >> (32 - logM), sh);
            buf2[2 * jj + (i & 1)] = make_float2(d.hi, d.lo);
        }
    }
    if (bad) cg_flag(err, CG_ERR_NONFINITE);
    __syncthreads();
    smem_fft_df<RADIX, SWZ>(buf, logM, twdf, -1, r2);
    OUT *out = spec + ((size_t)s * n_q + qi) * (M + 1);
    for (int k = threadIdx.x; k <= M; k += blockDim.x) {
        const dfc zk = dfc_load(buf[fft_slot<SWZ>(k & (M - 1), sh)]);
        const dfc zm = dfc_conj(dfc_load(buf[fft_slot<SWZ>((M - k) & (M - 1), sh)]));
        const dfc e = dfc_add(zk, zm);                  // 2 E
        const dfc dd = dfc_sub(zk, zm);                 // 2 i O
        const dfc o = dfc{dd.im, df_neg(dd.re)};        // 2 O = -i (2 i O)
        const dfc yk = dfc_add(e, dfc_mul(dfc_load(twdf[k]), o)); // 2 Y_k
        const float2 mw = modew_df[k];
        const dfl m = df_scale(dfl{mw.x, mw.y}, 0.5f);
        // conjugate; the double-float transform keeps the high modes' rounding
        // noise (which the growing Gamma-ratio kernel amplifies) at FP64 level
        store_spec(out + k, dfc{df_mul(yk.re, m), df_neg(df_mul(yk.im, m))});
    }
}

// ---- mixed path, double-float inverse transforms (COFFE_GPU_TABLES_DF):
// tables to ~1e-7 of their scale instead of the FP32 transforms' ~1e-6
// the half-length complex input of a real inverse transform:
// Fe + i Fo, Fe = X_k + conj(X_{M-k}), Fo = (X_k - conj(X_{M-k})) conj(w_k)
__device__ __forceinline__ dfc c2r_pre(dfc xa, dfc xb, float4 w)
{
    const dfc xbc = dfc_conj(xb);
    const dfc fe = dfc_add(xa, xbc);
    const dfc fo = dfc_mul(dfc_sub(xa, xbc), dfc_conj(dfc_load(w)));
    return dfc{df_sub(fe.re, fo.im), df_add(fe.im, fo.re)};
}

template <int RADIX, bool SWZ>
__global__ void fftlog_inverse_df_kernel(GridPar g, const float4 *__restrict__ spec,
                                         const int *__restrict__ term_q, int n_q, int n_terms,
                                         const float4 *__restrict__ mcoef_df,
                                         const float2 *__restrict__ postf_df,
                                         const float4 *__restrict__ twdf, float *__restrict__ tab,
                                         int *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float4 *buf = reinterpret_cast<float4 *>(smem_raw);
    const int s = blockIdx.x, t = blockIdx.y;
    const int N = g.N, M = N / 2;
    const int logM = 31 - __clz(M);
    const int sh = logM > 6 ? logM - 6 : 0;
    const float4 *in = spec + ((size_t)s * n_q + term_q[t]) * (M + 1);
    const float4 *mc = mcoef_df + (size_t)t * (M + 1);
    // z_k = Fe_k + i Fo_k from X_k and conj(X_{M-k}), X = spectrum x kernel;
    // one thread makes z_k and z_{M-k} from the same two products
    for (int k = threadIdx.x; k <= M / 2; k += blockDim.x) {
        const int km = M - k;
        dfc xa = dfc_mul(dfc_load(in[k]), dfc_load(mc[k]));
        dfc xb = dfc_mul(dfc_load(in[km]), dfc_load(mc[km]));
        if (k == 0) {
            xa.im = dfl{0.f, 0.f};
            xb.im = dfl{0.f, 0.f};
        }
        buf[fft_slot<SWZ>(__brev((unsigned)k) >> (32 - logM), sh)] =
            dfc_pack(c2r_pre(xa, xb, twdf[k]));
        if (k > 0 && k < M / 2)
            buf[fft_slot<SWZ>(__brev((unsigned)km) >> (32 - logM), sh)] =
                dfc_pack(c2r_pre(xb, xa, twdf[km]));
    }
    __syncthreads();
    smem_fft_df<RADIX, SWZ>(buf, logM, twdf, +1);
    const size_t len = (size_t)N + CG_N_SMALL_R + 1;
    float *o = tab + ((size_t)s * n_terms + t) * len + CG_N_SMALL_R + 1;
    const float2 *pf = postf_df + (size_t)t * N;
    bool bad = false;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const float4 z = buf[fft_slot<SWZ>(i >> 1, sh)];
        const dfl u = (i & 1) ? dfl{z.z, z.w} : dfl{z.x, z.y};
        const float2 p = pf[i];
        const dfl r = df_mul(u, dfl{p.x, p.y});
        const float v = r.hi + r.lo;
        if (!isfinite(v)) bad = true;
        o[i] = v;
    }
    if (bad) cg_flag(err, CG_ERR_NONFINITE);
}

// ---- mixed path, inverse transforms in FP32 (the default)
//
// The c2r transform of (forward spectrum x Gamma-ratio kernel) needs no more
// than float precision: its rounding error stays ~1e-7 of the outputs' scale
// (unlike the forward transform's, which the kernel's growth at high modes
// amplifies), so it runs in plain FP32 on float twiddles, kernel and
// prefactors rounded from their FP64 values.

__device__ __forceinline__ float2 c32_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 c32_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 c32_mul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 c32_conj(float2 a) { return make_float2(a.x, -a.y); }

// (re, im) of a complex float as one packed f32x2 value: the butterflies'
// complex additions as one add/sub.rn.f32x2 each (the same per-lane rounding as
// two scalar ones, so the same results)
__device__ __forceinline__ f2 c32_pk(float2 a) { return f2_pack(a.x, a.y); }
__device__ __forceinline__ float2 c32_unpk(f2 a)
{
    float2 r;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(r.x), "=f"(r.y) : "l"(a.v));
    return r;
}

// Shared-memory layout of the FP32 transforms (8-byte elements, 16 per
// 128-byte bank row): element i at i ^ f(i >> 4), f(x) = (x ^ 8x ^ (x >> 4))
// mod 16, a permutation within each row that makes the bit-reversed scatter
// and the butterfly strides conflict-free (two-way in one stage at most).
template <bool SWZ> __device__ __forceinline__ int slot32(int i)
{
    if (!SWZ) return i;
    const int x = i >> 4;
    return i ^ ((x ^ (x << 3) ^ (x >> 4)) & 15);
}

// In-place DIT FFTs of `nact` <= G sequences of M = 2^logM complex floats
// (bit-reversed input) at buf + j M: radix-4 butterflies, after one radix-2
// stage when logM is odd; tw[j] = exp(-2 pi i j / (2M)), j <= M; sign +1
// (backward) conjugates the twiddles.  The G transforms share each twiddle
// load and give every thread G independent butterflies between barriers.
template <bool SWZ, int G>
__device__ void smem_fft_f32(float2 *buf, int logM, int nact, const float2 *__restrict__ tw,
                             int sign)
{
    const int M = 1 << logM;
    int st = 1;
    if (logM & 1) {
        for (int b = threadIdx.x; b < M / 2; b += blockDim.x) {
            const int p0 = slot32<SWZ>(2 * b), p1 = slot32<SWZ>(2 * b + 1);
#pragma unroll
            for (int j = 0; j < G; ++j) {
                if (j >= nact) break;
                float2 *bj = buf + j * M;
                const f2 u = c32_pk(bj[p0]), v = c32_pk(bj[p1]);
                bj[p0] = c32_unpk(f2_add(u, v));
                bj[p1] = c32_unpk(f2_sub(u, v));
            }
        }
        __syncthreads();
        st = 2;
    }
    for (; st < logM; st += 2) {
        const int half = 1 << (st - 1);
        const int step = M >> st;
        for (int b = threadIdx.x; b < M / 4; b += blockDim.x) {
            const int pos = b & (half - 1);
            const int i0 = ((b >> (st - 1)) << (st + 1)) + pos;
            const int p0 = slot32<SWZ>(i0), p1 = slot32<SWZ>(i0 + half);
            const int p2 = slot32<SWZ>(i0 + 2 * half), p3 = slot32<SWZ>(i0 + 3 * half);
            float2 w1 = make_float2(1.f, 0.f), w2 = w1, w3 = w1;
            if (half > 1) {
                const int jj = pos * step, j3 = 3 * jj;
                w1 = tw[2 * jj];
                w2 = tw[jj];
                w3 = j3 <= M ? tw[j3] : make_float2(-tw[j3 - M].x, -tw[j3 - M].y);
                if (sign > 0) {
                    w1 = c32_conj(w1);
                    w2 = c32_conj(w2);
                    w3 = c32_conj(w3);
                }
            }
#pragma unroll
            for (int j = 0; j < G; ++j) {
                if (j >= nact) break;
                float2 *bj = buf + j * M;
                const float2 x0 = bj[p0];
                float2 x1 = bj[p1], x2 = bj[p2], x3 = bj[p3];
                if (half > 1) {
                    x1 = c32_mul(x1, w1);
                    x2 = c32_mul(x2, w2);
                    x3 = c32_mul(x3, w3);
                }
                const f2 X0 = c32_pk(x0), X1 = c32_pk(x1), X2 = c32_pk(x2), X3 = c32_pk(x3);
                const f2 t0 = f2_add(X0, X1), t2 = f2_add(X2, X3);
                const float2 t1 = c32_unpk(f2_sub(X0, X1)), t3 = c32_unpk(f2_sub(X2, X3));
                // w_{4 half}^half = -i forward, +i backward (a lane swap: scalar)
                const float2 r = sign < 0 ? make_float2(t3.y, -t3.x) : make_float2(-t3.y, t3.x);
                bj[p0] = c32_unpk(f2_add(t0, t2));
                bj[p1] = c32_add(t1, r);
                bj[p2] = c32_unpk(f2_sub(t0, t2));
                bj[p3] = c32_sub(t1, r);
            }
        }
        __syncthreads();
    }
}

// the half-length complex input of a real inverse transform:
// Fe + i Fo, Fe = X_k + conj(X_{M-k}), Fo = (X_k - conj(X_{M-k})) conj(w_k)
__device__ __forceinline__ float2 c2r_pre32(float2 xa, float2 xb, float2 w)
{
    const float2 xbc = c32_conj(xb);
    const float2 fe = c32_add(xa, xbc);
    const float2 fo = c32_mul(c32_sub(xa, xbc), c32_conj(w));
    return make_float2(fe.x - fo.y, fe.y + fo.x);
}

// Up to G inverse transforms of one spectrum that share their forward half
// spectrum (terms with the same q): block (s, g) makes the tables of the
// terms group[g] = (q, t0, t1, t2) (-1: unused) of spectrum s.  The half
// spectrum is read once for the G products with the terms' kernels.
// fill_small != 0 also writes NaN into the 43 entries before the FFTLog part
// (r = 0 and the sub-Mpc points, not computed).
template <bool SWZ, int G>
__global__ void fftlog_inverse_f32_kernel(GridPar g, const float2 *__restrict__ spec,
                                          const int4 *__restrict__ groups, int n_q, int n_terms,
                                          const float2 *__restrict__ mcoef32,
                                          const float *__restrict__ postf32,
                                          const float2 *__restrict__ tw32,
                                          float *__restrict__ tab, int fill_small, int *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *buf = reinterpret_cast<float2 *>(smem_raw);
    const int s = blockIdx.x;
    const int4 gr = groups[blockIdx.y];
    const int ts[3] = {gr.y, gr.z, gr.w};
    const int nact = ts[0] < 0 ? 0 : (ts[1] < 0 ? 1 : (ts[2] < 0 ? 2 : 3));
    const int N = g.N, M = N / 2;
    const int logM = 31 - __clz(M);
    const float2 *in = spec + ((size_t)s * n_q + gr.x) * (M + 1);
    // z_k = Fe_k + i Fo_k from X_k and conj(X_{M-k}), X = spectrum x kernel;
    // one thread makes z_k and z_{M-k} of every term from the same two loads
    for (int k = threadIdx.x; k <= M / 2; k += blockDim.x) {
        const int km = M - k;
        const float2 ik = in[k], ikm = in[km], wk = tw32[k], wkm = tw32[km];
        const int pk = slot32<SWZ>(__brev((unsigned)k) >> (32 - logM));
        const int pkm = slot32<SWZ>(__brev((unsigned)km) >> (32 - logM));
#pragma unroll
        for (int j = 0; j < G; ++j) {
            if (j >= nact) break;
            const float2 *mc = mcoef32 + (size_t)ts[j] * (M + 1);
            float2 xa = c32_mul(ik, mc[k]);
            float2 xb = c32_mul(ikm, mc[km]);
            if (k == 0) {
                xa.y = 0.f;
                xb.y = 0.f;
            }
            buf[j * M + pk] = c2r_pre32(xa, xb, wk);
            if (k > 0 && k < M / 2) buf[j * M + pkm] = c2r_pre32(xb, xa, wkm);
        }
    }
    __syncthreads();
    smem_fft_f32<SWZ, G>(buf, logM, nact, tw32, +1);
    const size_t len = (size_t)N + CG_N_SMALL_R + 1;
    bool bad = false;
#pragma unroll
    for (int j = 0; j < G; ++j) {
        if (j >= nact) break;
        float *o = tab + ((size_t)s * n_terms + ts[j]) * len + CG_N_SMALL_R + 1;
        const float *pf = postf32 + (size_t)ts[j] * N;
        const float2 *bj = buf + j * M;
        if (fill_small && threadIdx.x <= CG_N_SMALL_R)
            o[(int)threadIdx.x - CG_N_SMALL_R - 1] = cg_nan<float>();
#pragma unroll 4
        for (int i = threadIdx.x; i < N; i += blockDim.x) {
            const float2 z = bj[slot32<SWZ>(i >> 1)];
            const float v = ((i & 1) ? z.y : z.x) * pf[i];
            if (!isfinite(v)) bad = true;
            o[i] = v;
        }
    }
    if (bad) cg_flag(err, CG_ERR_NONFINITE);
}

// ---- mixed path, the whole table stage of one spectrum in one block
//
// The three kernels above (spline band product, double-float forward
// transform, FP32 inverse transforms) each wait on global memory between
// short bursts of work (their top stall: loads from L2/HBM), and pass their
// results through global memory.  Here one block per (spectrum, q) keeps
// everything in shared memory: the spectrum's double-float knots, its spline
// coefficients, the forward transform, the half spectrum and the inverse
// transforms of every term of that q, writing only the tables.  Same
// arithmetic as the separate kernels, so the same results.
//
// Shared memory (bytes; nk >= N/2 + 1 is required):
//   phase 1: knots (hi, lo) [0, 8 nk) | spline c [FUS_C, +4 nk) |
//            forward buffer [FUS_F, +max(16 M, 4 (nk + 2 CS_BAND + 8))) (the
//            spline right-hand sides, nk + 2 CS_BAND - 2 floats, live there
//            before the sampling, and the band product's window reads up to
//            3 floats past them)
//   phase 2: half spectrum [0, 8 (M + 1)) | inverse buffers [FUS_I, +8 G M)
struct FusedLayout {
    size_t c, f, i, total;
};
__host__ __device__ inline FusedLayout fused_layout(int nk, int M, int G)
{
    auto up = [](size_t x) { return (x + 15) & ~(size_t)15; };
    FusedLayout l;
    l.c = up(sizeof(float2) * (size_t)nk);
    l.f = up(l.c + sizeof(float) * (size_t)nk);
    l.i = up(sizeof(float2) * (size_t)(M + 1));
    const size_t fwd = sizeof(float4) * (size_t)M;
    const size_t rhs = sizeof(float) * ((size_t)nk + 2 * CS_BAND + 8);
    const size_t t1 = l.f + (fwd > rhs ? fwd : rhs);
    const size_t t2 = l.i + sizeof(float2) * (size_t)M * G;
    l.total = t1 > t2 ? t1 : t2;
    return l;
}

#define FUSED_THREADS 512
template <int RADIX, bool SWZ, int G>
__global__ void __launch_bounds__(FUSED_THREADS, 2)
    fftlog_tables_fused_kernel(GridPar g, const double *__restrict__ pk,
                               const double *__restrict__ pk_end,
                               const float *__restrict__ band_t, BandFac bfac,
                               const float *__restrict__ fac32,
                               const int *__restrict__ idx, const float2 *__restrict__ tdf,
                               const float4 *__restrict__ sf32, const float2 *__restrict__ qfac_df,
                               const float2 *__restrict__ modew_df,
                               const float4 *__restrict__ twdf, const int4 *__restrict__ groups,
                               int n_grp, int n_terms, const float2 *__restrict__ mcoef32,
                               const float *__restrict__ postf32, const float2 *__restrict__ tw32,
                               float *__restrict__ tab, int fill_small, int *err)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // a kernel launched after this one with programmatic stream serialization
    // (the per-request background fit, which does not read the tables) may
    // start once every block of this grid has started, and waits for this
    // grid's completion itself before it exits
    asm volatile("griddepcontrol.launch_dependents;");
    const int s = blockIdx.x, qi = blockIdx.y;
    const int N = g.N, M = N / 2, nk = g.nk, m = nk - 2;
    const int logM = 31 - __clz(M);
    const int sh = logM > 6 ? logM - 6 : 0;
    const FusedLayout L = fused_layout(nk, M, G);
    float2 *ydf = reinterpret_cast<float2 *>(smem_raw);
    float *cs = reinterpret_cast<float *>(smem_raw + L.c);
    float4 *fbuf = reinterpret_cast<float4 *>(smem_raw + L.f);
    float2 *fbuf2 = reinterpret_cast<float2 *>(smem_raw + L.f);
    float *rhs = reinterpret_cast<float *>(smem_raw + L.f);
    const int tid = threadIdx.x, bd = blockDim.x;
    // knots as (hi, lo) pairs, split with integer operations.  The spectrum's
    // FP64 row comes into shared memory by one bulk asynchronous copy (into the
    // spline-coefficient and transform region, free until the band product;
    // from the 16-byte boundary at or below the row to the one at or above its
    // end), instead of nk / blockDim dependent rounds of loads from memory.
    // A row whose rounded end would pass the end of the P(k) array (the last
    // one, when that end is not 16-byte aligned) is read with plain loads.
    const double *p = pk + (size_t)s * nk;
    const uintptr_t a = reinterpret_cast<uintptr_t>(p), a0 = a & ~(uintptr_t)15;
    const unsigned bytes = (unsigned)(((a - a0) + sizeof(double) * (size_t)nk + 15) & ~(size_t)15);
    if (a0 + bytes <= reinterpret_cast<uintptr_t>(pk_end)) {
        __shared__ __align__(8) unsigned long long kbar;
        double *stage = reinterpret_cast<double *>(smem_raw + L.c);
        if (tid == 0) bulk_begin(&kbar, stage, reinterpret_cast<const void *>(a0), bytes);
        __syncthreads(); // the barrier is initialised before it is waited on
        bool ok = bulk_wait(&kbar);
        if (__syncthreads_or(!ok)) { // given up: wait once more for the copy, then leave
            if (!ok) ok = bulk_wait(&kbar);
            if (tid == 0) cg_flag(err, CG_ERR_WAIT);
            __syncthreads();
            return;
        }
        const double *row = stage + (a - a0) / sizeof(double);
        for (int i = tid; i < nk; i += bd) {
            const dfl d = df_from_double_bits(row[i]);
            ydf[i] = make_float2(d.hi, d.lo);
        }
    } else {
        for (int i = tid; i < nk; i += bd) {
            const dfl d = df_from_double_bits(p[i]);
            ydf[i] = make_float2(d.hi, d.lo);
        }
    }
    __syncthreads();
    // natural-spline right-hand sides (float, from the high parts), padded by
    // CS_BAND zeros on both sides
    const float *gi = fac32 + 2 * nk;
    for (int t = tid; t < m + 2 * CS_BAND; t += bd) {
        const int j = t - CS_BAND;
        float v = 0.f;
        if (j >= 0 && j < m) {
            const float ya = ydf[j].x, yb = ydf[j + 1].x, yc = ydf[j + 2].x;
            const float gj = __ldg(gi + j);
            v = 3.f * ((yc - yb) * __ldg(gi + j + 1) - (yb - ya) * gj);
            if (bfac.ok) v *= gj; // the factorised band: g_j rhs_j
        }
        rhs[t] = v;
    }
    __syncthreads();
    // spline coefficients: the band of the inverse spline matrix times the
    // right-hand sides (cspline_band_kernel's product), BR consecutive rows per
    // thread with their right-hand sides in registers: on a geometric grid
    // (bfac.ok) the 2 CS_BAND + 1 constants of the factorised band and, for the
    // 2 CS_BAND end rows, their own coefficients; otherwise the band rows as
    // aligned float4 (row stride a multiple of 8, zero-padded).  The window of
    // the last rows reads up to 3 floats past the m + 2 CS_BAND right-hand
    // sides (inside the region fused_layout reserves), for rows past m, whose
    // results are not kept.
    {
        constexpr int BR = 4, BW = BR + 2 * CS_BAND; // rows per thread, window
        const int ms = cs_band_stride(m);
        const float *edge = band_t + (size_t)(2 * CS_BAND + 1) * ms;
        for (int i0 = BR * tid; i0 < m; i0 += BR * bd) {
            float win[BW];
#pragma unroll
            for (int k = 0; k < BW / 4; ++k) {
                const float4 v = reinterpret_cast<const float4 *>(rhs + i0)[k];
                win[4 * k] = v.x;
                win[4 * k + 1] = v.y;
                win[4 * k + 2] = v.z;
                win[4 * k + 3] = v.w;
            }
            float acc[BR];
#pragma unroll
            for (int j = 0; j < BR; ++j) acc[j] = 0.f;
            if (!bfac.ok) {
#pragma unroll
                for (int d = 0; d <= 2 * CS_BAND; ++d) {
                    const float4 b0 =
                        __ldg(reinterpret_cast<const float4 *>(band_t + (size_t)d * ms + i0));
                    const float bw[4] = {b0.x, b0.y, b0.z, b0.w};
#pragma unroll
                    for (int j = 0; j < BR; ++j) acc[j] = fmaf(bw[j], win[j + d], acc[j]);
                }
            } else if (i0 >= CS_BAND && i0 + BR <= m - CS_BAND) { // interior rows
#pragma unroll
                for (int d = 0; d <= 2 * CS_BAND; ++d)
#pragma unroll
                    for (int j = 0; j < BR; ++j) acc[j] = fmaf(bfac.tau[d], win[j + d], acc[j]);
            } else { // rows near the ends: their own coefficients
#pragma unroll
                for (int j = 0; j < BR; ++j) {
                    const int i = i0 + j;
                    // (rows past m, not kept, take the constants: no loads past the end rows)
                    const bool end = i < m && (i < CS_BAND || i >= m - CS_BAND);
                    const float *e =
                        edge + (size_t)(!end ? 0 : i < CS_BAND ? i : i - m + 2 * CS_BAND) *
                                   (2 * CS_BAND + 1);
#pragma unroll
                    for (int d = 0; d <= 2 * CS_BAND; ++d)
                        acc[j] = fmaf(end ? __ldg(e + d) : bfac.tau[d], win[j + d], acc[j]);
                }
            }
#pragma unroll
            for (int j = 0; j < BR; ++j)
                if (i0 + j < m) cs[i0 + j + 1] = acc[j];
        }
    }
    if (tid == 0) {
        cs[0] = 0.f;
        cs[nk - 1] = 0.f;
    }
    __syncthreads();
    // forward transform input (double-float sampling), bit-reversed
    const bool r2 = RADIX == 4 && (logM & 1);
    bool bad = false;
    if (r2) {
        bad = fill_forward_r2<SWZ>(fbuf, logM, ydf, cs, idx, tdf, sf32,
                                   qfac_df + (size_t)qi * N);
    } else {
        for (int i = tid; i < N; i += bd) {
            const dfl d = sample_input_df(ydf, cs, idx, tdf, sf32, qfac_df + (size_t)qi * N, i);
            if (!isfinite(d.hi)) bad = true;
            const int jj = fft_slot<SWZ>(__brev((unsigned)(i >> 1)) >> (32 - logM), sh);
            fbuf2[2 * jj + (i & 1)] = make_float2(d.hi, d.lo);
        }
    }
    __syncthreads();
    smem_fft_df<RADIX, SWZ>(fbuf, logM, twdf, -1, r2);
    // half spectrum, rounded to float (phase 2 starts: the knots are dead)
    float2 *spec = reinterpret_cast<float2 *>(smem_raw);
    for (int k = tid; k <= M; k += bd) {
        const dfc zk = dfc_load(fbuf[fft_slot<SWZ>(k & (M - 1), sh)]);
        const dfc zm = dfc_conj(dfc_load(fbuf[fft_slot<SWZ>((M - k) & (M - 1), sh)]));
        const dfc e = dfc_add(zk, zm);
        const dfc dd = dfc_sub(zk, zm);
        const dfc o = dfc{dd.im, df_neg(dd.re)};
        const dfc yk = dfc_add(e, dfc_mul(dfc_load(twdf[k]), o));
        const float2 mw = modew_df[k];
        const dfl mm = df_scale(dfl{mw.x, mw.y}, 0.5f);
        const dfl re = df_mul(yk.re, mm), im = df_mul(yk.im, mm);
        spec[k] = make_float2(re.hi + re.lo, -(im.hi + im.lo));
    }
    __syncthreads();
    // the inverse transforms of this q's terms, G at a time
    float2 *buf = reinterpret_cast<float2 *>(smem_raw + L.i);
    const size_t len = (size_t)N + CG_N_SMALL_R + 1;
    for (int gi2 = 0; gi2 < n_grp; ++gi2) {
        const int4 gr = groups[gi2];
        if (gr.x != qi) continue;
        const int ts[3] = {gr.y, gr.z, gr.w};
        const int nact = ts[0] < 0 ? 0 : (ts[1] < 0 ? 1 : (ts[2] < 0 ? 2 : 3));
        for (int k = tid; k <= M / 2; k += bd) {
            const int km = M - k;
            const float2 ik = spec[k], ikm = spec[km], wk = tw32[k], wkm = tw32[km];
            const int pk0 = slot32<SWZ>(__brev((unsigned)k) >> (32 - logM));
            const int pkm = slot32<SWZ>(__brev((unsigned)km) >> (32 - logM));
#pragma unroll
            for (int j = 0; j < G; ++j) {
                if (j >= nact) break;
                const float2 *mc = mcoef32 + (size_t)ts[j] * (M + 1);
                float2 xa = c32_mul(ik, mc[k]);
                float2 xb = c32_mul(ikm, mc[km]);
                if (k == 0) {
                    xa.y = 0.f;
                    xb.y = 0.f;
                }
                buf[j * M + pk0] = c2r_pre32(xa, xb, wk);
                if (k > 0 && k < M / 2) buf[j * M + pkm] = c2r_pre32(xb, xa, wkm);
            }
        }
        __syncthreads();
        smem_fft_f32<SWZ, G>(buf, logM, nact, tw32, +1);
#pragma unroll
        for (int j = 0; j < G; ++j) {
            if (j >= nact) break;
            float *o = tab + ((size_t)s * n_terms + ts[j]) * len + CG_N_SMALL_R + 1;
            const float *pf = postf32 + (size_t)ts[j] * N;
            const float2 *bj = buf + j * M;
            if (fill_small && tid <= CG_N_SMALL_R) o[tid - CG_N_SMALL_R - 1] = cg_nan<float>();
#pragma unroll 4
            for (int i = tid; i < N; i += bd) {
                const float2 z = bj[slot32<SWZ>(i >> 1)];
                const float v = ((i & 1) ? z.y : z.x) * pf[i];
                if (!isfinite(v)) bad = true;
                o[i] = v;
            }
        }
        __syncthreads(); // the buffers are refilled by the next group
    }
    if (bad) cg_flag(err, CG_ERR_NONFINITE);
}

// ------------------------------------------------- r = 0 and sub-Mpc points

// j_l(x): ascending series below max(1, l + 1), upward recurrence above
__device__ double sph_bessel(int l, double x)
{
    const double thr = (l < 1 ? 1.0 : (double)l + 1.0);
    if (x < thr) {
        double pref = 1.0;
        for (int k = 1; k <= l; ++k) pref *= x / (2.0 * k + 1.0);
        const double yy = -0.5 * x * x;
        double term = 1.0, sum = 1.0;
        for (int k = 1; k < 200; ++k) {
            term *= yy / ((double)k * (2.0 * l + 2.0 * k + 1.0));
            sum += term;
            if (fabs(term) < 1e-17 * fabs(sum)) break;
        }
        return pref * sum;
    }
    double sn, cs;
    sincos(x, &sn, &cs);
    double j0 = sn / x;
    if (l == 0) return j0;
    double j1 = (sn / x - cs) / x;
    for (int k = 1; k < l; ++k) {
        const double j2 = (2.0 * k + 1.0) / x * j1 - j0;
        j0 = j1;
        j1 = j2;
    }
    return j1;
}

// Akima spline of the input P(k) (power_spectrum_norm, interp_method default)
struct PkAkima {
    const double *x, *y;
    int n;
    __device__ double operator()(double k) const
    {
        if (!(k >= x[0] && k <= x[n - 1])) return cg_nan<double>();
        int lo = 0, hi = n - 1;
        while (hi > lo + 1) {
            const int mid = (lo + hi) / 2;
            if (x[mid] > k)
                hi = mid;
            else
                lo = mid;
        }
        return akima_eval_at<double>(x, y, n, lo, k);
    }
};

// k^2 P(k) j_l(k r) / (k r)^n  (integrals.c:280-325)
struct BesselIntegrand {
    PkAkima pk;
    double r;
    int n, l;
    __device__ double operator()(double k) const
    {
        const double bf = sph_bessel(l, k * r) / pow(k * r, (double)n);
        return k * k * pk(k) * bf;
    }
};

// k^(2+l-n) P(k)  (integrals.c:238-269)
struct PrefactorIntegrand {
    PkAkima pk;
    int n, l;
    __device__ double operator()(double k) const { return pow(k, 2.0 + l - n) * pk(k); }
};

#define SR_WARPS 4
#define SR_CAP 256

// One warp per (spectrum, term, point j): j = 0 is r = 0, j = 1..42 the
// sub-Mpc separations (integrals.c:524-562), GK61 QAG with epsrel 1e-5.
template <typename TO>
__global__ void __launch_bounds__(32 * SR_WARPS)
    small_r_kernel(const double *__restrict__ kx, const double *__restrict__ pk, int nk,
                   int n_spectra, int n_terms, const int *__restrict__ tn,
                   const int *__restrict__ tl, const double *__restrict__ tab_x, size_t len,
                   TO *__restrict__ tab, int *err)
{
    __shared__ double sa[SR_WARPS][SR_CAP], sb[SR_WARPS][SR_CAP], sr[SR_WARPS][SR_CAP],
        se[SR_WARPS][SR_CAP];
    const int w = threadIdx.x >> 5;
    const long item = (long)blockIdx.x * SR_WARPS + w;
    const long total = (long)n_spectra * n_terms * (CG_N_SMALL_R + 1);
    if (item >= total) return;
    const int j = (int)(item % (CG_N_SMALL_R + 1));
    const long st_ = item / (CG_N_SMALL_R + 1);
    const int t = (int)(st_ % n_terms);
    const int s = (int)(st_ / n_terms);
    const int n = tn[t], l = tl[t];
    if (l < 0) { // half-integer table: the r = 0 and sub-Mpc entries stay NaN
        if ((threadIdx.x & 31) == 0) tab[((size_t)s * n_terms + t) * len + j] = cg_nan<TO>();
        return;
    }
    PkAkima P{kx, pk + (size_t)s * nk, nk};
    QagStore<double> store{sa[w], sb[w], sr[w], se[w], SR_CAP};
    int status = 0;
    double v;
    const double kmin = kx[0], kmax = kx[nk - 1];
    if (j == 0) {
        if (n >= l) {
            PrefactorIntegrand f{P, n, l};
            const double res = qag61_warp<double>(f, kmin, kmax, 0.0, 1e-5, store, 50000, &status);
            const double coeff = sqrt(CG_PI / 2.) / pow(2.0, l + 0.5) / tgamma(l + 1.5);
            v = res / 2. / CG_PI / CG_PI * coeff;
        } else {
            v = 0.0;
        }
    } else {
        const double r = tab_x[j];
        BesselIntegrand f{P, r, n, l};
        double res = qag61_warp<double>(f, kmin, kmax, 0.0, 1e-5, store, 50000, &status);
        if (n >= l) res = res * pow(r, (double)(n - l));
        v = res / 2. / CG_PI / CG_PI;
    }
    if ((threadIdx.x & 31) == 0) {
        if (status == 1) cg_flag(err, CG_ERR_QAG_LIMIT);
        if (!isfinite(v)) cg_flag(err, CG_ERR_NONFINITE);
        tab[((size_t)s * n_terms + t) * len + j] = (TO)v;
    }
}

// (n, l) of the tables whose sub-Mpc entries an adjoint call differentiates
struct SmallRTerms {
    int n[8], l[8];
};

// Adjoint of small_r_kernel for one (spectrum, table t, point j): the table
// cotangent gY[(s * n_at + t) * len + j] carried into dL/dP(k).  With the
// final QAG partition of the entry fixed (recomputed here as small_r_kernel
// found it; it changes only where an error estimate crosses a threshold), the
// entry is sum over the partition's GK61 nodes of weight x kernel(k) x P(k), P
// the Akima spline of the input spectrum: the node cotangents go to the
// spline's knots through its exact partials.
__global__ void __launch_bounds__(32 * SR_WARPS)
    small_r_adjoint_kernel(const double *__restrict__ kx, const double *__restrict__ pk, int nk,
                           int n_spectra, int n_at, SmallRTerms tm,
                           const double *__restrict__ tab_x, size_t len,
                           const double *__restrict__ gY, double *__restrict__ gpk, int *err)
{
    __shared__ double sa[SR_WARPS][SR_CAP], sb[SR_WARPS][SR_CAP], sr[SR_WARPS][SR_CAP],
        se[SR_WARPS][SR_CAP];
    const int w = threadIdx.x >> 5;
    const long item = (long)blockIdx.x * SR_WARPS + w;
    const long total = (long)n_spectra * n_at * (CG_N_SMALL_R + 1);
    if (item >= total) return;
    const int j = (int)(item % (CG_N_SMALL_R + 1));
    const long st_ = item / (CG_N_SMALL_R + 1);
    const int t = (int)(st_ % n_at);
    const int s = (int)(st_ / n_at);
    const double cot = gY[((size_t)s * n_at + t) * len + j];
    const int n = tm.n[t], l = tm.l[t];
    if (cot == 0.0 || l < 0 || (j == 0 && n < l)) return; // whole warps leave together
    const double *ps = pk + (size_t)s * nk;
    PkAkima P{kx, ps, nk};
    QagStore<double> store{sa[w], sb[w], sr[w], se[w], SR_CAP};
    int status = 0, nf = 1;
    const double kmin = kx[0], kmax = kx[nk - 1];
    const double r = tab_x[j];
    double scale;
    if (j == 0) {
        PrefactorIntegrand f{P, n, l};
        qag61_warp<double>(f, kmin, kmax, 0.0, 1e-5, store, 50000, &status, &nf);
        const double coeff = sqrt(CG_PI / 2.) / pow(2.0, l + 0.5) / tgamma(l + 1.5);
        scale = coeff / 2. / CG_PI / CG_PI;
    } else {
        BesselIntegrand f{P, r, n, l};
        qag61_warp<double>(f, kmin, kmax, 0.0, 1e-5, store, 50000, &status, &nf);
        scale = (n >= l ? pow(r, (double)(n - l)) : 1.0) / 2. / CG_PI / CG_PI;
    }
    if (status == 1 && (threadIdx.x & 31) == 0) cg_flag(err, CG_ERR_QAG_LIMIT);
    // the integrand without P(k)
    auto kernel = [&](double k) {
        if (j == 0) return pow(k, 2.0 + l - n);
        return k * k * sph_bessel(l, k * r) / pow(k * r, (double)n);
    };
    // one GK61 node at k with weight wgt (the Kronrod result is
    // half_length x sum wgk f)
    auto scatter = [&](double k, double wgt) {
        int lo = 0, hi = nk - 1;
        while (hi > lo + 1) {
            const int mid = (lo + hi) / 2;
            if (kx[mid] > k)
                hi = mid;
            else
                lo = mid;
        }
        const D6 v = akima_eval_d6(kx, ps, nk, lo, k);
        const double g = cot * scale * wgt * kernel(k);
        double *dst = gpk + (size_t)s * nk + d6_base(nk, lo);
        for (int q = 0; q < 6; ++q)
            if (v.g[q] != 0.0) atomicAdd(dst + q, g * v.g[q]);
    };
    const GkLane<double> gl = gk_lane<double>();
    for (int p = 0; p < nf; ++p) {
        const double a = nf == 1 ? kmin : store.a[p], b = nf == 1 ? kmax : store.b[p];
        const double center = 0.5 * (a + b), half = 0.5 * (b - a);
        if (gl.centre) {
            scatter(center, half * gl.wk);
        } else if (gl.active) {
            const double absc = half * gl.x;
            scatter(center - absc, half * gl.wk);
            scatter(center + absc, half * gl.wk);
        }
    }
}

// ---------------------------------------------- divergent I^4_0 (integrals.c:773-914)
// The integrands of the divergent integral: P (1 - j0(kr)^2) / k^2 (its r = 0
// renormalisation, integrals.c:390-404) and P j0(k chi1) j0(k chi2) / k^2 (the
// renormalisation term, integrals.c:406-422); the integral itself is
// BesselIntegrand with n = 4, l = 0.
struct RenormIntegrand {
    PkAkima pk;
    double r1, r2;
    bool zero; // the r = 0 form
    __device__ double operator()(double k) const
    {
        const double j1 = sph_bessel(0, k * r1);
        const double w = zero ? 1.0 - j1 * j1 : j1 * sph_bessel(0, k * r2);
        return pk(k) * w / k / k;
    }
};

// One warp per item, GK61 QAG at relative 1e-5 over [kmin, kmax] (the
// reference's coffe_integrate_1d_prec_gsl).  grid == 0: items 0..n1-1 are
// r^4 I^4_0(r1[i]) / 2 pi^2, items n1..2 n1-1 the r^4-scaled r = 0
// renormalisation integral / 2 pi^2 (integrals.c:803-826), each with a
// DIV_CAP-interval store in `scratch` (below r ~ 1e-4 Mpc the reference's
// 1 - j0(kr)^2 is rounding noise and QAG bisects ~1000 times before it stops);
// grid != 0: item b * n1 + a is the renormalisation term at (r1[a], r2[b]) /
// 2 pi^2 (under 30 intervals: a shared-memory store).
#define DIV_CAP 4096
#define DIV_CHUNK 1024
__global__ void __launch_bounds__(32 * SR_WARPS)
    divergent_kernel(const double *__restrict__ kx, const double *__restrict__ pk, int nk,
                     double kmin, double kmax, const double *__restrict__ r1,
                     const double *__restrict__ r2, long n1, long item0, long n_items,
                     int grid, double *__restrict__ scratch, double *__restrict__ out, int *err)
{
    __shared__ double sa[SR_WARPS][SR_CAP], sb[SR_WARPS][SR_CAP], sr[SR_WARPS][SR_CAP],
        se[SR_WARPS][SR_CAP];
    const int w = threadIdx.x >> 5;
    const long item = item0 + (long)blockIdx.x * SR_WARPS + w;
    if (item >= n_items) return;
    PkAkima P{kx, pk, nk};
    // launches of at most DIV_CHUNK items: the store of item sits at item - item0
    double *g = scratch + (size_t)(item - item0) * 4 * DIV_CAP;
    const QagStore<double> store =
        grid ? QagStore<double>{sa[w], sb[w], sr[w], se[w], SR_CAP}
             : QagStore<double>{g, g + DIV_CAP, g + 2 * DIV_CAP, g + 3 * DIV_CAP, DIV_CAP};
    int status = 0;
    double v;
    if (grid) {
        RenormIntegrand f{P, r1[item % n1], r2[item / n1], false};
        v = qag61_warp<double>(f, kmin, kmax, 0.0, 1e-5, store, 50000, &status);
    } else if (item < n1) {
        const double r = r1[item];
        BesselIntegrand f{P, r, 4, 0};
        v = qag61_warp<double>(f, kmin, kmax, 0.0, 1e-5, store, 50000, &status) * pow(r, 4.0);
    } else {
        const double r = r1[item - n1];
        RenormIntegrand f{P, r, 0.0, true};
        v = qag61_warp<double>(f, kmin, kmax, 0.0, 1e-5, store, 50000, &status) * pow(r, 4.0);
    }
    v = v / 2. / CG_PI / CG_PI;
    if ((threadIdx.x & 31) == 0) {
        if (status == 1) cg_flag(err, CG_ERR_QAG_LIMIT);
        if (!isfinite(v)) cg_flag(err, CG_ERR_NONFINITE);
        out[item] = v;
    }
}

template <typename TO> __global__ void fill_nan_kernel(TO *tab, size_t len, long count)
{
    const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count * (CG_N_SMALL_R + 1)) return;
    const long tb = i / (CG_N_SMALL_R + 1), j = i % (CG_N_SMALL_R + 1);
    tab[tb * len + j] = (TO)cg_nan<double>();
}

__global__ void table_eval_kernel(const double *__restrict__ x, const double *__restrict__ y,
                                  int n, const double *__restrict__ r, int nq,
                                  double *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const double v = r[i];
    if (!(v >= x[0] && v <= x[n - 1])) {
        out[i] = cg_nan<double>();
        return;
    }
    int lo = 0, hi = n - 1;
    while (hi > lo + 1) {
        const int mid = (lo + hi) / 2;
        if (x[mid] > v)
            hi = mid;
        else
            lo = mid;
    }
    out[i] = akima_eval_at<double>(x, y, n, lo, v);
}

__global__ void table_f32_to_f64_kernel(const float *__restrict__ in, double *__restrict__ out,
                                        size_t n)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (double)in[i];
}

bool same_grid(const coffe_gpu_ctx *ctx, const double *k, size_t nk, size_t N,
               const std::vector<int> &terms)
{
    if (ctx->grid_N != N || ctx->grid_nk != nk || ctx->grid_terms != terms) return false;
    if (ctx->grid_k.size() != nk) return false;
    return std::memcmp(ctx->grid_k.data(), k, sizeof(double) * nk) == 0;
}

} // namespace

// Byte offsets of the mixed path's per-grid arrays in ctx->term_df, each
// rounded up to 256 bytes (float4 accesses need 16-byte alignment, and
// N/2 + 1 entries of 8 bytes are not a multiple of 16)
struct TermDfLayout {
    size_t wdf, tw32, m32, mdf, pdf, p32, total;
};
static TermDfLayout term_df_layout(int M, int N, int n_terms)
{
    auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
    TermDfLayout l;
    l.wdf = 0;
    l.tw32 = up(l.wdf + sizeof(float2) * (M + 1));
    l.m32 = up(l.tw32 + sizeof(float2) * (M + 1));
    l.mdf = up(l.m32 + sizeof(float2) * (size_t)(M + 1) * n_terms);
    l.pdf = up(l.mdf + sizeof(float4) * (size_t)(M + 1) * n_terms);
    l.p32 = up(l.pdf + sizeof(float2) * (size_t)N * n_terms);
    l.total = up(l.p32 + sizeof(float) * (size_t)N * n_terms);
    return l;
}

int integrals_build(coffe_gpu_ctx *ctx, const double *k, const double *pk, int n_spectra,
                    size_t nk, const int *n, const int *l, const int *half, int n_terms, size_t N,
                    int precision, unsigned flags)
{
    if (!k || !pk || !n || !l || n_spectra < 1 || n_terms < 1 || n_terms > CG_MAX_TERMS) {
        cg_set_error(ctx, "integrals: bad arguments (n_spectra=%d, n_terms=%d)", n_spectra,
                     n_terms);
        return COFFE_GPU_EINVAL;
    }
    if (N < 64 || N > 16384 || (N & (N - 1))) {
        cg_set_error(ctx, "integrals: N must be a power of two in [64, 16384] (got %zu)", N);
        return COFFE_GPU_EINVAL;
    }
    if (nk < 5 || nk > (1u << 22)) {
        cg_set_error(ctx, "integrals: need 5 <= nk <= 2^22 k samples (got %zu)", nk);
        return COFFE_GPU_EINVAL;
    }
    if (precision != COFFE_GPU_FP64 && precision != COFFE_GPU_MIXED) {
        cg_set_error(ctx, "integrals: unknown precision %d", precision);
        return COFFE_GPU_EINVAL;
    }
    for (size_t i = 0; i < nk; ++i)
        if (!(k[i] > 0) || (i > 0 && !(k[i] > k[i - 1]))) {
            cg_set_error(ctx, "integrals: k must be positive and strictly increasing");
            return COFFE_GPU_EINVAL;
        }
    for (int t = 0; t < n_terms; ++t) {
        const int hf = half ? half[t] : 0;
        if (hf != 0 && hf != 1) {
            cg_set_error(ctx, "integrals: half[%d] must be 0 or 1", t);
            return COFFE_GPU_EINVAL;
        }
        const int lmax = hf ? 33 : 16, nmin = hf ? -8 : -4, nmax = hf ? 33 : 16;
        if (l[t] < 0 || l[t] > lmax || n[t] < nmin || n[t] > nmax) {
            cg_set_error(ctx, "integrals: unsupported term (n=%d, l=%d%s)", n[t], l[t],
                         hf ? ", half-integer numerators" : "");
            return COFFE_GPU_EINVAL;
        }
    }
    cg_timing_begin(ctx);
    const bool mixed = precision == COFFE_GPU_MIXED;
    const bool tables_df = mixed && (flags & COFFE_GPU_TABLES_DF) != 0;
    const int M = (int)N / 2;
    const size_t len = N + CG_N_SMALL_R + 1;
    int st;
    ctx->int_ready = false;

    // distinct total biases q + nu
    std::vector<double> qvals;
    std::vector<int> term_q(n_terms);
    std::vector<double> tq(n_terms), tl(n_terms), tn(n_terms);
    for (int t = 0; t < n_terms; ++t) {
        // half-integer terms (integrals.c:189-207): n, l are numerators of n/2, l/2
        const int hf = half ? half[t] : 0;
        const double lt = hf ? l[t] / 2.0 : (double)l[t], nt = hf ? n[t] / 2.0 : (double)n[t];
        const double qnu = select_qnu(lt, nt);
        const double qt = qnu + nt;
        int qi = -1;
        for (size_t j = 0; j < qvals.size(); ++j)
            if (qvals[j] == qt) qi = (int)j;
        if (qi < 0) {
            qi = (int)qvals.size();
            qvals.push_back(qt);
        }
        term_q[t] = qi;
        tq[t] = qnu;
        tl[t] = lt;
        tn[t] = nt;
        ctx->term_n[t] = n[t];
        ctx->term_l[t] = l[t];
        ctx->term_half[t] = hf;
        ctx->term_q[t] = qi;
    }
    const int n_q = (int)qvals.size();
    std::vector<int> terms_key;
    for (int t = 0; t < n_terms; ++t) {
        terms_key.push_back(n[t]);
        terms_key.push_back(l[t]);
        terms_key.push_back(half ? half[t] : 0);
    }

    GridPar g{k[0], k[nk - 1], k[0], 1.0, (int)N, (int)nk};
    const bool grid_cached = same_grid(ctx, k, nk, N, terms_key);
    // device buffers
    const bool pk_on_device = (flags & COFFE_GPU_PK_DEVICE) != 0;
    if ((!pk_on_device || (flags & COFFE_GPU_SMALL_R)) &&
        (st = cg_ensure(ctx, ctx->pk, sizeof(double) * nk * n_spectra)))
        return st;
    if ((st = cg_ensure(ctx, ctx->csc, sizeof(double) * nk * n_spectra))) return st;
    if ((st = cg_ensure(ctx, ctx->spec, sizeof(double2) * (M + 1) * (size_t)n_spectra * n_q)))
        return st;
    if ((st = cg_ensure(ctx, ctx->tab_y, (mixed ? sizeof(float) : sizeof(double)) * len *
                                             (size_t)n_spectra * n_terms)))
        return st;
    if (!grid_cached) {
        if ((st = cg_ensure(ctx, ctx->kgrid, sizeof(double) * nk))) return st;
        if ((st = cg_ensure(ctx, ctx->csfac, sizeof(double) * 3 * nk))) return st;
        if ((st = cg_ensure(ctx, ctx->samp_idx, sizeof(int) * N))) return st;
        if ((st = cg_ensure(ctx, ctx->samp_dx, sizeof(double) * N))) return st;
        if ((st = cg_ensure(ctx, ctx->samp_f32, sizeof(float4) * N))) return st;
        if ((st = cg_ensure(ctx, ctx->csfac32, sizeof(float) * 4 * nk))) return st;
        if ((st = cg_ensure(ctx, ctx->samp_tdf, sizeof(float2) * N))) return st;
        if ((st = cg_ensure(ctx, ctx->qfac_df, sizeof(float2) * N * n_q))) return st;
        if ((st = cg_ensure(ctx, ctx->qfac, sizeof(double) * N * n_q))) return st;
        if ((st = cg_ensure(ctx, ctx->modec, sizeof(double2) * (M + 1) * n_terms + sizeof(double) * (M + 1)))) return st;
        if ((st = cg_ensure(ctx, ctx->postf, sizeof(double) * N * n_terms))) return st;
        if ((st = cg_ensure(ctx, ctx->twid, sizeof(double2) * (M + 1)))) return st;
        if ((st = cg_ensure(ctx, ctx->twid32, sizeof(float4) * (M + 1)))) return st;
        if ((st = cg_ensure(ctx, ctx->term_df, term_df_layout(M, (int)N, n_terms).total)))
            return st;
        if ((st = cg_ensure(ctx, ctx->tab_x, sizeof(double) * len))) return st;
        if ((st = cg_ensure(ctx, ctx->tab_x32, sizeof(float) * len))) return st;
    }
    // term metadata (small, staged through the request buffer)
    struct TermMeta {
        double q[CG_MAX_TERMS], l[CG_MAX_TERMS], n[CG_MAX_TERMS], qv[CG_MAX_TERMS];
        int tq[CG_MAX_TERMS], tn[CG_MAX_TERMS], tl[CG_MAX_TERMS];
        int4 grp[CG_MAX_TERMS]; // FP32 inverse transforms: (q, up to 3 terms of that q)
    } meta;
    // terms sharing a forward spectrum go through the FP32 inverse kernel
    // together, inv_g of them per block (one per block when three do not fit
    // the shared memory twice over)
    const int inv_g = 3 * sizeof(float2) * (size_t)M <= 112 * 1024 ? 3 : 1;
    int n_grp = 0;
    for (int q = 0; q < (int)qvals.size(); ++q) {
        int cur[3] = {-1, -1, -1}, nc = 0;
        for (int t = 0; t <= n_terms; ++t) {
            if (t < n_terms && term_q[t] == q) cur[nc++] = t;
            if (nc == inv_g || (t == n_terms && nc > 0)) {
                meta.grp[n_grp++] = make_int4(q, cur[0], cur[1], cur[2]);
                cur[0] = cur[1] = cur[2] = -1;
                nc = 0;
            }
        }
    }
    for (int t = 0; t < n_terms; ++t) {
        meta.q[t] = tq[t];
        meta.l[t] = tl[t];
        meta.n[t] = tn[t];
        meta.tq[t] = term_q[t];
        meta.tn[t] = n[t];
        meta.tl[t] = (half && half[t]) ? -1 : l[t]; // -1: no sub-Mpc QAG entries
    }
    for (int q = 0; q < n_q; ++q) meta.qv[q] = qvals[q];
    if ((st = cg_ensure(ctx, ctx->term_meta, sizeof(TermMeta)))) return st;
    TermMeta *d_meta = (TermMeta *)ctx->term_meta.p;
    if (!grid_cached)
        CG_CUDA(ctx, cudaMemcpyAsync(d_meta, &meta, sizeof(TermMeta), cudaMemcpyHostToDevice,
                                     ctx->stream));
    const double *d_pk = pk_on_device ? pk : (const double *)ctx->pk.p;
    // (host P(k) is uploaded below, once the launch configuration is known)
    if (pk_on_device && (flags & COFFE_GPU_SMALL_R)) // kept for the adjoint of the sub-Mpc entries
        CG_CUDA(ctx, cudaMemcpyAsync(ctx->pk.p, pk, sizeof(double) * nk * n_spectra,
                                     cudaMemcpyDeviceToDevice, ctx->stream));

    double2 *mcoef = (double2 *)ctx->modec.p;
    double *modew = (double *)((char *)ctx->modec.p + sizeof(double2) * (M + 1) * n_terms);
    // mixed path: mode taper (double-float), twiddles, kernel and prefactors
    // (float, and double-float for COFFE_GPU_TABLES_DF)
    const TermDfLayout lay = term_df_layout(M, (int)N, n_terms);
    char *tdb = (char *)ctx->term_df.p;
    float2 *wdf = (float2 *)(tdb + lay.wdf);
    float2 *tw32 = (float2 *)(tdb + lay.tw32);
    float2 *m32 = (float2 *)(tdb + lay.m32);
    float4 *mdf = (float4 *)(tdb + lay.mdf);
    float2 *pdf = (float2 *)(tdb + lay.pdf);
    float *p32 = (float *)(tdb + lay.p32);
    if (!grid_cached) {
        CG_CUDA(ctx, cudaMemcpyAsync(ctx->kgrid.p, k, sizeof(double) * nk, cudaMemcpyHostToDevice,
                                     ctx->stream));
        double hx[CG_N_SMALL_R + 1];
        hx[0] = 0.0;
        for (int i = 0; i < CG_N_SMALL_R; ++i) hx[i + 1] = h_min_sep[i];
        float hx32[CG_N_SMALL_R + 1];
        for (int i = 0; i <= CG_N_SMALL_R; ++i) hx32[i] = (float)hx[i];
        CG_CUDA(ctx, cudaMemcpyAsync(ctx->tab_x.p, hx, sizeof(hx), cudaMemcpyHostToDevice,
                                     ctx->stream));
        CG_CUDA(ctx, cudaMemcpyAsync(ctx->tab_x32.p, hx32, sizeof(hx32), cudaMemcpyHostToDevice,
                                     ctx->stream));
        // spline factors and the band of the inverse spline matrix, computed
        // on the host; the host arrays live in the context, so the copies need
        // no synchronisation for their sake
        csfac_host(k, (int)nk, ctx->grid_fac_host, ctx->grid_fac32_host);
        cspline_band_host(std::vector<double>(k, k + nk), ctx->grid_band_host);
        {
            std::vector<float> edge;
            const BandFac bfac =
                cspline_band_factor(std::vector<double>(k, k + nk), ctx->grid_band_host, edge);
            ctx->grid_band_ok = bfac.ok;
            for (int d = 0; d <= 2 * CS_BAND; ++d) ctx->grid_band_tau[d] = bfac.tau[d];
            // the end rows' coefficients follow the band rows
            ctx->grid_band_host.insert(ctx->grid_band_host.end(), edge.begin(), edge.end());
        }
        if ((st = cg_ensure(ctx, ctx->csband, sizeof(float) * ctx->grid_band_host.size())))
            return st;
        CG_CUDA(ctx, cudaMemcpyAsync(ctx->csfac.p, ctx->grid_fac_host.data(),
                                     sizeof(double) * ctx->grid_fac_host.size(),
                                     cudaMemcpyHostToDevice, ctx->stream));
        CG_CUDA(ctx, cudaMemcpyAsync(ctx->csfac32.p, ctx->grid_fac32_host.data(),
                                     sizeof(float) * ctx->grid_fac32_host.size(),
                                     cudaMemcpyHostToDevice, ctx->stream));
        CG_CUDA(ctx, cudaMemcpyAsync(ctx->csband.p, ctx->grid_band_host.data(),
                                     sizeof(float) * ctx->grid_band_host.size(),
                                     cudaMemcpyHostToDevice, ctx->stream));
        const int tb = 256;
        sampling_kernel<<<((int)N + tb) / tb, tb, 0, ctx->stream>>>(
            g, (const double *)ctx->kgrid.p, (int *)ctx->samp_idx.p, (double *)ctx->samp_dx.p,
            (float4 *)ctx->samp_f32.p, n_q, d_meta->qv, (double *)ctx->qfac.p, modew,
            (double *)ctx->tab_x.p, (float *)ctx->tab_x32.p, (float2 *)ctx->samp_tdf.p,
            (float2 *)ctx->qfac_df.p);
        if ((st = cg_after_launch(ctx, "sampling_kernel"))) return st;
        dim3 tg(((int)N + tb - 1) / tb + 1, n_terms);
        term_tables_kernel<<<tg, tb, 0, ctx->stream>>>(g, n_terms, d_meta->q, d_meta->l,
                                                        d_meta->n, mcoef, (double *)ctx->postf.p,
                                                        ctx->d_err);
        if ((st = cg_after_launch(ctx, "term_tables_kernel"))) return st;
        twiddle_kernel<<<(M + 1 + tb - 1) / tb, tb, 0, ctx->stream>>>(
            (int)N, (double2 *)ctx->twid.p, (float4 *)ctx->twid32.p);
        if ((st = cg_after_launch(ctx, "twiddle_kernel"))) return st;
        term_tables_df_kernel<<<tg, tb, 0, ctx->stream>>>(
            M, (int)N, n_terms, mcoef, (const double *)ctx->postf.p, modew,
            (const double2 *)ctx->twid.p, wdf, m32, p32, tw32, mdf, pdf);
        if ((st = cg_after_launch(ctx, "term_tables_df_kernel"))) return st;
        if ((st = cg_check_device_errors(ctx, "FFTLog coefficient tables"))) return st;
        ctx->grid_N = N;
        ctx->grid_nk = nk;
        ctx->grid_k.assign(k, k + nk);
        ctx->grid_terms = terms_key;
    }
    // per spectrum: natural-spline coefficients, forward FFTs, inverse FFTs
    if (mixed && (st = cg_ensure(ctx, ctx->pk_df, sizeof(float2) * nk * n_spectra))) return st;
    const size_t smem = sizeof(double2) * M; // == sizeof(float4) * M
    const size_t smem32 = sizeof(float2) * M * (size_t)inv_g;
    const dim3 gf(n_spectra, n_q), gi(n_spectra, n_terms), gg(n_spectra, n_grp);
    // the FP32 inverse kernel fills the 43 uncomputed entries itself
    const int fill_small = (flags & COFFE_GPU_SMALL_R) ? 0 : 1;
    // the fused mixed table kernel: one block per (spectrum, q), everything in
    // shared memory, where that fits
    const FusedLayout fl = fused_layout((int)nk, M, inv_g);
    const bool fused_ok = mixed && !tables_df && nk >= (size_t)M + 1 && nk <= 8192 &&
                          N <= 8192 && fl.total <= 200 * 1024;
    BandFac bfac;
    bfac.ok = ctx->grid_band_ok;
    for (int d = 0; d <= 2 * CS_BAND; ++d) bfac.tau[d] = ctx->grid_band_tau[d];
    // the fused kernel over spectra [s0, s0 + ns), P(k) of spectrum s0 at pks
    // (occ: only the kernel's resident blocks per SM, nothing launched)
    auto launch_fused = [&](const coffe_gpu_tuning_t &tu, int s0, int ns, const double *pks,
                            int *occ) -> int {
        int s2;
        const dim3 gfc(ns, n_q);
        float *tab0 = (float *)ctx->tab_y.p + (size_t)s0 * n_terms * (N + CG_N_SMALL_R + 1);
#define FUSED_LAUNCH(R, W, G)                                                                     \
    {                                                                                             \
        CG_CUDA(ctx, cudaFuncSetAttribute(fftlog_tables_fused_kernel<R, W, G>,                    \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,            \
                                          (int)fl.total));                                        \
        if (occ) {                                                                                \
            CG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(                           \
                             occ, fftlog_tables_fused_kernel<R, W, G>, FUSED_THREADS, fl.total)); \
            return COFFE_GPU_OK;                                                                  \
        }                                                                                         \
        fftlog_tables_fused_kernel<R, W, G><<<gfc, FUSED_THREADS, fl.total, ctx->stream>>>(       \
            g, pks, d_pk + nk * (size_t)n_spectra, (const float *)ctx->csband.p, bfac,            \
            (const float *)ctx->csfac32.p,                                                        \
            (const int *)ctx->samp_idx.p, (const float2 *)ctx->samp_tdf.p,                        \
            (const float4 *)ctx->samp_f32.p, (const float2 *)ctx->qfac_df.p, wdf,                 \
            (const float4 *)ctx->twid32.p, d_meta->grp, n_grp, n_terms, m32, p32, tw32, tab0,     \
            fill_small, ctx->d_err);                                                              \
        if ((s2 = cg_after_launch(ctx, "fftlog_tables_fused_kernel"))) return s2;                 \
    }
        const bool swz = tu.fft_swizzle && M >= 64;
        if (inv_g == 3) {
            if (tu.fft_radix == 2) {
                if (swz) FUSED_LAUNCH(2, true, 3) else FUSED_LAUNCH(2, false, 3)
            } else {
                if (swz) FUSED_LAUNCH(4, true, 3) else FUSED_LAUNCH(4, false, 3)
            }
        } else {
            if (tu.fft_radix == 2) {
                if (swz) FUSED_LAUNCH(2, true, 1) else FUSED_LAUNCH(2, false, 1)
            } else {
                if (swz) FUSED_LAUNCH(4, true, 1) else FUSED_LAUNCH(4, false, 1)
            }
        }
#undef FUSED_LAUNCH
        return COFFE_GPU_OK;
    };
    auto stage = [&](const coffe_gpu_tuning_t &tu) -> int {
        int s2;
        if (fused_ok && tu.fft_fused) return launch_fused(tu, 0, n_spectra, d_pk, nullptr);
        if (mixed) {
            const dim3 gb(((int)nk - 2 + CS_TILE - 1) / CS_TILE,
                          (n_spectra + tu.spline_group - 1) / tu.spline_group);
#define CS_LAUNCH(G)                                                                              \
    cspline_band_kernel<G><<<gb, CS_TILE, 0, ctx->stream>>>(                                      \
        d_pk, (const float *)ctx->csband.p, (const float *)ctx->csfac32.p, (int)nk, n_spectra,    \
        (float2 *)ctx->pk_df.p, (float *)ctx->csc.p)
            if (tu.spline_group == 2)
                CS_LAUNCH(2);
            else if (tu.spline_group == 4)
                CS_LAUNCH(4);
            else
                CS_LAUNCH(8);
#undef CS_LAUNCH
            if ((s2 = cg_after_launch(ctx, "cspline_band_kernel"))) return s2;
#define DF_LAUNCH(R, W)                                                                           \
    {                                                                                             \
        if (tables_df) {                                                                          \
            CG_CUDA(ctx, cudaFuncSetAttribute(fftlog_forward_df_kernel<R, W, float4>,             \
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,        \
                                              (int)smem));                                        \
            CG_CUDA(ctx, cudaFuncSetAttribute(fftlog_inverse_df_kernel<R, W>,                     \
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,        \
                                              (int)smem));                                        \
            fftlog_forward_df_kernel<R, W, float4><<<gf, tu.fft_threads_fwd, smem, ctx->stream>>>( \
                g, (const float2 *)ctx->pk_df.p, (const float *)ctx->csc.p,                       \
                (const int *)ctx->samp_idx.p, (const float2 *)ctx->samp_tdf.p,                    \
                (const float4 *)ctx->samp_f32.p, (const float2 *)ctx->qfac_df.p, wdf,             \
                (const float4 *)ctx->twid32.p, n_q, (float4 *)ctx->spec.p, ctx->d_err);           \
            if ((s2 = cg_after_launch(ctx, "fftlog_forward_df_kernel"))) return s2;               \
            fftlog_inverse_df_kernel<R, W><<<gi, tu.fft_threads, smem, ctx->stream>>>(            \
                g, (const float4 *)ctx->spec.p, d_meta->tq, n_q, n_terms, mdf, pdf,               \
                (const float4 *)ctx->twid32.p, (float *)ctx->tab_y.p, ctx->d_err);                \
            if ((s2 = cg_after_launch(ctx, "fftlog_inverse_df_kernel"))) return s2;               \
        } else {                                                                                  \
            CG_CUDA(ctx, cudaFuncSetAttribute(fftlog_forward_df_kernel<R, W, float2>,             \
                                              cudaFuncAttributeMaxDynamicSharedMemorySize,        \
                                              (int)smem));                                        \
            if (inv_g == 3)                                                                       \
                CG_CUDA(ctx, cudaFuncSetAttribute(fftlog_inverse_f32_kernel<W, 3>,                \
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                                                  (int)smem32));                                  \
            else                                                                                  \
                CG_CUDA(ctx, cudaFuncSetAttribute(fftlog_inverse_f32_kernel<W, 1>,                \
                                                  cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                                                  (int)smem32));                                  \
            fftlog_forward_df_kernel<R, W, float2><<<gf, tu.fft_threads_fwd, smem, ctx->stream>>>( \
                g, (const float2 *)ctx->pk_df.p, (const float *)ctx->csc.p,                       \
                (const int *)ctx->samp_idx.p, (const float2 *)ctx->samp_tdf.p,                    \
                (const float4 *)ctx->samp_f32.p, (const float2 *)ctx->qfac_df.p, wdf,             \
                (const float4 *)ctx->twid32.p, n_q, (float2 *)ctx->spec.p, ctx->d_err);           \
            if ((s2 = cg_after_launch(ctx, "fftlog_forward_df_kernel"))) return s2;               \
            if (inv_g == 3)                                                                       \
                fftlog_inverse_f32_kernel<W, 3><<<gg, tu.fft_threads, smem32, ctx->stream>>>(     \
                    g, (const float2 *)ctx->spec.p, d_meta->grp, n_q, n_terms, m32, p32, tw32,    \
                    (float *)ctx->tab_y.p, fill_small, ctx->d_err);                               \
            else                                                                                  \
                fftlog_inverse_f32_kernel<W, 1><<<gg, tu.fft_threads, smem32, ctx->stream>>>(     \
                    g, (const float2 *)ctx->spec.p, d_meta->grp, n_q, n_terms, m32, p32, tw32,    \
                    (float *)ctx->tab_y.p, fill_small, ctx->d_err);                               \
            if ((s2 = cg_after_launch(ctx, "fftlog_inverse_f32_kernel"))) return s2;              \
        }                                                                                         \
    }
            const bool swz = tu.fft_swizzle && M >= 64;
            if (tu.fft_radix == 2) {
                if (swz) DF_LAUNCH(2, true) else DF_LAUNCH(2, false)
            } else {
                if (swz) DF_LAUNCH(4, true) else DF_LAUNCH(4, false)
            }
#undef DF_LAUNCH
            return COFFE_GPU_OK;
        }
        cspline_c_kernel<<<(n_spectra + 3) / 4, 128, 0, ctx->stream>>>(
            (const double *)ctx->kgrid.p, d_pk, (const double *)ctx->csfac.p, (int)nk, n_spectra,
            (double *)ctx->csc.p);
        if ((s2 = cg_after_launch(ctx, "cspline_c_kernel"))) return s2;
        CG_CUDA(ctx, cudaFuncSetAttribute(fftlog_forward_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        CG_CUDA(ctx, cudaFuncSetAttribute(fftlog_inverse_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        fftlog_forward_kernel<<<gf, tu.fft_threads_fwd, smem, ctx->stream>>>(
            g, (const double *)ctx->kgrid.p, d_pk, (const double *)ctx->csc.p,
            (const double *)ctx->csfac.p, (const int *)ctx->samp_idx.p,
            (const double *)ctx->samp_dx.p, (const double *)ctx->qfac.p, modew,
            (const double2 *)ctx->twid.p, n_q, (double2 *)ctx->spec.p, ctx->d_err);
        if ((s2 = cg_after_launch(ctx, "fftlog_forward_kernel"))) return s2;
        fftlog_inverse_kernel<<<gi, tu.fft_threads, smem, ctx->stream>>>(
            g, (const double2 *)ctx->spec.p, d_meta->tq, n_q, n_terms, mcoef,
            (const double *)ctx->postf.p, (const double2 *)ctx->twid.p, (double *)ctx->tab_y.p,
            ctx->d_err);
        return cg_after_launch(ctx, "fftlog_inverse_kernel");
    };
    // candidate launch shapes of this table stage
    std::vector<coffe_gpu_tuning_t> cands;
    for (int fu : {0, 1})
    for (int ff : {256, 512})
    for (int ft : {128, 256, 512})
        for (int rad : {2, 4})
            for (int sw : {0, 1})
                for (int grp : {2, 4, 8}) {
                    coffe_gpu_tuning_t c = ctx->tuning;
                    c.fft_threads = ft;
                    c.fft_threads_fwd = ff;
                    c.fft_fused = fu;
                    // the fused kernel has fixed block shapes and no spline grouping
                    if (fu && (!fused_ok || ft != 256 || ff != 512 || grp != 8)) continue;
                    if (mixed) {
                        if (sw && M < 64) continue;
                        c.fft_radix = rad;
                        c.fft_swizzle = sw;
                        c.spline_group = grp;
                    } else if (rad != 2 || sw || grp != 2) {
                        continue; // the FP64 transforms have only the thread count
                    }
                    cands.push_back(c);
                }
    const std::array<long long, 6> key{1, (long long)N, n_spectra, n_terms, n_q,
                                       mixed ? (tables_df ? 2 : 1) : 0};
    coffe_gpu_tuning_t tu = ctx->tuning;
    bool known = !ctx->autotune;
    {
        const auto it = ctx->tune_cache.find(key);
        if (it != ctx->tune_cache.end()) {
            tu = it->second;
            known = true;
        }
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    CG_CUDA(ctx, cudaStreamIsCapturing(ctx->stream, &cap));
    // host P(k) for the fused kernel with a known configuration: uploaded in
    // two parts on the copy stream, so that the tables of the first wave of
    // spectra (the blocks the device holds at once) are made while the rest
    // is on its way
    int first = n_spectra;
    if (!pk_on_device && known && fused_ok && tu.fft_fused && !(flags & COFFE_GPU_SMALL_R) &&
        cap == cudaStreamCaptureStatusNone) {
        int occ = 0;
        if ((st = launch_fused(tu, 0, 0, nullptr, &occ))) return st;
        if (ctx->sm_count <= 0)
            CG_CUDA(ctx, cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount,
                                                ctx->device));
        first = std::min(n_spectra, std::max(1, occ * ctx->sm_count / n_q));
    }
    if (first < n_spectra) {
        if ((st = cg_copy_stream(ctx))) return st;
        const size_t row = sizeof(double) * nk;
        double *dst = (double *)ctx->pk.p;
        CG_CUDA(ctx, cudaEventRecord(ctx->copy_ev[0], ctx->stream)); // earlier readers of ctx->pk
        CG_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->copy_ev[0], 0));
        CG_CUDA(ctx, cudaMemcpyAsync(dst, pk, row * first, cudaMemcpyHostToDevice,
                                     ctx->copy_stream));
        CG_CUDA(ctx, cudaEventRecord(ctx->copy_ev[1], ctx->copy_stream));
        CG_CUDA(ctx, cudaMemcpyAsync(dst + (size_t)first * nk, pk + (size_t)first * nk,
                                     row * (n_spectra - first), cudaMemcpyHostToDevice,
                                     ctx->copy_stream));
        CG_CUDA(ctx, cudaEventRecord(ctx->copy_ev[2], ctx->copy_stream)); // P(k) consumed
        CG_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->copy_ev[1], 0));
        if ((st = launch_fused(tu, 0, first, dst, nullptr))) return st;
        CG_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->copy_ev[2], 0));
        if ((st = launch_fused(tu, first, n_spectra - first, dst + (size_t)first * nk, nullptr)))
            return st;
    } else {
        if (!pk_on_device) {
            CG_CUDA(ctx, cudaMemcpyAsync(ctx->pk.p, pk, sizeof(double) * nk * n_spectra,
                                         cudaMemcpyHostToDevice, ctx->stream));
            if ((st = cg_copy_stream(ctx))) return st;
            CG_CUDA(ctx, cudaEventRecord(ctx->copy_ev[2], ctx->stream)); // P(k) consumed
        }
        if ((st = cg_tuned(ctx, key, cands, stage, &tu, /*cold=*/true))) return st;
        if ((st = stage(tu))) return st;
    }
    ctx->last_tuning.fft_threads = tu.fft_threads;
    ctx->last_tuning.fft_threads_fwd = tu.fft_threads_fwd;
    if (mixed) {
        ctx->last_tuning.fft_radix = tu.fft_radix;
        ctx->last_tuning.fft_swizzle = tu.fft_swizzle;
        ctx->last_tuning.spline_group = tu.spline_group;
        ctx->last_tuning.fft_fused = fused_ok && tu.fft_fused;
    }
    // r = 0 and sub-Mpc entries
    const long tables = (long)n_spectra * n_terms;
    if (flags & COFFE_GPU_SMALL_R) {
        const long items = tables * (CG_N_SMALL_R + 1);
        const int blocks = (int)((items + SR_WARPS - 1) / SR_WARPS);
        if (mixed)
            small_r_kernel<float><<<blocks, 32 * SR_WARPS, 0, ctx->stream>>>(
                (const double *)ctx->kgrid.p, d_pk, (int)nk, n_spectra,
                n_terms, d_meta->tn, d_meta->tl, (const double *)ctx->tab_x.p, len,
                (float *)ctx->tab_y.p, ctx->d_err);
        else
            small_r_kernel<double><<<blocks, 32 * SR_WARPS, 0, ctx->stream>>>(
                (const double *)ctx->kgrid.p, d_pk, (int)nk, n_spectra,
                n_terms, d_meta->tn, d_meta->tl, (const double *)ctx->tab_x.p, len,
                (double *)ctx->tab_y.p, ctx->d_err);
        if ((st = cg_after_launch(ctx, "small_r_kernel"))) return st;
    } else if (!mixed || tables_df) {
        const long items = tables * (CG_N_SMALL_R + 1);
        if (mixed)
            fill_nan_kernel<float><<<(int)((items + 255) / 256), 256, 0, ctx->stream>>>(
                (float *)ctx->tab_y.p, len, tables);
        else
            fill_nan_kernel<double><<<(int)((items + 255) / 256), 256, 0, ctx->stream>>>(
                (double *)ctx->tab_y.p, len, tables);
        if ((st = cg_after_launch(ctx, "fill_nan_kernel"))) return st;
    }
    ctx->n_spectra = n_spectra;
    ctx->n_terms = n_terms;
    ctx->n_q = n_q;
    ctx->N = N;
    ctx->nk = nk;
    ctx->kmin = k[0];
    ctx->kmax = k[nk - 1];
    ctx->int_precision = precision;
    ctx->int_small_r = (flags & COFFE_GPU_SMALL_R) != 0;
    ctx->int_ready = true;
    return COFFE_GPU_OK;
}

// Evaluates table (spectrum, term) with the Akima spline at host separations.
int integrals_eval(coffe_gpu_ctx *ctx, int spectrum, int term, const double *r, size_t nq,
                   double *out)
{
    if (!ctx->int_ready) {
        cg_set_error(ctx, "integrals not initialised");
        return COFFE_GPU_ESTATE;
    }
    if (spectrum < 0 || spectrum >= ctx->n_spectra || term < 0 || term >= ctx->n_terms) {
        cg_set_error(ctx, "integral (spectrum %d, term %d) out of range", spectrum, term);
        return COFFE_GPU_EINVAL;
    }
    if (nq == 0) return COFFE_GPU_OK;
    const size_t len = ctx->N + CG_N_SMALL_R + 1;
    int st;
    DevBuf tmp;
    const size_t bytes = sizeof(double) * (len + 2 * nq);
    if (cudaMalloc(&tmp.p, bytes) != cudaSuccess) {
        cg_set_error(ctx, "cudaMalloc of %zu bytes failed", bytes);
        return COFFE_GPU_ENOMEM;
    }
    double *y = (double *)tmp.p, *dr = y + len, *dout = dr + nq;
    const size_t off = ((size_t)spectrum * ctx->n_terms + term) * len;
    if (ctx->int_precision == COFFE_GPU_MIXED) {
        table_f32_to_f64_kernel<<<(int)((len + 255) / 256), 256, 0, ctx->stream>>>(
            (const float *)ctx->tab_y.p + off, y, len);
        if ((st = cg_after_launch(ctx, "table_f32_to_f64_kernel"))) {
            cudaFree(tmp.p);
            return st;
        }
    } else {
        cudaMemcpyAsync(y, (const double *)ctx->tab_y.p + off, sizeof(double) * len,
                        cudaMemcpyDeviceToDevice, ctx->stream);
    }
    cudaMemcpyAsync(dr, r, sizeof(double) * nq, cudaMemcpyHostToDevice, ctx->stream);
    table_eval_kernel<<<(int)((nq + 255) / 256), 256, 0, ctx->stream>>>(
        (const double *)ctx->tab_x.p, y, (int)len, dr, (int)nq, dout);
    st = cg_after_launch(ctx, "table_eval_kernel");
    if (!st) {
        cudaError_t e = cudaMemcpyAsync(out, dout, sizeof(double) * nq, cudaMemcpyDeviceToHost,
                                        ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) {
            cg_set_error(ctx, "integral_eval copy: %s", cudaGetErrorString(e));
            st = COFFE_GPU_ECUDA;
        }
    }
    cudaFree(tmp.p);
    return st;
}

// The divergent integral on host separations r (all > 0) or, with r2, the
// renormalisation grid over host chi1 x chi2 (all >= 0): P(k) = Akima of
// (k, pk) on the host, integrated over [kmin, kmax] inside its range.
int divergent_run(coffe_gpu_ctx *ctx, const double *k, const double *pk, size_t nk, double kmin,
                  double kmax, const double *r1, size_t n1, const double *r2, size_t n2,
                  double *out_a, double *out_b)
{
    if (!k || !pk || !r1 || nk < 5 || nk > (1u << 22) || n1 < 1 || (r2 && n2 < 1) ||
        n1 > (r2 ? (1u << 24) : (1u << 16)) || n2 > (1u << 24) || !out_a || (!r2 && !out_b)) {
        cg_set_error(ctx, "divergent integral: bad arguments");
        return COFFE_GPU_EINVAL;
    }
    for (size_t i = 0; i < nk; ++i)
        if (!(k[i] > 0) || (i > 0 && !(k[i] > k[i - 1])) || !std::isfinite(pk[i])) {
            cg_set_error(ctx, "divergent integral: k must be positive and strictly increasing, "
                              "P(k) finite");
            return COFFE_GPU_EINVAL;
        }
    if (!(kmin >= k[0] && kmax <= k[nk - 1] && kmin < kmax)) {
        cg_set_error(ctx, "divergent integral: need k[0] <= kmin < kmax <= k[nk-1]");
        return COFFE_GPU_EINVAL;
    }
    for (size_t i = 0; i < n1; ++i)
        if (!(r2 ? r1[i] >= 0 : r1[i] > 0) || !std::isfinite(r1[i])) {
            cg_set_error(ctx, "divergent integral: separations must be %s",
                         r2 ? "non-negative" : "positive");
            return COFFE_GPU_EINVAL;
        }
    for (size_t i = 0; r2 && i < n2; ++i)
        if (!(r2[i] >= 0) || !std::isfinite(r2[i])) {
            cg_set_error(ctx, "divergent integral: separations must be non-negative");
            return COFFE_GPU_EINVAL;
        }
    const long items = r2 ? (long)(n1 * n2) : 2 * (long)n1;
    const size_t scratch = r2 ? 0 : (size_t)std::min<long>(items, DIV_CHUNK) * 4 * DIV_CAP;
    const size_t bytes =
        sizeof(double) * (2 * nk + n1 + (r2 ? n2 : 0) + (size_t)items + scratch);
    int st = cg_ensure(ctx, ctx->div_buf, bytes);
    if (st) return st;
    double *d = (double *)ctx->div_buf.p;
    double *dk = d, *dp = dk + nk, *d1 = dp + nk, *d2 = d1 + n1;
    double *dout = d2 + (r2 ? n2 : 0), *dscr = dout + items;
    CG_CUDA(ctx, cudaMemcpyAsync(dk, k, sizeof(double) * nk, cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(dp, pk, sizeof(double) * nk, cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(d1, r1, sizeof(double) * n1, cudaMemcpyHostToDevice, ctx->stream));
    if (r2)
        CG_CUDA(ctx, cudaMemcpyAsync(d2, r2, sizeof(double) * n2, cudaMemcpyHostToDevice,
                                     ctx->stream));
    const long chunk = r2 ? items : DIV_CHUNK;
    for (long i0 = 0; i0 < items; i0 += chunk) {
        const long n = std::min(chunk, items - i0);
        divergent_kernel<<<(unsigned)((n + SR_WARPS - 1) / SR_WARPS), 32 * SR_WARPS, 0,
                           ctx->stream>>>(dk, dp, (int)nk, kmin, kmax, d1, d2, (long)n1, i0,
                                          items, r2 ? 1 : 0, dscr, dout, ctx->d_err);
        if ((st = cg_after_launch(ctx, "divergent_kernel"))) return st;
    }
    if (r2) {
        CG_CUDA(ctx, cudaMemcpyAsync(out_a, dout, sizeof(double) * items, cudaMemcpyDeviceToHost,
                                     ctx->stream));
    } else {
        CG_CUDA(ctx, cudaMemcpyAsync(out_a, dout, sizeof(double) * n1, cudaMemcpyDeviceToHost,
                                     ctx->stream));
        CG_CUDA(ctx, cudaMemcpyAsync(out_b, dout + n1, sizeof(double) * n1,
                                     cudaMemcpyDeviceToHost, ctx->stream));
    }
    return cg_check_device_errors(ctx, "divergent integral");
}

// gY: table cotangents [n_spectra][n_at][N + CG_N_SMALL_R + 1]; adds the part
// of dL/dP that flows through the r = 0 and sub-Mpc entries to grad_pk
int small_r_adjoint_run(coffe_gpu_ctx *ctx, const double *gY, int n_at, const int *term,
                        double *grad_pk)
{
    if (n_at > 8) return COFFE_GPU_EINVAL;
    SmallRTerms tm;
    for (int t = 0; t < 8; ++t) {
        tm.n[t] = t < n_at ? ctx->term_n[term[t]] : 0;
        tm.l[t] = t < n_at ? (ctx->term_half[term[t]] ? -1 : ctx->term_l[term[t]]) : -1;
    }
    const long items = (long)ctx->n_spectra * n_at * (CG_N_SMALL_R + 1);
    const int blocks = (int)((items + SR_WARPS - 1) / SR_WARPS);
    small_r_adjoint_kernel<<<blocks, 32 * SR_WARPS, 0, ctx->stream>>>(
        (const double *)ctx->kgrid.p, (const double *)ctx->pk.p, (int)ctx->nk, ctx->n_spectra,
        n_at, tm, (const double *)ctx->tab_x.p, ctx->N + CG_N_SMALL_R + 1, gY, grad_pk,
        ctx->d_err);
    return cg_after_launch(ctx, "small_r_adjoint_kernel");
}
