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
// Work split: one thread owns one (request, separation) pair and evaluates the
// whole first GK61 panel on [0, 1] itself -- 61 integrand values, summed in
// QUADPACK's order, no cross-lane reductions.  The panel's abscissae, weights
// and P_l(mu_k) are the same for every pair, so they sit in constant memory
// and are read as warp-uniform broadcasts.  xi does not depend on l, so all
// requested multipoles share the 61 evaluations (the reference recomputes the
// integrand once per l).  Each l gets QUADPACK's error estimate and tolerance
// test; an l whose first panel misses the tolerance is appended to a retry
// list that a second kernel finishes with the full adaptive QAG, one warp per
// entry (qag.cuh).  For the den/RSD integrand the first panel converges for
// practically every pair, so the retry kernel is nearly idle.
//
// FP64 path: the reference's arithmetic in double.  Mixed path: the same
// algorithm with float splines, integrand and Legendre values, and a
// Kahan-compensated float sum for the panel result.
#include <algorithm>
#include <mutex>
#include <vector>

#include "ctx.cuh"
#include "dfloat.cuh"
#include "f32x2.cuh"
#include "qag.cuh"

namespace {

#define MP_MAX_L 8
#define MP_MAX_LDEG 8
#define MP_LANE_THREADS 128
#define MP_RETRY_WARPS 4
#define MP_CAP 128

// ------------------------------------------------ first-panel constant tables
// The 61 nodes of the first panel on [0, 1] are stored in "slots": slot 2p and
// 2p+1 are the pair x = 0.5 -+ 0.5 xgk[g_p] with g_p = 2p+1 (Gauss nodes,
// p < 15) or 2(p-15) (Kronrod-only), slot 60 the centre.  The integrand is
// evaluated in ascending mu (order[]), which makes the two z(chi) lookups of a
// thread monotone sweeps; the sums use the weight x P_l products per slot.
template <typename T> struct PanelTables {
    T mu[61];                       // mu = 2x - 1 per slot
    T wk[61];                       // Kronrod weight per slot
    T wkP[MP_MAX_LDEG + 1][61];     // wk P_l(mu)
    T wgP[MP_MAX_LDEG + 1][61];     // wg P_l(mu) (0 on Kronrod-only slots)
    T wkA[MP_MAX_LDEG + 1][61];     // wk |P_l(mu)|
    T Pl[MP_MAX_LDEG + 1][61];      // P_l(mu)
    T mu_sorted[61];                // mu in ascending order
    int order[61];                  // slot of the k-th smallest mu
};
// P_l(x) by the upward recurrence (gsl_sf_legendre_Pl), host side
double host_legendre(int l, double x)
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

const double h_xgk[31] = CG_GK61_XGK_INIT;
const double h_wgk[31] = CG_GK61_WGK_INIT;
const double h_wg[15] = CG_GK61_WG_INIT;

// first-panel tables in FP64, built once on the host
const PanelTables<double> &panel_tables()
{
    static PanelTables<double> t64;
    static bool built = false;
    if (built) return t64;
    // node positions and weights exactly as QUADPACK's qk61 forms them on [0, 1]
    const double center = 0.5, half_length = 0.5;
    double wg[61];
    for (int p = 0; p < 30; ++p) {
        const int g = p < 15 ? 2 * p + 1 : 2 * (p - 15);
        const double absc = half_length * h_xgk[g];
        t64.mu[2 * p] = 2 * (center - absc) - 1;
        t64.mu[2 * p + 1] = 2 * (center + absc) - 1;
        t64.wk[2 * p] = t64.wk[2 * p + 1] = h_wgk[g];
        wg[2 * p] = wg[2 * p + 1] = p < 15 ? h_wg[p] : 0.0;
    }
    t64.mu[60] = 2 * center - 1;
    t64.wk[60] = h_wgk[30];
    wg[60] = 0.0;
    for (int sl = 0; sl < 61; ++sl)
        for (int l = 0; l <= MP_MAX_LDEG; ++l) {
            const double P = host_legendre(l, t64.mu[sl]);
            t64.Pl[l][sl] = P;
            t64.wkP[l][sl] = t64.wk[sl] * P;
            t64.wgP[l][sl] = wg[sl] * P;
            t64.wkA[l][sl] = t64.wk[sl] * fabs(P);
        }
    std::vector<int> ord(61);
    for (int i = 0; i < 61; ++i) ord[i] = i;
    std::sort(ord.begin(), ord.end(), [&](int a, int b) { return t64.mu[a] < t64.mu[b]; });
    for (int i = 0; i < 61; ++i) {
        t64.order[i] = ord[i];
        t64.mu_sorted[i] = t64.mu[ord[i]];
    }
    built = true;
    return t64;
}

// The node table of mp_fast_kernel (layout FastLayout<NL>, in T): the mirror
// rule's rows mu >= 0 ascending with the mu-only RSD coefficients
template <typename T> void build_node_table_fast(int NL, const int *ls, std::vector<T> &out)
{
    const PanelTables<double> &P = panel_tables();
    const int R1 = ((8 + 3 * NL) + 3) / 4 * 4, R2 = ((1 + NL) + 3) / 4 * 4;
    out.assign((size_t)31 * (R1 + R2), T(0));
    for (int k = 0; k < 31; ++k) {
        const int sl = P.order[30 + k];
        const double mult = sl == 60 ? 1.0 : 2.0;
        const double mu = P.mu_sorted[30 + k], mu2 = mu * mu, omm = 1.0 - mu2;
        T *r = out.data() + (size_t)k * R1;
        r[0] = (T)mu;
        r[1] = (T)mu2;
        r[2] = (T)omm;
        r[3] = (T)(0.75 * omm * omm + 4.0 * mu2 * omm + 12.0 * mu2 * mu2);  // a2
        r[4] = (T)(-2.5 * omm * omm - 20.0 * mu2 * omm);                   // a1
        r[5] = (T)(4.75 * omm * omm - 8.0 * mu2 * omm - 4.0 * mu2 * mu2);  // a0
        r[6] = (T)(11.0 - 9.0 * omm);                                      // b2
        r[7] = (T)(9.0 * omm);                                             // -b1
        for (int j = 0; j < NL; ++j) {
            r[8 + j] = (T)(mult * P.wkP[ls[j]][sl]);
            r[8 + NL + j] = (T)(mult * P.wgP[ls[j]][sl]);
            r[8 + 2 * NL + j] = (T)(mult * P.wkA[ls[j]][sl]);
        }
        T *r2 = out.data() + (size_t)31 * R1 + (size_t)k * R2;
        r2[0] = (T)(mult * P.wk[sl]);
        for (int j = 0; j < NL; ++j) r2[1 + j] = (T)P.Pl[ls[j]][sl];
    }
}

// ------------------------------------------ integrand as a polynomial in mu^2
//
// For the fast kernels' case (unit biases, even multipoles, equal tracers) the
// den/RSD integrand at a node is a polynomial in w = mu^2 times powers of
// 1/D, D = 2 chi1 chi2 = 2 chi^2 (1 - w r^2 / (4 chi^2)): the background
// polynomials are polynomials in t^2 = rho^2 w (their odd parts pair up into
// even products), the mu-only RSD coefficients are quadratics in w, and 1/D
// is a geometric series in w r^2 / (4 chi^2) <= (r / 2 chi)^2 < 0.01 here.
// mp_poly_kernel therefore forms, once per (request, separation), the
// coefficients of the integrand in w up to MP_PJ (the 1/D series to MP_PS
// terms; truncation < 1e-12 of the integrand over 5 <= r <= 375 Mpc,
// chi >= 1300 Mpc), and the Kronrod and Gauss sums of the first panel
// become dot products of those coefficients with the rule's moments
// sum_k w_k P_l(mu_k) mu_k^(2j) (host, FP64).  Only QUADPACK's |f| and
// |f - mean| sums still need the integrand at the 31 nodes: a Horner
// evaluation each.
#define MP_PJ 8
#define MP_PS 4
#define MP_FAST_MAX_L 4
template <typename T> struct PolyMom {
    T mk[MP_FAST_MAX_L][MP_PJ + 1]; // sum_k mult wk P_l mu_k^(2j)
    T mg[MP_FAST_MAX_L][MP_PJ + 1]; // sum_k mult wg P_l mu_k^(2j)
};
template <typename T> PolyMom<T> poly_moments(int NL, const int *ls)
{
    const PanelTables<double> &P = panel_tables();
    PolyMom<T> m;
    for (int j = 0; j < NL; ++j) {
        double sk[MP_PJ + 1] = {0}, sg[MP_PJ + 1] = {0};
        for (int k = 0; k < 31; ++k) {
            const int sl = P.order[30 + k];
            const double mult = sl == 60 ? 1.0 : 2.0;
            const double w = P.mu_sorted[30 + k] * P.mu_sorted[30 + k];
            double wp = 1.0;
            for (int e = 0; e <= MP_PJ; ++e, wp *= w) {
                sk[e] += mult * P.wkP[ls[j]][sl] * wp;
                sg[e] += mult * P.wgP[ls[j]][sl] * wp;
            }
        }
        for (int e = 0; e <= MP_PJ; ++e) {
            m.mk[j][e] = (T)sk[e];
            m.mg[j][e] = (T)sg[e];
        }
    }
    for (int j = NL; j < MP_FAST_MAX_L; ++j)
        for (int e = 0; e <= MP_PJ; ++e) m.mk[j][e] = m.mg[j][e] = T(0);
    return m;
}
// node rows of mp_poly_kernel: w = mu^2, mult wk, P_l (NL), mult wk |P_l| (NL)
template <int NL> struct PolyLayout {
    static constexpr int R = (2 + 2 * NL + 3) / 4 * 4;
    static constexpr int ROWS = 31;
    static constexpr int COUNT = ROWS * R;
};
template <typename T> void build_node_table_poly(int NL, const int *ls, std::vector<T> &out)
{
    const PanelTables<double> &P = panel_tables();
    const int R = (2 + 2 * NL + 3) / 4 * 4;
    out.assign((size_t)31 * R, T(0));
    for (int k = 0; k < 31; ++k) {
        const int sl = P.order[30 + k];
        const double mult = sl == 60 ? 1.0 : 2.0;
        const double mu = P.mu_sorted[30 + k];
        T *r = out.data() + (size_t)k * R;
        r[0] = (T)(mu * mu);
        r[1] = (T)(mult * P.wk[sl]);
        for (int j = 0; j < NL; ++j) {
            r[2 + j] = (T)P.Pl[ls[j]][sl];
            r[2 + NL + j] = (T)(mult * P.wkA[ls[j]][sl]);
        }
    }
}

// The node table of mp_fast2_kernel (layout Fast2Layout<NL>): every constant of
// the rows mu >= 0 stored twice, as the packed pair (c, c) both lanes of a
// packed FP32 operation use; pass-1 pairs mu, -mu, -mu^2, 1 - mu^2, a2, a1, a0,
// -b2, -b1, wk P_l (NL), wg P_l (NL), wk |P_l| (NL); pass-2 pairs wk, P_l (NL)
void build_node_table_fast2(int NL, const int *ls, std::vector<float> &out)
{
    const PanelTables<double> &P = panel_tables();
    const int F1 = (2 * (9 + 3 * NL) + 3) / 4 * 4, F2 = (2 * (1 + NL) + 3) / 4 * 4;
    out.assign((size_t)31 * (F1 + F2), 0.f);
    for (int k = 0; k < 31; ++k) {
        const int sl = P.order[30 + k];
        const double mult = sl == 60 ? 1.0 : 2.0;
        const double mu = P.mu_sorted[30 + k], mu2 = mu * mu, omm = 1.0 - mu2;
        double c[9 + 3 * MP_MAX_L];
        c[0] = mu;
        c[1] = -mu;
        c[2] = -mu2;
        c[3] = omm;
        c[4] = 0.75 * omm * omm + 4.0 * mu2 * omm + 12.0 * mu2 * mu2; // a2
        c[5] = -2.5 * omm * omm - 20.0 * mu2 * omm;                   // a1
        c[6] = 4.75 * omm * omm - 8.0 * mu2 * omm - 4.0 * mu2 * mu2;  // a0
        c[7] = -(11.0 - 9.0 * omm);                                   // -b2
        c[8] = 9.0 * omm;                                             // -b1
        for (int j = 0; j < NL; ++j) {
            c[9 + j] = mult * P.wkP[ls[j]][sl];
            c[9 + NL + j] = mult * P.wgP[ls[j]][sl];
            c[9 + 2 * NL + j] = mult * P.wkA[ls[j]][sl];
        }
        float *r = out.data() + (size_t)k * F1;
        for (int i = 0; i < 9 + 3 * NL; ++i) r[2 * i] = r[2 * i + 1] = (float)c[i];
        float *r2 = out.data() + (size_t)31 * F1 + (size_t)k * F2;
        r2[0] = r2[1] = (float)(mult * P.wk[sl]);
        for (int j = 0; j < NL; ++j) r2[2 + 2 * j] = r2[3 + 2 * j] = (float)P.Pl[ls[j]][sl];
    }
}

// The node table of one launch (layout NodeLayout<NL>), in T, for multipoles ls[0..NL)
template <typename T>
void build_node_table(int NL, const int *ls, std::vector<T> &out, bool mirror = false)
{
    const PanelTables<double> &P = panel_tables();
    const int R1 = ((2 + 3 * NL) + 3) / 4 * 4, R2 = ((1 + NL) + 3) / 4 * 4;
    if (mirror) {
        // rows: mu >= 0 ascending (the centre, then the 30 positive nodes); the
        // value slot of pair p (slots 2p, 2p+1) is p, of the centre 30
        out.assign((size_t)31 * (R1 + R2), T(0));
        for (int k = 0; k < 31; ++k) {
            const int sl = P.order[30 + k];
            const double mult = sl == 60 ? 1.0 : 2.0;
            const int pidx = sl == 60 ? 30 : sl >> 1;
            T *r = out.data() + (size_t)k * R1;
            r[0] = (T)P.mu_sorted[30 + k];
            r[1] = (T)pidx;
            for (int j = 0; j < NL; ++j) {
                r[2 + j] = (T)(mult * P.wkP[ls[j]][sl]);
                r[2 + NL + j] = (T)(mult * P.wgP[ls[j]][sl]);
                r[2 + 2 * NL + j] = (T)(mult * P.wkA[ls[j]][sl]);
            }
            T *r2 = out.data() + (size_t)31 * R1 + (size_t)pidx * R2;
            r2[0] = (T)(mult * P.wk[sl]);
            for (int j = 0; j < NL; ++j) r2[1 + j] = (T)P.Pl[ls[j]][sl];
        }
        return;
    }
    out.assign((size_t)61 * (R1 + R2), T(0));
    for (int k = 0; k < 61; ++k) {
        const int sl = P.order[k];
        T *r = out.data() + (size_t)k * R1;
        r[0] = (T)P.mu_sorted[k];
        r[1] = (T)sl;
        for (int j = 0; j < NL; ++j) {
            r[2 + j] = (T)P.wkP[ls[j]][sl];
            r[2 + NL + j] = (T)P.wgP[ls[j]][sl];
            r[2 + 2 * NL + j] = (T)P.wkA[ls[j]][sl];
        }
    }
    for (int sl = 0; sl < 61; ++sl) {
        T *r = out.data() + (size_t)61 * R1 + (size_t)sl * R2;
        r[0] = (T)P.wk[sl];
        for (int j = 0; j < NL; ++j) r[1 + j] = (T)P.Pl[ls[j]][sl];
    }
}

// ------------------------------------------------------ background access
template <typename T> struct ZRec; // f and D1 coefficients of one z interval
template <> struct ZRec<double> { double4_32a f, d; };
template <> struct ZRec<float> { float4 f, d; };

__device__ __forceinline__ ZRec<double> ldg_zrec(const ZRec<double> *p)
{
    ZRec<double> r;
    r.f = ldg_c4(&p->f);
    r.d = ldg_c4(&p->d);
    return r;
}
__device__ __forceinline__ ZRec<float> ldg_zrec(const ZRec<float> *p)
{
    ZRec<float> r;
    r.f = __ldg(&p->f);
    r.d = __ldg(&p->d);
    return r;
}

template <typename T, typename S> struct Bg {
    S z_of_chi, f, D1, b1, b2;
    const ZRec<T> *zrec; // fused f / D1 records on a uniform z grid (or null)
    T z0, zn, dz, inv_dz;
    int nz, has_b1, has_b2;

    // f(z) and D1(z), one interval search for both
    __device__ __forceinline__ void fD1(T z, T &fv, T &dv) const
    {
        if (zrec) {
            if (!(z >= z0 && z <= zn)) {
                fv = dv = cg_nan<T>();
                return;
            }
            int i = (int)((z - z0) * inv_dz);
            i = i < 0 ? 0 : (i > nz - 2 ? nz - 2 : i);
            const T dx = z - (z0 + (T)i * dz);
            const ZRec<T> r = ldg_zrec(zrec + i);
            fv = r.f.x + dx * (r.f.y + dx * (r.f.z + r.f.w * dx));
            dv = r.d.x + dx * (r.d.y + dx * (r.d.z + r.d.w * dx));
        } else {
            fv = spl_eval(f, z);
            dv = spl_eval(D1, z);
        }
    }
};

// xi(z_mean, mu, r) of the den/rsd terms in the cancellation-free form:
// with D = 2 chi^2 - mu^2 r^2 / 2 (= 2 chi1 chi2) and s = 1 - cos(theta) =
// r^2 (1 - mu^2) / D, the reference's cos(theta)- and chi/r-expressions
// become the polynomials below (identical algebra; the reference's I04
// coefficient cancels two terms of size (chi/r)^4).
// 1/x: IEEE division in double; the MUFU reciprocal (2 ulp) in the float path
__device__ __forceinline__ double rcp_t(double x) { return 1.0 / x; }
__device__ __forceinline__ float rcp_t(float x) { return __fdividef(1.0f, x); }

template <typename T, typename S> struct Xi {
    Bg<T, S> bg;
    T chi_mean, sep, I00, I02, I04;
    int contrib;

    __device__ __forceinline__ T operator()(T mu) const
    {
        const T chi1 = chi_mean - sep * mu * T(0.5);
        const T chi2 = chi_mean + sep * mu * T(0.5);
        return combine(mu, chi1, chi2, spl_eval(bg.z_of_chi, chi1), spl_eval(bg.z_of_chi, chi2));
    }

    // xi from the two line-of-sight distances and their redshifts
    __device__ __forceinline__ T combine(T mu, T chi1, T chi2, T z1, T z2) const
    {
        const T mu2 = mu * mu;
        const T omm = T(1) - mu2;
        const T D = T(2) * chi_mean * chi_mean - mu2 * sep * sep * T(0.5);
        const T inv_D = rcp_t(D);
        const T s = sep * sep * omm * inv_D;
        const T c = T(1) - s;
        T f1, f2, g1, g2;
        bg.fD1(z1, f1, g1);
        bg.fD1(z2, f2, g2);
        const T b1 = bg.has_b1 ? spl_eval(bg.b1, z1) : T(1);
        const T b2 = bg.has_b2 ? spl_eval(bg.b2, z2) : T(1);
        T result = T(0);
        const bool autos = !(contrib & COFFE_GPU_ONLY_CROSS); // functions.c:129-133, 230-234
        if ((contrib & COFFE_GPU_DEN) && autos) result += b1 * b2 * I00;
        if ((contrib & COFFE_GPU_RSD) && autos) {
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
        return result * g1 * g2;
    }
};

// P_l(x) by the upward recurrence, 1/k as a product (device; adaptive path)
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

// integrand of one multipole at x in [0, 1] (adaptive continuation)
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
template <typename T, bool FAST = false>
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
    return akima_eval_at<T, FAST>(x, y, n, i, r);
}

// The three tables I00, I02, I04 (rows y0, y1, y2 on the knots x) at one r:
// table_lookup's interval and Akima coefficients, with the interval search,
// the knot loads and the secant denominators (as reciprocals) shared by the
// three; the FAST float path divides through the approximate reciprocal as
// __fdividef does.
template <typename T>
__device__ __forceinline__ void table_lookup3(const T *__restrict__ x, const T *__restrict__ y0,
                                              const T *__restrict__ y1, const T *__restrict__ y2,
                                              int n, T inv_dlog, T r, T &v0, T &v1, T &v2)
{
    if (!(r >= x[0] && r <= x[n - 1])) {
        v0 = v1 = v2 = cg_nan<T>();
        return;
    }
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
    if (i < 2 || i > n - 4) { // the end rule of the Akima secants: the general path
        v0 = akima_eval_at<T, true>(x, y0, n, i, r);
        v1 = akima_eval_at<T, true>(x, y1, n, i, r);
        v2 = akima_eval_at<T, true>(x, y2, n, i, r);
        return;
    }
    T ih[5]; // 1 / (x_{k+1} - x_k), k = i - 2 .. i + 2
#pragma unroll
    for (int k = 0; k < 5; ++k) ih[k] = akima_div<T, true>(T(1), x[i - 1 + k] - x[i - 2 + k]);
    const T dx = r - x[i];
    const T ih2 = ih[2] * ih[2];
    auto eval = [&](const T *__restrict__ y) {
        T m[5];
        T yp = y[i - 2];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const T yn = y[i - 1 + k];
            m[k] = (yn - yp) * ih[k];
            yp = yn;
        }
        const T t0 = akima_node_slope<T, true>(m[0], m[1], m[2], m[3]);
        const T t1 = akima_node_slope<T, true>(m[1], m[2], m[3], m[4]);
        const T c = (T(3) * m[2] - T(2) * t0 - t1) * ih[2];
        const T d = (t0 + t1 - T(2) * m[2]) * ih2;
        return y[i] + dx * (t0 + dx * (c + d * dx));
    };
    v0 = eval(y0);
    v1 = eval(y1);
    v2 = eval(y2);
}

struct MpArgs {
    int n_req, n_l, contrib;
    int t00, t02, t04;
    int n_terms, tab_len;
    double inv_dlog; // N / ln(kmax/kmin), r0 = 1
    double epsrel;
    long long retry_cap;
    int ls[MP_MAX_L];
    int out_staged = 0; // out is mapped host memory: store whole lines (mp_fast_kernel)
};

// request of each separation: largest q with req_offset[q] <= item
__device__ __forceinline__ int find_request(const int64_t *__restrict__ req_offset, int n_req,
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

// find_request for a whole warp whose lanes hold consecutive items (every lane
// active): a 32-way search for the request of lane 0's item (three rounds of
// one coalesced load for 3072 requests, instead of twelve dependent ones per
// lane), then each lane walks forward over the few boundaries its warp spans.
// Same result as find_request: the last request q with req_offset[q] <= item.
__device__ __forceinline__ int find_request_warp(const int64_t *__restrict__ req_offset,
                                                 int n_req, long long item)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const long long first = __shfl_sync(full, item, 0);
    int lo = 0, hi = n_req; // req_offset[lo] <= first (req_offset[0] = 0)
    while (hi - lo > 1) {
        const int step = (hi - lo + 31) >> 5;
        const int probe = lo + lane * step;
        const unsigned m = __ballot_sync(full, probe < hi && req_offset[probe] <= first);
        const int nlo = lo + (31 - __clz(m)) * step;
        hi = min(hi, nlo + step);
        lo = nlo;
    }
    int q = lo;
    while (q + 1 < n_req && req_offset[q + 1] <= item) ++q;
    return q;
}

template <typename T, typename S, typename TT>
__device__ __forceinline__ Xi<T, S> make_xi(const MpArgs &a, const Bg<T, S> &bg, const S &chi_of_z,
                                            const TT *__restrict__ tab_x,
                                            const TT *__restrict__ tab_y, int s, T zm, T r)
{
    Xi<T, S> xi;
    xi.bg = bg;
    xi.sep = r;
    xi.contrib = a.contrib;
    const TT *y0 = tab_y + ((size_t)s * a.n_terms) * a.tab_len;
    xi.I00 = (T)table_lookup<TT>(tab_x, y0 + (size_t)a.t00 * a.tab_len, a.tab_len, (TT)a.inv_dlog, (TT)r);
    xi.I02 = (T)table_lookup<TT>(tab_x, y0 + (size_t)a.t02 * a.tab_len, a.tab_len, (TT)a.inv_dlog, (TT)r);
    xi.I04 = (T)table_lookup<TT>(tab_x, y0 + (size_t)a.t04 * a.tab_len, a.tab_len, (TT)a.inv_dlog, (TT)r);
    xi.chi_mean = spl_eval(chi_of_z, zm);
    return xi;
}

// --------------------------------------------------------------- fast path

// A monotone cursor over the knots of the z(chi) spline: along the mu-sorted
// node sweep chi1 = chi - r mu / 2 only decreases and chi2 = chi + r mu / 2
// only increases, so each lookup moves the previous interval by a step or
// two instead of searching.  The interval reached is the one a binary search
// returns (x_i <= v < x_{i+1}).  Range checks are done once per pair by the
// caller (the sweep stays inside [chi - r mu_max / 2, chi + r mu_max / 2]).
template <typename T> struct Cursor {
    int i;
    T xa, xb; // x_i, x_{i+1}
};

template <typename S>
__device__ __forceinline__ Cursor<typename SplTraits<S>::T> cursor_at(const S &s,
                                                                      typename SplTraits<S>::T v)
{
    Cursor<typename SplTraits<S>::T> c;
    c.i = spl_interval(s, v);
    c.xa = __ldg(s.x + c.i);
    c.xb = __ldg(s.x + c.i + 1);
    return c;
}

template <typename S>
__device__ __forceinline__ typename SplTraits<S>::T cursor_up(const S &s,
                                                              Cursor<typename SplTraits<S>::T> &c,
                                                              typename SplTraits<S>::T v)
{
    typedef typename SplTraits<S>::T T;
    while (c.i < s.n - 2 && c.xb <= v) {
        ++c.i;
        c.xa = c.xb;
        c.xb = __ldg(s.x + c.i + 1);
    }
    const T dx = v - c.xa;
    const typename SplTraits<S>::C4 q = ldg_c4(s.c + c.i);
    return q.x + dx * (q.y + dx * (q.z + q.w * dx));
}

template <typename S>
__device__ __forceinline__ typename SplTraits<S>::T cursor_down(const S &s,
                                                                Cursor<typename SplTraits<S>::T> &c,
                                                                typename SplTraits<S>::T v)
{
    typedef typename SplTraits<S>::T T;
    while (c.i > 0 && c.xa > v) {
        --c.i;
        c.xb = c.xa;
        c.xa = __ldg(s.x + c.i);
    }
    const T dx = v - c.xa;
    const typename SplTraits<S>::C4 q = ldg_c4(s.c + c.i);
    return q.x + dx * (q.y + dx * (q.z + q.w * dx));
}

// Per-launch node table for the requested multipoles (NL of them), staged in
// shared memory so every node reads its constants as broadcast vector loads:
//   pass-1 record k (ascending mu): mu, slot, wk P_l, wg P_l, wk |P_l| per l;
//   pass-2 record per slot: wk, P_l per l.
// With MIRROR the integrand is even in mu (equal tracers, even multipoles:
// functions.c's xi swaps chi1 <-> chi2 under mu -> -mu), so only the 31 nodes
// with mu >= 0 are evaluated; the weights of the 30 nodes off the centre are
// doubled (the Kronrod, Gauss, |f| and resasc sums are unchanged).
template <int NL, bool MIRROR = false> struct NodeLayout {
    static constexpr int R1 = ((2 + 3 * NL) + 3) / 4 * 4;
    static constexpr int R2 = ((1 + NL) + 3) / 4 * 4;
    static constexpr int ROWS = MIRROR ? 31 : 61;
    static constexpr int COUNT = ROWS * (R1 + R2);
};

template <typename T, int R> __device__ __forceinline__ void lds_rec(const T *p, T (&r)[R]);
template <int R> __device__ __forceinline__ void lds_rec(const float *p, float (&r)[R])
{
#pragma unroll
    for (int i = 0; i < R / 4; ++i) {
        const float4 v = reinterpret_cast<const float4 *>(p)[i];
        r[4 * i] = v.x;
        r[4 * i + 1] = v.y;
        r[4 * i + 2] = v.z;
        r[4 * i + 3] = v.w;
    }
}
template <int R> __device__ __forceinline__ void lds_rec(const double *p, double (&r)[R])
{
#pragma unroll
    for (int i = 0; i < R / 2; ++i) {
        const double2 v = reinterpret_cast<const double2 *>(p)[i];
        r[2 * i] = v.x;
        r[2 * i + 1] = v.y;
    }
}

// First-panel results of one separation: QUADPACK's acceptance test of the
// 61-point panel (gsl qag.c) per multipole; accepted values are written,
// the others queued for the adaptive continuation.
__device__ __forceinline__ double to_f64(double x) { return x; }
__device__ __forceinline__ double to_f64(float x) { return f64_of_bits(x); }

template <int NL, typename T>
__device__ __forceinline__ void first_panel_value(const MpArgs &a, T epsrel, long long item,
                                                  bool finite, const T (&K)[NL], const T (&G)[NL],
                                                  const T (&A)[NL], const T (&asc)[NL],
                                                  double (&res)[NL], bool (&have)[NL],
                                                  int *__restrict__ retry_count,
                                                  int2 *__restrict__ retry, int *err)
{
#pragma unroll
    for (int j = 0; j < NL; ++j) {
        const int l = a.ls[j];
        QkOut<T> o;
        o.result = K[j] * T(0.5);
        o.resabs = A[j] * T(0.5);
        o.resasc = asc[j] * T(0.5);
        o.abserr = qk_rescale_error((K[j] - G[j]) * T(0.5), o.resabs, o.resasc);
        const T tolerance = epsrel * fabs(o.result);
        const T round_off = T(50) * qk_eps<T>() * o.resabs;
        const bool roundoff_fail = o.abserr <= round_off && o.abserr > tolerance;
        const bool ok = (o.abserr <= tolerance && o.abserr != o.resasc) || o.abserr == T(0);
        have[j] = true;
        if (!finite) {
            cg_flag(err, CG_ERR_NONFINITE);
            res[j] = cg_nan<double>();
        } else if (ok || roundoff_fail) {
            res[j] = to_f64(T(2 * l + 1) * o.result);
            if (!isfinite(res[j])) cg_flag(err, CG_ERR_NONFINITE);
        } else { // the retry kernel writes this entry
            have[j] = false;
            res[j] = cg_nan<double>();
            const int slot = atomicAdd(retry_count, 1);
            if (slot < a.retry_cap)
                retry[slot] = make_int2((int)item, j);
            else
                cg_flag(err, CG_ERR_QAG_LIMIT);
        }
    }
}

template <int NL, typename T>
__device__ __forceinline__ void first_panel_out(const MpArgs &a, T epsrel, long long item, bool finite,
                                                const T (&K)[NL], const T (&G)[NL],
                                                const T (&A)[NL], const T (&asc)[NL],
                                                double *__restrict__ out,
                                                int *__restrict__ retry_count,
                                                int2 *__restrict__ retry, int *err)
{
    double res[NL];
    bool have[NL];
    first_panel_value<NL, T>(a, epsrel, item, finite, K, G, A, asc, res, have, retry_count, retry,
                             err);
#pragma unroll
    for (int j = 0; j < NL; ++j)
        if (have[j]) out[item * NL + j] = res[j];
}

template <int NL, typename T, typename S, typename TT, bool MIRROR = false>
__global__ void __launch_bounds__(MP_LANE_THREADS)
    mp_lane_kernel(MpArgs a, Bg<T, S> bg, S chi_of_z, const TT *__restrict__ tab_x,
                   const TT *__restrict__ tab_y, const int *__restrict__ req_spectrum,
                   const double *__restrict__ req_z_mean, const int64_t *__restrict__ req_offset,
                   const double *__restrict__ sep, long long total,
                   const T *__restrict__ nodes, double *__restrict__ out,
                   int *__restrict__ retry_count, int2 *__restrict__ retry, int *err)
{
    typedef NodeLayout<NL, MIRROR> LY;
    extern __shared__ __align__(16) unsigned char mp_smem[];
    T *tab1 = reinterpret_cast<T *>(mp_smem);  // [ROWS][R1]
    T *tab2 = tab1 + LY::ROWS * LY::R1;         // [ROWS][R2]
    T *xs = tab2 + LY::ROWS * LY::R2;           // [ROWS slots][blockDim.x] integrand values
    for (int i = threadIdx.x; i < LY::COUNT; i += blockDim.x) tab1[i] = nodes[i];
    __syncthreads();
    const long long item = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= total) return;
    const int q = find_request(req_offset, a.n_req, item);
    const int s = req_spectrum[q];
    const T r = (T)sep[item];
    const T zm = (T)req_z_mean[q];
    const Xi<T, S> xi = make_xi<T, S, TT>(a, bg, chi_of_z, tab_x, tab_y, s, zm, r);
    const int bd = blockDim.x, tid = threadIdx.x;
    T K[NL], Kc[NL], G[NL], A[NL];
#pragma unroll
    for (int j = 0; j < NL; ++j) K[j] = Kc[j] = G[j] = A[j] = T(0);
    const T half_r = r * T(0.5);
    // the sweep covers chi -+ r mu_max / 2: outside the chi knots every node of
    // the reference's integrand is NaN, so the whole pair is
    const T mu0 = tab1[0]; // first node of the sweep
    const T span = fabs(tab1[(LY::ROWS - 1) * LY::R1]) * half_r; // largest |mu|
    const bool inside = (xi.chi_mean - span >= bg.z_of_chi.x0) && (xi.chi_mean + span <= bg.z_of_chi.xn);
    bool finite = inside && isfinite(xi.I00) && isfinite(xi.I02) && isfinite(xi.I04);
    if (inside) {
        Cursor<T> c1 = cursor_at(bg.z_of_chi, xi.chi_mean - mu0 * half_r);
        Cursor<T> c2 = cursor_at(bg.z_of_chi, xi.chi_mean + mu0 * half_r);
        // integrand at the 61 nodes in ascending mu; Kronrod, Gauss and |f| sums
#pragma unroll 1
        for (int k = 0; k < LY::ROWS; ++k) {
            T rec[LY::R1];
            lds_rec<LY::R1>(tab1 + k * LY::R1, rec);
            const T mu = rec[0];
            const int slot = (int)rec[1];
            const T chi1 = xi.chi_mean - mu * half_r;
            const T chi2 = xi.chi_mean + mu * half_r;
            const T z1 = cursor_down(bg.z_of_chi, c1, chi1);
            const T z2 = cursor_up(bg.z_of_chi, c2, chi2);
            const T v = xi.combine(mu, chi1, chi2, z1, z2);
            xs[slot * bd + tid] = v;
            const T av = fabs(v);
#pragma unroll
            for (int j = 0; j < NL; ++j) {
                const T term = rec[2 + j] * v;
                if (sizeof(T) == 4) { // Kahan-compensated float sum of the Kronrod estimate
                    const T yk = term - Kc[j];
                    const T tk = K[j] + yk;
                    Kc[j] = (tk - K[j]) - yk;
                    K[j] = tk;
                } else {
                    K[j] += term;
                }
                G[j] += rec[2 + NL + j] * v;
                A[j] += rec[2 + 2 * NL + j] * av;
            }
        }
    }
    T asc[NL];
#pragma unroll
    for (int j = 0; j < NL; ++j) asc[j] = T(0);
    if (inside) {
#pragma unroll 1
        for (int sl = 0; sl < LY::ROWS; ++sl) {
            T rec[LY::R2];
            lds_rec<LY::R2>(tab2 + sl * LY::R2, rec);
            const T v = xs[sl * bd + tid];
#pragma unroll
            for (int j = 0; j < NL; ++j) asc[j] += rec[0] * fabs(v * rec[1 + j] - K[j] * T(0.5));
        }
    }
    first_panel_out<NL, T>(a, (T)a.epsrel, item, finite, K, G, A, asc, out, retry_count, retry, err);
}

// ------------------------------------------- mixed path, equal unit biases
//
// The same first panel for the common case of the mixed path: unit galaxy
// biases (so equal tracers and, with even multipoles, the 31-node mirror
// rule), density and/or RSD without the only-cross switch.  Two changes
// against mp_lane_kernel, both exact rearrangements up to float rounding:
//  * background: D1 and f D1 along the line of sight of a request as one
//    degree-5 polynomial each in t = x / X around the request's mean distance
//    (chi = chi_mean + x, |x| <= X = half its largest separation, clamped to
//    the background's range), interpolated at six Chebyshev points by
//    mp_bgfit_kernel from the uniform chi table of (D1, f D1) (ChiTab, filled
//    from the FP64 splines); a node evaluates the even and odd parts in t^2
//    (both ends from one evaluation, no loads).  Error: the interpolation's
//    ~(X/L)^6 of the background's scale L ~ Gpc (1e-8 at X = 190 Mpc), the
//    table's linear interpolation (~5e-9) and float rounding (~1e-7 relative
//    in the float kernels);
//  * integrand: with G = D1 and F = f D1 at both ends, xi g1 g2 becomes
//      G1 G2 I00 + F1 F2 R(c) + (G1 F2 + F1 G2)(I00 - 2 I02)/3
//      + g I02 (G1 F2 chi1^2 + F1 G2 chi2^2),       g = (2 - s)(1 - mu^2)/D,
//    R(c) = (1 + 2c^2) I00/15 - (b2 c^2 + b1 c + 1) I02/21
//           + (a2 c^2 + a1 c + a0) I04/35,
//    where the mu-only coefficients a_i, b_i of the RSD polynomials (functions.c
//    :129-134 as rewritten for Xi::combine) sit in the node table.

// Per-request background polynomials: G(chi_mean + X t) = ge(t^2) + t go(t^2),
// F likewise, ge = (c0, c2, c4), go = (c1, c3, c5) in t; the fourth lanes hold
// 1/X, chi_mean, X.
template <typename T> struct BgFitT;
template <> struct BgFitT<float> {
    float4 ge, go, fe, fo; // (c0,c2,c4,1/X) (c1,c3,c5,chi_mean) (d0,d2,d4,X) (d1,d3,d5,-)
};
template <> struct BgFitT<double> {
    double4_32a ge, go, fe, fo;
};

template <typename T> __device__ __forceinline__ T from_f64(double x);
// double -> float without the FP64 pipe (1/64 of the FP32 rate)
template <> __device__ __forceinline__ float from_f64<float>(double x) { return f32_of_bits(x); }
template <> __device__ __forceinline__ double from_f64<double>(double x) { return x; }

__device__ __forceinline__ float4 mk4(float a, float b, float c, float d) { return make_float4(a, b, c, d); }
__device__ __forceinline__ double4_32a mk4(double a, double b, double c, double d)
{
    double4_32a v;
    v.x = a;
    v.y = b;
    v.z = c;
    v.w = d;
    return v;
}

// (D1, f D1) as functions of chi on a uniform grid of CG_CHI_TAB points over
// the background's chi range (multipoles_prepare_background evaluates the FP64
// splines there), read by linear interpolation: two independent loads where
// the splines need a chain of three lookups (z of chi, then D1 and f of z).
// Interpolation error ~ h^2 / 8 of the second derivative: ~5e-9 relative for
// the growth factor's Gpc scale at h = range / 16383.
#define CG_CHI_TAB 16384
template <typename T> struct V2T;
template <> struct V2T<double> { typedef double2 t; };
template <> struct V2T<float> { typedef float2 t; };
template <typename T> struct ChiTab {
    const typename V2T<T>::t *rec;
    T c0, cn, inv_dc;
};
template <typename T>
__device__ __forceinline__ void chi_tab_eval(const ChiTab<T> &tb, T chi, T &g, T &fg)
{
    if (!(chi >= tb.c0 && chi <= tb.cn)) {
        g = fg = cg_nan<T>();
        return;
    }
    const T u = (chi - tb.c0) * tb.inv_dc;
    int i = (int)u;
    i = i > CG_CHI_TAB - 2 ? CG_CHI_TAB - 2 : i;
    const T w = u - (T)i;
    const typename V2T<T>::t p = tb.rec[i], q = tb.rec[i + 1];
    g = fma(w, q.x - p.x, p.x);
    fg = fma(w, q.y - p.y, p.y);
}

// the Chebyshev points t_j = cos((2j + 1) pi / 12), j < 6, and the inverse of
// their Vandermonde matrix (monomial coefficients from the six values), both
// computed on the host in FP64
template <typename T> struct FitInvT {
    T t[6];
    T m[6][6];
};

// one warp per request (MP_FIT_WARPS per block): the largest separation, the
// background at the six Chebyshev points (lanes 0-5, the float background
// splines, as mp_lane_kernel reads them), then the coefficients (lanes 0-11:
// D1 and f D1) as rows of the inverse Vandermonde
#define MP_FIT_WARPS 4
template <typename T, typename S>
__global__ void __launch_bounds__(32 * MP_FIT_WARPS)
    mp_bgfit_kernel(S chi_of_z, ChiTab<T> tab, int n_req, FitInvT<T> vinv,
                    const double *__restrict__ req_z_mean, const int64_t *__restrict__ req_offset,
                    const double *__restrict__ sep, BgFitT<T> *__restrict__ fit,
                    int *__restrict__ retry_count)
{
    __shared__ T val[MP_FIT_WARPS][12];
    __shared__ T cof[MP_FIT_WARPS][12];
    // the multipole kernel launched after this one with programmatic stream
    // serialization may start (its node-table prologue) once every block of
    // this grid has started; it waits for this grid's completion before it
    // reads the fits.  The retry counter of that kernel starts at zero here
    // (the last kernel that read it completed before this grid began).
    asm volatile("griddepcontrol.launch_dependents;");
    if (retry_count && blockIdx.x == 0 && threadIdx.x == 0) *retry_count = 0;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int q = blockIdx.x * MP_FIT_WARPS + w;
    if (q < n_req) { // whole warps
        // a chain of dependent loads per warp: the separations are read eight per
        // lane at a time (one round for requests of up to 256), chi(z_mean) while
        // the first round is in flight, then (D1, f D1) at the six nodes from the
        // uniform chi table
        constexpr int U = 8;
        const long long o1 = req_offset[q + 1];
        long long i0 = req_offset[q] + lane;
        double sv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) sv[u] = i0 + 32 * u < o1 ? sep[i0 + 32 * u] : 0.0;
        const T chim = spl_eval(chi_of_z, from_f64<T>(req_z_mean[q]));
        T rmax = T(0);
        for (;;) {
#pragma unroll
            for (int u = 0; u < U; ++u) rmax = fmax(rmax, from_f64<T>(sv[u]));
            i0 += 32 * U;
            if (i0 >= o1) break;
#pragma unroll
            for (int u = 0; u < U; ++u) sv[u] = i0 + 32 * u < o1 ? sep[i0 + 32 * u] : 0.0;
        }
        for (int o = 16; o > 0; o >>= 1) rmax = fmax(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
        T X = fmin(T(0.5) * rmax, fmin(chim - tab.c0, tab.cn - chim));
        if (!(X > T(1e-3))) X = T(1e-3); // empty request or no room: its pairs are outside anyway
        if (lane < 6) {
            T g, fg;
            chi_tab_eval(tab, fma(X, vinv.t[lane], chim), g, fg);
            val[w][lane] = g;
            val[w][6 + lane] = fg;
        }
        __syncwarp();
        if (lane < 12) {
            const int c = lane % 6, off = lane < 6 ? 0 : 6;
            T acc = T(0);
            for (int k = 0; k < 6; ++k) acc = fma(vinv.m[c][k], val[w][off + k], acc);
            cof[w][lane] = acc;
        }
        __syncwarp();
        if (lane == 0) {
            const T *c = cof[w];
            BgFitT<T> o;
            o.ge = mk4(c[0], c[2], c[4], T(1) / X);
            o.go = mk4(c[1], c[3], c[5], chim);
            o.fe = mk4(c[6], c[8], c[10], X);
            o.fo = mk4(c[7], c[9], c[11], T(0));
            fit[q] = o;
        }
    }
    // Launched right after the table kernel (programmatic dependent launch),
    // this grid may run while the table kernel's last blocks do; every thread
    // waits here for that kernel to complete and its writes to be visible, so
    // that work ordered after this grid sees the tables.  (Launched after
    // anything else, the wait returns at once.)
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// the inverse Vandermonde matrix of the six Chebyshev points (host, FP64)
template <typename T> FitInvT<T> fit_inverse()
{
    FitInvT<T> r;
    double V[6][12];
    for (int j = 0; j < 6; ++j) {
        const double t = cos((2 * j + 1) * CG_PI / 12.0);
        double p = 1.0;
        for (int c = 0; c < 6; ++c, p *= t) V[j][c] = p;
        for (int c = 0; c < 6; ++c) V[j][6 + c] = (c == j) ? 1.0 : 0.0;
    }
    for (int c = 0; c < 6; ++c) { // Gauss-Jordan with partial pivoting
        int piv = c;
        for (int r2 = c + 1; r2 < 6; ++r2)
            if (fabs(V[r2][c]) > fabs(V[piv][c])) piv = r2;
        for (int k = 0; k < 12; ++k) std::swap(V[c][k], V[piv][k]);
        const double d = V[c][c];
        for (int k = 0; k < 12; ++k) V[c][k] /= d;
        for (int r2 = 0; r2 < 6; ++r2)
            if (r2 != c) {
                const double m = V[r2][c];
                for (int k = 0; k < 12; ++k) V[r2][k] -= m * V[c][k];
            }
    }
    for (int j = 0; j < 6; ++j) {
        r.t[j] = (T)cos((2 * j + 1) * CG_PI / 12.0);
        for (int k = 0; k < 6; ++k) r.m[j][k] = (T)V[j][6 + k];
    }
    return r;
}

// node table of mp_fast_kernel, rows mu >= 0 ascending:
//   row k: mu, mu^2, 1 - mu^2, a2, a1, a0, b2, -b1, wk P_l (NL), wg P_l (NL), wk |P_l| (NL)
//   then per row: wk, P_l (NL)
template <int NL> struct FastLayout {
    static constexpr int R1 = ((8 + 3 * NL) + 3) / 4 * 4;
    static constexpr int R2 = ((1 + NL) + 3) / 4 * 4;
    static constexpr int ROWS = 31;
    static constexpr int COUNT = ROWS * (R1 + R2);
    // the integrand rows start 16-byte aligned and hold a block's NL double
    // results when mp_fast_kernel stages its output
    static_assert(COUNT % 4 == 0 && ROWS * sizeof(float) >= NL * sizeof(double), "layout");
};

#define MP_FAST_MAX_THREADS 256

// 1/x: the MUFU reciprocal (2 ulp) on the float path, IEEE division in double
__device__ __forceinline__ float fast_rcp(float x) { return __fdividef(1.f, x); }
__device__ __forceinline__ double fast_rcp(double x) { return 1.0 / x; }

// Compensated (Kahan) Kronrod sum on the float path; plain sums in double
template <typename T> struct KSum;
template <> struct KSum<float> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float y)
    {
        const float yk = y - c;
        const float t = s + yk;
        c = (t - s) - yk;
        s = t;
    }
};
template <> struct KSum<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double y) { s += y; }
};

// T = float: the mixed path.  T = double: the same algorithm (background
// polynomials, regrouped integrand) in FP64, the precision-only baseline of
// the mixed path (COFFE_GPU_FP64_FASTALG).
template <int NL, int CONTRIB, int UNROLL, typename T>
__global__ void __launch_bounds__(MP_FAST_MAX_THREADS)
    mp_fast_kernel(MpArgs a, const BgFitT<T> *__restrict__ fit, T chi_lo, T chi_hi,
                   const T *__restrict__ tab_x, const T *__restrict__ tab_y,
                   const int *__restrict__ req_spectrum, const double *__restrict__ req_z_mean,
                   const int64_t *__restrict__ req_offset, const double *__restrict__ sep,
                   long long total, const T *__restrict__ nodes, double *__restrict__ out,
                   int *__restrict__ retry_count, int2 *__restrict__ retry, int *err)
{
    typedef FastLayout<NL> LY;
    extern __shared__ __align__(16) unsigned char mp_smem[];
    T *tab1 = reinterpret_cast<T *>(mp_smem); // [ROWS][R1]
    T *tab2 = tab1 + LY::ROWS * LY::R1;       // [ROWS][R2]
    T *xs = tab2 + LY::ROWS * LY::R2;         // [ROWS][blockDim.x] integrand values
    for (int i = threadIdx.x; i < LY::COUNT; i += blockDim.x) tab1[i] = nodes[i];
    __syncthreads();
    const long long item0 = (long long)blockIdx.x * blockDim.x;
    const long long item = item0 + threadIdx.x;
    const int qw = find_request_warp(req_offset, a.n_req, item); // every lane takes part
    if (item >= total && !a.out_staged) return; // the staged store needs every thread
    const bool valid = item < total;
    const int q = valid ? qw : 0;
    const int s = req_spectrum[q];
    const T r = valid ? from_f64<T>(sep[item]) : T(1);
    const BgFitT<T> bf = fit[q];
    const T chim = bf.go.w;
    const T *y0 = tab_y + ((size_t)s * a.n_terms) * a.tab_len;
    const T idl = from_f64<T>(a.inv_dlog);
    const int tl = a.tab_len;
    T I00, I02, I04;
    table_lookup3<T>(tab_x, y0 + (size_t)a.t00 * tl, y0 + (size_t)a.t02 * tl,
                     y0 + (size_t)a.t04 * tl, tl, idl, r, I00, I02, I04);
    const int bd = blockDim.x, tid = threadIdx.x;
    KSum<T> K[NL];
    T G[NL], A[NL];
#pragma unroll
    for (int j = 0; j < NL; ++j) G[j] = A[j] = T(0);
    const T half_r = T(0.5) * r;
    const T span = tab1[(LY::ROWS - 1) * LY::R1] * half_r; // largest mu
    const bool inside = valid && (chim - span >= chi_lo) && (chim + span <= chi_hi);
    const bool finite = inside && isfinite(I00) && isfinite(I02) && isfinite(I04);
    if (inside) {
        const T A2 = T(2) * chim * chim, Br = T(0.5) * r * r, r2 = r * r;
        const T e00 = I00 * T(1.0 / 15.0), e02 = I02 * T(1.0 / 21.0), e04 = I04 * T(1.0 / 35.0);
        const T e00x2 = T(2) * e00, e0d = e00 - e02;
        const T K1 = (I00 - T(2) * I02) * T(1.0 / 3.0);
        const T rho = half_r * bf.ge.w; // t = mu rho in [-1, 1] for inside pairs
#pragma unroll UNROLL
        for (int k = 0; k < LY::ROWS; ++k) {
            T rec[LY::R1];
            lds_rec<LY::R1>(tab1 + k * LY::R1, rec);
            const T mu = rec[0], mu2 = rec[1], omm = rec[2];
            const T chi1 = fma(-mu, half_r, chim), chi2 = fma(mu, half_r, chim);
            // background at chi_mean -/+ mu r/2: even and odd parts in t
            const T t = mu * rho, u = t * t;
            const T gE = fma(fma(bf.ge.z, u, bf.ge.y), u, bf.ge.x);
            const T gO = fma(fma(bf.go.z, u, bf.go.y), u, bf.go.x);
            const T fE = fma(fma(bf.fe.z, u, bf.fe.y), u, bf.fe.x);
            const T fO = fma(fma(bf.fo.z, u, bf.fo.y), u, bf.fo.x);
            const T G1 = fma(-t, gO, gE), G2 = fma(t, gO, gE);
            const T F1 = fma(-t, fO, fE), F2 = fma(t, fO, fE);
            const T D = fma(-mu2, Br, A2); // 2 chi1 chi2
            const T inv_D = fast_rcp(D);
            const T sv = r2 * omm * inv_D;
            const T c = T(1) - sv;
            T v = T(0);
            if (CONTRIB & COFFE_GPU_DEN) v = G1 * G2 * I00;
            if (CONTRIB & COFFE_GPU_RSD) {
                const T g2c = fma(rec[3], e04, fma(-rec[6], e02, e00x2));
                const T g1c = fma(rec[4], e04, rec[7] * e02);
                const T g0c = fma(rec[5], e04, e0d);
                v = fma(F1 * F2, fma(fma(g2c, c, g1c), c, g0c), v);
            }
            if ((CONTRIB & COFFE_GPU_DEN) && (CONTRIB & COFFE_GPU_RSD)) {
                const T gf = G1 * F2, fg = F1 * G2;
                const T g = (T(1) + c) * omm * inv_D;
                v = fma(gf + fg, K1, v);
                v = fma(g * I02, fma(gf, chi1 * chi1, fg * (chi2 * chi2)), v);
            }
            xs[k * bd + tid] = v;
            const T av = fabs(v);
#pragma unroll
            for (int j = 0; j < NL; ++j) {
                K[j].add(rec[8 + j] * v);
                G[j] = fma(rec[8 + NL + j], v, G[j]);
                A[j] = fma(rec[8 + 2 * NL + j], av, A[j]);
            }
        }
    }
    T Ks[NL], asc[NL];
#pragma unroll
    for (int j = 0; j < NL; ++j) {
        Ks[j] = K[j].s;
        asc[j] = T(0);
    }
    if (inside) {
#pragma unroll 1
        for (int k = 0; k < LY::ROWS; ++k) {
            T rec[LY::R2];
            lds_rec<LY::R2>(tab2 + k * LY::R2, rec);
            const T v = xs[k * bd + tid];
#pragma unroll
            for (int j = 0; j < NL; ++j)
                asc[j] = fma(rec[0], fabs(fma(v, rec[1 + j], T(-0.5) * Ks[j])), asc[j]);
        }
    }
    if (!a.out_staged) {
        first_panel_out<NL, T>(a, from_f64<T>(a.epsrel), item, finite, Ks, G, A, asc, out,
                               retry_count, retry, err);
        return;
    }
    // out in page-locked host memory: the block's results go through shared
    // memory (the xs rows, no longer read) and leave as consecutive 16-byte
    // stores, whole lines over the host link instead of 8-byte pieces
    double res[NL];
    bool have[NL];
    if (valid)
        first_panel_value<NL, T>(a, from_f64<T>(a.epsrel), item, finite, Ks, G, A, asc, res,
                                 have, retry_count, retry, err);
    __syncthreads();
    double *stage = reinterpret_cast<double *>(xs);
    if (valid) {
#pragma unroll
        for (int j = 0; j < NL; ++j) stage[tid * NL + j] = res[j]; // retried: NaN until retried
    }
    __syncthreads();
    const int n = (int)min((long long)bd, total - item0) * NL;
    double *o = out + item0 * NL;
    if ((reinterpret_cast<uintptr_t>(o) & 15) == 0) {
        const double2 *s2 = reinterpret_cast<const double2 *>(stage);
        double2 *o2 = reinterpret_cast<double2 *>(o);
        for (int i = tid; i < n / 2; i += bd) o2[i] = s2[i];
        if ((n & 1) && tid == 0) o[n - 1] = stage[n - 1];
    } else {
        for (int i = tid; i < n; i += bd) o[i] = stage[i];
    }
}

// o += a b, truncated to the NO lowest coefficients
template <int NA, int NB, int NO, typename T>
__device__ __forceinline__ void poly_fma(const T (&a)[NA], const T (&b)[NB], T (&o)[NO])
{
#pragma unroll
    for (int i = 0; i < NA; ++i)
#pragma unroll
        for (int j = 0; j < NB; ++j)
            if (i + j < NO) o[i + j] = fma(a[i], b[j], o[i + j]);
}

// The first-panel integrand of one (request, separation) as coefficients of
// w = mu^2 (mp_fast_kernel's algebra, functions.c:129-362, 670-771, expanded):
//   v = G1 G2 I00 + F1 F2 R(c) + (G1 F2 + F1 G2) K1 + g I02 (G1 F2 chi1^2 + F1 G2 chi2^2)
// with G1 G2 = gE^2 - rho^2 w gO^2, F1 F2 = fE^2 - rho^2 w fO^2,
// G1 F2 + F1 G2 = 2 A, A = gE fE - rho^2 w gO fO, and
// G1 F2 chi1^2 + F1 G2 chi2^2 = 2 A (chi^2 + w r^2 / 4) - 2 rho r chi w B,
// B = gE fO - gO fE; c = 1 - r^2 (1 - w) / D, g = (1 + c)(1 - w) / D.
template <int CONTRIB, typename T>
__device__ __forceinline__ void poly_integrand(const BgFitT<T> &bf, T chim, T r, T rho, T I00,
                                               T I02, T I04, T (&v)[MP_PJ + 1])
{
    constexpr int N = MP_PJ + 1;
#pragma unroll
    for (int j = 0; j < N; ++j) v[j] = T(0);
    const T p2 = rho * rho, p4 = p2 * p2;
    const T gE[3] = {bf.ge.x, bf.ge.y * p2, bf.ge.z * p4};
    const T gO[3] = {bf.go.x, bf.go.y * p2, bf.go.z * p4};
    const T fE[3] = {bf.fe.x, bf.fe.y * p2, bf.fe.z * p4};
    const T fO[3] = {bf.fo.x, bf.fo.y * p2, bf.fo.z * p4};
    // a w-shifted product: o[j + 1] += s a[i] b[j - i]
    auto shifted = [&](const T(&a)[3], const T(&b)[3], T sc, T(&o)[6]) {
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) o[i + j + 1] = fma(sc * a[i], b[j], o[i + j + 1]);
    };
    if (CONTRIB & COFFE_GPU_DEN) {
        T GG[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
        poly_fma(gE, gE, GG);
        shifted(gO, gO, -p2, GG);
#pragma unroll
        for (int j = 0; j < 6; ++j) v[j] = GG[j] * I00;
    }
    if (CONTRIB & COFFE_GPU_RSD) {
        const T h = T(0.5) / (chim * chim), x = r * r * T(0.5) * h; // 1/(2 chi^2), r^2/(4 chi^2)
        T iD[MP_PS + 1];
        iD[0] = h;
#pragma unroll
        for (int n = 1; n <= MP_PS; ++n) iD[n] = iD[n - 1] * x;
        // s = r^2 (1 - w) / D, c = 1 - s
        T c[MP_PS + 2];
        const T rr = r * r;
        c[0] = T(1) - rr * iD[0];
#pragma unroll
        for (int n = 1; n <= MP_PS; ++n) c[n] = rr * (iD[n - 1] - iD[n]);
        c[MP_PS + 1] = rr * iD[MP_PS];
        T c2[N];
#pragma unroll
        for (int j = 0; j < N; ++j) c2[j] = T(0);
        poly_fma(c, c, c2);
        const T e00 = I00 * T(1.0 / 15.0), e02 = I02 * T(1.0 / 21.0), e04 = I04 * T(1.0 / 35.0);
        // R(c) = g2c c^2 + g1c c + g0c with the quadratics in w of the node table
        const T g2c[3] = {fma(T(0.75), e04, fma(T(-2), e02, T(2) * e00)),
                          fma(T(2.5), e04, T(-9) * e02), T(8.75) * e04};
        const T g1c[3] = {fma(T(-2.5), e04, T(9) * e02), fma(T(-15), e04, T(-9) * e02),
                          T(17.5) * e04};
        const T g0c[3] = {fma(T(4.75), e04, e00 - e02), T(-17.5) * e04, T(8.75) * e04};
        T R[N] = {g0c[0], g0c[1], g0c[2]};
#pragma unroll
        for (int j = 3; j < N; ++j) R[j] = T(0);
        poly_fma(g2c, c2, R);
        poly_fma(g1c, c, R);
        T FF[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
        poly_fma(fE, fE, FF);
        shifted(fO, fO, -p2, FF);
        poly_fma(FF, R, v);
        if (CONTRIB & COFFE_GPU_DEN) {
            T Am[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
            poly_fma(gE, fE, Am);
            shifted(gO, fO, -p2, Am);
            T Bm[5] = {T(0), T(0), T(0), T(0), T(0)};
            poly_fma(gE, fO, Bm);
            const T mgO[3] = {-gO[0], -gO[1], -gO[2]};
            poly_fma(mgO, fE, Bm);
            const T K1 = (I00 - T(2) * I02) * T(1.0 / 3.0);
#pragma unroll
            for (int j = 0; j < 6; ++j) v[j] = fma(T(2) * K1, Am[j], v[j]);
            // Q = 2 A (chi^2 + w r^2/4) - 2 rho r chi w B
            T Q[7];
            const T cq0 = T(2) * chim * chim, cq1 = T(0.5) * rr, cb = T(-2) * rho * r * chim;
            Q[0] = cq0 * Am[0];
#pragma unroll
            for (int j = 1; j < 6; ++j) Q[j] = fma(cq0, Am[j], fma(cq1, Am[j - 1], cb * Bm[j - 1]));
            Q[6] = cq1 * Am[5];
            // g = (2 - s)(1 - w) / D = (1 + c)(1 - w) / D
            T om[MP_PS + 3];
            const T cp0 = T(1) + c[0];
            om[0] = cp0;
#pragma unroll
            for (int n = 1; n <= MP_PS + 1; ++n)
                om[n] = c[n] - (n == 1 ? cp0 : c[n - 1]);
            om[MP_PS + 2] = -c[MP_PS + 1];
            T g[N];
#pragma unroll
            for (int j = 0; j < N; ++j) g[j] = T(0);
            poly_fma(om, iD, g);
#pragma unroll
            for (int j = 0; j < N; ++j) g[j] *= I02;
            poly_fma(g, Q, v);
        }
    }
}

// Mixed path (T = float) and its FP64 baseline (T = double), unit biases and
// even multipoles: mp_fast_kernel's first panel with the integrand as the
// polynomial of poly_integrand (Kronrod and Gauss sums as moments; the |f|
// and |f - mean| sums from a Horner evaluation at each node).  The float
// kernel is held to 48 registers (five blocks of 256 per SM instead of four,
// a few spilled values: 50.3 against 52.4 us on the 512-spectrum batch); the
// FP64 one keeps its own allocation.
template <int NL, int CONTRIB, int UNROLL, typename T>
__global__ void __launch_bounds__(MP_FAST_MAX_THREADS, sizeof(T) == sizeof(float) ? 5 : 1)
    mp_poly_kernel(MpArgs a, const BgFitT<T> *__restrict__ fit, T chi_lo, T chi_hi,
                   const T *__restrict__ tab_x, const T *__restrict__ tab_y,
                   const int *__restrict__ req_spectrum, const double *__restrict__ req_z_mean,
                   const int64_t *__restrict__ req_offset, const double *__restrict__ sep,
                   long long total, const T *__restrict__ nodes, PolyMom<T> mom,
                   double *__restrict__ out, int *__restrict__ retry_count,
                   int2 *__restrict__ retry, int *err)
{
    typedef PolyLayout<NL> LY;
    extern __shared__ __align__(16) unsigned char mp_smem[];
    T *tab = reinterpret_cast<T *>(mp_smem);                           // [ROWS][R]
    double *stage = reinterpret_cast<double *>(tab + LY::COUNT);      // [blockDim][NL]
    for (int i = threadIdx.x; i < LY::COUNT; i += blockDim.x) tab[i] = nodes[i];
    // launched as a dependent of the background fit: the fits (and, through
    // the fit's own wait, the tables) are complete and visible after this
    // (otherwise it returns at once)
    asm volatile("griddepcontrol.wait;" ::: "memory");
    __syncthreads();
    const long long item0 = (long long)blockIdx.x * blockDim.x;
    const long long item = item0 + threadIdx.x;
    const int qw = find_request_warp(req_offset, a.n_req, item); // every lane takes part
    if (item >= total && !a.out_staged) return; // the staged store needs every thread
    const bool valid = item < total;
    const int q = valid ? qw : 0;
    const int s = req_spectrum[q];
    const T r = valid ? from_f64<T>(sep[item]) : T(1);
    const BgFitT<T> bf = fit[q];
    const T chim = bf.go.w;
    const T *y0 = tab_y + ((size_t)s * a.n_terms) * a.tab_len;
    const T idl = from_f64<T>(a.inv_dlog);
    const int tl = a.tab_len;
    T I00, I02, I04;
    table_lookup3<T>(tab_x, y0 + (size_t)a.t00 * tl, y0 + (size_t)a.t02 * tl,
                     y0 + (size_t)a.t04 * tl, tl, idl, r, I00, I02, I04);
    T K[NL], G[NL], A[NL], asc[NL];
#pragma unroll
    for (int j = 0; j < NL; ++j) K[j] = G[j] = A[j] = asc[j] = T(0);
    const T half_r = T(0.5) * r;
    const T span = half_r * sqrt(tab[(LY::ROWS - 1) * LY::R]); // largest mu
    const bool inside = valid && (chim - span >= chi_lo) && (chim + span <= chi_hi);
    const bool finite = inside && isfinite(I00) && isfinite(I02) && isfinite(I04);
    if (inside) {
        T v[MP_PJ + 1];
        poly_integrand<CONTRIB, T>(bf, chim, r, half_r * bf.ge.w, I00, I02, I04, v);
        T Kh[NL];
#pragma unroll
        for (int j = 0; j < NL; ++j) {
            T k = T(0), g = T(0);
#pragma unroll
            for (int e = MP_PJ; e >= 0; --e) {
                k = fma(v[e], mom.mk[j][e], k);
                g = fma(v[e], mom.mg[j][e], g);
            }
            K[j] = k;
            G[j] = g;
            Kh[j] = T(-0.5) * k;
        }
#pragma unroll UNROLL
        for (int n = 0; n < LY::ROWS; ++n) {
            T rec[LY::R];
            lds_rec<LY::R>(tab + n * LY::R, rec);
            const T w = rec[0];
            T f = v[MP_PJ];
#pragma unroll
            for (int e = MP_PJ - 1; e >= 0; --e) f = fma(f, w, v[e]);
            const T af = fabs(f);
#pragma unroll
            for (int j = 0; j < NL; ++j) {
                A[j] = fma(rec[2 + NL + j], af, A[j]);
                asc[j] = fma(rec[1], fabs(fma(f, rec[2 + j], Kh[j])), asc[j]);
            }
        }
    }
    if (!a.out_staged) {
        first_panel_out<NL, T>(a, from_f64<T>(a.epsrel), item, finite, K, G, A, asc, out,
                               retry_count, retry, err);
        return;
    }
    // out in page-locked host memory: staged in shared memory, stored as
    // consecutive 16-byte words (mp_fast_kernel's epilogue)
    double res[NL];
    bool have[NL];
    if (valid)
        first_panel_value<NL, T>(a, from_f64<T>(a.epsrel), item, finite, K, G, A, asc, res, have,
                                 retry_count, retry, err);
    const int tid = threadIdx.x, bd = blockDim.x;
    if (valid) {
#pragma unroll
        for (int j = 0; j < NL; ++j) stage[tid * NL + j] = res[j];
    }
    __syncthreads();
    const int n = (int)min((long long)bd, total - item0) * NL;
    double *o = out + item0 * NL;
    if ((reinterpret_cast<uintptr_t>(o) & 15) == 0) {
        const double2 *s2 = reinterpret_cast<const double2 *>(stage);
        double2 *o2 = reinterpret_cast<double2 *>(o);
        for (int i = tid; i < n / 2; i += bd) o2[i] = s2[i];
        if ((n & 1) && tid == 0) o[n - 1] = stage[n - 1];
    } else {
        for (int i = tid; i < n; i += bd) o[i] = stage[i];
    }
}

// ---------------------------------- mixed path, two separations per thread
//
// mp_fast_kernel's algorithm (float) with every per-node operation on packed
// FP32 pairs: each thread evaluates two (request, separation) pairs, lane lo
// the separation item0 + tid and lane hi item0 + blockDim + tid, so one
// fma/add/mul.rn.f32x2 issue serves both.  The kernel is bound by instruction
// issue, not by the FMA pipe, so halving the FP32 instructions is the lever.
// The results are those of the one-pair kernel up to float rounding order.
template <int NL> struct Fast2Layout {
    static constexpr int P1 = 9 + 3 * NL;  // packed constants of pass 1
    static constexpr int P2 = 1 + NL;      // and of pass 2
    static constexpr int F1 = (2 * P1 + 3) / 4 * 4;
    static constexpr int F2 = (2 * P2 + 3) / 4 * 4;
    static constexpr int ROWS = 31;
    static constexpr int COUNT = ROWS * (F1 + F2); // floats
    // the rows of integrand pairs (8 bytes per thread and node) hold the
    // block's 2 blockDim x NL double results when the output is staged
    static_assert(COUNT % 4 == 0 && ROWS * 8 >= 2 * NL * 8, "layout");
};

// row of packed pairs from shared memory (16-byte loads)
template <int F> __device__ __forceinline__ void lds_pairs(const float *p, f2 (&r)[F / 2])
{
#pragma unroll
    for (int i = 0; i < F / 4; ++i) {
        const ulonglong2 v = reinterpret_cast<const ulonglong2 *>(p)[i];
        r[2 * i].v = v.x;
        r[2 * i + 1].v = v.y;
    }
}

template <int NL, int CONTRIB, int UNROLL>
__global__ void __launch_bounds__(MP_FAST_MAX_THREADS)
    mp_fast2_kernel(MpArgs a, const BgFitT<float> *__restrict__ fit, float chi_lo, float chi_hi,
                    const float *__restrict__ tab_x, const float *__restrict__ tab_y,
                    const int *__restrict__ req_spectrum, const double *__restrict__ req_z_mean,
                    const int64_t *__restrict__ req_offset, const double *__restrict__ sep,
                    long long total, const float *__restrict__ nodes, double *__restrict__ out,
                    int *__restrict__ retry_count, int2 *__restrict__ retry, int *err)
{
    typedef Fast2Layout<NL> LY;
    extern __shared__ __align__(16) unsigned char mp_smem[];
    float *tab1 = reinterpret_cast<float *>(mp_smem); // [ROWS][F1]
    float *tab2 = tab1 + LY::ROWS * LY::F1;           // [ROWS][F2]
    f2 *xs = reinterpret_cast<f2 *>(tab2 + LY::ROWS * LY::F2); // [ROWS][blockDim.x]
    for (int i = threadIdx.x; i < LY::COUNT; i += blockDim.x) tab1[i] = nodes[i];
    __syncthreads();
    const int bd = blockDim.x, tid = threadIdx.x;
    const long long item0 = (long long)blockIdx.x * 2 * bd;
    const long long it[2] = {item0 + tid, item0 + bd + tid};
    if (it[0] >= total && !a.out_staged) return; // the staged store needs every thread
    const float idl = f32_of_bits(a.inv_dlog);
    const int tl = a.tab_len;
    const float mu_max = tab1[(LY::ROWS - 1) * LY::F1]; // largest mu
    // per lane: the separation, its request's background polynomials and the
    // three table values
    float r[2], chim[2], rho[2], I00[2], I02[2], I04[2];
    float4 ge[2], go[2], fe[2], fo[2];
    bool valid[2], inside[2], finite[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        valid[h] = it[h] < total;
        const int q = valid[h] ? find_request(req_offset, a.n_req, it[h]) : 0;
        const int s = req_spectrum[q];
        r[h] = valid[h] ? f32_of_bits(sep[it[h]]) : 1.f;
        const BgFitT<float> bf = fit[q];
        ge[h] = bf.ge;
        go[h] = bf.go;
        fe[h] = bf.fe;
        fo[h] = bf.fo;
        chim[h] = bf.go.w;
        rho[h] = 0.5f * r[h] * bf.ge.w;
        const float *y0 = tab_y + ((size_t)s * a.n_terms) * tl;
        I00[h] = table_lookup<float, true>(tab_x, y0 + (size_t)a.t00 * tl, tl, idl, r[h]);
        I02[h] = table_lookup<float, true>(tab_x, y0 + (size_t)a.t02 * tl, tl, idl, r[h]);
        I04[h] = table_lookup<float, true>(tab_x, y0 + (size_t)a.t04 * tl, tl, idl, r[h]);
        const float span = mu_max * 0.5f * r[h];
        inside[h] = valid[h] && (chim[h] - span >= chi_lo) && (chim[h] + span <= chi_hi);
        finite[h] = inside[h] && isfinite(I00[h]) && isfinite(I02[h]) && isfinite(I04[h]);
    }
    f2 K[NL], nKc[NL], G[NL], A[NL];
#pragma unroll
    for (int j = 0; j < NL; ++j) K[j] = nKc[j] = G[j] = A[j] = f2_dup(0.f);
    const bool any = inside[0] || inside[1];
    if (any) {
        const f2 hr = f2_pack(0.5f * r[0], 0.5f * r[1]);
        const f2 cm = f2_pack(chim[0], chim[1]);
        const f2 A2 = f2_pack(2.f * chim[0] * chim[0], 2.f * chim[1] * chim[1]);
        const f2 Br = f2_pack(0.5f * r[0] * r[0], 0.5f * r[1] * r[1]);
        const f2 r2 = f2_pack(r[0] * r[0], r[1] * r[1]);
        const f2 rh = f2_pack(rho[0], rho[1]);
        const f2 gex = f2_pack(ge[0].x, ge[1].x), gey = f2_pack(ge[0].y, ge[1].y),
                 gez = f2_pack(ge[0].z, ge[1].z);
        const f2 gox = f2_pack(go[0].x, go[1].x), goy = f2_pack(go[0].y, go[1].y),
                 goz = f2_pack(go[0].z, go[1].z);
        const f2 fex = f2_pack(fe[0].x, fe[1].x), fey = f2_pack(fe[0].y, fe[1].y),
                 fez = f2_pack(fe[0].z, fe[1].z);
        const f2 fox = f2_pack(fo[0].x, fo[1].x), foy = f2_pack(fo[0].y, fo[1].y),
                 foz = f2_pack(fo[0].z, fo[1].z);
        const f2 i00 = f2_pack(I00[0], I00[1]), i02 = f2_pack(I02[0], I02[1]);
        const f2 e00 = f2_mul(i00, f2_dup(1.f / 15.f)), e02 = f2_mul(i02, f2_dup(1.f / 21.f)),
                 e04 = f2_pack(I04[0] * (1.f / 35.f), I04[1] * (1.f / 35.f));
        const f2 e00x2 = f2_add(e00, e00), e0d = f2_sub(e00, e02);
        const f2 K1 = f2_mul(f2_sub(i00, f2_add(i02, i02)), f2_dup(1.f / 3.f));
        const f2 one = f2_dup(1.f);
#pragma unroll UNROLL
        for (int k = 0; k < LY::ROWS; ++k) {
            f2 c[LY::F1 / 2];
            lds_pairs<LY::F1>(tab1 + k * LY::F1, c);
            const f2 mu = c[0], nmu = c[1], nmu2 = c[2], omm = c[3];
            const f2 chi1 = f2_fma(nmu, hr, cm), chi2 = f2_fma(mu, hr, cm);
            // background at chi_mean -/+ mu r/2: even and odd parts in t
            const f2 t = f2_mul(mu, rh), tn = f2_mul(nmu, rh), u = f2_mul(t, t);
            const f2 gE = f2_fma(f2_fma(gez, u, gey), u, gex);
            const f2 gO = f2_fma(f2_fma(goz, u, goy), u, gox);
            const f2 fE = f2_fma(f2_fma(fez, u, fey), u, fex);
            const f2 fO = f2_fma(f2_fma(foz, u, foy), u, fox);
            const f2 G1 = f2_fma(tn, gO, gE), G2 = f2_fma(t, gO, gE);
            const f2 F1 = f2_fma(tn, fO, fE), F2 = f2_fma(t, fO, fE);
            const f2 D = f2_fma(nmu2, Br, A2); // 2 chi1 chi2
            const f2 inv_D = f2_rcp(D);
            const f2 sv = f2_mul(f2_mul(r2, omm), inv_D);
            const f2 cc = f2_sub(one, sv);
            f2 v = f2_dup(0.f);
            if (CONTRIB & COFFE_GPU_DEN) v = f2_mul(f2_mul(G1, G2), i00);
            if (CONTRIB & COFFE_GPU_RSD) {
                const f2 g2c = f2_fma(c[4], e04, f2_fma(c[7], e02, e00x2));
                const f2 g1c = f2_fma(c[5], e04, f2_mul(c[8], e02));
                const f2 g0c = f2_fma(c[6], e04, e0d);
                v = f2_fma(f2_mul(F1, F2), f2_fma(f2_fma(g2c, cc, g1c), cc, g0c), v);
            }
            if ((CONTRIB & COFFE_GPU_DEN) && (CONTRIB & COFFE_GPU_RSD)) {
                const f2 gf = f2_mul(G1, F2), fg = f2_mul(F1, G2);
                const f2 g = f2_mul(f2_mul(f2_add(one, cc), omm), inv_D);
                v = f2_fma(f2_add(gf, fg), K1, v);
                v = f2_fma(f2_mul(g, i02),
                           f2_fma(gf, f2_mul(chi1, chi1), f2_mul(fg, f2_mul(chi2, chi2))), v);
            }
            xs[k * bd + tid] = v;
            const f2 av = f2_abs(v);
#pragma unroll
            for (int j = 0; j < NL; ++j) { // Kahan-compensated Kronrod sum, -c kept
                const f2 yk = f2_fma(c[9 + j], v, nKc[j]);
                const f2 tk = f2_add(K[j], yk);
                nKc[j] = f2_sub(yk, f2_sub(tk, K[j]));
                K[j] = tk;
                G[j] = f2_fma(c[9 + NL + j], v, G[j]);
                A[j] = f2_fma(c[9 + 2 * NL + j], av, A[j]);
            }
        }
    }
    f2 asc[NL], nhK[NL];
#pragma unroll
    for (int j = 0; j < NL; ++j) {
        asc[j] = f2_dup(0.f);
        nhK[j] = f2_mul(K[j], f2_dup(-0.5f));
    }
    if (any) {
#pragma unroll 1
        for (int k = 0; k < LY::ROWS; ++k) {
            f2 c[LY::F2 / 2];
            lds_pairs<LY::F2>(tab2 + k * LY::F2, c);
            const f2 v = xs[k * bd + tid];
#pragma unroll
            for (int j = 0; j < NL; ++j)
                asc[j] = f2_fma(c[0], f2_abs(f2_fma(v, c[1 + j], nhK[j])), asc[j]);
        }
    }
    float Kl[2][NL], Gl[2][NL], Al[2][NL], Sl[2][NL];
#pragma unroll
    for (int j = 0; j < NL; ++j) {
        Kl[0][j] = f2_lo(K[j]);
        Kl[1][j] = f2_hi(K[j]);
        Gl[0][j] = f2_lo(G[j]);
        Gl[1][j] = f2_hi(G[j]);
        Al[0][j] = f2_lo(A[j]);
        Al[1][j] = f2_hi(A[j]);
        Sl[0][j] = f2_lo(asc[j]);
        Sl[1][j] = f2_hi(asc[j]);
    }
    const float eps = f32_of_bits(a.epsrel);
    if (!a.out_staged) {
#pragma unroll
        for (int h = 0; h < 2; ++h)
            if (valid[h])
                first_panel_out<NL, float>(a, eps, it[h], finite[h], Kl[h], Gl[h], Al[h], Sl[h],
                                           out, retry_count, retry, err);
        return;
    }
    // out in page-locked host memory: the block's 2 blockDim results go
    // through shared memory (the integrand rows, no longer read) and leave as
    // consecutive 16-byte stores
    double res[2][NL];
    bool have[2][NL];
#pragma unroll
    for (int h = 0; h < 2; ++h)
        if (valid[h])
            first_panel_value<NL, float>(a, eps, it[h], finite[h], Kl[h], Gl[h], Al[h], Sl[h],
                                         res[h], have[h], retry_count, retry, err);
    __syncthreads();
    double *stage = reinterpret_cast<double *>(xs);
#pragma unroll
    for (int h = 0; h < 2; ++h)
        if (valid[h]) {
#pragma unroll
            for (int j = 0; j < NL; ++j) stage[(h * bd + tid) * NL + j] = res[h][j];
        }
    __syncthreads();
    const int n = (int)min((long long)(2 * bd), total - item0) * NL;
    double *o = out + item0 * NL;
    if ((reinterpret_cast<uintptr_t>(o) & 15) == 0) {
        const double2 *s2 = reinterpret_cast<const double2 *>(stage);
        double2 *o2 = reinterpret_cast<double2 *>(o);
        for (int i = tid; i < n / 2; i += bd) o2[i] = s2[i];
        if ((n & 1) && tid == 0) o[n - 1] = stage[n - 1];
    } else {
        for (int i = tid; i < n; i += bd) o[i] = stage[i];
    }
}

// ------------------------------------------------- correlation function
// xi(z_mean, mu, r) of the nonintegrated den/rsd terms (corrfunc.c:55-141,
// signal.c:511-518: functions_nonintegrated at the requested mu), one thread
// per (separation, mu): out[item * n_mu + m].
template <typename T, typename S, typename TT>
__global__ void cf_nonint_kernel(MpArgs a, Bg<T, S> bg, S chi_of_z, const TT *__restrict__ tab_x,
                                 const TT *__restrict__ tab_y, const int *__restrict__ req_spectrum,
                                 const double *__restrict__ req_z_mean,
                                 const int64_t *__restrict__ req_offset,
                                 const double *__restrict__ sep, const double *__restrict__ mu,
                                 int n_mu, long long total, double *__restrict__ out, int *err)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total * n_mu) return;
    const long long item = t / n_mu;
    const int m = (int)(t - item * n_mu);
    const int q = find_request(req_offset, a.n_req, item);
    const Xi<T, S> xi = make_xi<T, S, TT>(a, bg, chi_of_z, tab_x, tab_y, req_spectrum[q],
                                         (T)req_z_mean[q], (T)sep[item]);
    const double res = to_f64(xi((T)mu[m]));
    if (!isfinite(res)) cg_flag(err, CG_ERR_NONFINITE);
    out[t] = res;
}

// ------------------------------------------ redshift-averaged multipoles
// Expansion of every (window, separation) into n_z Gauss-Legendre redshift
// nodes (average_multipoles.c:69-156; signal.c:241-310): node k of separation
// item sits at z = z1 + (z2 - z1) v_k, z1 = z(chi(z_min) + r/2),
// z2 = z(chi(z_max) - r/2), with weight (w_k / 2) H0 h / (conformal_H(z) (1 + z)).
// The expanded entries are single-separation requests for multipoles_run.
__global__ void avg_expand_kernel(Spl64 chi_of_z, Spl64 z_of_chi, Spl64 confH, double H0h,
                                  const int *__restrict__ win_spectrum,
                                  const double *__restrict__ z_min, const double *__restrict__ z_max,
                                  const int64_t *__restrict__ win_offset, int n_win,
                                  const double *__restrict__ sep, long long total,
                                  const double *__restrict__ gl, int n_z,
                                  int *__restrict__ e_spec, double *__restrict__ e_z,
                                  int64_t *__restrict__ e_off, double *__restrict__ e_sep,
                                  double *__restrict__ e_w)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= total * n_z) return;
    const long long item = e / n_z;
    const int k = (int)(e - item * n_z);
    const int q = find_request(win_offset, n_win, item);
    const double r = sep[item];
    const double z1 = spl_eval(z_of_chi, spl_eval(chi_of_z, z_min[q]) + 0.5 * r);
    const double z2 = spl_eval(z_of_chi, spl_eval(chi_of_z, z_max[q]) - 0.5 * r);
    const double v = 0.5 * (gl[k] + 1.0);
    const double z = (z2 - z1) * v + z1;
    e_spec[e] = win_spectrum[q];
    e_z[e] = z;
    e_sep[e] = r;
    e_off[e] = e;
    if (e == total * n_z - 1) e_off[e + 1] = e + 1;
    e_w[e] = 0.5 * gl[n_z + k] * H0h / (spl_eval(confH, z) * (1.0 + z));
}

// out[item][j] = sum_k w[item, k] mp[(item, k)][j]
__global__ void avg_reduce_kernel(const double *__restrict__ e_w, const double *__restrict__ e_out,
                                  long long total, int n_z, int n_l, double *__restrict__ out,
                                  int *err)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= total * n_l) return;
    const long long item = t / n_l;
    const int j = (int)(t - item * n_l);
    double acc = 0.0;
    for (int k = 0; k < n_z; ++k)
        acc += e_w[item * n_z + k] * e_out[(item * n_z + k) * n_l + j];
    if (!isfinite(acc)) cg_flag(err, CG_ERR_NONFINITE);
    out[t] = acc;
}

// ------------------------------------------------------- adaptive retries
template <typename T, typename S, typename TT>
__global__ void __launch_bounds__(32 * MP_RETRY_WARPS)
    mp_retry_kernel(MpArgs a, Bg<T, S> bg, S chi_of_z, const TT *__restrict__ tab_x,
                    const TT *__restrict__ tab_y, const int *__restrict__ req_spectrum,
                    const double *__restrict__ req_z_mean, const int64_t *__restrict__ req_offset,
                    const double *__restrict__ sep, double *__restrict__ out,
                    const int *__restrict__ retry_count, const int2 *__restrict__ retry, int *err)
{
    __shared__ T sa[MP_RETRY_WARPS][MP_CAP], sb[MP_RETRY_WARPS][MP_CAP],
        sr[MP_RETRY_WARPS][MP_CAP], se[MP_RETRY_WARPS][MP_CAP];
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    int count = *retry_count;
    if (count > a.retry_cap) count = (int)a.retry_cap;
    const int nw = gridDim.x * MP_RETRY_WARPS;
    for (int e = blockIdx.x * MP_RETRY_WARPS + w; e < count; e += nw) {
        const int2 ent = retry[e];
        const long long item = ent.x;
        const int li = ent.y;
        const int l = a.ls[li];
        const int q = find_request(req_offset, a.n_req, item);
        const Xi<T, S> xi =
            make_xi<T, S, TT>(a, bg, chi_of_z, tab_x, tab_y, req_spectrum[q], (T)req_z_mean[q],
                              (T)sep[item]);
        MpIntegrand<T, S> fn{xi, l};
        QagStore<T> store{sa[w], sb[w], sr[w], se[w], MP_CAP};
        int status = 0;
        const T v = qag61_warp<T>(fn, T(0), T(1), T(0), (T)a.epsrel, store, 50000, &status);
        if (lane == 0) {
            if (status == 1) cg_flag(err, CG_ERR_QAG_LIMIT);
            const double res = (double)(T(2 * l + 1) * v);
            if (!isfinite(res)) cg_flag(err, CG_ERR_NONFINITE);
            out[item * a.n_l + li] = res;
        }
    }
}

// The cached node table of (multipole list, precision, layout), uploaded on
// first use: layout 0 / 1 = NodeLayout without / with the mirror rule,
// 2 = FastLayout, 3 = Fast2Layout (packed pairs).  *dev receives its device
// address.
template <typename Build>
int node_slot(coffe_gpu_ctx *ctx, int n_l, const int *ls, int prec_tag, int layout, Build build,
              const void **dev)
{
    for (auto &sl : ctx->mp_node_slots) {
        bool same = sl.buf.p && sl.nl == n_l && sl.prec == prec_tag && sl.mirror == layout;
        for (int j = 0; same && j < n_l; ++j) same = sl.ls[j] == ls[j];
        if (same) {
            *dev = sl.buf.p;
            return COFFE_GPU_OK;
        }
    }
    coffe_gpu_ctx::NodeSlot *slot = &ctx->mp_node_slots[ctx->mp_node_next];
    ctx->mp_node_next = (ctx->mp_node_next + 1) % coffe_gpu_ctx::CG_NODE_SLOTS;
    std::vector<unsigned char> bytes;
    build(bytes);
    slot->nl = 0; // invalid until the upload below has finished
    int st = cg_ensure(ctx, slot->buf, bytes.size());
    if (st) return st;
    CG_CUDA(ctx, cudaMemcpyAsync(slot->buf.p, bytes.data(), bytes.size(), cudaMemcpyHostToDevice,
                                 ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream)); // bytes is a host temporary
    slot->nl = n_l;
    slot->prec = prec_tag;
    slot->mirror = layout;
    for (int j = 0; j < n_l; ++j) slot->ls[j] = ls[j];
    *dev = slot->buf.p;
    return COFFE_GPU_OK;
}

// mp_fast_kernel for a validated call with unit biases, even multipoles (at
// most four) and no only-cross switch, then the retries: T = float for the
// mixed path, double for its FP64 baseline (COFFE_GPU_FP64_FASTALG)
template <typename T, typename S>
int launch_fast(coffe_gpu_ctx *ctx, const MpArgs &a, const Bg<T, S> &bg, const S &chi_of_z,
                const T *tab_x, const T *tab_y, const int *req_spectrum, const double *req_z_mean,
                const int64_t *req_offset, const double *sep, long long total, double *out)
{
    int *d_count = (int *)ctx->mp_retry.p;
    int2 *d_retry = (int2 *)((char *)ctx->mp_retry.p + 256);
    const void *dn = nullptr;
    const int prec_tag = sizeof(T) == sizeof(float) ? COFFE_GPU_MIXED : COFFE_GPU_FP64_FASTALG;
    int st = node_slot(ctx, a.n_l, a.ls, prec_tag, 2,
                       [&](std::vector<unsigned char> &bytes) {
                           std::vector<T> tab;
                           build_node_table_fast<T>(a.n_l, a.ls, tab);
                           bytes.assign((const unsigned char *)tab.data(),
                                        (const unsigned char *)(tab.data() + tab.size()));
                       },
                       &dn);
    if (st) return st;
    if ((st = cg_ensure(ctx, ctx->mp_bgfit, sizeof(BgFitT<T>) * (size_t)a.n_req))) return st;
    BgFitT<T> *d_fit = (BgFitT<T> *)ctx->mp_bgfit.p;
    static const FitInvT<T> vinv = fit_inverse<T>();
    const int contrib = a.contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD);
    // first panel (with lt threads per block) and the adaptive retries
    // the packed two-separation kernel (float only) and its node table
    const bool can_pack = sizeof(T) == sizeof(float);
    const void *dn2 = nullptr;
    if (can_pack &&
        (st = node_slot(ctx, a.n_l, a.ls, COFFE_GPU_MIXED, 3,
                        [&](std::vector<unsigned char> &bytes) {
                            std::vector<float> tab;
                            build_node_table_fast2(a.n_l, a.ls, tab);
                            bytes.assign((const unsigned char *)tab.data(),
                                         (const unsigned char *)(tab.data() + tab.size()));
                        },
                        &dn2)))
        return st;
    // the polynomial kernel's node rows and the rule's moments
    const void *dnp = nullptr;
    if ((st = node_slot(ctx, a.n_l, a.ls, prec_tag, 4,
                        [&](std::vector<unsigned char> &bytes) {
                            std::vector<T> tab;
                            build_node_table_poly<T>(a.n_l, a.ls, tab);
                            bytes.assign((const unsigned char *)tab.data(),
                                         (const unsigned char *)(tab.data() + tab.size()));
                        },
                        &dnp)))
        return st;
    const PolyMom<T> mom = poly_moments<T>(a.n_l, a.ls);
    // the per-request background polynomials (independent of the launch
    // shape); on ctx->prep_stream when the caller gives one (its uploads of
    // the requests run there), so that they overlap earlier work on the stream
    {
        cudaStream_t fs = ctx->prep_stream ? ctx->prep_stream : ctx->stream;
        ChiTab<T> tab;
        tab.rec = (const typename V2T<T>::t *)(sizeof(T) == sizeof(double) ? ctx->chi_tab64.p
                                                                         : ctx->chi_tab32.p);
        tab.c0 = (T)ctx->chi_t0;
        tab.cn = (T)ctx->chi_tn;
        tab.inv_dc = (T)((CG_CHI_TAB - 1) / (ctx->chi_tn - ctx->chi_t0));
        // on the library's stream it may start while the preceding table kernel
        // finishes (programmatic dependent launch: that kernel signals once all
        // its blocks are resident, and this one waits for its completion before
        // it exits)
        cudaLaunchConfig_t lc = {};
        lc.gridDim = dim3((a.n_req + MP_FIT_WARPS - 1) / MP_FIT_WARPS);
        lc.blockDim = dim3(32 * MP_FIT_WARPS);
        lc.stream = fs;
        cudaLaunchAttribute la[1];
        la[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        la[0].val.programmaticStreamSerializationAllowed = 1;
        lc.attrs = la;
        lc.numAttrs = fs == ctx->stream ? 1 : 0;
        CG_CUDA(ctx, cudaLaunchKernelEx(&lc, mp_bgfit_kernel<T, S>, chi_of_z, tab, a.n_req, vinv,
                                        req_z_mean, req_offset, sep, d_fit, d_count));
        if ((st = cg_after_launch(ctx, "mp_bgfit_kernel"))) return st;
        if (ctx->prep_stream) {
            CG_CUDA(ctx, cudaEventRecord(ctx->copy_ev[1], fs));
            CG_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->copy_ev[1], 0));
        }
    }
    // the first launch after the fit finds the retry counter zeroed by it and,
    // when the fit ran on this stream, follows it as a programmatic dependent
    // launch (the polynomial kernel); later launches (the tuner's candidates)
    // clear the counter themselves
    bool after_fit = true;
    const bool dependent = !ctx->prep_stream && !ctx->timing;
    auto run = [&](const coffe_gpu_tuning_t &tu) -> int {
        const int lt = tu.lane_threads;
        const bool pack = can_pack && tu.lane_pack == 2 && !tu.lane_poly;
        const long long blocks = (total + (pack ? 2 : 1) * lt - 1) / ((pack ? 2 : 1) * lt);
        const bool first = after_fit;
        after_fit = false;
        if (!first) CG_CUDA(ctx, cudaMemsetAsync(d_count, 0, sizeof(int), ctx->stream));
#define MP_FAST_U(NLV, CV, UV)                                                                    \
    if (tu.lane_poly) {                                                                           \
        const size_t smem = sizeof(T) * PolyLayout<NLV>::COUNT + sizeof(double) * NLV * lt;       \
        CG_CUDA(ctx, cudaFuncSetAttribute(mp_poly_kernel<NLV, CV, UV, T>,                         \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,            \
                                          (int)smem));                                            \
        cudaLaunchConfig_t lc = {};                                                               \
        lc.gridDim = dim3((unsigned)blocks);                                                      \
        lc.blockDim = dim3(lt);                                                                   \
        lc.dynamicSmemBytes = smem;                                                               \
        lc.stream = ctx->stream;                                                                  \
        cudaLaunchAttribute la[1];                                                                \
        la[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;                            \
        la[0].val.programmaticStreamSerializationAllowed = 1;                                     \
        lc.attrs = la;                                                                            \
        lc.numAttrs = first && dependent ? 1 : 0;                                                 \
        CG_CUDA(ctx, cudaLaunchKernelEx(&lc, mp_poly_kernel<NLV, CV, UV, T>, a, d_fit,            \
                                        (T)bg.z_of_chi.x0, (T)bg.z_of_chi.xn, tab_x, tab_y,       \
                                        req_spectrum, req_z_mean, req_offset, sep, total,         \
                                        (const T *)dnp, mom, out, d_count, d_retry,               \
                                        ctx->d_err));                                             \
    } else if (pack) {                                                                            \
        const size_t smem = sizeof(float) * Fast2Layout<NLV>::COUNT +                             \
                            sizeof(f2) * Fast2Layout<NLV>::ROWS * lt;                             \
        CG_CUDA(ctx, cudaFuncSetAttribute(mp_fast2_kernel<NLV, CV, UV>,                           \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,            \
                                          (int)smem));                                            \
        mp_fast2_kernel<NLV, CV, UV><<<(unsigned)blocks, lt, smem, ctx->stream>>>(                \
            a, (const BgFitT<float> *)d_fit, (float)bg.z_of_chi.x0, (float)bg.z_of_chi.xn,        \
            (const float *)tab_x, (const float *)tab_y, req_spectrum, req_z_mean, req_offset,     \
            sep, total, (const float *)dn2, out, d_count, d_retry, ctx->d_err);                   \
    } else {                                                                                      \
        const size_t smem = sizeof(T) * (FastLayout<NLV>::COUNT + FastLayout<NLV>::ROWS * lt);    \
        CG_CUDA(ctx, cudaFuncSetAttribute(mp_fast_kernel<NLV, CV, UV, T>,                         \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,            \
                                          (int)smem));                                            \
        mp_fast_kernel<NLV, CV, UV, T><<<(unsigned)blocks, lt, smem, ctx->stream>>>(              \
            a, d_fit, bg.z_of_chi.x0, bg.z_of_chi.xn, tab_x, tab_y, req_spectrum, req_z_mean,     \
            req_offset, sep, total, (const T *)dn, out, d_count, d_retry, ctx->d_err);            \
    }
#define MP_FAST(NLV, CV)                                                                          \
    if (a.n_l == NLV && contrib == CV) {                                                          \
        if (tu.lane_unroll == 2)                                                                  \
            MP_FAST_U(NLV, CV, 2)                                                                 \
        else                                                                                      \
            MP_FAST_U(NLV, CV, 1)                                                                 \
    }
#define MP_FAST_NL(NLV) MP_FAST(NLV, 1) MP_FAST(NLV, 2) MP_FAST(NLV, 3)
        MP_FAST_NL(1)
        MP_FAST_NL(2)
        MP_FAST_NL(3)
        MP_FAST_NL(4)
#undef MP_FAST_NL
#undef MP_FAST
#undef MP_FAST_U
        int s2 = cg_after_launch(ctx, tu.lane_poly ? "mp_poly_kernel" : "mp_fast_kernel");
        if (s2) return s2;
        mp_retry_kernel<T, S, T><<<ctx->sm_count * 2, 32 * MP_RETRY_WARPS, 0, ctx->stream>>>(
            a, bg, chi_of_z, tab_x, tab_y, req_spectrum, req_z_mean, req_offset, sep, out,
            d_count, d_retry, ctx->d_err);
        return cg_after_launch(ctx, "mp_retry_kernel");
    };
    std::vector<coffe_gpu_tuning_t> cands;
    for (int po : {1, 0})
        for (int pk : {1, 2})
            for (int lt : {64, 128, 256})
                for (int un : {1, 2}) {
                    if (pk == 2 && (!can_pack || po)) continue;
                    coffe_gpu_tuning_t c = ctx->tuning;
                    c.lane_threads = lt;
                    c.lane_unroll = un;
                    c.lane_pack = pk;
                    c.lane_poly = po;
                    cands.push_back(c);
                }
    coffe_gpu_tuning_t tu;
    long long bucket = 0;
    while ((1ll << bucket) < total) ++bucket;
    const std::array<long long, 6> key{2, a.n_l, contrib, bucket, prec_tag, 0};
    if ((st = cg_tuned(ctx, key, cands, run, &tu))) return st;
    ctx->last_tuning.lane_threads = tu.lane_threads;
    ctx->last_tuning.lane_unroll = tu.lane_unroll;
    ctx->last_tuning.lane_pack = can_pack && !tu.lane_poly ? tu.lane_pack : 1;
    ctx->last_tuning.lane_poly = tu.lane_poly;
    return run(tu);
}

template <typename T, typename S, typename TT>
int launch(coffe_gpu_ctx *ctx, const MpArgs &a, const Bg<T, S> &bg, const S &chi_of_z,
           const TT *tab_x, const TT *tab_y, const int *req_spectrum, const double *req_z_mean,
           const int64_t *req_offset, const double *sep, long long total, double *out)
{
    int *d_count = (int *)ctx->mp_retry.p;
    int2 *d_retry = (int2 *)((char *)ctx->mp_retry.p + 256);
    CG_CUDA(ctx, cudaMemsetAsync(d_count, 0, sizeof(int), ctx->stream));
    // xi is even in mu when both tracers share one galaxy bias (or density is
    // off); then even multipoles need only the nodes with mu >= 0
    bool mirror = !(a.contrib & COFFE_GPU_DEN) || (!ctx->bias_set[0] && !ctx->bias_set[1]) ||
                  (ctx->bias_set[0] && ctx->bias_set[1] && ctx->bias_host[0] == ctx->bias_host[1]);
    for (int j = 0; j < a.n_l; ++j) mirror = mirror && (a.ls[j] % 2 == 0);
    // node table of these multipoles: one cached table per (l list,
    // precision, layout), built on first use
    const T *d_nodes = nullptr;
    {
        const void *dn = nullptr;
        int st0 = node_slot(ctx, a.n_l, a.ls, sizeof(T) == 8 ? COFFE_GPU_FP64 : COFFE_GPU_MIXED,
                            (int)mirror,
                            [&](std::vector<unsigned char> &bytes) {
                                std::vector<T> tab;
                                build_node_table<T>(a.n_l, a.ls, tab, mirror);
                                bytes.assign((const unsigned char *)tab.data(),
                                             (const unsigned char *)(tab.data() + tab.size()));
                            },
                            &dn);
        if (st0) return st0;
        d_nodes = (const T *)dn;
    }
    const long long blocks = (total + MP_LANE_THREADS - 1) / MP_LANE_THREADS;
#define MP_LAUNCH_MIR(NLV, MIR)                                                                  \
    {                                                                                            \
        const size_t smem = sizeof(T) * (NodeLayout<NLV, MIR>::COUNT +                           \
                                         NodeLayout<NLV, MIR>::ROWS * MP_LANE_THREADS);          \
        CG_CUDA(ctx, cudaFuncSetAttribute(mp_lane_kernel<NLV, T, S, TT, MIR>,                   \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,           \
                                          (int)smem));                                           \
        mp_lane_kernel<NLV, T, S, TT, MIR>                                                       \
            <<<(unsigned)blocks, MP_LANE_THREADS, smem, ctx->stream>>>(                          \
                a, bg, chi_of_z, tab_x, tab_y, req_spectrum, req_z_mean, req_offset, sep, total, \
                d_nodes, out, d_count, d_retry, ctx->d_err);                                     \
    }
#define MP_LAUNCH_NL(NLV)                                                                        \
    case NLV:                                                                                    \
        if (mirror)                                                                              \
            MP_LAUNCH_MIR(NLV, true)                                                             \
        else                                                                                     \
            MP_LAUNCH_MIR(NLV, false)                                                            \
        break;
    switch (a.n_l) {
        MP_LAUNCH_NL(1)
        MP_LAUNCH_NL(2)
        MP_LAUNCH_NL(3)
        MP_LAUNCH_NL(4)
        MP_LAUNCH_NL(5)
        MP_LAUNCH_NL(6)
        MP_LAUNCH_NL(7)
        MP_LAUNCH_NL(8)
    default:
        cg_set_error(ctx, "multipoles: unsupported number of multipoles %d", a.n_l);
        return COFFE_GPU_EINVAL;
    }
#undef MP_LAUNCH_NL
#undef MP_LAUNCH_MIR
    int st = cg_after_launch(ctx, "mp_lane_kernel");
    if (st) return st;
    mp_retry_kernel<T, S, TT><<<ctx->sm_count * 2, 32 * MP_RETRY_WARPS, 0, ctx->stream>>>(
        a, bg, chi_of_z, tab_x, tab_y, req_spectrum, req_z_mean, req_offset, sep, out, d_count,
        d_retry, ctx->d_err);
    return cg_after_launch(ctx, "mp_retry_kernel");
}

// (D1, f D1) at chi_j = c0 + j (cn - c0) / (CG_CHI_TAB - 1) from the FP64 splines
__global__ void chi_tab_kernel(Spl64 z_of_chi, Spl64 D1, Spl64 f, double c0, double cn,
                               double2 *__restrict__ t64, float2 *__restrict__ t32)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= CG_CHI_TAB) return;
    const double chi = j == CG_CHI_TAB - 1 ? cn : c0 + (cn - c0) * ((double)j / (CG_CHI_TAB - 1));
    const double z = spl_eval(z_of_chi, chi);
    const double g = spl_eval(D1, z), fg = spl_eval(f, z) * g;
    t64[j] = make_double2(g, fg);
    t32[j] = make_float2((float)g, (float)fg);
}

__global__ void zrec_kernel(const double4_32a *__restrict__ f64, const double4_32a *__restrict__ d64,
                            const float4 *__restrict__ f32, const float4 *__restrict__ d32, int n,
                            ZRec<double> *__restrict__ r64, ZRec<float> *__restrict__ r32)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    r64[i].f = f64[i];
    r64[i].d = d64[i];
    r32[i].f = f32[i];
    r32[i].d = d32[i];
}

} // namespace

// Fused f/D1 records when f and D1 share a uniform z grid (background_init's
// grid z_i = 15 i / (bins - 1)); called after the background splines exist.
int multipoles_prepare_background(coffe_gpu_ctx *ctx)
{
    const int n = ctx->bg_bins;
    ctx->z_uniform = false;
    {
        const Spl64 zc = ctx->bg[BG_Z_OF_CHI].v64();
        int st = cg_ensure(ctx, ctx->chi_tab64, sizeof(double2) * CG_CHI_TAB);
        if (st || (st = cg_ensure(ctx, ctx->chi_tab32, sizeof(float2) * CG_CHI_TAB))) return st;
        chi_tab_kernel<<<(CG_CHI_TAB + 255) / 256, 256, 0, ctx->stream>>>(
            zc, ctx->bg[BG_D1].v64(), ctx->bg[BG_F].v64(), zc.x0, zc.xn,
            (double2 *)ctx->chi_tab64.p, (float2 *)ctx->chi_tab32.p);
        if ((st = cg_after_launch(ctx, "chi_tab_kernel"))) return st;
        ctx->chi_t0 = zc.x0;
        ctx->chi_tn = zc.xn;
    }
    std::vector<double> z(n);
    CG_CUDA(ctx, cudaMemcpyAsync(z.data(), ctx->bg_nodes.p, sizeof(double) * n,
                                 cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const double dz = (z[n - 1] - z[0]) / (n - 1);
    bool uni = dz > 0;
    for (int i = 0; i < n && uni; ++i)
        if (fabs(z[i] - (z[0] + i * dz)) > 1e-12 * (fabs(z[i]) + dz)) uni = false;
    if (!uni) return COFFE_GPU_OK;
    int st = cg_ensure(ctx, ctx->zrec64, sizeof(ZRec<double>) * (n - 1));
    if (st) return st;
    if ((st = cg_ensure(ctx, ctx->zrec32, sizeof(ZRec<float>) * (n - 1)))) return st;
    zrec_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(
        ctx->bg[BG_F].c64, ctx->bg[BG_D1].c64, ctx->bg[BG_F].c32, ctx->bg[BG_D1].c32, n,
        (ZRec<double> *)ctx->zrec64.p, (ZRec<float> *)ctx->zrec32.p);
    if ((st = cg_after_launch(ctx, "zrec_kernel"))) return st;
    ctx->z_uniform = true;
    ctx->z0 = z[0];
    ctx->zn = z[n - 1];
    ctx->dz = dz;
    return COFFE_GPU_OK;
}

static int multipoles_nonintegrated(coffe_gpu_ctx *ctx, const MpArgs &a, int precision,
                                    const int *req_spectrum, const double *req_z_mean,
                                    const int64_t *req_offset, const double *sep, double *out,
                                    long long total);

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
    if (precision != ctx->int_precision &&
        !(precision == COFFE_GPU_FP64_FASTALG && ctx->int_precision == COFFE_GPU_FP64)) {
        cg_set_error(ctx, "multipoles: precision %d differs from the integrals' (%d)", precision,
                     ctx->int_precision);
        return COFFE_GPU_EINVAL;
    }
    if (!(contrib & 7) || (contrib & ~15)) {
        cg_set_error(ctx, "multipoles: contrib must select den, rsd and/or len (+ only-cross)");
        return COFFE_GPU_EINVAL;
    }
    if (!(epsrel > 0)) {
        cg_set_error(ctx, "multipoles: epsrel must be positive");
        return COFFE_GPU_EINVAL;
    }
    if (total > (long long)INT32_MAX) {
        cg_set_error(ctx, "multipoles: at most 2^31-1 separations per call");
        return COFFE_GPU_EINVAL;
    }
    MpArgs a;
    a.n_req = n_req;
    a.n_l = n_l;
    a.contrib = contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD | COFFE_GPU_ONLY_CROSS);
    a.out_staged = ctx->out_host;
    a.t00 = cg_find_term(ctx, 0, 0);
    a.t02 = cg_find_term(ctx, 0, 2);
    a.t04 = cg_find_term(ctx, 0, 4);
    if (a.t00 < 0 || a.t02 < 0 || a.t04 < 0) {
        cg_set_error(ctx, "multipoles: integrals (0,0), (0,2), (0,4) are required");
        return COFFE_GPU_ESTATE;
    }
    a.n_terms = ctx->n_terms;
    a.tab_len = (int)(ctx->N + CG_N_SMALL_R + 1);
    a.inv_dlog = (double)ctx->N / log(ctx->kmax / ctx->kmin);
    a.epsrel = epsrel;
    for (int i = 0; i < MP_MAX_L; ++i) a.ls[i] = 0;
    for (int i = 0; i < n_l; ++i) {
        if (l[i] < 0 || l[i] > MP_MAX_LDEG) {
            cg_set_error(ctx, "multipoles: l = %d out of range [0, %d]", l[i], MP_MAX_LDEG);
            return COFFE_GPU_EINVAL;
        }
        a.ls[i] = l[i];
    }
    if (total <= 0) return COFFE_GPU_OK;
    int st;
    if (ctx->sm_count <= 0)
        CG_CUDA(ctx, cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount,
                                            ctx->device));
    cg_timing_begin(ctx);
    if (!(contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD))) {
        // lensing only: no nonintegrated terms (signal.c:472-520 returns 0)
        CG_CUDA(ctx, cudaMemsetAsync(out, 0, sizeof(double) * (size_t)total * n_l, ctx->stream));
        return lensing_run(ctx, contrib, precision, epsrel, n_req, req_spectrum, req_z_mean,
                           req_offset, sep, n_l, l, out, total);
    }
    a.retry_cap = total * n_l;
    if ((st = cg_ensure(ctx, ctx->mp_retry, 256 + sizeof(int2) * (size_t)a.retry_cap))) return st;
    if ((st = multipoles_nonintegrated(ctx, a, precision, req_spectrum, req_z_mean, req_offset,
                                       sep, out, total)))
        return st;
    return lensing_run(ctx, contrib, precision, epsrel, n_req, req_spectrum, req_z_mean,
                       req_offset, sep, n_l, l, out, total);
}

// the den/rsd nonintegrated multipoles of a validated call
static int multipoles_nonintegrated(coffe_gpu_ctx *ctx, const MpArgs &a, int precision,
                                    const int *req_spectrum, const double *req_z_mean,
                                    const int64_t *req_offset, const double *sep, double *out,
                                    long long total)
{
    if (precision == COFFE_GPU_MIXED) {
        Bg<float, Spl32> bg;
        bg.z_of_chi = ctx->bg[BG_Z_OF_CHI].v32();
        bg.f = ctx->bg[BG_F].v32();
        bg.D1 = ctx->bg[BG_D1].v32();
        bg.b1 = ctx->bias[0].v32();
        bg.b2 = ctx->bias[1].v32();
        bg.has_b1 = ctx->bias_set[0];
        bg.has_b2 = ctx->bias_set[1];
        bg.zrec = ctx->z_uniform ? (const ZRec<float> *)ctx->zrec32.p : nullptr;
        bg.z0 = (float)ctx->z0;
        bg.zn = (float)ctx->zn;
        bg.dz = (float)ctx->dz;
        bg.inv_dz = (float)(1.0 / ctx->dz);
        bg.nz = ctx->bg_bins;
        bool fast = a.n_l <= 4 && !ctx->bias_set[0] && !ctx->bias_set[1] &&
                    !(a.contrib & COFFE_GPU_ONLY_CROSS);
        for (int j = 0; j < a.n_l; ++j) fast = fast && a.ls[j] % 2 == 0;
        if (fast)
            return launch_fast<float, Spl32>(ctx, a, bg, ctx->bg[BG_CHI_OF_Z].v32(),
                                             (const float *)ctx->tab_x32.p,
                                             (const float *)ctx->tab_y.p, req_spectrum,
                                             req_z_mean, req_offset, sep, total, out);
        return launch<float, Spl32, float>(ctx, a, bg, ctx->bg[BG_CHI_OF_Z].v32(),
                                           (const float *)ctx->tab_x32.p,
                                           (const float *)ctx->tab_y.p, req_spectrum, req_z_mean,
                                           req_offset, sep, total, out);
    }
    Bg<double, Spl64> bg;
    bg.z_of_chi = ctx->bg[BG_Z_OF_CHI].v64();
    bg.f = ctx->bg[BG_F].v64();
    bg.D1 = ctx->bg[BG_D1].v64();
    bg.b1 = ctx->bias[0].v64();
    bg.b2 = ctx->bias[1].v64();
    bg.has_b1 = ctx->bias_set[0];
    bg.has_b2 = ctx->bias_set[1];
    bg.zrec = ctx->z_uniform ? (const ZRec<double> *)ctx->zrec64.p : nullptr;
    bg.z0 = ctx->z0;
    bg.zn = ctx->zn;
    bg.dz = ctx->dz;
    bg.inv_dz = 1.0 / ctx->dz;
    bg.nz = ctx->bg_bins;
    if (precision == COFFE_GPU_FP64_FASTALG) {
        bool fast = a.n_l <= 4 && !ctx->bias_set[0] && !ctx->bias_set[1] &&
                    !(a.contrib & COFFE_GPU_ONLY_CROSS);
        for (int j = 0; j < a.n_l; ++j) fast = fast && a.ls[j] % 2 == 0;
        if (fast)
            return launch_fast<double, Spl64>(ctx, a, bg, ctx->bg[BG_CHI_OF_Z].v64(),
                                              (const double *)ctx->tab_x.p,
                                              (const double *)ctx->tab_y.p, req_spectrum,
                                              req_z_mean, req_offset, sep, total, out);
    }
    return launch<double, Spl64, double>(ctx, a, bg, ctx->bg[BG_CHI_OF_Z].v64(),
                                         (const double *)ctx->tab_x.p,
                                         (const double *)ctx->tab_y.p, req_spectrum, req_z_mean,
                                         req_offset, sep, total, out);
}

// Redshift-averaged multipoles of a call to coffe_gpu_average_multipoles (all
// arrays on the device except l): the multipoles at the n_z redshift nodes of
// every (window, separation) by multipoles_run, then their weighted sums.
int average_multipoles_run(coffe_gpu_ctx *ctx, int contrib, int precision, double epsrel,
                           int n_win, const int *win_spectrum, const double *z_min,
                           const double *z_max, const int64_t *win_offset, const double *sep,
                           int n_l, const int *l, int n_z, double *out, long long total)
{
    if (!ctx->bg_ready) {
        cg_set_error(ctx, "average_multipoles: background not initialised");
        return COFFE_GPU_ESTATE;
    }
    if (n_z < 1 || n_z > 256 || n_l < 1 || n_l > MP_MAX_L || n_win < 1) {
        cg_set_error(ctx, "average_multipoles: need 1 <= n_z <= 256, 1 <= n_l <= %d, n_win >= 1",
                     MP_MAX_L);
        return COFFE_GPU_EINVAL;
    }
    if (total <= 0) return COFFE_GPU_OK;
    const long long E = total * n_z;
    if (E > (long long)INT32_MAX) {
        cg_set_error(ctx, "average_multipoles: too many (separation, redshift node) entries");
        return COFFE_GPU_EINVAL;
    }
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t b_gl = sizeof(double) * 2 * n_z, b_spec = sizeof(int) * E,
                 b_z = sizeof(double) * E, b_off = sizeof(int64_t) * (E + 1),
                 b_sep = sizeof(double) * E, b_w = sizeof(double) * E,
                 b_out = sizeof(double) * E * n_l;
    int st = cg_ensure(ctx, ctx->avg_buf, al(b_gl) + al(b_spec) + al(b_z) + al(b_off) +
                                              al(b_sep) + al(b_w) + al(b_out));
    if (st) return st;
    char *p = (char *)ctx->avg_buf.p;
    double *d_gl = (double *)p;
    p += al(b_gl);
    int *e_spec = (int *)p;
    p += al(b_spec);
    double *e_z = (double *)p;
    p += al(b_z);
    int64_t *e_off = (int64_t *)p;
    p += al(b_off);
    double *e_sep = (double *)p;
    p += al(b_sep);
    double *e_w = (double *)p;
    p += al(b_w);
    double *e_out = (double *)p;
    std::vector<double> gl(2 * (size_t)n_z);
    gauss_legendre_nodes(n_z, gl.data(), gl.data() + n_z);
    CG_CUDA(ctx, cudaMemcpyAsync(d_gl, gl.data(), b_gl, cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream)); // gl is a host temporary
    avg_expand_kernel<<<(unsigned)((E + 255) / 256), 256, 0, ctx->stream>>>(
        ctx->bg[BG_CHI_OF_Z].v64(), ctx->bg[BG_Z_OF_CHI].v64(), ctx->bg[BG_CONFH].v64(),
        CG_H0 * ctx->h, win_spectrum, z_min, z_max, win_offset, n_win, sep, total, d_gl, n_z,
        e_spec, e_z, e_off, e_sep, e_w);
    if ((st = cg_after_launch(ctx, "avg_expand_kernel"))) return st;
    if ((st = multipoles_run(ctx, contrib, precision, epsrel, (int)E, e_spec, e_z, e_off, e_sep,
                             n_l, l, e_out, E)))
        return st;
    avg_reduce_kernel<<<(unsigned)((total * n_l + 255) / 256), 256, 0, ctx->stream>>>(
        e_w, e_out, total, n_z, n_l, out, ctx->d_err);
    return cg_after_launch(ctx, "avg_reduce_kernel");
}

// The correlation function of a call to coffe_gpu_corrfunc (all arrays on the
// device except mu_host, the same n_mu values as mu): the nonintegrated
// den/rsd terms, then the lensing terms added by corrfunc_lensing_run.
int corrfunc_run(coffe_gpu_ctx *ctx, int contrib, int precision, int n_req,
                 const int *req_spectrum, const double *req_z_mean, const int64_t *req_offset,
                 const double *sep, int n_mu, const double *mu, const double *mu_host,
                 double *out, long long total)
{
    if (!ctx->bg_ready || !ctx->int_ready) {
        cg_set_error(ctx, "corrfunc: %s not initialised", ctx->bg_ready ? "integrals" : "background");
        return COFFE_GPU_ESTATE;
    }
    if (precision != ctx->int_precision) {
        cg_set_error(ctx, "corrfunc: precision %d differs from the integrals' (%d)", precision,
                     ctx->int_precision);
        return COFFE_GPU_EINVAL;
    }
    if (!(contrib & 7) || (contrib & ~15)) {
        cg_set_error(ctx, "corrfunc: contrib must select den, rsd and/or len (+ only-cross)");
        return COFFE_GPU_EINVAL;
    }
    if (n_req < 1 || n_mu < 1 || n_mu > 1024) {
        cg_set_error(ctx, "corrfunc: need n_req >= 1 and 1 <= n_mu <= 1024");
        return COFFE_GPU_EINVAL;
    }
    for (int m = 0; m < n_mu; ++m)
        if (!(mu_host[m] >= -1.0 && mu_host[m] <= 1.0)) {
            cg_set_error(ctx, "corrfunc: mu must lie in [-1, 1]");
            return COFFE_GPU_EINVAL;
        }
    if (total * n_mu > (long long)INT32_MAX * 32) {
        cg_set_error(ctx, "corrfunc: too many (separation, mu) outputs in one call");
        return COFFE_GPU_EINVAL;
    }
    if (total <= 0) return COFFE_GPU_OK;
    int st;
    if (contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD)) {
        MpArgs a;
        a.n_req = n_req;
        a.n_l = 1;
        a.contrib = contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD | COFFE_GPU_ONLY_CROSS);
        a.t00 = cg_find_term(ctx, 0, 0);
        a.t02 = cg_find_term(ctx, 0, 2);
        a.t04 = cg_find_term(ctx, 0, 4);
        if (a.t00 < 0 || a.t02 < 0 || a.t04 < 0) {
            cg_set_error(ctx, "corrfunc: integrals (0,0), (0,2), (0,4) are required");
            return COFFE_GPU_ESTATE;
        }
        a.n_terms = ctx->n_terms;
        a.tab_len = (int)(ctx->N + CG_N_SMALL_R + 1);
        a.inv_dlog = (double)ctx->N / log(ctx->kmax / ctx->kmin);
        a.epsrel = 1e-5;
        a.retry_cap = 0;
        for (int i = 0; i < MP_MAX_L; ++i) a.ls[i] = 0;
        const long long n_out = total * n_mu;
        const unsigned blocks = (unsigned)((n_out + 255) / 256);
        if (precision == COFFE_GPU_MIXED) {
            Bg<float, Spl32> bg;
            bg.z_of_chi = ctx->bg[BG_Z_OF_CHI].v32();
            bg.f = ctx->bg[BG_F].v32();
            bg.D1 = ctx->bg[BG_D1].v32();
            bg.b1 = ctx->bias[0].v32();
            bg.b2 = ctx->bias[1].v32();
            bg.has_b1 = ctx->bias_set[0];
            bg.has_b2 = ctx->bias_set[1];
            bg.zrec = ctx->z_uniform ? (const ZRec<float> *)ctx->zrec32.p : nullptr;
            bg.z0 = (float)ctx->z0;
            bg.zn = (float)ctx->zn;
            bg.dz = (float)ctx->dz;
            bg.inv_dz = (float)(1.0 / ctx->dz);
            bg.nz = ctx->bg_bins;
            cf_nonint_kernel<float, Spl32, float><<<blocks, 256, 0, ctx->stream>>>(
                a, bg, ctx->bg[BG_CHI_OF_Z].v32(), (const float *)ctx->tab_x32.p,
                (const float *)ctx->tab_y.p, req_spectrum, req_z_mean, req_offset, sep, mu, n_mu,
                total, out, ctx->d_err);
        } else {
            Bg<double, Spl64> bg;
            bg.z_of_chi = ctx->bg[BG_Z_OF_CHI].v64();
            bg.f = ctx->bg[BG_F].v64();
            bg.D1 = ctx->bg[BG_D1].v64();
            bg.b1 = ctx->bias[0].v64();
            bg.b2 = ctx->bias[1].v64();
            bg.has_b1 = ctx->bias_set[0];
            bg.has_b2 = ctx->bias_set[1];
            bg.zrec = ctx->z_uniform ? (const ZRec<double> *)ctx->zrec64.p : nullptr;
            bg.z0 = ctx->z0;
            bg.zn = ctx->zn;
            bg.dz = ctx->dz;
            bg.inv_dz = 1.0 / ctx->dz;
            bg.nz = ctx->bg_bins;
            cf_nonint_kernel<double, Spl64, double><<<blocks, 256, 0, ctx->stream>>>(
                a, bg, ctx->bg[BG_CHI_OF_Z].v64(), (const double *)ctx->tab_x.p,
                (const double *)ctx->tab_y.p, req_spectrum, req_z_mean, req_offset, sep, mu, n_mu,
                total, out, ctx->d_err);
        }
        if ((st = cg_after_launch(ctx, "cf_nonint_kernel"))) return st;
    } else {
        CG_CUDA(ctx, cudaMemsetAsync(out, 0, sizeof(double) * (size_t)(total * n_mu), ctx->stream));
    }
    if (!(contrib & COFFE_GPU_LEN)) return COFFE_GPU_OK;
    return corrfunc_lensing_run(ctx, contrib, precision, n_req, req_spectrum, req_z_mean,
                                req_offset, sep, n_mu, mu_host, out, total);
}

// ============================================================================
// coffe_gpu_multipoles_noalloc: the multipole kernels above with every byte of
// their scratch taken from one fixed array in the library's device memory.
//
// Some callers cannot let the library allocate while they run: a process that
// hands all device memory to a pool at start-up (PyTorch's caching allocator, a
// service reserving its HBM) could see a growing buffer fail mid-run, and
// cudaMalloc/cudaFree synchronise the whole device, stalling every other
// stream.  multipoles_run grows its retry list and node table on demand; this
// variant never calls cudaMalloc, cudaFree or any allocating routine.
//
// Scratch layout (noalloc_scratch, 256-byte aligned):
//   [0, 256)                    retry counter (int) -- must start at zero, so
//                               every call clears it on its stream first;
//   [256, 256 + 20480)          first-panel node table, rewritten every call
//                               by mp_node_table_kernel;
//   [20736, + 8 * max outputs)  retry list, one int2 per (separation, l).
// One array serves every call on a device, so calls whose work overlaps in
// time race on it; callers serialise them (one stream does).
// ============================================================================
namespace {

#define MP_NOALLOC_NODE_BYTES 20480
#define MP_NOALLOC_LIST_OFFSET (256 + MP_NOALLOC_NODE_BYTES)
#define MP_NOALLOC_BYTES \
    (MP_NOALLOC_LIST_OFFSET + sizeof(int2) * (size_t)COFFE_GPU_NOALLOC_MAX_OUTPUTS)
static_assert(sizeof(double) * NodeLayout<MP_MAX_L>::COUNT <= MP_NOALLOC_NODE_BYTES,
              "node table of the largest multipole list must fit the scratch slot");
static_assert(MP_NOALLOC_LIST_OFFSET % 256 == 0, "retry list alignment");

static __device__ __align__(256) unsigned char noalloc_scratch[MP_NOALLOC_BYTES];

// Device address of noalloc_scratch in the current context.  Looked up on
// every call rather than cached, so a call after cudaDeviceReset or under
// another context never reuses a stale address; once the module is loaded
// (noalloc_prepare) the lookup allocates nothing.
int noalloc_scratch_address(coffe_gpu_ctx *ctx, unsigned char **addr)
{
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, noalloc_scratch);
    if (e != cudaSuccess || !p) {
        cg_set_error(ctx, "multipoles_noalloc: cannot resolve the scratch array on device %d: %s",
                     ctx->device, cudaGetErrorString(e));
        return COFFE_GPU_ECUDA;
    }
    *addr = (unsigned char *)p;
    return COFFE_GPU_OK;
}

// P_l(x) by the upward recurrence, as host_legendre forms it
__device__ double node_legendre(int l, double x)
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

// The node table of build_node_table (layout NodeLayout<a.n_l>), computed on
// the device so that no host staging buffer is needed: thread sl owns slot sl,
// finds its rank in ascending mu and writes its pass-1 and pass-2 records.
template <typename T> __global__ void __launch_bounds__(64) mp_node_table_kernel(MpArgs a, T *out)
{
    __shared__ double mus[64];
    const int sl = threadIdx.x;
    double mu = 0.0, wk = 0.0, wg = 0.0;
    if (sl < 60) { // slots 2p, 2p+1: x = 0.5 -+ 0.5 xgk[g_p]
        const int p = sl >> 1;
        const int g = p < 15 ? 2 * p + 1 : 2 * (p - 15);
        const double absc = 0.5 * cg_gk_xgk[g];
        mu = (sl & 1) ? 2.0 * (0.5 + absc) - 1.0 : 2.0 * (0.5 - absc) - 1.0;
        wk = cg_gk_wgk[g];
        wg = p < 15 ? cg_gk_wg[p] : 0.0;
    } else if (sl == 60) { // centre
        wk = cg_gk_wgk[30];
    }
    mus[sl] = sl < 61 ? mu : 2.0;
    __syncthreads();
    if (sl >= 61) return;
    int rank = 0;
    for (int i = 0; i < 61; ++i) rank += (mus[i] < mu) || (mus[i] == mu && i < sl);
    const int NL = a.n_l;
    const int R1 = ((2 + 3 * NL) + 3) / 4 * 4, R2 = ((1 + NL) + 3) / 4 * 4;
    T *r1 = out + (size_t)rank * R1;
    T *r2 = out + (size_t)61 * R1 + (size_t)sl * R2;
    for (int i = 0; i < R1; ++i) r1[i] = T(0);
    for (int i = 0; i < R2; ++i) r2[i] = T(0);
    r1[0] = (T)mu;
    r1[1] = (T)sl;
    r2[0] = (T)wk;
    for (int j = 0; j < NL; ++j) {
        const double P = node_legendre(a.ls[j], mu);
        r1[2 + j] = (T)(wk * P);
        r1[2 + NL + j] = (T)(wg * P);
        r1[2 + 2 * NL + j] = (T)(wk * fabs(P));
        r2[1 + j] = (T)P;
    }
}

// Background views of the context for the multipole kernels.
template <typename T, typename S> Bg<T, S> noalloc_bg(const coffe_gpu_ctx *ctx);
template <> Bg<float, Spl32> noalloc_bg<float, Spl32>(const coffe_gpu_ctx *ctx)
{
    Bg<float, Spl32> bg;
    bg.z_of_chi = ctx->bg[BG_Z_OF_CHI].v32();
    bg.f = ctx->bg[BG_F].v32();
    bg.D1 = ctx->bg[BG_D1].v32();
    bg.b1 = ctx->bias[0].v32();
    bg.b2 = ctx->bias[1].v32();
    bg.has_b1 = ctx->bias_set[0];
    bg.has_b2 = ctx->bias_set[1];
    bg.zrec = ctx->z_uniform ? (const ZRec<float> *)ctx->zrec32.p : nullptr;
    bg.z0 = (float)ctx->z0;
    bg.zn = (float)ctx->zn;
    bg.dz = (float)ctx->dz;
    bg.inv_dz = (float)(1.0 / ctx->dz);
    bg.nz = ctx->bg_bins;
    return bg;
}
template <> Bg<double, Spl64> noalloc_bg<double, Spl64>(const coffe_gpu_ctx *ctx)
{
    Bg<double, Spl64> bg;
    bg.z_of_chi = ctx->bg[BG_Z_OF_CHI].v64();
    bg.f = ctx->bg[BG_F].v64();
    bg.D1 = ctx->bg[BG_D1].v64();
    bg.b1 = ctx->bias[0].v64();
    bg.b2 = ctx->bias[1].v64();
    bg.has_b1 = ctx->bias_set[0];
    bg.has_b2 = ctx->bias_set[1];
    bg.zrec = ctx->z_uniform ? (const ZRec<double> *)ctx->zrec64.p : nullptr;
    bg.z0 = ctx->z0;
    bg.zn = ctx->zn;
    bg.dz = ctx->dz;
    bg.inv_dz = 1.0 / ctx->dz;
    bg.nz = ctx->bg_bins;
    return bg;
}

// The launches of `launch` with the counter, node table and retry list in the
// fixed scratch.
template <typename T, typename S, typename TT>
int launch_noalloc(coffe_gpu_ctx *ctx, const MpArgs &a, const S &chi_of_z, const TT *tab_x,
                   const TT *tab_y, const int *req_spectrum, const double *req_z_mean,
                   const int64_t *req_offset, const double *sep, long long total, double *out,
                   unsigned char *scratch)
{
    const Bg<T, S> bg = noalloc_bg<T, S>(ctx);
    int *d_count = (int *)scratch;
    T *d_nodes = (T *)(scratch + 256);
    int2 *d_retry = (int2 *)(scratch + MP_NOALLOC_LIST_OFFSET);
    CG_CUDA(ctx, cudaMemsetAsync(d_count, 0, sizeof(int), ctx->stream));
    mp_node_table_kernel<T><<<1, 64, 0, ctx->stream>>>(a, d_nodes);
    int st = cg_after_launch(ctx, "mp_node_table_kernel");
    if (st) return st;
    const long long blocks = (total + MP_LANE_THREADS - 1) / MP_LANE_THREADS;
#define MP_NOALLOC_NL(NLV)                                                                       \
    case NLV: {                                                                                  \
        const size_t smem = sizeof(T) * (NodeLayout<NLV>::COUNT + 61 * MP_LANE_THREADS);         \
        CG_CUDA(ctx, cudaFuncSetAttribute(mp_lane_kernel<NLV, T, S, TT>,                        \
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,           \
                                          (int)smem));                                           \
        mp_lane_kernel<NLV, T, S, TT><<<(unsigned)blocks, MP_LANE_THREADS, smem, ctx->stream>>>( \
            a, bg, chi_of_z, tab_x, tab_y, req_spectrum, req_z_mean, req_offset, sep, total,    \
            d_nodes, out, d_count, d_retry, ctx->d_err);                                         \
        break;                                                                                   \
    }
    switch (a.n_l) {
        MP_NOALLOC_NL(1)
        MP_NOALLOC_NL(2)
        MP_NOALLOC_NL(3)
        MP_NOALLOC_NL(4)
        MP_NOALLOC_NL(5)
        MP_NOALLOC_NL(6)
        MP_NOALLOC_NL(7)
        MP_NOALLOC_NL(8)
    default:
        cg_set_error(ctx, "multipoles_noalloc: unsupported number of multipoles %d", a.n_l);
        return COFFE_GPU_EINVAL;
    }
#undef MP_NOALLOC_NL
    if ((st = cg_after_launch(ctx, "mp_lane_kernel"))) return st;
    mp_retry_kernel<T, S, TT><<<ctx->sm_count * 2, 32 * MP_RETRY_WARPS, 0, ctx->stream>>>(
        a, bg, chi_of_z, tab_x, tab_y, req_spectrum, req_z_mean, req_offset, sep, out, d_count,
        d_retry, ctx->d_err);
    return cg_after_launch(ctx, "mp_retry_kernel");
}

// Loads every kernel launch_noalloc<T, S, TT> launches (lazy loading would
// otherwise load them, allocating their code, at the first call).
template <typename T, typename S, typename TT> int noalloc_load_kernels(coffe_gpu_ctx *ctx)
{
    cudaFuncAttributes fa;
    CG_CUDA(ctx, cudaFuncGetAttributes(&fa, mp_node_table_kernel<T>));
    CG_CUDA(ctx, cudaFuncGetAttributes(&fa, mp_lane_kernel<1, T, S, TT>));
    CG_CUDA(ctx, cudaFuncGetAttributes(&fa, mp_lane_kernel<2, T, S, TT>));
    CG_CUDA(ctx, cudaFuncGetAttributes(&fa, mp_lane_kernel<3, T, S, TT>));
    CG_CUDA(ctx, cudaFuncGetAttributes(&fa, mp_lane_kernel<4, T, S, TT>));
    CG_CUDA(ctx, cudaFuncGetAttributes(&fa, mp_lane_kernel<5, T, S, TT>));
    CG_CUDA(ctx, cudaFuncGetAttributes(&fa, mp_lane_kernel<6, T, S, TT>));
    CG_CUDA(ctx, cudaFuncGetAttributes(&fa, mp_lane_kernel<7, T, S, TT>));
    CG_CUDA(ctx, cudaFuncGetAttributes(&fa, mp_lane_kernel<8, T, S, TT>));
    CG_CUDA(ctx, cudaFuncGetAttributes(&fa, mp_retry_kernel<T, S, TT>));
    return COFFE_GPU_OK;
}

} // namespace

// Called by coffe_gpu_ctx_create with ctx->device current: loads this file's
// module (which places noalloc_scratch in device memory) and the kernels of
// coffe_gpu_multipoles_noalloc, so that the entry point itself never triggers
// an allocation.
int multipoles_noalloc_prepare(coffe_gpu_ctx *ctx)
{
    unsigned char *p = nullptr;
    int st = noalloc_scratch_address(ctx, &p);
    if (st) return st;
    if ((st = noalloc_load_kernels<float, Spl32, float>(ctx))) return st;
    return noalloc_load_kernels<double, Spl64, double>(ctx);
}

extern "C" int coffe_gpu_multipoles_noalloc(coffe_gpu_ctx_t *ctx, int contrib, int precision,
                                            double epsrel, int n_req, int64_t n_sep,
                                            const int *req_spectrum, const double *req_z_mean,
                                            const int64_t *req_offset, const double *sep, int n_l,
                                            const int *l, double *out)
{
    if (!ctx || !req_spectrum || !req_z_mean || !req_offset || !l || n_req < 1 || n_sep < 0 ||
        (n_sep > 0 && (!sep || !out)))
        return COFFE_GPU_EINVAL;
    if (!ctx->bg_ready || !ctx->int_ready) {
        cg_set_error(ctx, "multipoles_noalloc: %s not initialised",
                     ctx->bg_ready ? "integrals" : "background");
        return COFFE_GPU_ESTATE;
    }
    if (n_l < 1 || n_l > MP_MAX_L) {
        cg_set_error(ctx, "multipoles_noalloc: need 1 <= n_l <= %d", MP_MAX_L);
        return COFFE_GPU_EINVAL;
    }
    if ((long long)n_sep * n_l > (long long)COFFE_GPU_NOALLOC_MAX_OUTPUTS) {
        cg_set_error(ctx,
                     "multipoles_noalloc: %lld separations x %d multipoles = %lld outputs exceed "
                     "the fixed scratch limit of %d outputs per call; split the requests",
                     (long long)n_sep, n_l, (long long)n_sep * n_l, COFFE_GPU_NOALLOC_MAX_OUTPUTS);
        return COFFE_GPU_EINVAL;
    }
    if (precision != ctx->int_precision) {
        cg_set_error(ctx, "multipoles_noalloc: precision %d differs from the integrals' (%d)",
                     precision, ctx->int_precision);
        return COFFE_GPU_EINVAL;
    }
    if (!(contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD)) || (contrib & ~3)) {
        cg_set_error(ctx, "multipoles_noalloc: contrib must select den and/or rsd (the lensing "
                          "terms need per-call buffers)");
        return COFFE_GPU_EINVAL;
    }
    if (!(epsrel > 0)) {
        cg_set_error(ctx, "multipoles_noalloc: epsrel must be positive");
        return COFFE_GPU_EINVAL;
    }
    MpArgs a;
    a.n_req = n_req;
    a.n_l = n_l;
    a.contrib = contrib & (COFFE_GPU_DEN | COFFE_GPU_RSD);
    a.t00 = cg_find_term(ctx, 0, 0);
    a.t02 = cg_find_term(ctx, 0, 2);
    a.t04 = cg_find_term(ctx, 0, 4);
    if (a.t00 < 0 || a.t02 < 0 || a.t04 < 0) {
        cg_set_error(ctx, "multipoles_noalloc: integrals (0,0), (0,2), (0,4) are required");
        return COFFE_GPU_ESTATE;
    }
    a.n_terms = ctx->n_terms;
    a.tab_len = (int)(ctx->N + CG_N_SMALL_R + 1);
    a.inv_dlog = (double)ctx->N / log(ctx->kmax / ctx->kmin);
    a.epsrel = epsrel;
    for (int i = 0; i < MP_MAX_L; ++i) a.ls[i] = 0;
    for (int i = 0; i < n_l; ++i) {
        if (l[i] < 0 || l[i] > MP_MAX_LDEG) {
            cg_set_error(ctx, "multipoles_noalloc: l = %d out of range [0, %d]", l[i], MP_MAX_LDEG);
            return COFFE_GPU_EINVAL;
        }
        a.ls[i] = l[i];
    }
    a.retry_cap = (long long)n_sep * n_l;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    unsigned char *scratch = nullptr;
    int st = noalloc_scratch_address(ctx, &scratch);
    if (st) return st;
    if (n_sep == 0) return COFFE_GPU_OK;
    if (ctx->sm_count <= 0)
        CG_CUDA(ctx, cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount,
                                            ctx->device));
    if (precision == COFFE_GPU_MIXED)
        return launch_noalloc<float, Spl32, float>(
            ctx, a, ctx->bg[BG_CHI_OF_Z].v32(), (const float *)ctx->tab_x32.p,
            (const float *)ctx->tab_y.p, req_spectrum, req_z_mean, req_offset, sep, n_sep, out,
            scratch);
    return launch_noalloc<double, Spl64, double>(
        ctx, a, ctx->bg[BG_CHI_OF_Z].v64(), (const double *)ctx->tab_x.p,
        (const double *)ctx->tab_y.p, req_spectrum, req_z_mean, req_offset, sep, n_sep, out,
        scratch);
}
