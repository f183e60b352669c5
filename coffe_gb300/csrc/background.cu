// Background of a flat LCDM cosmology on the device (replaces
// coffe_background_init, background.c:301-696, for w0 = -1, wa = 0).
//
// Node i sits at z_i = 15 i / (bins - 1).  chi(z_i) is the GK61 QAG integral of
// 1/E(z) (background.c:485-502) computed by one warp per node; D1 and f come
// from the growth ODE (background.c:196-211, 430-481) from a = 0.05,
// (D, D') = (0.05, 1): one trajectory of 950 classical RK4 steps of 1e-3 in a
// up to a = 1, integrated on the host (a sequential recurrence of ~10^4
// operations), then read at every node by cubic Hermite interpolation between
// the two steps around a_i, with the ODE's own derivatives (error ~h^4/384 of
// the fourth derivative, far below the RK4 error).  The reference integrates
// every node separately with GSL's adaptive rk2; both agree with it to its
// tolerance.  The ODE's x(z) = Om/(1-Om) (1+z)^3 is read through the same
// linear interpolation on 16385 points in [0, 100] as the reference's xint
// spline (background.c:337-412).
#include <vector>

#include "ctx.cuh"
#include "qag.cuh"

namespace {

#define BG_XINT_BINS 16384
#define BG_XINT_ZMAX 100.0

struct BgPar {
    double om, og, ode, h;
};

#define BG_ODE_A0 0.05
#define BG_ODE_STEPS 950 // (1 - 0.05) / 1e-3

// x(z) through the linear interpolation of the reference's xint spline
double xint_lin(const BgPar &p, double z)
{
    const double dz = BG_XINT_ZMAX / BG_XINT_BINS;
    const double ratio = p.om / (1.0 - p.om);
    const double u = z / dz;
    long i = (long)u;
    if (i >= BG_XINT_BINS) i = BG_XINT_BINS - 1;
    const double z0 = BG_XINT_ZMAX * (double)i / BG_XINT_BINS;
    const double z1 = BG_XINT_ZMAX * (double)(i + 1) / BG_XINT_BINS;
    const double x0 = ratio * (1 + z0) * (1 + z0) * (1 + z0);
    const double x1 = ratio * (1 + z1) * (1 + z1) * (1 + z1);
    return x0 + (z - z0) * ((x1 - x0) / (z1 - z0));
}

void growth_rhs(const BgPar &p, double a, double y0, double y1, double &f0, double &f1)
{
    const double z = 1. / a - 1;
    const double w = -1.0;
    const double x = xint_lin(p, z);
    f0 = y1;
    f1 = -3. / 2 * (1 - w / (1 + x)) * y1 / a + 3. / 2 * x / (1 + x) * y0 / (a * a);
}

// the growth trajectory at a_s = a0 + s h, s = 0..BG_ODE_STEPS: (D, D', and
// their derivatives from the ODE) per step point, host side
void growth_trajectory(const BgPar &p, std::vector<double4_32a> &tr)
{
    const double h = (1.0 - BG_ODE_A0) / BG_ODE_STEPS;
    tr.resize(BG_ODE_STEPS + 1);
    double y0 = 0.05, y1 = 1.0;
    for (int s = 0; s <= BG_ODE_STEPS; ++s) {
        const double a = BG_ODE_A0 + h * (double)s;
        double k10, k11;
        growth_rhs(p, a, y0, y1, k10, k11);
        tr[s].x = y0;
        tr[s].y = y1;
        tr[s].z = k10;
        tr[s].w = k11;
        if (s == BG_ODE_STEPS) break;
        double k20, k21, k30, k31, k40, k41;
        growth_rhs(p, a + 0.5 * h, y0 + 0.5 * h * k10, y1 + 0.5 * h * k11, k20, k21);
        growth_rhs(p, a + 0.5 * h, y0 + 0.5 * h * k20, y1 + 0.5 * h * k21, k30, k31);
        growth_rhs(p, a + h, y0 + h * k30, y1 + h * k31, k40, k41);
        y0 += h / 6.0 * (k10 + 2.0 * k20 + 2.0 * k30 + k40);
        y1 += h / 6.0 * (k11 + 2.0 * k21 + 2.0 * k31 + k41);
    }
}

__global__ void bg_nodes_kernel(BgPar p, int bins, const double4_32a *__restrict__ tr,
                                double *__restrict__ nodes)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= bins) return;
    double *z_ = nodes, *D1_ = nodes + 2 * bins, *f_ = nodes + 3 * bins, *a_ = nodes + 4 * bins,
           *cH_ = nodes + 5 * bins, *H_ = nodes + 6 * bins, *cHp_ = nodes + 7 * bins;
    const double zi = 15. * i / (double)(bins - 1);
    const double ai = 1. / (1. + zi);
    // cubic Hermite interpolation of the trajectory between the steps around ai
    const double h = (1.0 - BG_ODE_A0) / BG_ODE_STEPS;
    int s = (int)floor((ai - BG_ODE_A0) / h);
    s = s < 0 ? 0 : (s > BG_ODE_STEPS - 1 ? BG_ODE_STEPS - 1 : s);
    const double t = (ai - (BG_ODE_A0 + h * (double)s)) / h;
    const double4_32a u = tr[s], v = tr[s + 1];
    const double t2 = t * t, t3 = t2 * t;
    const double h00 = 2 * t3 - 3 * t2 + 1, h10 = t3 - 2 * t2 + t, h01 = -2 * t3 + 3 * t2,
                 h11 = t3 - t2;
    const double y0 = h00 * u.x + h10 * h * u.z + h01 * v.x + h11 * h * v.z;
    const double y1 = h00 * u.y + h10 * h * u.w + h01 * v.y + h11 * h * v.w;
    const double Hi = sqrt(p.om * pow(1 + zi, 3) + p.og * pow(1 + zi, 4) + p.ode * 1.0) * p.h * CG_H0;
    z_[i] = zi;
    a_[i] = ai;
    D1_[i] = y0; // normalised by bg_normalise_kernel
    f_[i] = y1 * ai / y0;
    H_[i] = Hi;
    cH_[i] = ai * Hi;
    cHp_[i] = -(pow(1 + zi, 3) * (2 * (1 + zi) * p.og + p.om) + (1 + 3 * (-1.0)) * p.ode * 1.0) /
              pow(1 + zi, 2) / 2. * pow(p.h * CG_H0, 2);
}

struct InvE {
    BgPar p;
    __device__ double operator()(double z) const
    {
        return 1. / sqrt(p.om * pow(1 + z, 3) + p.og * pow(1 + z, 4) + p.ode * 1.0);
    }
};

#define BG_QAG_CAP 128
#define BG_WARPS 4

__global__ void __launch_bounds__(32 * BG_WARPS) bg_chi_kernel(BgPar p, int bins,
                                                                 double *__restrict__ nodes,
                                                                 int *err)
{
    __shared__ double sa[BG_WARPS][BG_QAG_CAP], sb[BG_WARPS][BG_QAG_CAP],
        sr[BG_WARPS][BG_QAG_CAP], se[BG_WARPS][BG_QAG_CAP];
    const int w = threadIdx.x >> 5;
    const int i = blockIdx.x * BG_WARPS + w;
    if (i >= bins) return;
    const double zi = 15. * i / (double)(bins - 1);
    QagStore<double> st{sa[w], sb[w], sr[w], se[w], BG_QAG_CAP};
    int status = 0;
    InvE f{p};
    const double v = qag61_warp<double>(f, 0.0, zi, 0.0, 1e-5, st, 50000, &status);
    if ((threadIdx.x & 31) == 0) {
        if (status == 1) cg_flag(err, CG_ERR_QAG_LIMIT);
        const double chi = v / (p.h * CG_H0);
        if (!isfinite(chi)) cg_flag(err, CG_ERR_NONFINITE);
        nodes[bins + i] = chi;
    }
}

__global__ void bg_normalise_kernel(int bins, double *__restrict__ nodes)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= bins) return;
    // D1 row: divide by its value at z = 0 (node 0, rewritten by the next launch)
    const double D0 = nodes[2 * bins];
    if (i > 0) nodes[2 * bins + i] /= D0;
}

__global__ void bg_normalise_first_kernel(int bins, double *__restrict__ nodes)
{
    nodes[2 * bins] = 1.0;
}

} // namespace

int bg_init_device(coffe_gpu_ctx *ctx, const coffe_gpu_cosmology_t *c)
{
    const int bins = c->bins;
    if (bins < 5 || bins > (1 << 24)) {
        cg_set_error(ctx, "background bins must be in [5, 2^24] (got %d)", bins);
        return COFFE_GPU_EINVAL;
    }
    if (!(c->h > 0) || !(c->Omega0_cdm + c->Omega0_baryon > 0) ||
        !(c->Omega0_cdm + c->Omega0_baryon < 1)) {
        cg_set_error(ctx, "invalid cosmology (h > 0, 0 < Omega0_m < 1 required)");
        return COFFE_GPU_EINVAL;
    }
    int st = cg_ensure(ctx, ctx->bg_nodes, sizeof(double) * 8 * (size_t)bins);
    if (st) return st;
    BgPar p{c->Omega0_cdm + c->Omega0_baryon, c->Omega0_gamma, c->Omega0_de, c->h};
    double *nodes = (double *)ctx->bg_nodes.p;
    growth_trajectory(p, ctx->bg_traj_host);
    if ((st = cg_ensure(ctx, ctx->bg_traj, sizeof(double4_32a) * ctx->bg_traj_host.size())))
        return st;
    CG_CUDA(ctx, cudaMemcpyAsync(ctx->bg_traj.p, ctx->bg_traj_host.data(),
                                 sizeof(double4_32a) * ctx->bg_traj_host.size(),
                                 cudaMemcpyHostToDevice, ctx->stream));
    bg_nodes_kernel<<<(bins + 127) / 128, 128, 0, ctx->stream>>>(
        p, bins, (const double4_32a *)ctx->bg_traj.p, nodes);
    if ((st = cg_after_launch(ctx, "bg_nodes_kernel"))) return st;
    bg_chi_kernel<<<(bins + BG_WARPS - 1) / BG_WARPS, 32 * BG_WARPS, 0, ctx->stream>>>(
        p, bins, nodes, ctx->d_err);
    if ((st = cg_after_launch(ctx, "bg_chi_kernel"))) return st;
    // the whole grid must read node 0 before it is overwritten: two launches
    bg_normalise_kernel<<<(bins + 255) / 256, 256, 0, ctx->stream>>>(bins, nodes);
    if ((st = cg_after_launch(ctx, "bg_normalise_kernel"))) return st;
    bg_normalise_first_kernel<<<1, 1, 0, ctx->stream>>>(bins, nodes);
    if ((st = cg_after_launch(ctx, "bg_normalise_first_kernel"))) return st;
    if ((st = cg_check_device_errors(ctx, "background"))) return st;
    ctx->bg_bins = bins;
    ctx->Omega0_m = c->Omega0_cdm + c->Omega0_baryon;
    ctx->h = c->h;
    ctx->bg_has_H = true;
    return bg_build_splines(ctx);
}

int bg_build_splines(coffe_gpu_ctx *ctx)
{
    const int bins = ctx->bg_bins;
    const double *nodes = (const double *)ctx->bg_nodes.p;
    const double *z = nodes, *chi = nodes + bins, *D1 = nodes + 2 * bins, *f = nodes + 3 * bins,
                 *a = nodes + 4 * bins, *cH = nodes + 5 * bins;
    int st;
    ctx->bg_ready = false;
    if ((st = spline_build(ctx, ctx->bg[BG_CHI_OF_Z], z, chi, bins))) return st;
    if ((st = spline_build(ctx, ctx->bg[BG_Z_OF_CHI], chi, z, bins))) return st;
    if ((st = spline_build(ctx, ctx->bg[BG_D1], z, D1, bins))) return st;
    if ((st = spline_build(ctx, ctx->bg[BG_F], z, f, bins))) return st;
    if ((st = spline_build(ctx, ctx->bg[BG_A], z, a, bins))) return st;
    if ((st = spline_build(ctx, ctx->bg[BG_CONFH], z, cH, bins))) return st;
    if ((st = multipoles_prepare_background(ctx))) return st;
    ctx->bg_ready = true;
    return COFFE_GPU_OK;
}
