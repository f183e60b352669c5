// C ABI entry points (include/coffe_gpu.h): argument checks, host<->device
// staging, error mapping.  The numerical work lives in the other .cu files.
#include <string.h>

#include <algorithm>
#include <vector>

#include "ctx.cuh"

void cg_set_error(coffe_gpu_ctx *ctx, const char *fmt, ...)
{
    if (!ctx) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(ctx->last_error, sizeof(ctx->last_error), fmt, ap);
    va_end(ap);
}

int cg_ensure(coffe_gpu_ctx *ctx, DevBuf &b, size_t bytes)
{
    if (b.bytes >= bytes && b.p) return COFFE_GPU_OK;
    if (b.p) {
        // the stream may still use the old buffer
        cudaStreamSynchronize(ctx->stream);
        cudaFree(b.p);
    }
    b.p = nullptr;
    b.bytes = 0;
    if (bytes == 0) return COFFE_GPU_OK;
    // injected failure (coffe_gpu_debug_fail_alloc): this allocation fails as
    // an exhausted device would make it fail, without calling cudaMalloc
    if (ctx->fail_alloc_in > 0 && --ctx->fail_alloc_in == 0) {
        cg_set_error(ctx, "cudaMalloc of %zu bytes failed (injected)", bytes);
        return COFFE_GPU_ENOMEM;
    }
    if (cudaMalloc(&b.p, bytes) != cudaSuccess) {
        cudaGetLastError();
        cg_set_error(ctx, "cudaMalloc of %zu bytes failed", bytes);
        return COFFE_GPU_ENOMEM;
    }
    b.bytes = bytes;
    return COFFE_GPU_OK;
}

void cg_release(DevBuf &b)
{
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.bytes = 0;
}

// Kernel timing mode (coffe_gpu_set_kernel_timing): an event recorded on the
// stream after every launch (and one at the start of each table or multipole
// call); the interval between consecutive events of a call is charged to the
// kernel launched between them.  Nothing is recorded while the stream is
// being captured.
static bool cg_timing_active(coffe_gpu_ctx *ctx)
{
    if (!ctx->timing) return false;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(ctx->stream, &cap) == cudaSuccess &&
           cap == cudaStreamCaptureStatusNone;
}

static void cg_timing_record(coffe_gpu_ctx *ctx, const char *what)
{
    if (ctx->timing_marks.size() >= 4096) return; // read them with coffe_gpu_kernel_times
    const size_t i = ctx->timing_marks.size();
    if (i == ctx->timing_events.size()) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) {
            cudaGetLastError();
            return;
        }
        ctx->timing_events.push_back(e);
    }
    if (cudaEventRecord(ctx->timing_events[i], ctx->stream) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    ctx->timing_marks.push_back(what);
}

void cg_timing_begin(coffe_gpu_ctx *ctx)
{
    if (cg_timing_active(ctx)) cg_timing_record(ctx, nullptr);
}

int cg_after_launch(coffe_gpu_ctx *ctx, const char *what)
{
    ctx->launches++;
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        cg_set_error(ctx, "launch of %s failed: %s", what, cudaGetErrorString(e));
        return COFFE_GPU_ECUDA;
    }
    if (cg_timing_active(ctx) && !ctx->timing_marks.empty()) cg_timing_record(ctx, what);
    return COFFE_GPU_OK;
}

// Flags CG_ERR_BADSEP if any of the n separations is not > 0 (NaN included):
// the check of a host-array call, on the device copy (5 MB of separations
// read at HBM speed instead of a serial host scan).
__global__ void sep_check_kernel(const double *__restrict__ sep, long long n, int *err)
{
    bool bad = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        bad |= !(sep[i] > 0);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) cg_flag(err, CG_ERR_BADSEP);
}

static int sep_check(coffe_gpu_ctx *ctx, const double *d_sep, long long n, cudaStream_t stream)
{
    if (n <= 0) return COFFE_GPU_OK;
    if (ctx->sm_count <= 0)
        CG_CUDA(ctx, cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount,
                                            ctx->device));
    const long long blocks = std::min<long long>((n + 255) / 256, 4LL * ctx->sm_count);
    sep_check_kernel<<<(unsigned)blocks, 256, 0, stream>>>(d_sep, n, ctx->d_err);
    return cg_after_launch(ctx, "sep_check_kernel");
}

// The device address of `bytes` of page-locked host memory at p when both its
// first and last byte are mapped into this device's address space as one
// range, else nullptr (pageable memory, or a range the check cannot vouch for).
static void *mapped_device_pointer(const void *p, size_t bytes)
{
    cudaPointerAttributes a0, a1;
    const char *last = (const char *)p + bytes - 1;
    const bool ok = cudaPointerGetAttributes(&a0, p) == cudaSuccess &&
                    a0.type == cudaMemoryTypeHost && a0.devicePointer &&
                    cudaPointerGetAttributes(&a1, last) == cudaSuccess &&
                    a1.type == cudaMemoryTypeHost && a1.devicePointer &&
                    (const char *)a1.devicePointer - (const char *)a0.devicePointer ==
                        last - (const char *)p;
    cudaGetLastError(); // an unregistered pointer is an answer, not an error
    return ok ? a0.devicePointer : nullptr;
}

int cg_check_device_errors(coffe_gpu_ctx *ctx, const char *where)
{
    CG_CUDA(ctx, cudaMemcpyAsync(ctx->h_err, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const int bits = *ctx->h_err;
    if (!bits) return COFFE_GPU_OK;
    CG_CUDA(ctx, cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream));
    *ctx->h_err = 0;
    if (bits & CG_ERR_WAIT) {
        cg_set_error(ctx, "%s: an asynchronous copy into shared memory did not complete", where);
        return COFFE_GPU_ECUDA;
    }
    if (bits & CG_ERR_BADSEP) { // before NONFINITE: such separations give NaN
        cg_set_error(ctx, "%s: separations must be positive", where);
        return COFFE_GPU_EINVAL;
    }
    if (bits & CG_ERR_NONFINITE) {
        cg_set_error(ctx, "%s: non-finite value produced (device flags 0x%x)", where, bits);
        return COFFE_GPU_ENONFINITE;
    }
    if (bits & CG_ERR_QAG_LIMIT) {
        cg_set_error(ctx, "%s: adaptive quadrature exhausted its subintervals", where);
        return COFFE_GPU_ELIMIT;
    }
    if (bits & CG_ERR_BOUNDS) {
        cg_set_error(ctx, "%s: an input was outside the supported range (device flags 0x%x)", where,
                     bits);
        return COFFE_GPU_EINVAL;
    }
    cg_set_error(ctx, "%s: device error flags 0x%x", where, bits);
    return COFFE_GPU_EINVAL;
}

namespace {
// reads 16-byte words of buf; the sum only keeps the loads alive
__global__ void l2_read_kernel(const uint4 *__restrict__ buf, size_t n, unsigned *sink)
{
    unsigned acc = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const uint4 v = buf[i];
        acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
    if (acc == 0x9e3779b9u) atomicAdd(sink, 1u); // practically never taken
}
} // namespace

int cg_copy_stream(coffe_gpu_ctx *ctx)
{
    if (!ctx->copy_stream)
        CG_CUDA(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    for (cudaEvent_t &e : ctx->copy_ev)
        if (!e) CG_CUDA(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return COFFE_GPU_OK;
}

int cg_l2_evict(coffe_gpu_ctx *ctx, void *buf, size_t bytes, int value)
{
    CG_CUDA(ctx, cudaMemsetAsync(buf, value, bytes, ctx->stream));
    if (ctx->sm_count <= 0)
        CG_CUDA(ctx, cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount,
                                            ctx->device));
    l2_read_kernel<<<ctx->sm_count * 4, 512, 0, ctx->stream>>>((const uint4 *)buf, bytes / 16,
                                                               (unsigned *)buf);
    CG_CUDA(ctx, cudaGetLastError());
    return COFFE_GPU_OK;
}

extern "C" {

const char *coffe_gpu_strerror(int status)
{
    switch (status) {
    case COFFE_GPU_OK: return "success";
    case COFFE_GPU_EINVAL: return "invalid argument";
    case COFFE_GPU_ECUDA: return "CUDA runtime error";
    case COFFE_GPU_ENOMEM: return "device out of memory";
    case COFFE_GPU_ENONFINITE: return "non-finite value in a result";
    case COFFE_GPU_ESTATE: return "missing prerequisite (background or integrals)";
    case COFFE_GPU_ELIMIT: return "adaptive quadrature subinterval limit reached";
    default: return "unknown status";
    }
}

int coffe_gpu_ctx_create(int device, coffe_gpu_ctx_t **out)
{
    if (!out) return COFFE_GPU_EINVAL;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        return COFFE_GPU_ECUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess) return COFFE_GPU_ECUDA;
    coffe_gpu_ctx *ctx = new coffe_gpu_ctx();
    ctx->device = device;
    if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&ctx->d_err, sizeof(int)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_err, sizeof(int)) != cudaSuccess) {
        coffe_gpu_ctx_destroy(ctx);
        return COFFE_GPU_ECUDA;
    }
    ctx->stream = ctx->own_stream;
    *ctx->h_err = 0;
    if (cudaMemsetAsync(ctx->d_err, 0, sizeof(int), ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
        coffe_gpu_ctx_destroy(ctx);
        return COFFE_GPU_ECUDA;
    }
    if (multipoles_noalloc_prepare(ctx) != COFFE_GPU_OK) {
        coffe_gpu_ctx_destroy(ctx);
        return COFFE_GPU_ECUDA;
    }
    *out = ctx;
    return COFFE_GPU_OK;
}

int coffe_gpu_ctx_destroy(coffe_gpu_ctx_t *ctx)
{
    if (!ctx) return COFFE_GPU_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (int i = 0; i < BG_NFN; ++i) spline_free(ctx->bg[i]);
    for (int i = 0; i < 4; ++i) {
        spline_free(ctx->bias[i]);
        cg_release(ctx->bias_nodes[i]);
    }
    DevBuf *bufs[] = {&ctx->bg_nodes, &ctx->tab_x,  &ctx->tab_x32, &ctx->tab_y,  &ctx->pk,
                      &ctx->kgrid,    &ctx->csc,    &ctx->csfac,   &ctx->samp_idx, &ctx->samp_dx,
                      &ctx->qfac,     &ctx->modec,  &ctx->postf,   &ctx->twid,   &ctx->twid32,
                      &ctx->spec,     &ctx->req_buf, &ctx->term_meta, &ctx->zrec64,
                      &ctx->zrec32,   &ctx->mp_retry, &ctx->term_df, &ctx->chi_tab64, &ctx->chi_tab32,
                      &ctx->samp_f32, &ctx->csfac32,
                      &ctx->lens_rule, &ctx->lens_rec, &ctx->lens_part,
                      &ctx->cov_buf,  &ctx->cov_out, &ctx->adj_buf, &ctx->csband,
                      &ctx->samp_tdf, &ctx->qfac_df, &ctx->pk_df, &ctx->mp_bgfit,
                      &ctx->cf_rule, &ctx->avg_buf, &ctx->div_buf, &ctx->peak_buf,
                      &ctx->bg_traj};
    spline_free(ctx->cov_pk);
    for (DevBuf *b : bufs) cg_release(*b);
    for (auto &slot : ctx->mp_node_slots) cg_release(slot.buf);
    for (cudaEvent_t ev : ctx->timing_events) cudaEventDestroy(ev);
    if (ctx->d_err) cudaFree(ctx->d_err);
    if (ctx->h_err) cudaFreeHost(ctx->h_err);
    for (cudaEvent_t e : ctx->copy_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return COFFE_GPU_OK;
}

const char *coffe_gpu_last_error(const coffe_gpu_ctx_t *ctx)
{
    return ctx ? ctx->last_error : "no context";
}

int coffe_gpu_synchronize(coffe_gpu_ctx_t *ctx)
{
    if (!ctx) return COFFE_GPU_EINVAL;
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return cg_check_device_errors(ctx, "synchronize");
}

int coffe_gpu_set_stream(coffe_gpu_ctx_t *ctx, void *stream)
{
    if (!ctx) return COFFE_GPU_EINVAL;
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return COFFE_GPU_OK;
}

int coffe_gpu_set_kernel_timing(coffe_gpu_ctx_t *ctx, int enable)
{
    if (!ctx) return COFFE_GPU_EINVAL;
    ctx->timing = enable != 0;
    return COFFE_GPU_OK;
}

int coffe_gpu_kernel_times(coffe_gpu_ctx_t *ctx, const char **names, long long *launches,
                           double *total_ms, int cap, int reset)
{
    if (!ctx || cap < 0 || (cap > 0 && (!names || !launches || !total_ms)))
        return COFFE_GPU_EINVAL;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    if (!ctx->timing_marks.empty()) {
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (size_t i = 1; i < ctx->timing_marks.size(); ++i) {
            const char *what = ctx->timing_marks[i];
            if (!what) continue; // the start of a call
            float ms = 0.f;
            CG_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->timing_events[i - 1],
                                              ctx->timing_events[i]));
            auto &acc = ctx->timing_totals[what];
            acc.first += 1;
            acc.second += ms;
        }
        ctx->timing_marks.clear();
    }
    // the names handed out live in a snapshot that the next call replaces
    ctx->timing_names.clear();
    for (const auto &kv : ctx->timing_totals) ctx->timing_names.push_back(kv.first);
    int n = 0;
    for (const auto &kv : ctx->timing_totals) {
        if (n < cap) {
            names[n] = ctx->timing_names[n].c_str();
            launches[n] = kv.second.first;
            total_ms[n] = kv.second.second;
        }
        ++n;
    }
    if (reset) ctx->timing_totals.clear();
    return n;
}

int coffe_gpu_debug_fail_alloc(coffe_gpu_ctx_t *ctx, int nth)
{
    if (!ctx || nth < 0) return COFFE_GPU_EINVAL;
    ctx->fail_alloc_in = nth;
    return COFFE_GPU_OK;
}

long long coffe_gpu_launch_count(const coffe_gpu_ctx_t *ctx) { return ctx ? ctx->launches : -1; }

long long coffe_gpu_multipoles_retries(coffe_gpu_ctx_t *ctx)
{
    if (!ctx || !ctx->mp_retry.p) return -1;
    int count = 0;
    if (cudaMemcpyAsync(&count, ctx->mp_retry.p, sizeof(int), cudaMemcpyDeviceToHost,
                        ctx->stream) != cudaSuccess ||
        cudaStreamSynchronize(ctx->stream) != cudaSuccess)
        return -1;
    return count;
}

int coffe_gpu_background_init(coffe_gpu_ctx_t *ctx, const coffe_gpu_cosmology_t *c)
{
    if (!ctx || !c) return COFFE_GPU_EINVAL;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    const int st = bg_init_device(ctx, c);
    if (st) return st;
    return cg_check_device_errors(ctx, "background_init");
}

int coffe_gpu_background_set(coffe_gpu_ctx_t *ctx, const double *z, const double *chi,
                             const double *D1, const double *f, const double *a,
                             const double *conformal_Hz, size_t bins, double Omega0_m, double h)
{
    if (!ctx || !z || !chi || !D1 || !f || !a || !conformal_Hz) return COFFE_GPU_EINVAL;
    if (bins < 5 || bins > (1u << 24)) {
        cg_set_error(ctx, "background_set: bins must be in [5, 2^24]");
        return COFFE_GPU_EINVAL;
    }
    for (size_t i = 1; i < bins; ++i)
        if (!(z[i] > z[i - 1]) || !(chi[i] > chi[i - 1])) {
            cg_set_error(ctx, "background_set: z and chi must be strictly increasing");
            return COFFE_GPU_EINVAL;
        }
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    int st = cg_ensure(ctx, ctx->bg_nodes, sizeof(double) * 8 * bins);
    if (st) return st;
    double *d = (double *)ctx->bg_nodes.p;
    const double *src[6] = {z, chi, D1, f, a, conformal_Hz};
    const int row[6] = {0, 1, 2, 3, 4, 5};
    for (int i = 0; i < 6; ++i)
        CG_CUDA(ctx, cudaMemcpyAsync(d + row[i] * bins, src[i], sizeof(double) * bins,
                                     cudaMemcpyHostToDevice, ctx->stream));
    ctx->bg_bins = (int)bins;
    ctx->Omega0_m = Omega0_m;
    ctx->h = h;
    ctx->bg_has_H = false;
    st = bg_build_splines(ctx);
    if (st) return st;
    return cg_check_device_errors(ctx, "background_set");
}

int coffe_gpu_background_get(coffe_gpu_ctx_t *ctx, double *z, double *chi, double *D1, double *f,
                             double *a, double *Hz, double *conformal_Hz,
                             double *conformal_Hz_prime)
{
    if (!ctx) return COFFE_GPU_EINVAL;
    if (ctx->bg_bins <= 0) {
        cg_set_error(ctx, "background_get: no background");
        return COFFE_GPU_ESTATE;
    }
    if ((Hz || conformal_Hz_prime) && !ctx->bg_has_H) {
        cg_set_error(ctx, "background_get: H and H' exist only after background_init");
        return COFFE_GPU_ESTATE;
    }
    const size_t bins = (size_t)ctx->bg_bins;
    const double *d = (const double *)ctx->bg_nodes.p;
    double *dst[8] = {z, chi, D1, f, a, conformal_Hz, Hz, conformal_Hz_prime};
    for (int i = 0; i < 8; ++i)
        if (dst[i])
            CG_CUDA(ctx, cudaMemcpyAsync(dst[i], d + i * bins, sizeof(double) * bins,
                                         cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return COFFE_GPU_OK;
}

int coffe_gpu_set_bias(coffe_gpu_ctx_t *ctx, int which, const double *z, const double *value,
                       size_t n)
{
    if (!ctx || which < 0 || which > 3) return COFFE_GPU_EINVAL;
    if (!z || !value || n < 5 || n > (1u << 24)) {
        cg_set_error(ctx, "set_bias: need at least 5 (z, value) samples");
        return COFFE_GPU_EINVAL;
    }
    for (size_t i = 1; i < n; ++i)
        if (!(z[i] > z[i - 1])) {
            cg_set_error(ctx, "set_bias: z must be strictly increasing");
            return COFFE_GPU_EINVAL;
        }
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    int st = cg_ensure(ctx, ctx->bias_nodes[which], sizeof(double) * 2 * n);
    if (st) return st;
    double *d = (double *)ctx->bias_nodes[which].p;
    CG_CUDA(ctx, cudaMemcpyAsync(d, z, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(d + n, value, sizeof(double) * n, cudaMemcpyHostToDevice,
                                 ctx->stream));
    ctx->bias_set[which] = false;
    st = spline_build(ctx, ctx->bias[which], d, d + n, (int)n);
    if (st) return st;
    ctx->bias_set[which] = true;
    ctx->bias_host[which].assign(z, z + n);
    ctx->bias_host[which].insert(ctx->bias_host[which].end(), value, value + n);
    return cg_check_device_errors(ctx, "set_bias");
}

// the fixed separations (Mpc) of the divergent integral's spline
// (integrals.c:76-103): a table the spline's knots must reproduce
static const double cg_div_sep[] = {
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

size_t coffe_gpu_divergent_separations(double *out, size_t cap)
{
    const size_t n = sizeof(cg_div_sep) / sizeof(cg_div_sep[0]);
    for (size_t i = 0; out && i < n && i < cap; ++i) out[i] = cg_div_sep[i];
    return n;
}

int coffe_gpu_divergent_integral(coffe_gpu_ctx_t *ctx, const double *k, const double *pk,
                                 size_t nk, double kmin, double kmax, const double *sep,
                                 size_t n_sep, double *result, double *result0)
{
    if (!ctx) return COFFE_GPU_EINVAL;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    return divergent_run(ctx, k, pk, nk, kmin, kmax, sep, n_sep, nullptr, 0, result, result0);
}

int coffe_gpu_renormalization_grid(coffe_gpu_ctx_t *ctx, const double *k, const double *pk,
                                   size_t nk, double kmin, double kmax, const double *chi1,
                                   size_t n1, const double *chi2, size_t n2, double *out)
{
    if (!ctx) return COFFE_GPU_EINVAL;
    if (!chi2) {
        cg_set_error(ctx, "renormalization grid: chi2 is required");
        return COFFE_GPU_EINVAL;
    }
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    return divergent_run(ctx, k, pk, nk, kmin, kmax, chi1, n1, chi2, n2, out, nullptr);
}

int coffe_gpu_set_autotune(coffe_gpu_ctx_t *ctx, int enable)
{
    if (!ctx) return COFFE_GPU_EINVAL;
    ctx->autotune = enable != 0;
    return COFFE_GPU_OK;
}

int coffe_gpu_get_tuning(const coffe_gpu_ctx_t *ctx, coffe_gpu_tuning_t *out)
{
    if (!ctx || !out) return COFFE_GPU_EINVAL;
    *out = ctx->last_tuning;
    return COFFE_GPU_OK;
}

int coffe_gpu_set_tuning(coffe_gpu_ctx_t *ctx, const coffe_gpu_tuning_t *t)
{
    if (!ctx || !t) return COFFE_GPU_EINVAL;
    const int ft = t->fft_threads, lt = t->lane_threads, g = t->spline_group;
    const int ff = t->fft_threads_fwd;
    if (!(ft == 128 || ft == 256 || ft == 512 || ft == 1024) ||
        !(ff == 128 || ff == 256 || ff == 512 || ff == 1024) ||
        !(t->fft_radix == 2 || t->fft_radix == 4) || !(t->fft_swizzle == 0 || t->fft_swizzle == 1) ||
        !(g == 2 || g == 4 || g == 8) || !(lt == 64 || lt == 128 || lt == 256) ||
        !(t->lane_unroll == 1 || t->lane_unroll == 2) ||
        !(t->lane_pack == 1 || t->lane_pack == 2) || !(t->fft_fused == 0 || t->fft_fused == 1) ||
        !(t->lane_poly == 0 || t->lane_poly == 1)) {
        cg_set_error(ctx, "set_tuning: fft_threads(_fwd) 128/256/512/1024, fft_radix 2/4, "
                          "fft_swizzle 0/1, spline_group 2/4/8, lane_threads 64/128/256, "
                          "lane_unroll 1/2, lane_pack 1/2, fft_fused 0/1, lane_poly 0/1");
        return COFFE_GPU_EINVAL;
    }
    ctx->tuning = *t;
    ctx->tune_cache.clear();
    return COFFE_GPU_OK;
}

size_t coffe_gpu_integral_table_len(size_t N) { return N + CG_N_SMALL_R + 1; }

int coffe_gpu_integrals_init(coffe_gpu_ctx_t *ctx, const double *k, const double *pk,
                             int n_spectra, size_t nk, const int *n, const int *l, int n_terms,
                             size_t N, int precision, unsigned flags)
{
    return coffe_gpu_integrals_init_ex(ctx, k, pk, n_spectra, nk, n, l, nullptr, n_terms, N,
                                       precision, flags);
}

int coffe_gpu_integrals_init_ex(coffe_gpu_ctx_t *ctx, const double *k, const double *pk,
                                int n_spectra, size_t nk, const int *n, const int *l,
                                const int *half, int n_terms, size_t N, int precision,
                                unsigned flags)
{
    if (!ctx) return COFFE_GPU_EINVAL;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    const int st = integrals_build(ctx, k, pk, n_spectra, nk, n, l, half, n_terms, N, precision,
                                   flags);
    if (st) {
        ctx->int_ready = false;
        return st;
    }
    if (flags & COFFE_GPU_ASYNC) {
        // host P(k): returns once it has been copied, so the caller may reuse it
        if (!(flags & COFFE_GPU_PK_DEVICE) && ctx->copy_ev[2])
            CG_CUDA(ctx, cudaEventSynchronize(ctx->copy_ev[2]));
        return COFFE_GPU_OK;
    }
    const int st2 = cg_check_device_errors(ctx, "integrals_init");
    if (st2) ctx->int_ready = false;
    return st2;
}

int coffe_gpu_integral_get(coffe_gpu_ctx_t *ctx, int spectrum, int term, double *x, double *y)
{
    if (!ctx) return COFFE_GPU_EINVAL;
    if (!ctx->int_ready) {
        cg_set_error(ctx, "integral_get: integrals not initialised");
        return COFFE_GPU_ESTATE;
    }
    if (spectrum < 0 || spectrum >= ctx->n_spectra || term < 0 || term >= ctx->n_terms) {
        cg_set_error(ctx, "integral_get: (spectrum %d, term %d) out of range", spectrum, term);
        return COFFE_GPU_EINVAL;
    }
    const size_t len = ctx->N + CG_N_SMALL_R + 1;
    const size_t off = ((size_t)spectrum * ctx->n_terms + term) * len;
    if (x)
        CG_CUDA(ctx, cudaMemcpyAsync(x, ctx->tab_x.p, sizeof(double) * len, cudaMemcpyDeviceToHost,
                                     ctx->stream));
    if (y) {
        if (ctx->int_precision == COFFE_GPU_MIXED) {
            std::vector<float> tmp(len);
            CG_CUDA(ctx, cudaMemcpyAsync(tmp.data(), (const float *)ctx->tab_y.p + off,
                                         sizeof(float) * len, cudaMemcpyDeviceToHost, ctx->stream));
            CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            for (size_t i = 0; i < len; ++i) y[i] = tmp[i];
        } else {
            CG_CUDA(ctx, cudaMemcpyAsync(y, (const double *)ctx->tab_y.p + off,
                                         sizeof(double) * len, cudaMemcpyDeviceToHost, ctx->stream));
        }
    }
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return COFFE_GPU_OK;
}

int coffe_gpu_integral_eval(coffe_gpu_ctx_t *ctx, int spectrum, int term, const double *r,
                            size_t nq, double *out)
{
    if (!ctx || (nq && (!r || !out))) return COFFE_GPU_EINVAL;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    const int st = integrals_eval(ctx, spectrum, term, r, nq, out);
    if (st) return st;
    return cg_check_device_errors(ctx, "integral_eval");
}

int coffe_gpu_multipoles(coffe_gpu_ctx_t *ctx, int contrib, int precision, double epsrel,
                         int n_req, const int *req_spectrum, const double *req_z_mean,
                         const int64_t *req_offset, const double *sep, int n_l, const int *l,
                         double *out, int arrays_on_device)
{
    if (!ctx || !req_spectrum || !req_z_mean || !req_offset || !l || n_req < 1 || n_l < 1)
        return COFFE_GPU_EINVAL;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    if (arrays_on_device) {
        int ls[64];
        if (n_l > 64) return COFFE_GPU_EINVAL;
        CG_CUDA(ctx, cudaMemcpyAsync(ls, l, sizeof(int) * n_l, cudaMemcpyDeviceToHost,
                                     ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        int64_t total = 0;
        CG_CUDA(ctx, cudaMemcpyAsync(&total, req_offset + n_req, sizeof(int64_t),
                                     cudaMemcpyDeviceToHost, ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const int st = multipoles_run(ctx, contrib, precision, epsrel, n_req, req_spectrum,
                                      req_z_mean, req_offset, sep, n_l, ls, out, total);
        if (st) return st;
        return cg_check_device_errors(ctx, "multipoles");
    }
    // host arrays: validate, stage, run, copy back
    if (!ctx->bg_ready || !ctx->int_ready) {
        cg_set_error(ctx, "multipoles: %s not initialised", ctx->bg_ready ? "integrals" : "background");
        return COFFE_GPU_ESTATE;
    }
    if (req_offset[0] != 0) {
        cg_set_error(ctx, "multipoles: req_offset[0] must be 0");
        return COFFE_GPU_EINVAL;
    }
    for (int q = 0; q < n_req; ++q) {
        if (req_offset[q + 1] < req_offset[q]) {
            cg_set_error(ctx, "multipoles: req_offset must be non-decreasing");
            return COFFE_GPU_EINVAL;
        }
        if (req_spectrum[q] < 0 || req_spectrum[q] >= ctx->n_spectra) {
            cg_set_error(ctx, "multipoles: request %d names spectrum %d of %d", q, req_spectrum[q],
                         ctx->n_spectra);
            return COFFE_GPU_EINVAL;
        }
        if (!(req_z_mean[q] >= 0)) {
            cg_set_error(ctx, "multipoles: request %d has a bad mean redshift", q);
            return COFFE_GPU_EINVAL;
        }
    }
    const int64_t total = req_offset[n_req];
    if (total > 0 && (!sep || !out)) return COFFE_GPU_EINVAL;
    // a page-locked, mapped output is written by the kernels directly (no
    // device copy and download; the den/rsd kernels store it in whole lines)
    double *out_mapped = total > 0 && !(contrib & COFFE_GPU_LEN)
                             ? (double *)mapped_device_pointer(out, sizeof(double) * total * n_l)
                             : nullptr;
    const size_t b_spec = sizeof(int) * n_req, b_z = sizeof(double) * n_req,
                 b_off = sizeof(int64_t) * (n_req + 1), b_sep = sizeof(double) * total,
                 b_out = out_mapped ? 0 : sizeof(double) * total * n_l;
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t bytes = al(b_spec) + al(b_z) + al(b_off) + al(b_sep) + al(b_out);
    int st = cg_ensure(ctx, ctx->req_buf, bytes);
    if (st) return st;
    char *base = (char *)ctx->req_buf.p;
    int *d_spec = (int *)base;
    double *d_z = (double *)(base + al(b_spec));
    int64_t *d_off = (int64_t *)(base + al(b_spec) + al(b_z));
    double *d_sep = (double *)(base + al(b_spec) + al(b_z) + al(b_off));
    double *d_out = out_mapped ? out_mapped
                               : (double *)(base + al(b_spec) + al(b_z) + al(b_off) + al(b_sep));
    // the uploads go through the copy stream, so that they overlap work still
    // running on the context's stream (the tables of an ASYNC integrals_init);
    // the request buffer is free: every host-array call ends synchronised
    if ((st = cg_copy_stream(ctx))) return st;
    cudaStream_t up = ctx->copy_stream;
    CG_CUDA(ctx, cudaMemcpyAsync(d_spec, req_spectrum, b_spec, cudaMemcpyHostToDevice, up));
    CG_CUDA(ctx, cudaMemcpyAsync(d_z, req_z_mean, b_z, cudaMemcpyHostToDevice, up));
    CG_CUDA(ctx, cudaMemcpyAsync(d_off, req_offset, b_off, cudaMemcpyHostToDevice, up));
    if (total > 0) CG_CUDA(ctx, cudaMemcpyAsync(d_sep, sep, b_sep, cudaMemcpyHostToDevice, up));
    // the separations are checked on the device copy, after the uploads (a
    // non-positive one cannot make a kernel read out of bounds: its lookups
    // give NaN); the flag surfaces as EINVAL after the work has run
    if ((st = sep_check(ctx, d_sep, total, up))) return st;
    CG_CUDA(ctx, cudaEventRecord(ctx->copy_ev[0], up));
    CG_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->copy_ev[0], 0));
    ctx->out_host = out_mapped != nullptr;
    // work that needs only the requests may run on the upload stream (per-kernel
    // timing keeps everything on one stream)
    ctx->prep_stream = ctx->timing ? nullptr : up;
    st = multipoles_run(ctx, contrib, precision, epsrel, n_req, d_spec, d_z, d_off, d_sep, n_l, l,
                        d_out, total);
    ctx->prep_stream = nullptr;
    ctx->out_host = false;
    if (st) {
        cudaStreamSynchronize(ctx->stream); // no kernel may write `out` after return
        return st;
    }
    if (total > 0 && !out_mapped)
        CG_CUDA(ctx, cudaMemcpyAsync(out, d_out, b_out, cudaMemcpyDeviceToHost, ctx->stream));
    return cg_check_device_errors(ctx, "multipoles"); // also clears the device flags
}

int coffe_gpu_average_multipoles(coffe_gpu_ctx_t *ctx, int contrib, int precision,
                                 double epsrel, int n_win, const int *win_spectrum,
                                 const double *z_min, const double *z_max,
                                 const int64_t *win_offset, const double *sep, int n_l,
                                 const int *l, int n_z, double *out, int arrays_on_device)
{
    if (!ctx || !win_spectrum || !z_min || !z_max || !win_offset || !l || n_win < 1 || n_l < 1)
        return COFFE_GPU_EINVAL;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    if (arrays_on_device) {
        int64_t total = 0;
        CG_CUDA(ctx, cudaMemcpyAsync(&total, win_offset + n_win, sizeof(int64_t),
                                     cudaMemcpyDeviceToHost, ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const int st = average_multipoles_run(ctx, contrib, precision, epsrel, n_win, win_spectrum,
                                              z_min, z_max, win_offset, sep, n_l, l, n_z, out,
                                              total);
        if (st) return st;
        return cg_check_device_errors(ctx, "average_multipoles");
    }
    if (!ctx->bg_ready || !ctx->int_ready) {
        cg_set_error(ctx, "average_multipoles: %s not initialised",
                     ctx->bg_ready ? "integrals" : "background");
        return COFFE_GPU_ESTATE;
    }
    if (win_offset[0] != 0) {
        cg_set_error(ctx, "average_multipoles: win_offset[0] must be 0");
        return COFFE_GPU_EINVAL;
    }
    for (int q = 0; q < n_win; ++q) {
        if (win_offset[q + 1] < win_offset[q]) {
            cg_set_error(ctx, "average_multipoles: win_offset must be non-decreasing");
            return COFFE_GPU_EINVAL;
        }
        if (win_spectrum[q] < 0 || win_spectrum[q] >= ctx->n_spectra) {
            cg_set_error(ctx, "average_multipoles: window %d names spectrum %d of %d", q,
                         win_spectrum[q], ctx->n_spectra);
            return COFFE_GPU_EINVAL;
        }
        if (!(z_min[q] >= 0 && z_max[q] > z_min[q])) {
            cg_set_error(ctx, "average_multipoles: window %d needs 0 <= z_min < z_max", q);
            return COFFE_GPU_EINVAL;
        }
    }
    const int64_t total = win_offset[n_win];
    if (total > 0 && (!sep || !out)) return COFFE_GPU_EINVAL;
    for (int64_t i = 0; i < total; ++i)
        if (!(sep[i] > 0)) {
            cg_set_error(ctx, "average_multipoles: separations must be positive");
            return COFFE_GPU_EINVAL;
        }
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t b_spec = sizeof(int) * n_win, b_z = sizeof(double) * n_win,
                 b_off = sizeof(int64_t) * (n_win + 1), b_sep = sizeof(double) * total,
                 b_out = sizeof(double) * total * n_l;
    int st = cg_ensure(ctx, ctx->req_buf, al(b_spec) + 2 * al(b_z) + al(b_off) + al(b_sep) +
                                              al(b_out));
    if (st) return st;
    char *base = (char *)ctx->req_buf.p;
    int *d_spec = (int *)base;
    double *d_zmin = (double *)(base + al(b_spec));
    double *d_zmax = (double *)(base + al(b_spec) + al(b_z));
    int64_t *d_off = (int64_t *)(base + al(b_spec) + 2 * al(b_z));
    double *d_sep = (double *)(base + al(b_spec) + 2 * al(b_z) + al(b_off));
    double *d_out = (double *)(base + al(b_spec) + 2 * al(b_z) + al(b_off) + al(b_sep));
    CG_CUDA(ctx, cudaMemcpyAsync(d_spec, win_spectrum, b_spec, cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(d_zmin, z_min, b_z, cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(d_zmax, z_max, b_z, cudaMemcpyHostToDevice, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(d_off, win_offset, b_off, cudaMemcpyHostToDevice, ctx->stream));
    if (total > 0)
        CG_CUDA(ctx, cudaMemcpyAsync(d_sep, sep, b_sep, cudaMemcpyHostToDevice, ctx->stream));
    st = average_multipoles_run(ctx, contrib, precision, epsrel, n_win, d_spec, d_zmin, d_zmax,
                                d_off, d_sep, n_l, l, n_z, d_out, total);
    if (st) return st;
    if (total > 0)
        CG_CUDA(ctx, cudaMemcpyAsync(out, d_out, b_out, cudaMemcpyDeviceToHost, ctx->stream));
    return cg_check_device_errors(ctx, "average_multipoles");
}

int coffe_gpu_corrfunc(coffe_gpu_ctx_t *ctx, int contrib, int precision, int n_req,
                       const int *req_spectrum, const double *req_z_mean,
                       const int64_t *req_offset, const double *sep, int n_mu, const double *mu,
                       double *out, int arrays_on_device)
{
    if (!ctx || !req_spectrum || !req_z_mean || !req_offset || !mu || n_req < 1 || n_mu < 1 ||
        n_mu > 1024)
        return COFFE_GPU_EINVAL;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    int64_t total = 0;
    if (arrays_on_device) {
        CG_CUDA(ctx, cudaMemcpyAsync(&total, req_offset + n_req, sizeof(int64_t),
                                     cudaMemcpyDeviceToHost, ctx->stream));
        CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    } else {
        if (!ctx->bg_ready || !ctx->int_ready) {
            cg_set_error(ctx, "corrfunc: %s not initialised", ctx->bg_ready ? "integrals" : "background");
            return COFFE_GPU_ESTATE;
        }
        if (req_offset[0] != 0) {
            cg_set_error(ctx, "corrfunc: req_offset[0] must be 0");
            return COFFE_GPU_EINVAL;
        }
        for (int q = 0; q < n_req; ++q) {
            if (req_offset[q + 1] < req_offset[q]) {
                cg_set_error(ctx, "corrfunc: req_offset must be non-decreasing");
                return COFFE_GPU_EINVAL;
            }
            if (req_spectrum[q] < 0 || req_spectrum[q] >= ctx->n_spectra) {
                cg_set_error(ctx, "corrfunc: request %d names spectrum %d of %d", q,
                             req_spectrum[q], ctx->n_spectra);
                return COFFE_GPU_EINVAL;
            }
            if (!(req_z_mean[q] >= 0)) {
                cg_set_error(ctx, "corrfunc: request %d has a bad mean redshift", q);
                return COFFE_GPU_EINVAL;
            }
        }
        total = req_offset[n_req];
        for (int64_t i = 0; i < total; ++i)
            if (!(sep[i] > 0)) {
                cg_set_error(ctx, "corrfunc: separations must be positive");
                return COFFE_GPU_EINVAL;
            }
    }
    if (total > 0 && (!sep || !out)) return COFFE_GPU_EINVAL;
    // mu on the device (a host array in both modes), then the inputs
    auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t b_mu = sizeof(double) * n_mu;
    size_t bytes = al(b_mu);
    const size_t b_spec = sizeof(int) * n_req, b_z = sizeof(double) * n_req,
                 b_off = sizeof(int64_t) * (n_req + 1), b_sep = sizeof(double) * total,
                 b_out = sizeof(double) * total * n_mu;
    if (!arrays_on_device) bytes += al(b_spec) + al(b_z) + al(b_off) + al(b_sep) + al(b_out);
    int st = cg_ensure(ctx, ctx->req_buf, bytes);
    if (st) return st;
    char *base = (char *)ctx->req_buf.p;
    double *d_mu = (double *)base;
    CG_CUDA(ctx, cudaMemcpyAsync(d_mu, mu, b_mu, cudaMemcpyHostToDevice, ctx->stream));
    if (arrays_on_device) {
        st = corrfunc_run(ctx, contrib, precision, n_req, req_spectrum, req_z_mean, req_offset, sep,
                          n_mu, d_mu, mu, out, total);
        if (st) return st;
        return cg_check_device_errors(ctx, "corrfunc");
    }
    base += al(b_mu);
    int *d_spec = (int *)base;
    double *d_z = (double *)(base + al(b_spec));
    int64_t *d_off = (int64_t *)(base + al(b_spec) + al(b_z));
    double *d_sep = (double *)(base + al(b_spec) + al(b_z) + al(b_off));
    double *d_out = (double *)(base + al(b_spec) + al(b_z) + al(b_off) + al(b_sep));
    // the uploads go through the copy stream, so that they overlap work still
    // running on the context's stream (the tables of an ASYNC integrals_init);
    // the request buffer is free: every host-array call ends synchronised
    if ((st = cg_copy_stream(ctx))) return st;
    cudaStream_t up = ctx->copy_stream;
    CG_CUDA(ctx, cudaMemcpyAsync(d_spec, req_spectrum, b_spec, cudaMemcpyHostToDevice, up));
    CG_CUDA(ctx, cudaMemcpyAsync(d_z, req_z_mean, b_z, cudaMemcpyHostToDevice, up));
    CG_CUDA(ctx, cudaMemcpyAsync(d_off, req_offset, b_off, cudaMemcpyHostToDevice, up));
    if (total > 0) CG_CUDA(ctx, cudaMemcpyAsync(d_sep, sep, b_sep, cudaMemcpyHostToDevice, up));
    CG_CUDA(ctx, cudaEventRecord(ctx->copy_ev[0], up));
    CG_CUDA(ctx, cudaStreamWaitEvent(ctx->stream, ctx->copy_ev[0], 0));
    st = corrfunc_run(ctx, contrib, precision, n_req, d_spec, d_z, d_off, d_sep, n_mu, d_mu, mu,
                      d_out, total);
    if (st) return st;
    if (total > 0)
        CG_CUDA(ctx, cudaMemcpyAsync(out, d_out, b_out, cudaMemcpyDeviceToHost, ctx->stream));
    return cg_check_device_errors(ctx, "corrfunc");
}

int coffe_gpu_multipoles_scaled(coffe_gpu_ctx_t *ctx, int contrib, int n_req, int64_t n_sep,
                                const int *req_spectrum, const double *req_z_mean,
                                const int64_t *req_offset, const double *sep, int n_l,
                                const int *l, const double *bias_scale,
                                const double *growth_scale, double *out)
{
    if (!ctx || !req_spectrum || !req_z_mean || !req_offset || !l || n_sep < 0 ||
        (n_sep > 0 && (!sep || !out)))
        return COFFE_GPU_EINVAL;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    const int st = multipoles_adjoint_run(ctx, contrib, n_req, req_spectrum, req_z_mean,
                                          req_offset, sep, n_sep, n_l, l, bias_scale,
                                          growth_scale, nullptr, out, nullptr, nullptr, nullptr);
    if (st) return st;
    return cg_check_device_errors(ctx, "multipoles_scaled");
}

int coffe_gpu_multipoles_adjoint(coffe_gpu_ctx_t *ctx, int contrib, int n_req, int64_t n_sep,
                                 const int *req_spectrum, const double *req_z_mean,
                                 const int64_t *req_offset, const double *sep, int n_l,
                                 const int *l, const double *bias_scale,
                                 const double *growth_scale, const double *grad_out,
                                 double *grad_pk, double *grad_bias_scale,
                                 double *grad_growth_scale)
{
    if (!ctx || !req_spectrum || !req_z_mean || !req_offset || !l || n_sep < 0 ||
        (n_sep > 0 && (!sep || !grad_out)) || !grad_pk)
        return COFFE_GPU_EINVAL;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    const int st = multipoles_adjoint_run(ctx, contrib, n_req, req_spectrum, req_z_mean,
                                          req_offset, sep, n_sep, n_l, l, bias_scale,
                                          growth_scale, grad_out, nullptr, grad_pk,
                                          grad_bias_scale, grad_growth_scale);
    if (st) return st;
    return cg_check_device_errors(ctx, "multipoles_adjoint");
}

int coffe_gpu_set_flatsky(coffe_gpu_ctx_t *ctx, int local_nonlocal, int nonlocal)
{
    if (!ctx) return COFFE_GPU_EINVAL;
    ctx->flat_local_nonlocal = local_nonlocal != 0;
    ctx->flat_nonlocal = nonlocal != 0;
    return COFFE_GPU_OK;
}

int coffe_gpu_set_lensing_rule(coffe_gpu_ctx_t *ctx, int n_mu, int n_x)
{
    if (!ctx) return COFFE_GPU_EINVAL;
    if (n_mu < 2 || n_mu > 4096 || n_x < 2 || n_x > 4096) {
        cg_set_error(ctx, "set_lensing_rule: need 2 <= n_mu, n_x <= 4096 (got %d, %d)", n_mu, n_x);
        return COFFE_GPU_EINVAL;
    }
    ctx->lens_n_mu = n_mu;
    ctx->lens_n_x = n_x;
    return COFFE_GPU_OK;
}

int coffe_gpu_multipoles_async(coffe_gpu_ctx_t *ctx, int contrib, int precision, double epsrel,
                               int n_req, int64_t n_sep, const int *req_spectrum,
                               const double *req_z_mean, const int64_t *req_offset,
                               const double *sep, int n_l, const int *l, double *out)
{
    if (!ctx || !req_spectrum || !req_z_mean || !req_offset || !l || n_req < 1 || n_l < 1 ||
        n_sep < 0 || (n_sep > 0 && (!sep || !out)))
        return COFFE_GPU_EINVAL;
    return multipoles_run(ctx, contrib, precision, epsrel, n_req, req_spectrum, req_z_mean,
                          req_offset, sep, n_l, l, out, n_sep);
}

} // extern "C"
