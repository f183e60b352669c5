// Measured arithmetic rates of the device: the roofline denominators of the
// compute-bound kernels of this library.  No counterpart in the reference.
//
// Each kernel runs CHAINS independent fused multiply-add chains per thread
// (enough independent work to cover the pipe latency at the launch's
// occupancy) over a grid of 8 blocks of 256 threads per SM, and writes one
// value per thread so nothing is dead code.  The rate is the FMA count x 2
// over the CUDA-event time of one launch, after a warm-up launch.
//   FP64  fma.rn.f64              (the FP64 multipole and FFTLog path)
//   FP32  fma.rn.f32              (the mixed path's integrand arithmetic)
//   FP32X2 fma.rn.f32x2           (packed pair: two FP32 FMAs per instruction)
// The chain x <- x * b + c with b = 1 - 2^-12, c = 2^-12 stays near 1, so no
// input becomes denormal or overflows whatever the iteration count.
#include "ctx.cuh"

namespace {

constexpr int PEAK_CHAINS = 8;
constexpr int PEAK_THREADS = 256;
constexpr int PEAK_BLOCKS_PER_SM = 8;

__device__ __forceinline__ unsigned long long pk_f32x2(float lo, float hi)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}

__device__ __forceinline__ float sum_f32x2(unsigned long long v)
{
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
    return lo + hi;
}

__global__ void __launch_bounds__(PEAK_THREADS) peak_fp64_kernel(int iters, double *out)
{
    double x[PEAK_CHAINS];
    const double b = 1.0 - 0x1p-12, c = 0x1p-12;
#pragma unroll
    for (int j = 0; j < PEAK_CHAINS; ++j) x[j] = 1.0 + j * 0x1p-20 + threadIdx.x * 0x1p-30;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int j = 0; j < PEAK_CHAINS; ++j) x[j] = fma(x[j], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < PEAK_CHAINS; ++j) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(PEAK_THREADS) peak_fp32_kernel(int iters, double *out)
{
    float x[PEAK_CHAINS];
    const float b = 1.f - 0x1p-12f, c = 0x1p-12f;
#pragma unroll
    for (int j = 0; j < PEAK_CHAINS; ++j) x[j] = 1.f + j * 0x1p-20f + threadIdx.x * 0x1p-22f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int j = 0; j < PEAK_CHAINS; ++j) x[j] = fmaf(x[j], b, c);
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < PEAK_CHAINS; ++j) s += x[j];
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void __launch_bounds__(PEAK_THREADS) peak_fp32x2_kernel(int iters, double *out)
{
    unsigned long long x[PEAK_CHAINS];
    const unsigned long long b = pk_f32x2(1.f - 0x1p-12f, 1.f - 0x1p-12f);
    const unsigned long long c = pk_f32x2(0x1p-12f, 0x1p-12f);
#pragma unroll
    for (int j = 0; j < PEAK_CHAINS; ++j)
        x[j] = pk_f32x2(1.f + j * 0x1p-20f, 1.f + threadIdx.x * 0x1p-22f);
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int j = 0; j < PEAK_CHAINS; ++j)
                asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[j]) : "l"(b), "l"(c));
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < PEAK_CHAINS; ++j) s += sum_f32x2(x[j]);
    out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

} // namespace

extern "C" int coffe_gpu_measure_peak(coffe_gpu_ctx_t *ctx, int kind, double *flops_per_s)
{
    if (!ctx || !flops_per_s || kind < COFFE_GPU_PEAK_FP64 || kind > COFFE_GPU_PEAK_FP32X2)
        return COFFE_GPU_EINVAL;
    *flops_per_s = 0.0;
    CG_CUDA(ctx, cudaSetDevice(ctx->device));
    if (ctx->sm_count <= 0)
        CG_CUDA(ctx, cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount,
                                            ctx->device));
    const int blocks = ctx->sm_count * PEAK_BLOCKS_PER_SM;
    const size_t threads = (size_t)blocks * PEAK_THREADS;
    DevBuf &buf = ctx->peak_buf;
    int st = cg_ensure(ctx, buf, threads * sizeof(double));
    if (st) return st;
    // FMAs per thread = iters x 4 x CHAINS (x 2 lanes for the packed kind);
    // sized for launches of ~10 ms at the nominal rates
    const int iters = kind == COFFE_GPU_PEAK_FP64 ? 640 : 20000;
    const double fma_per_thread =
        (double)iters * 4 * PEAK_CHAINS * (kind == COFFE_GPU_PEAK_FP32X2 ? 2 : 1);
    auto launch = [&]() {
        double *o = (double *)buf.p;
        if (kind == COFFE_GPU_PEAK_FP64)
            peak_fp64_kernel<<<blocks, PEAK_THREADS, 0, ctx->stream>>>(iters, o);
        else if (kind == COFFE_GPU_PEAK_FP32)
            peak_fp32_kernel<<<blocks, PEAK_THREADS, 0, ctx->stream>>>(iters, o);
        else
            peak_fp32x2_kernel<<<blocks, PEAK_THREADS, 0, ctx->stream>>>(iters, o);
        return cg_after_launch(ctx, "peak kernel");
    };
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    CG_CUDA(ctx, cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        cg_set_error(ctx, "measure_peak: cudaEventCreate failed");
        return COFFE_GPU_ECUDA;
    }
    float best = 3.0e38f;
    if (!(st = launch())) { // warm-up
        for (int rep = 0; rep < 3 && !st; ++rep) {
            cudaEventRecord(e0, ctx->stream);
            st = launch();
            cudaEventRecord(e1, ctx->stream);
            float ms = 0.f;
            if (!st && (cudaEventSynchronize(e1) != cudaSuccess ||
                        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess))
                st = COFFE_GPU_ECUDA;
            if (!st && ms < best) best = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st) return st;
    *flops_per_s = 2.0 * fma_per_thread * (double)threads / (best * 1e-3);
    return COFFE_GPU_OK;
}
