// Spline construction kernels: Akima coefficient records and search hints.
#include "ctx.cuh"

namespace {

__global__ void akima_records_kernel(const double *__restrict__ x, const double *__restrict__ y,
                                     int n, double4_32a *__restrict__ c64, float4 *__restrict__ c32,
                                     float *__restrict__ x32)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x32[i] = (float)x[i];
    if (i >= n - 1) return;
    double b, c, d;
    akima_interval<double>(x, y, n, i, b, c, d);
    c64[i] = make_double4_32a(y[i], b, c, d);
    c32[i] = make_float4((float)y[i], (float)b, (float)c, (float)d);
}

// hint[j] = the interval a binary search returns for the left edge of bin j
__global__ void hint_kernel(const double *__restrict__ x, int n, double x0, double xn, int nh,
                            int *__restrict__ hint)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nh) return;
    const double edge = x0 + (xn - x0) * ((double)j / (double)nh);
    int lo = 0, hi = n - 1;
    while (hi > lo + 1) {
        const int mid = (lo + hi) / 2;
        if (x[mid] > edge)
            hi = mid;
        else
            lo = mid;
    }
    hint[j] = lo;
}

} // namespace

int spline_build(coffe_gpu_ctx *ctx, SplineBuf &s, const double *d_x, const double *d_y, int n)
{
    if (n < 5) {
        cg_set_error(ctx, "spline needs at least 5 knots (got %d)", n);
        return COFFE_GPU_EINVAL;
    }
    double x0, xn;
    CG_CUDA(ctx, cudaMemcpyAsync(&x0, d_x, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CG_CUDA(ctx, cudaMemcpyAsync(&xn, d_x + n - 1, sizeof(double), cudaMemcpyDeviceToHost,
                                 ctx->stream));
    CG_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (!(xn > x0)) {
        cg_set_error(ctx, "spline knots are not increasing");
        return COFFE_GPU_EINVAL;
    }
    if (s.n != n) {
        spline_free(s);
        const int nh = 2 * n;
        if (cudaMalloc(&s.x, sizeof(double) * n) != cudaSuccess ||
            cudaMalloc(&s.c64, sizeof(double4_32a) * (n - 1)) != cudaSuccess ||
            cudaMalloc(&s.x32, sizeof(float) * n) != cudaSuccess ||
            cudaMalloc(&s.c32, sizeof(float4) * (n - 1)) != cudaSuccess ||
            cudaMalloc(&s.hint, sizeof(int) * nh) != cudaSuccess) {
            spline_free(s);
            cg_set_error(ctx, "cudaMalloc failed for a spline of %d knots", n);
            return COFFE_GPU_ENOMEM;
        }
        s.n = n;
        s.nh = nh;
    }
    s.x0 = x0;
    s.xn = xn;
    CG_CUDA(ctx, cudaMemcpyAsync(s.x, d_x, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                 ctx->stream));
    const int tb = 256;
    akima_records_kernel<<<(n + tb - 1) / tb, tb, 0, ctx->stream>>>(d_x, d_y, n, s.c64, s.c32,
                                                                    s.x32);
    int st = cg_after_launch(ctx, "akima_records_kernel");
    if (st) return st;
    hint_kernel<<<(s.nh + tb - 1) / tb, tb, 0, ctx->stream>>>(d_x, n, x0, xn, s.nh, s.hint);
    return cg_after_launch(ctx, "hint_kernel");
}

void spline_free(SplineBuf &s)
{
    cudaFree(s.x);
    cudaFree(s.c64);
    cudaFree(s.x32);
    cudaFree(s.c32);
    cudaFree(s.hint);
    s = SplineBuf();
}
