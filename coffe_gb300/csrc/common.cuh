// Shared device/host helpers of the coffe_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "../../include/coffe_gpu.h"

#ifndef CG_PI
#define CG_PI 3.14159265358979323846
#endif
#define CG_SQRT_PI 1.7724538509055160272981674833411451827975494561224
#define CG_H0 (1. / 2997.92458) /* H0 in h/Mpc (COFFE_H0, common.h:76) */
#define CG_DBL_EPS 2.2204460492503131e-16
#define CG_DBL_MIN 2.2250738585072014e-308

// Device-side error flags, OR-ed into ctx->d_err by kernels.
enum cg_err_bits {
    CG_ERR_NONFINITE = 1,
    CG_ERR_QAG_LIMIT = 2,
    CG_ERR_BOUNDS = 4,
    CG_ERR_BADSEP = 16, // a separation of a host-array call is not > 0
    CG_ERR_WAIT = 32    // a bounded wait for an asynchronous copy gave up
};

__device__ __forceinline__ void cg_flag(int *err, int bit)
{
    if (err) atomicOr(err, bit);
}

template <typename T> __device__ __forceinline__ T cg_nan();
template <> __device__ __forceinline__ double cg_nan<double>() { return __longlong_as_double(0x7ff8000000000000ULL); }
template <> __device__ __forceinline__ float cg_nan<float>() { return __int_as_float(0x7fc00000); }

template <typename T> __device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Compensated (two-sum) warp reduction: each lane carries (s, c); the result
// is s + c with the rounding errors of every pairwise addition kept in c.
__device__ __forceinline__ float warp_sum_comp(float s, float c)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float so = __shfl_xor_sync(0xffffffffu, s, o);
        const float co = __shfl_xor_sync(0xffffffffu, c, o);
        const float t = s + so;
        const float bp = t - s;
        const float err = (s - (t - bp)) + (so - bp);
        s = t;
        c = c + co + err;
    }
    return s + c;
}

__device__ __forceinline__ double warp_sum_comp(double s, double c)
{
    return warp_sum(s) + warp_sum(c);
}

// Host-side: wrap a CUDA call, record the message on the context, return status.
#define CG_CUDA(ctx, call)                                                        \
    do {                                                                          \
        cudaError_t e_ = (call);                                                  \
        if (e_ != cudaSuccess) {                                                  \
            cg_set_error((ctx), "%s:%d %s: %s", __FILE__, __LINE__, #call,        \
                         cudaGetErrorString(e_));                                 \
            return COFFE_GPU_ECUDA;                                               \
        }                                                                         \
    } while (0)
