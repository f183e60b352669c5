// Shared-memory complex FFT used by the FFTLog tables and their adjoint.
#pragma once

#include "common.cuh"

namespace {

template <typename T2> __device__ __forceinline__ T2 cmul(T2 a, T2 b)
{
    T2 r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}

// In-place radix-2 DIT FFT of M = 2^logM points already in bit-reversed
// order; tw[j] = exp(-2 pi i j / (2M)), so the M-point twiddle w_M^e is
// tw[2e].  sign = -1 forward, +1 backward (conjugate twiddles).
template <typename T2>
__device__ void smem_fft(T2 *buf, int logM, const T2 *__restrict__ tw, int sign)
{
    const int M = 1 << logM;
    for (int s = 1; s <= logM; ++s) {
        const int half = 1 << (s - 1);
        const int stride = M >> (s - 1); // index step in tw (2 * M / (2 half))
        for (int b = threadIdx.x; b < M / 2; b += blockDim.x) {
            const int pos = b & (half - 1);
            const int i0 = ((b >> (s - 1)) << s) + pos;
            const int i1 = i0 + half;
            T2 w = tw[pos * stride];
            if (sign > 0) w.y = -w.y;
            const T2 u = buf[i0];
            const T2 t = cmul(w, buf[i1]);
            buf[i0].x = u.x + t.x;
            buf[i0].y = u.y + t.y;
            buf[i1].x = u.x - t.x;
            buf[i1].y = u.y - t.y;
        }
        __syncthreads();
    }
}

} // namespace
