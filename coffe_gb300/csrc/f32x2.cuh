// Packed FP32 pairs (sm_100 family): two independent float lanes in one 64-bit
// register pair, operated on by add/sub/mul/fma.rn.f32x2 -- one instruction
// issue for two FP32 operations.  The FP32 lane throughput is unchanged (the
// measured rate of fma.rn.f32x2 equals fma.rn.f32's), so the gain is in issue
// slots: kernels bound by instruction issue rather than by the FMA pipe.
#pragma once

#include <cuda_runtime.h>

struct f2 {
    unsigned long long v;
};

__device__ __forceinline__ f2 f2_pack(float lo, float hi)
{
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ f2 f2_dup(float x) { return f2_pack(x, x); }
__device__ __forceinline__ float f2_lo(f2 a) { return __uint_as_float((unsigned)(a.v & 0xFFFFFFFFull)); }
__device__ __forceinline__ float f2_hi(f2 a) { return __uint_as_float((unsigned)(a.v >> 32)); }
__device__ __forceinline__ f2 f2_add(f2 a, f2 b)
{
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b)
{
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b)
{
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
// a b + c, each lane rounded once
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c)
{
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}
// |a| per lane (clears both sign bits)
__device__ __forceinline__ f2 f2_abs(f2 a)
{
    f2 r;
    r.v = a.v & 0x7FFFFFFF7FFFFFFFull;
    return r;
}
// approximate reciprocal per lane (the MUFU rcp, 1 ulp; normal inputs)
__device__ __forceinline__ f2 f2_rcp(f2 a)
{
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a.v));
    float rl, rh;
    asm("rcp.approx.f32 %0, %1;" : "=f"(rl) : "f"(lo));
    asm("rcp.approx.f32 %0, %1;" : "=f"(rh) : "f"(hi));
    return f2_pack(rl, rh);
}
