// One-shot bulk asynchronous copies global -> shared memory (the TMA engine's
// untiled cp.async.bulk, sm_90 and later) completed on a shared-memory
// mbarrier, with a bounded wait.
//
// Use, in a block: bulk_begin by one thread (initialises the barrier, declares
// the byte count, issues the copy), __syncthreads, then bulk_wait by every
// thread.  Source and destination 16-byte aligned, size a multiple of 16.
#pragma once

#include <cstdint>

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
    return (unsigned)__cvta_generic_to_shared(p);
}

// thread 0 of the block: barrier at bar (8 bytes of shared memory), copy of
// bytes from src (global) to dst (shared)
__device__ __forceinline__ void bulk_begin(unsigned long long *bar, void *dst, const void *src,
                                           unsigned bytes)
{
    const unsigned b = smem_addr(bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    // the initialised barrier visible to the copy engine
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], "
                 "%2, [%3];" ::"r"(smem_addr(dst)),
                 "l"((unsigned long long)__cvta_generic_to_global(src)), "r"(bytes), "r"(b)
                 : "memory");
}

// wait for phase 0 of the barrier: true once the copy has landed, false after
// BULK_WAIT_TRIES polls (each try_wait suspends the thread for a
// hardware-chosen time; the limit is seconds, far beyond a copy's
// microseconds)
#define BULK_WAIT_TRIES (1 << 22)
__device__ __forceinline__ bool bulk_wait(unsigned long long *bar)
{
    const unsigned b = smem_addr(bar);
    for (int it = 0; it < BULK_WAIT_TRIES; ++it) {
        unsigned done;
        asm volatile("{\n\t.reg .pred p;\n\t"
                     "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done)
                     : "r"(b)
                     : "memory");
        if (done) return true;
    }
    return false;
}
