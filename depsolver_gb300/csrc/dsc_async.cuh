// dsc_async.cuh -- mbarriers and bulk asynchronous copies (sm_90+ PTX) for
// the pipelined kernels of libdepsolver_cuda.
//
// Every wait is bounded: after kSpin clock cycles (about 2 s) it gives up,
// records a code in the caller's error word and returns false, so that a
// kernel can drain and return instead of hanging.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace dsc {

constexpr long long kSpin = 4000000000LL;  // clock cycles before a wait gives up

__device__ __forceinline__ uint32_t su32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *b, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *b)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *b, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(su32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait for the phase of parity `parity`; false (and *err = code)
// after kSpin cycles or when another thread has already failed.
__device__ __forceinline__ bool mbar_wait(uint64_t *b, uint32_t parity, int *err, int code)
{
    const long long t0 = clock64();
    while (!mbar_try(b, parity)) {
        if (*(volatile int *)err) return false;
        if (clock64() - t0 > kSpin) {
            atomicCAS(err, 0, code);
            return false;
        }
    }
    return true;
}

// Wait for the phase of parity `parity` for at most kSpin cycles, without
// reporting (the drain before a kernel returns after an error).
__device__ __forceinline__ void mbar_drain(uint64_t *b, uint32_t parity)
{
    const long long t0 = clock64();
    while (!mbar_try(b, parity) && clock64() - t0 < kSpin) {
    }
}

// bytes (a multiple of 16) from global src to shared dst (both 16-byte
// aligned); completion is counted on mbarrier bar as transaction bytes.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            su32(dst)),
        "l"(src), "r"(bytes), "r"(su32(bar))
        : "memory");
}

}  // namespace dsc
