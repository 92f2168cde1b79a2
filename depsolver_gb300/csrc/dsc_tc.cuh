// dsc_tc.cuh -- 5th-generation tensor-core building blocks (inline PTX for
// sm_100+): 2-D TMA loads, shared-memory matrix descriptors of 128-byte
// swizzled K-major tiles, instruction descriptors, tcgen05.mma / commit /
// fences and 32-column TMEM loads.  Shared by the products of dsc_tcgemm.cu
// and the field pass of dsc_field_tc.cu.
#pragma once

#include <cuda.h>
#include <stdint.h>

#include "dsc_async.cuh"

namespace dsc {

// A k-block is one swizzle row of kTcRowBytes bytes (128: 32 FP32 or 64
// fp16 values).
constexpr int kTcRowBytes = 128;

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x,
                                            int y)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%3, %4}], [%2];" ::"r"(su32(dst)),
        "l"((uint64_t)map), "r"(su32(bar)), "r"(x), "r"(y)
        : "memory");
}

// 2-D TMA store of the box at (x, y) from shared src (the tensor map's box
// layout); out-of-range parts of the box are not written.  The caller
// fences its generic writes to src (fence.proxy.async.shared::cta) first.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap *map, const void *src, int x, int y)
{
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                     (uint64_t)map),
                 "r"(su32(src)), "r"(x), "r"(y)
                 : "memory");
}

// Prefetch of the box at (x, y) into L2 (no shared memory, no completion).
__device__ __forceinline__ void tma_prefetch_2d(const CUtensorMap *map, int x, int y)
{
    asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global [%0, {%1, %2}];" ::"l"((uint64_t)map), "r"(x), "r"(y)
                 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// this thread's committed bulk stores have read their shared sources
__device__ __forceinline__ void bulk_wait_read0()
{
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

// this thread's committed bulk stores are complete
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major tile in the swizzled
// canonical layout: rows of kTcRowBytes bytes (the swizzle width), 8-row
// groups 8 rows apart.
__device__ __forceinline__ uint64_t sw_desc(const void *tile)
{
    const uint64_t a = su32(tile);
    uint64_t d = (a >> 4) & 0x3FFFull;                    // start address
    d |= (uint64_t)1 << 16;                               // leading byte offset (unused when swizzled)
    d |= (uint64_t)((8 * kTcRowBytes) >> 4) << 32;        // stride byte offset: 8 rows
    d |= (uint64_t)1 << 46;                               // descriptor version
    d |= (uint64_t)(kTcRowBytes == 128 ? 2 : 4) << 61;    // 128- or 64-byte swizzle
    return d;
}

// Instruction descriptor: D f32, A and B tf32, both K-major, N x M shape.
__host__ __device__ constexpr uint32_t idesc_tf32(int n, int m)
{
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}

// The same for kind::f16 with A and B both fp16 (type code 0).
__host__ __device__ constexpr uint32_t idesc_f16(int n, int m)
{
    return (1u << 4) | (0u << 7) | (0u << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                        uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

template <bool F16>
__device__ __forceinline__ void mma_op(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    if (F16) mma_f16(d, a, b, idesc, acc);
    else mma_tf32(d, a, b, idesc, acc);
}

__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     su32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// 32 consecutive accumulator columns of this warp's 32 TMEM lanes, waited
// for.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t *r)
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

}  // namespace dsc
