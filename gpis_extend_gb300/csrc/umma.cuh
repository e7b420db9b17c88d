// umma.cuh -- the pieces of the 5th-generation tensor-core path (tcgen05) that
// the learned proposal uses: tensor-memory allocation, shared-memory operand
// descriptors in the K-major no-swizzle layout, BF16 x BF16 -> FP32 MMAs issued by
// one thread with their completion signalled on an mbarrier, and tensor-memory
// loads into registers.  Inline PTX for sm_103a.
//
// Operand layout (K-major, no swizzle): 8 x 8 BF16 "core matrices" of 128 bytes
// (row r at byte 16 r); the core matrix of rows 8i.. and columns 8j.. of a tile
// with K columns sits at byte i * (K / 8) * 128 + j * 128.  An MMA of K = 16 reads
// two core matrices along K (leading byte offset 128) and M / 8 or N / 8 along
// the rows (stride byte offset K / 8 * 128).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gpis {
namespace umma {

// byte offset of element (row, k) in a K-major no-swizzle tile with `kdim` columns
__host__ __device__ __forceinline__ uint32_t tile_offset(uint32_t row, uint32_t k, uint32_t kdim)
{
    return (row >> 3) * (kdim >> 3) * 128u + (k >> 3) * 128u + (row & 7u) * 16u + (k & 7u) * 2u;
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M = 128 (bits: 4-5 D format, 7-9 A format, 10-12 B format, 15/16
// transposes, 17-22 N >> 3, 24-28 M >> 4)
__host__ __device__ __forceinline__ uint32_t idesc_bf16_m128(uint32_t n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((n >> 3) << 17) | ((128u >> 4) << 24);
}

// shared-memory descriptor: start address >> 4 (bits 0-13), leading byte offset >> 4
// (16-29), stride byte offset >> 4 (32-45), the fixed 0b001 at 46-48, base offset 0,
// no swizzle (61-63 = 0)
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// descriptor of the K = 16 block kb of a tile with kdim columns, starting at row r0
__device__ __forceinline__ uint64_t tile_desc(const void *tile, uint32_t r0, uint32_t kb, uint32_t kdim)
{
    const uint32_t a = smem_u32(tile) + (r0 >> 3) * (kdim >> 3) * 128u + kb * 256u;
    return sdesc(a, 128u, (kdim >> 3) * 128u);
}

// ---- tensor memory ----------------------------------------------------------------
// One warp allocates `cols` columns (a power of two >= 32) and writes the address to
// *slot; it gives up the allocation permit so that other CTAs of the SM can allocate.
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t cols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t cols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols));
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;"); }

// generic-proxy writes of shared memory made visible to the tensor core's reads
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[128 x N] (+)= A[128 x 16] * B[N x 16]^T, issued by one thread
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc, bool acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"((uint32_t)acc));
}

// the mbarrier at bar completes a phase when every MMA issued before by this thread has
__device__ __forceinline__ void commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void bar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// wait for the phase of parity `parity`, at most `limit` polls; false on time-out
__device__ __forceinline__ bool bar_wait(uint64_t *bar, uint32_t parity, uint32_t limit)
{
    const uint32_t a = smem_u32(bar);
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// 32 consecutive FP32 columns of this warp's 32 lanes (one row per thread); the wait
// for the load sits in the same statement, so no use of the values precedes it
__device__ __forceinline__ void ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 8 consecutive FP32 columns at each of four addresses (one row per thread), then
// the wait for all four loads, in one statement
__device__ __forceinline__ void ld4x8(uint32_t t0, uint32_t t1, uint32_t t2, uint32_t t3, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%32];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%33];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%34];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%24,%25,%26,%27,%28,%29,%30,%31}, [%35];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(t0), "r"(t1), "r"(t2), "r"(t3)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// barrier over `count` threads (a multiple of 32) on named barrier `id`, returning
// whether any of them passed true
__device__ __forceinline__ bool sync_or(uint32_t id, uint32_t count, bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.or.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id), "r"(count)
        : "memory");
    return r != 0;
}

}  // namespace umma
}  // namespace gpis
