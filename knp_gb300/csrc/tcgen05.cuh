// Minimal inline-PTX layer for 5th-generation tensor cores (tcgen05) on sm_103a: tensor-memory
// allocation, shared-memory matrix descriptors, BF16 MMA with FP32 accumulation in tensor memory,
// completion through an mbarrier, and tensor-memory loads. Every wait is bounded: it gives up after
// a fixed number of polls and reports failure, so a kernel can set an error flag and finish.
#pragma once

#include <cstdint>

namespace knp_gb300
{
namespace tc
{

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return static_cast<uint32_t>(__cvta_generic_to_shared(p)); }

// Shared-memory matrix descriptor for a K-major operand in the canonical layout without swizzle:
// the tile is made of 8-row x 16-byte core matrices stored as 128 contiguous bytes (row r of the
// core matrix at byte 16 r); core matrices adjacent along K are `lbo` bytes apart, adjacent along
// M (or N) `sbo` bytes apart. Element (r, k) of a BF16 tile is at
//   (r / 8) * sbo + (k / 8) * lbo + (r % 8) * 16 + (k % 8) * 2.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
    d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16;
    d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
    d |= 1ull << 46;  // descriptor version of tcgen05; base offset 0, no swizzle
    return d;
}

// Descriptor of a K-major operand in the 128-byte swizzled layout (the one a TMA load with
// SWIZZLE_128B writes): row r of the tile at r * 128 bytes, its 16-byte chunk j at chunk j ^ (r % 8),
// 8-row groups `sbo` bytes apart; the tile starts on a 1024-byte boundary, and the K step of an MMA
// inside the 128-byte row is an offset of the start address.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr, uint32_t sbo)
{
    uint64_t d = static_cast<uint64_t>((addr >> 4) & 0x3FFFu);
    d |= 1ull << 16;  // leading offset: unused for swizzled K-major operands
    d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32;
    d |= 1ull << 46;  // descriptor version of tcgen05
    d |= 2ull << 61;  // 128-byte swizzle
    return d;
}

__device__ __forceinline__ uint32_t core_offset(uint32_t r, uint32_t k, uint32_t lbo, uint32_t sbo)
{
    return (r >> 3) * sbo + (k >> 3) * lbo + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Instruction descriptor of tcgen05.mma kind::f16: A and B BF16, D FP32, both operands K-major.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int m, int n)
{
    return (1u << 4)                                    // D format F32
           | (1u << 7)                                  // A format BF16
           | (1u << 10)                                 // B format BF16
           | (static_cast<uint32_t>(n >> 3) << 17)      // N / 8
           | (static_cast<uint32_t>(m >> 4) << 24);     // M / 16
}

// Allocate `ncols` (power of two, >= 32) tensor-memory columns; one full warp executes it and the
// base address lands in *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Make generic-proxy shared-memory writes visible to the tensor core (async proxy).
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// D[tmem] (+)= A * B^T for one K = 16 slice; issued by a single thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                        uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// As mma_bf16 with the A operand in tensor memory: rows of A in lanes 0..M-1, K along columns, two
// 16-bit elements per 32-bit column (element 2c in the low half of column c).
__device__ __forceinline__ void mma_bf16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t b_desc, uint32_t idesc,
                                           uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}\n" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Thread t of warp w (w = warp index within its warpgroup) writes tensor-memory lane 32 w + t,
// 16 consecutive 32-bit columns starting at `taddr`'s column.
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t *v)
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
            taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]),
        "r"(v[9]), "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}

// This thread's earlier tcgen05.st have completed.
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// The mbarrier at `mbar` receives one arrival when every previously issued tcgen05.mma of this
// thread has completed.
__device__ __forceinline__ void commit(uint64_t *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Upper bound of one try_wait's suspension (ns): a waiting thread sleeps instead of spinning, so it
// does not take issue slots from the other warps of its SM sub-partition; it wakes when the phase
// completes.
constexpr uint32_t kSuspendNs = 4096;

// Wait for phase `parity` of the mbarrier to complete; false after `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity, uint32_t limit)
{
    const uint32_t a = smem_u32(mbar);
    for (uint32_t i = 0; i < limit; ++i)
    {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(parity), "r"(kSuspendNs)
            : "memory");
        if (done) return true;
    }
    return false;
}

// One poll of mbar_wait (suspends for at most kSuspendNs); true if the phase has completed.
__device__ __forceinline__ bool mbar_try_wait(uint64_t *mbar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity), "r"(kSuspendNs)
        : "memory");
    return done != 0;
}

// One poll of mbar_wait_cluster.
__device__ __forceinline__ bool mbar_try_wait_cluster(uint64_t *mbar, uint32_t parity)
{
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smem_u32(mbar)), "r"(parity), "r"(kSuspendNs)
        : "memory");
    return done != 0;
}

// 32-bit store into the shared memory of another CTA of the cluster (address from mapa).
__device__ __forceinline__ void st_cluster_u32(uint32_t remote_addr, uint32_t v)
{
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(remote_addr), "r"(v) : "memory");
}

__device__ __forceinline__ uint32_t cluster_nctarank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}

// As mbar_wait, with cluster-scope acquire: for phases completed by another CTA of the cluster
// (st.async with complete_tx into this CTA's shared memory).
__device__ __forceinline__ bool mbar_wait_cluster(uint64_t *mbar, uint32_t parity, uint32_t limit)
{
    const uint32_t a = smem_u32(mbar);
    for (uint32_t i = 0; i < limit; ++i)
    {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2, %3;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(parity), "r"(kSuspendNs)
            : "memory");
        if (done) return true;
    }
    return false;
}

// Address of the same shared-memory location in CTA `rank` of this cluster.
__device__ __forceinline__ uint32_t mapa(uint32_t addr, uint32_t rank)
{
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}

// 16-byte store into another CTA's shared memory; its mbarrier `remote_mbar` counts the bytes.
__device__ __forceinline__ void st_async_v4(uint32_t remote_addr, float a, float b, float c, float d,
                                            uint32_t remote_mbar)
{
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.v4.f32 [%0], {%1, %2, %3, %4}, [%5];" ::"r"(
                     remote_addr),
                 "f"(a), "f"(b), "f"(c), "f"(d), "r"(remote_mbar)
                 : "memory");
}

// One arrival (release, CTA scope) on a shared-memory mbarrier.
__device__ __forceinline__ void mbar_arrive(uint64_t *mbar)
{
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)) : "memory");
}

// Named barrier `id` over `n` threads (a multiple of 32) that also ANDs a predicate across them, so
// every participant leaves with the same decision.
__device__ __forceinline__ bool named_sync_and(uint32_t id, uint32_t n, bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"(static_cast<uint32_t>(v)), "r"(id), "r"(n)
        : "memory");
    return r != 0;
}

// Every thread of every CTA in the cluster arrives, then waits for all of them.
__device__ __forceinline__ void cluster_sync()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t cluster_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Thread t of warp w (w = warp index within its warpgroup) reads tensor-memory lane 32 w + t,
// 16 consecutive 32-bit columns starting at `taddr`'s column.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace knp_gb300
