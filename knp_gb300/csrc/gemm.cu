// BF16 GEMM on the tcgen05 tensor cores, pipelined: D[M x N] (FP32, row-major) = A[M x K] * B[N x K]^T
// with A and B BF16, row-major, K contiguous.
//
// One CTA computes one 128 x 128 tile of D over the whole K range in chunks of 64. Four warps copy
// the chunks of A and B into a ring of kStages shared-memory stages (cp.async, 16 bytes per thread
// and copy, zero-filled past the matrix edges) in the canonical no-swizzle K-major layout of
// tcgen05.cuh; one thread of a fifth warp issues the MMAs of each staged chunk (four K = 16 slices,
// FP32 accumulator in tensor memory) and commits them to the stage's `empty` barrier, so the copies
// of later chunks overlap the MMAs of earlier ones. The same four warps then read the accumulator
// (tcgen05.ld, one row per thread) and store it. Every wait is bounded: a timeout sets bit 0 of
// *err, stops the loops, drains the issued MMAs (bounded) and frees the tensor memory.
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "kernels.h"
#include "tcgen05.cuh"

namespace knp_gb300
{
namespace
{

constexpr int kBM = 128, kBN = 128, kBK = 64;
constexpr int kStages = 4;
constexpr int kCopyWarps = 4;
constexpr int kCopyThreads = 32 * kCopyWarps;
constexpr int kThreads = kCopyThreads + 32;  // + the MMA warp
constexpr uint32_t kTileBytes = kBM * kBK * 2;  // 16 KB: one operand chunk (kBN == kBM)
constexpr uint32_t kStageBytes = 2 * kTileBytes;
constexpr uint32_t kSbo = (kBK / 8) * 128;  // bytes between core matrices adjacent along M / N
constexpr uint32_t kLbo = 128;              // bytes between core matrices adjacent along K
constexpr uint32_t kWait = 1u << 22;        // polls (of up to tc::kSuspendNs each) before a wait gives up
static_assert(kBN == kBM, "A and B chunks share one layout");

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, uint32_t src_bytes)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Copies chunk [k0, k0 + 64) of rows [r0, r0 + 128) of a row-major [rows][K] BF16 matrix into the
// stage tile at `dst` (shared address). Copy thread t handles 16-byte units u = t + 128 i: row
// r0 + 8 (u / 64) + u % 8, K group (u / 8) % 8, so a warp's 32 units fill 512 contiguous bytes.
__device__ __forceinline__ void copy_chunk(const __nv_bfloat16 *__restrict__ m, int rows, int K, int r0, int k0,
                                           uint32_t dst, int t)
{
#pragma unroll
    for (int i = 0; i < (kBM * kBK / 8) / kCopyThreads; ++i)
    {
        const int u = t + kCopyThreads * i;
        const int r = 8 * (u >> 6) + (u & 7), g = (u >> 3) & 7;
        const int gr = r0 + r, gk = k0 + 8 * g;
        const int left = K - gk;
        const uint32_t bytes = (gr < rows && left > 0) ? (left >= 8 ? 16u : 2u * static_cast<uint32_t>(left)) : 0u;
        const __nv_bfloat16 *src = bytes ? m + static_cast<size_t>(gr) * K + gk : m;
        cp_async16(dst + tc::core_offset(r, 8 * g, kLbo, kSbo), src, bytes);
    }
}

// mbar_wait that also stops as soon as another role of the CTA has given up.
__device__ __forceinline__ bool wait_or_fail(uint64_t *mbar, uint32_t parity, const volatile int *fail)
{
    for (uint32_t i = 0; i < kWait; ++i)
    {
        if (tc::mbar_try_wait(mbar, parity)) return true;
        if (*fail) return false;
    }
    return false;
}

__global__ void __launch_bounds__(kThreads, 1) gemm_pipe_kernel(
    const __nv_bfloat16 *__restrict__ A, const __nv_bfloat16 *__restrict__ B, float *__restrict__ D, int M, int N,
    int K, unsigned int *err)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[kStages], empty[kStages], acc_full, drain;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kBN;
    const int nk = (K + kBK - 1) / kBK;
    if (warp == 0) tc::tmem_alloc(&tmem_slot, kBN);
    if (threadIdx.x == 0)
    {
        for (int s = 0; s < kStages; ++s)
        {
            tc::mbar_init(&full[s], kCopyThreads);
            tc::mbar_init(&empty[s], 1);
        }
        tc::mbar_init(&acc_full, 1);
        tc::mbar_init(&drain, 1);
        s_fail = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const uint32_t base = tc::smem_u32(smem);

    if (warp < kCopyWarps)
    {
        // Copies: chunk c into stage c % kStages once the MMAs of chunk c - kStages are done; the
        // stage is published (after its copies landed and are made visible to the tensor cores)
        // kStages - 1 chunks later, so that many chunks' copies are in flight.
        const int t = threadIdx.x;
        bool ok = true;
        int published = 0;
        auto publish = [&](int c)
        {
            tc::fence_async_smem();
            tc::mbar_arrive(&full[c % kStages]);
        };
        for (int c = 0; c < nk; ++c)
        {
            const int s = c % kStages;
            if (c >= kStages && ok && !wait_or_fail(&empty[s], ((c / kStages) - 1) & 1, &s_fail))
            {
                ok = false;
                s_fail = 1;
            }
            if (!ok || s_fail) break;  // no copies into a stage the tensor cores may still read
            copy_chunk(A, M, K, m0, c * kBK, base + s * kStageBytes, t);
            copy_chunk(B, N, K, n0, c * kBK, base + s * kStageBytes + kTileBytes, t);
            cp_async_commit();
            if (c >= kStages - 1)
            {
                cp_async_wait<kStages - 1>();
                publish(published++);
            }
        }
        cp_async_wait<0>();
        while (published < nk && ok && !s_fail) publish(published++);
        if (!ok) atomicOr(err, 1u);

        // Epilogue: thread t reads accumulator lane t (row m0 + t) and stores its kBN columns. The
        // decision to read is the same in all four warps (bar.red.and over their 128 threads).
        const bool done = wait_or_fail(&acc_full, 0, &s_fail);
        tc::fence_after_sync();
        if (tc::named_sync_and(1, kCopyThreads, done && !s_fail))
        {
            const int row = m0 + t;
            const uint32_t lane_base = static_cast<uint32_t>(32 * warp) << 16;
#pragma unroll 1
            for (int c0 = 0; c0 < kBN; c0 += 16)
            {
                float v[16];
                tc::tmem_ld16(tmem + lane_base + c0, v);
                if (row < M)
                {
                    float *d = D + static_cast<size_t>(row) * N + n0 + c0;
                    if (n0 + c0 + 16 <= N && (reinterpret_cast<uintptr_t>(d) & 15u) == 0)
                    {
#pragma unroll
                        for (int q = 0; q < 4; ++q)
                            reinterpret_cast<float4 *>(d)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                    }
                    else
                    {
#pragma unroll
                        for (int i = 0; i < 16; ++i)
                            if (n0 + c0 + i < N) d[i] = v[i];
                    }
                }
            }
        }
        else if (t == 0)
        {
            atomicOr(err, 1u);
        }
    }
    else if (lane == 0)
    {
        // MMA issuer: the four K = 16 slices of each staged chunk, then one commit that frees the stage.
        constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, kBN);
        for (int c = 0; c < nk; ++c)
        {
            const int s = c % kStages;
            if (!wait_or_fail(&full[s], (c / kStages) & 1, &s_fail))
            {
                s_fail = 1;
                break;
            }
            tc::fence_after_sync();
            const uint32_t sa = base + s * kStageBytes, sb = sa + kTileBytes;
#pragma unroll
            for (int j = 0; j < kBK / 16; ++j)
                tc::mma_bf16(tmem, tc::smem_desc(sa + j * 256, kLbo, kSbo), tc::smem_desc(sb + j * 256, kLbo, kSbo),
                             idesc, (c > 0 || j > 0) ? 1u : 0u);
            tc::commit(&empty[s]);
        }
        tc::commit(&acc_full);
        // Every issued MMA completes (bounded wait) before the tensor memory is freed.
        tc::commit(&drain);
        if (!tc::mbar_wait(&drain, 0, kWait)) s_fail = 1;
        if (s_fail) atomicOr(err, 1u);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kBN);
}

}  // namespace
}  // namespace knp_gb300

namespace knp_gb300
{
int bf16_gemm_tn_simple(const void *A, const void *B, float *D, int M, int N, int K, unsigned int *d_err, cudaStream_t s);

// D = A * B^T (see knp_gb300_bf16_gemm_tn). The pipelined kernel needs 16-byte aligned rows (K a
// multiple of 8, 16-byte aligned A and B); other shapes take the single-stage kernel.
int bf16_gemm_tn(const void *A, const void *B, float *D, int M, int N, int K, unsigned int *d_err, cudaStream_t s)
{
    if (M < 1 || N < 1 || K < 1 || !A || !B || !D || !d_err) return -1;
    const bool aligned = K % 8 == 0 && (reinterpret_cast<uintptr_t>(A) & 15u) == 0 && (reinterpret_cast<uintptr_t>(B) & 15u) == 0;
    if (!aligned) return bf16_gemm_tn_simple(A, B, D, M, N, K, d_err, s);
    static const cudaError_t attr =
        cudaFuncSetAttribute(gemm_pipe_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kStages * kStageBytes);
    if (attr != cudaSuccess) return -3;
    dim3 grid((M + kBM - 1) / kBM, (N + kBN - 1) / kBN);
    gemm_pipe_kernel<<<grid, kThreads, kStages * kStageBytes, s>>>(static_cast<const __nv_bfloat16 *>(A),
                                                                   static_cast<const __nv_bfloat16 *>(B), D, M, N, K, d_err);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
}  // namespace knp_gb300
