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
//
// When K is a multiple of 8, the chunks are loaded by TMA instead (gemm_tma_kernel): each operand is
// described to the TMA unit as a 2-D tensor (K, rows) whose 64 x 128 box (128 bytes of K per row)
// lands in shared memory in the 128-byte swizzled K-major layout the MMA reads directly; one thread
// issues the two copies of a stage and the stage's mbarrier counts their bytes; rows and K past the
// matrix edge arrive as zeros. Tiles are few when M and N are small and K large (weight gradients):
// the K range is then split over up to 16 CTAs per tile, each writing its partial tile to a
// workspace, and a second kernel adds the partials in split order, so results
// do not depend on scheduling.
#include <algorithm>
#include <cstdint>
#include <map>
#include <mutex>

#include <cuda.h>
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

__device__ __forceinline__ void mbar_expect_tx(uint64_t *mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(mbar)), "r"(bytes)
                 : "memory");
}

// TMA load of the 2-D box at (x, y) of `map` into shared memory at `dst`, completing its bytes on the
// mbarrier's transaction count.
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint64_t *mbar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(tc::smem_u32(mbar))
        : "memory");
}

constexpr int kTmaThreads = 128;

// Tile shapes of the TMA-fed kernel: 128 x kTN (kTN = 128, or 256 for large GEMMs: one MMA of
// N = 256 reads its 8 KB of A per 16-deep step for twice the work, halving shared-memory operand
// traffic per FLOP). Stages: as many as fit the 227 KB of shared memory.
template <int kTN>
struct TmaTile
{
    static constexpr uint32_t kBBytes = kTN * kBK * 2;
    static constexpr uint32_t kStage = kTileBytes + kBBytes;
    static constexpr int kStages = kTN == 128 ? 6 : 4;
    static constexpr uint32_t kSmem = kStages * kStage + 1024;  // + alignment slack
};

// One 128 x kTN tile of D (or of split blockIdx.z's partial, into `out` with row stride N) over
// chunks [blockIdx.z * cps, min(nk, (blockIdx.z + 1) * cps)). Warp 0 lane 0 issues the TMA copies,
// warp 1 lane 0 the MMAs; all four warps read the accumulator back.
template <int kTN>
__global__ void __launch_bounds__(kTmaThreads, 1) gemm_tma_kernel(
    const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, float *__restrict__ out, int M,
    int N, int K, int cps, size_t split_stride, unsigned int *err)
{
    using Tile = TmaTile<kTN>;
    constexpr int kTmaStages = Tile::kStages;
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t full[kTmaStages], empty[kTmaStages], acc_full, drain;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.x * kBM, n0 = blockIdx.y * kTN;
    const int nk = (K + kBK - 1) / kBK;
    const int c0 = blockIdx.z * cps, c1 = min(nk, c0 + cps);
    float *dst = out + blockIdx.z * split_stride;
    if (warp == 0) tc::tmem_alloc(&tmem_slot, kTN);
    if (threadIdx.x == 0)
    {
        for (int s = 0; s < kTmaStages; ++s)
        {
            tc::mbar_init(&full[s], 1);
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
    const uint32_t base = (tc::smem_u32(smem) + 1023u) & ~1023u;  // TMA boxes on 1024-byte boundaries

    if (warp == 0 && lane == 0)
    {
        int issued = 0;
        for (int c = c0; c < c1; ++c)
        {
            const int i = c - c0, s = i % kTmaStages;
            if (i >= kTmaStages && !wait_or_fail(&empty[s], ((i / kTmaStages) - 1) & 1, &s_fail))
            {
                s_fail = 1;
                break;
            }
            const uint32_t sa = base + s * Tile::kStage;
            mbar_expect_tx(&full[s], Tile::kStage);
            tma_load_2d(sa, &ta, c * kBK, m0, &full[s]);
            tma_load_2d(sa + kTileBytes, &tb, c * kBK, n0, &full[s]);
            issued = i + 1;
        }
        // Copies still in flight after a failed wait land before the CTA leaves (bounded).
        for (int i = max(0, issued - kTmaStages); i < issued; ++i)
            if (!tc::mbar_wait(&full[i % kTmaStages], (i / kTmaStages) & 1, kWait)) s_fail = 1;
    }
    else if (warp == 1 && lane == 0)
    {
        constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, kTN);
        for (int c = c0; c < c1; ++c)
        {
            const int i = c - c0, s = i % kTmaStages;
            if (!wait_or_fail(&full[s], (i / kTmaStages) & 1, &s_fail))
            {
                s_fail = 1;
                break;
            }
            tc::fence_after_sync();
            const uint32_t sa = base + s * Tile::kStage, sb = sa + kTileBytes;
#pragma unroll
            for (int j = 0; j < kBK / 16; ++j)
                tc::mma_bf16(tmem, tc::smem_desc_sw128(sa + j * 32, 1024), tc::smem_desc_sw128(sb + j * 32, 1024),
                             idesc, (i > 0 || j > 0) ? 1u : 0u);
            tc::commit(&empty[s]);
        }
        tc::commit(&acc_full);
        tc::commit(&drain);
        if (!tc::mbar_wait(&drain, 0, kWait)) s_fail = 1;
    }
    __syncwarp();
    // Epilogue: thread t reads accumulator lane t (row m0 + t); an empty chunk range leaves zeros.
    const bool done = c1 <= c0 || wait_or_fail(&acc_full, 0, &s_fail);
    tc::fence_after_sync();
    const bool ok = tc::named_sync_and(1, kTmaThreads, done && !s_fail);
    if (ok)
    {
        const int row = m0 + threadIdx.x;
        const uint32_t lane_base = static_cast<uint32_t>(32 * warp) << 16;
#pragma unroll 1
        for (int q0 = 0; q0 < kTN; q0 += 16)
        {
            float v[16];
            if (c1 > c0)
                tc::tmem_ld16(tmem + lane_base + q0, v);
            else
                for (int i = 0; i < 16; ++i) v[i] = 0.0f;
            if (row < M)
            {
                float *d = dst + static_cast<size_t>(row) * N + n0 + q0;
                if (n0 + q0 + 16 <= N && (reinterpret_cast<uintptr_t>(d) & 15u) == 0)
                {
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        reinterpret_cast<float4 *>(d)[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                }
                else
                {
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                        if (n0 + q0 + i < N) d[i] = v[i];
                }
            }
        }
    }
    else if (threadIdx.x == 0)
    {
        atomicOr(err, 1u);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, kTN);
}

// D = sum over the splits of ws[z] (split order), n elements.
__global__ void split_sum_kernel(const float *__restrict__ ws, float *__restrict__ D, size_t n, int splits)
{
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        float s = ws[i];
        for (int z = 1; z < splits; ++z) s = __fadd_rn(s, ws[z * n + i]);
        D[i] = s;
    }
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_tiled()
{
    static EncodeTiled fn = []
    {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
        {
            cudaGetLastError();
            return static_cast<EncodeTiled>(nullptr);
        }
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

// The (K, rows) view of a row-major [rows][K] BF16 matrix (K a multiple of 8), loaded in 64 x 128
// boxes with the 128-byte swizzle.
bool sw128_map(CUtensorMap *map, const void *ptr, int rows, int K, int box_rows = kBM)
{
    const EncodeTiled fn = encode_tiled();
    if (!fn) return false;
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(K), static_cast<cuuint64_t>(rows)};
    const cuuint64_t strides[1] = {static_cast<cuuint64_t>(K) * 2};
    const cuuint32_t box[2] = {kBK, static_cast<cuuint32_t>(box_rows)};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The kernel's dynamic shared memory limit raised once per (kernel, device): a per-device setting.
template <class Kernel>
cudaError_t smem_limit_once(Kernel kernel, int bytes, int dev)
{
    static std::mutex mu;
    static std::map<std::pair<const void *, int>, cudaError_t> done;
    std::lock_guard<std::mutex> lock(mu);
    const std::pair<const void *, int> key{reinterpret_cast<const void *>(kernel), dev};
    const auto it = done.find(key);
    if (it != done.end()) return it->second;
    return done[key] = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

// Stream-ordered pool of the split-K workspaces of device `dev` (memory kept by the pool between
// calls). Allocating on the call's stream keeps concurrent streams apart and lets a call be captured
// in a CUDA graph (the allocation becomes a graph memory node).
cudaMemPool_t split_pool(int dev)
{
    static std::mutex mu;
    static std::map<int, cudaMemPool_t> pools;
    std::lock_guard<std::mutex> lock(mu);
    const auto it = pools.find(dev);
    if (it != pools.end()) return it->second;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t pool = nullptr;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess)
    {
        cudaGetLastError();
        return pools[dev] = nullptr;
    }
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    return pools[dev] = pool;
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
    CUtensorMap ta, tb;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int tiles_m = (M + kBM - 1) / kBM;
    const int nk = (K + kBK - 1) / kBK;
    // 128 x 256 tiles when they alone fill every SM (large GEMMs; no K split then).
    if (N >= 256 && tiles_m * ((N + 255) / 256) >= sms && sw128_map(&ta, A, M, K) && sw128_map(&tb, B, N, K, 256))
    {
        if (smem_limit_once(gemm_tma_kernel<256>, static_cast<int>(TmaTile<256>::kSmem), dev) != cudaSuccess) return -3;
        dim3 grid(tiles_m, (N + 255) / 256, 1);
        gemm_tma_kernel<256><<<grid, kTmaThreads, TmaTile<256>::kSmem, s>>>(ta, tb, D, M, N, K, nk, 0, d_err);
        return cudaGetLastError() == cudaSuccess ? 0 : -3;
    }
    if (sw128_map(&ta, A, M, K) && sw128_map(&tb, B, N, K))
    {
        if (smem_limit_once(gemm_tma_kernel<128>, static_cast<int>(TmaTile<128>::kSmem), dev) != cudaSuccess) return -3;
        const int tiles_n = (N + kBN - 1) / kBN, tiles = tiles_m * tiles_n;
        // Split K when the tiles leave most SMs idle and each split keeps at least 4 chunks.
        int splits = 1;
        if (tiles * 2 <= sms) splits = std::max(1, std::min({16, nk / 4, sms / tiles}));
        const int cps = (nk + splits - 1) / splits;
        splits = (nk + cps - 1) / cps;
        const size_t mn = static_cast<size_t>(M) * N;
        float *ws = nullptr;
        if (splits > 1)
        {
            const cudaMemPool_t pool = split_pool(dev);
            if (!pool || cudaMallocFromPoolAsync(reinterpret_cast<void **>(&ws), mn * splits * sizeof(float), pool, s) !=
                             cudaSuccess)
            {
                cudaGetLastError();
                ws = nullptr;
                splits = 1;
            }
        }
        const int cps_used = splits > 1 ? cps : nk;
        dim3 grid(tiles_m, tiles_n, splits);
        gemm_tma_kernel<128><<<grid, kTmaThreads, TmaTile<128>::kSmem, s>>>(ta, tb, splits > 1 ? ws : D, M, N, K,
                                                                          cps_used, splits > 1 ? mn : 0, d_err);
        if (splits > 1)
        {
            const int blocks = static_cast<int>(std::min<size_t>((mn + 255) / 256, 8ull * sms));
            split_sum_kernel<<<blocks, 256, 0, s>>>(ws, D, mn, splits);
            cudaFreeAsync(ws, s);
        }
        return cudaGetLastError() == cudaSuccess ? 0 : -3;
    }
    if (smem_limit_once(gemm_pipe_kernel, static_cast<int>(kStages * kStageBytes), dev) != cudaSuccess) return -3;
    dim3 grid((M + kBM - 1) / kBM, (N + kBN - 1) / kBN);
    gemm_pipe_kernel<<<grid, kThreads, kStages * kStageBytes, s>>>(static_cast<const __nv_bfloat16 *>(A),
                                                                   static_cast<const __nv_bfloat16 *>(B), D, M, N, K, d_err);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}
}  // namespace knp_gb300
