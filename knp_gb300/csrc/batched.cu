// Batched form on 5th-generation tensor cores.
//
// bf16_gemm_tn: D[M x N] (FP32) = A[M x K] * B[N x K]^T with BF16 operands (row-major, K
// contiguous), tcgen05.mma kind::f16 with the accumulator in tensor memory. Used to validate the
// tcgen05 encodings and as a library GEMM of spike matrices.
#include <algorithm>
#include <cstdint>
#include <memory>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "kernels.h"
#include "tcgen05.cuh"

namespace knp_gb300
{
namespace
{

constexpr int kGemmM = 128;
constexpr int kGemmN = 64;
constexpr int kGemmK = 64;  // K chunk staged in shared memory
constexpr uint32_t kWaitLimit = 1u << 24;

// Stage rows [r0, r0 + rows) x K-chunk [k0, k0 + kGemmK) of a row-major BF16 matrix into the
// canonical no-swizzle K-major layout (zero outside the matrix).
__device__ __forceinline__ void stage_tile(
    const __nv_bfloat16 *__restrict__ src, int n_rows, int K, int r0, int k0, int rows, uint8_t *dst, uint32_t lbo,
    uint32_t sbo)
{
    // 16-byte units: (row, 8-element K group)
    const int groups = kGemmK / 8;
    for (int u = threadIdx.x; u < rows * groups; u += blockDim.x)
    {
        const int r = u / groups, g = u % groups;
        const int gr = r0 + r, gk = k0 + g * 8;
        uint4 v = make_uint4(0, 0, 0, 0);
        if (gr < n_rows)
        {
            if (gk + 8 <= K && (reinterpret_cast<uintptr_t>(src + static_cast<size_t>(gr) * K + gk) & 15u) == 0)
            {
                v = *reinterpret_cast<const uint4 *>(src + static_cast<size_t>(gr) * K + gk);
            }
            else
            {
                __nv_bfloat16 tmp[8];
#pragma unroll
                for (int e = 0; e < 8; ++e)
                    tmp[e] = (gk + e < K) ? src[static_cast<size_t>(gr) * K + gk + e] : __float2bfloat16(0.0f);
                v = *reinterpret_cast<uint4 *>(tmp);
            }
        }
        *reinterpret_cast<uint4 *>(dst + tc::core_offset(r, g * 8, lbo, sbo)) = v;
    }
}

__global__ void __launch_bounds__(128) gemm_tn_kernel(
    const __nv_bfloat16 *__restrict__ A, const __nv_bfloat16 *__restrict__ B, float *__restrict__ D, int M, int N,
    int K, unsigned int *err)
{
    __shared__ __align__(128) uint8_t sa[kGemmM * kGemmK * 2];
    __shared__ __align__(128) uint8_t sb[kGemmN * kGemmK * 2];
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) uint64_t mbar;
    const int m0 = blockIdx.x * kGemmM, n0 = blockIdx.y * kGemmN;
    const uint32_t lbo = 128, sbo_a = (kGemmK / 8) * 128, sbo_b = (kGemmK / 8) * 128;
    if (threadIdx.x < 32) tc::tmem_alloc(&tmem_slot, kGemmN);
    if (threadIdx.x == 0) tc::mbar_init(&mbar, 1);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kGemmM, kGemmN);
    bool ok = true;
    uint32_t phase = 0;
    for (int k0 = 0; k0 < K; k0 += kGemmK)
    {
        stage_tile(A, M, K, m0, k0, kGemmM, sa, lbo, sbo_a);
        stage_tile(B, N, K, n0, k0, kGemmN, sb, lbo, sbo_b);
        tc::fence_async_smem();
        __syncthreads();
        if (threadIdx.x == 0)
        {
            tc::fence_after_sync();
            for (int j = 0; j < kGemmK / 16; ++j)
            {
                const uint64_t da = tc::smem_desc(tc::smem_u32(sa) + j * 256, lbo, sbo_a);
                const uint64_t db = tc::smem_desc(tc::smem_u32(sb) + j * 256, lbo, sbo_b);
                tc::mma_bf16(tmem, da, db, idesc, (k0 > 0 || j > 0) ? 1u : 0u);
            }
            tc::commit(&mbar);
        }
        // Every thread waits for the MMAs of this chunk before the buffers are overwritten; the
        // outcome is made block-uniform so that no warp-collective instruction runs partially.
        const bool waited = tc::mbar_wait(&mbar, phase, kWaitLimit);
        phase ^= 1u;
        tc::fence_after_sync();
        ok = (__syncthreads_and(waited ? 1 : 0) != 0) && ok;
    }
    if (!ok)
    {
        if (threadIdx.x == 0) atomicOr(err, 1u);
    }
    else
    {
        const int row = m0 + (threadIdx.x >> 5) * 32 + (threadIdx.x & 31);
        const uint32_t lane_base = static_cast<uint32_t>((threadIdx.x >> 5) * 32) << 16;
        for (int c = 0; c < kGemmN; c += 16)
        {
            float v[16];
            tc::tmem_ld16(tmem + lane_base + c, v);
            if (row < M)
#pragma unroll
                for (int i = 0; i < 16; ++i)
                    if (n0 + c + i < N) D[static_cast<size_t>(row) * N + n0 + c + i] = v[i];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) tc::tmem_dealloc(tmem, kGemmN);
}

}  // namespace

int bf16_gemm_tn(const void *A, const void *B, float *D, int M, int N, int K, unsigned int *d_err, cudaStream_t s)
{
    if (M < 1 || N < 1 || K < 1 || !A || !B || !D || !d_err) return -1;
    dim3 grid((M + kGemmM - 1) / kGemmM, (N + kGemmN - 1) / kGemmN);
    gemm_tn_kernel<<<grid, 128, 0, s>>>(static_cast<const __nv_bfloat16 *>(A), static_cast<const __nv_bfloat16 *>(B),
                                        D, M, N, K, d_err);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // namespace knp_gb300

// ------------------------------------------------------------------------------------------------
// Batched LIF network (batched / precision form).
//
// B independent samples of a feed-forward LIF network (layers of sizes n_0 -> n_1 -> ... -> n_L,
// all-to-all, delay 1) advance together. Semantics per neuron are the reference LIF
// (knp/backends/cpu/cpu-library/include/knp/backends/cpu-library/impl/populations/lif/lif_impl.h:33-86):
// outside the refractory period V = V * leak + I, spike iff V > threshold, then V = reset and the
// counter = period; inside it the counter counts down and input is ignored. Layer l's input at
// step t is the spikes of layer l - 1 at step t - 1 times W_l (delay 1); layer 0 is the input,
// whose spike of source i for sample b at step t is the counter-based Bernoulli draw
// rand64(key, (t * B + b) * n_0 + i) >> 11 < rate[b][i] * 2^53. Sample b runs steps [0, T_b).
//
// Each step is a BF16 GEMM of the 0/1 spike matrix (exact in BF16) against BF16 weights with FP32
// accumulation in tensor memory. One CTA owns (layer, 128-sample tile, 32-neuron tile); its weight
// tile stays in shared memory and its neurons' LIF state in registers for the whole run.
//
// Spike matrices are kept in global memory already in the layout the tensor cores read: for each
// layer, step parity and 128-sample tile, the consumer's K range is cut into 128-input chunks of
// 32 KB each in the canonical no-swizzle K-major form (8 x 16-byte core matrices). A producer CTA
// writes its 128 x 32 block of 0/1 BF16 spikes there (512 16-byte stores), so a consumer needs no
// conversion: a loader thread streams the chunks into a 4-stage shared-memory ring with bulk copies
// (cp.async.bulk, completion on mbarriers), two issuer threads run the MMAs of alternate chunks
// into separate accumulators, and the other warps draw the next step's input spikes meanwhile.
// Samples are processed sorted by decreasing T, so finished samples leave whole M-tiles idle.
// Steps are separated by a grid barrier; the kernel is launched cooperatively (every CTA resident)
// and every wait is bounded.
namespace knp_gb300
{
namespace
{

constexpr int kBM = 128, kBN = 32, kBK = 128, kMaxLayers = 4, kMaxItems = 512;
constexpr int kPairN = 2 * kBN;  // neurons of a CTA pair's MMA tile; each CTA finalises kBN of them
constexpr int kIssuers = 2;                           // issuer q runs the MMAs of chunks c with c % 2 == q
constexpr int kMinStages = 3, kMaxStages = 5;        // operand ring depths the autotuner tries
constexpr uint32_t kChunkBytes = kBM * kBK * 2;       // one 128 x 128 BF16 chunk
constexpr uint32_t kSboA = (kBK / 8) * 128;           // row-group stride of a chunk (16 core matrices)
constexpr int kLoaderWarp = kIssuers;                 // lane 0 of this warp streams the chunks
constexpr int kFirstDrawWarp = kLoaderWarp + 1;       // warps from here on draw the input spikes
constexpr int kInCache = 12;                          // input words per drawing warp with cached thresholds
constexpr int kBatchThreads = 256;

struct BatchedNet
{
    int n_layers;
    uint32_t size[kMaxLayers + 1];
    uint32_t words[kMaxLayers + 1];   // ceil(size / 32)
    uint32_t kpad[kMaxLayers + 1];    // kpad[l] = size[l - 1] rounded up to 16 (layer l's K)
    uint32_t chunks[kMaxLayers + 1];  // chunks[l] = ceil(kpad[l] / 128)
    const __nv_bfloat16 *w[kMaxLayers];
    float leak[kMaxLayers], thr[kMaxLayers], reset[kMaxLayers];
    uint32_t refract[kMaxLayers];
    uint32_t batch;
    const uint32_t *perm;  // slot -> sample
    const uint32_t *act;   // [t_max]: slots still running at step t (slots sorted by decreasing T)
    const unsigned long long *rate_thr;  // [batch][size[0]] by sample: rate * 2^53, the draw's threshold
    // Optional per-sample layer sizes ([batch] by sample, <= size[l]); neurons and inputs beyond a
    // sample's size do not exist for it (never spike). Null: every sample has the full sizes.
    const uint32_t *sample_size[kMaxLayers + 1];
    unsigned long long key;
    uint32_t t_max;
    // spk[l][p]: spikes of layer l (l < n_layers) at steps of parity p, as layer l + 1's A operand:
    // [m tile][chunks[l + 1]][kChunkBytes].
    uint8_t *spk[kMaxLayers][2];
    int *counts;           // [batch][size[L]] by sample
    uint32_t *record;      // [t_max][sum_l batch * words[l]] by sample, or null
    unsigned long long rec_off[kMaxLayers + 1];
    unsigned long long rec_stride;
    unsigned long long *events;
    unsigned int *err;
    unsigned int *barrier;  // arrival counter of the grid barrier
    float *xbuf;                  // [n_items][kBM][kBN]: partial sums a CTA hands to its pair partner
    unsigned int *pair_flag;      // [n_items / 2]: arrivals of the pair exchange (2 per computed step)
    uint32_t n_items;
    uint16_t item_layer[kMaxItems];
    uint16_t item_m[kMaxItems];
    uint16_t item_n[kMaxItems];  // kPairN-neuron tile index
    uint8_t item_k[kMaxItems];   // K half: items 2i and 2i + 1 are the two halves of one tile
};

// Grid barrier on a counter that only grows: arrival k (0-based) belongs to barrier k / n_blocks,
// which completes when the counter reaches (k / n_blocks + 1) * n_blocks. One release add per CTA,
// acquire polls (bounded) until then.
__device__ __forceinline__ bool grid_sync(unsigned int *count, unsigned int n_blocks, uint32_t limit)
{
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        unsigned int old;
        asm volatile("atom.add.release.gpu.global.u32 %0, [%1], 1;" : "=r"(old) : "l"(count) : "memory");
        const unsigned int target = (old / n_blocks + 1) * n_blocks;
        int ok = 0;
        for (uint32_t i = 0; i < limit; ++i)
        {
            unsigned int cur;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(count) : "memory");
            if (static_cast<int>(cur - target) >= 0)
            {
                ok = 1;
                break;
            }
        }
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

// Exchange barrier of a CTA pair: both CTAs add 1 after writing their partial sums; a CTA goes on
// once the counter reaches `target + 2` (bounded polls). Returns false on timeout (block-uniform).
__device__ __forceinline__ bool pair_sync(unsigned int *flag, unsigned int target, uint32_t limit)
{
    __shared__ int pok_s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(flag) : "memory");
        int ok = 0;
        for (uint32_t i = 0; i < limit; ++i)
        {
            unsigned int cur;
            asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(flag) : "memory");
            if (static_cast<int>(cur - (target + 2u)) >= 0)
            {
                ok = 1;
                break;
            }
        }
        pok_s = ok;
    }
    __syncthreads();
    return pok_s != 0;
}

// Per (sample, input): the 53-bit threshold that the input draw is compared with.
__global__ void rate_threshold_kernel(const float *rates, unsigned long long *thr, size_t n)
{
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) thr[i] = static_cast<unsigned long long>(static_cast<double>(rates[i]) * 9007199254740992.0);
}

// Bulk copy global -> shared (both 16-byte aligned, size a multiple of 16) completing on `mbar`.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *mbar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     tc::smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(tc::smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(mbar)),
                 "r"(bytes)
                 : "memory");
}

// The low 8 bits of x as eight BF16 values 0 or 1.0 (0x3F80), bit i -> element i.
__device__ __forceinline__ uint4 bf16_bits(uint32_t x)
{
    uint4 v;
    v.x = ((x & 1u) ? 0x3F80u : 0u) | ((x & 2u) ? 0x3F800000u : 0u);
    v.y = ((x & 4u) ? 0x3F80u : 0u) | ((x & 8u) ? 0x3F800000u : 0u);
    v.z = ((x & 16u) ? 0x3F80u : 0u) | ((x & 32u) ? 0x3F800000u : 0u);
    v.w = ((x & 64u) ? 0x3F80u : 0u) | ((x & 128u) ? 0x3F800000u : 0u);
    return v;
}

// Byte offset of element (row r, input k) of a layer's spike matrix inside one 128-sample tile.
__device__ __forceinline__ uint32_t spk_offset(uint32_t r, uint32_t k)
{
    return (k / kBK) * kChunkBytes + (r >> 3) * kSboA + ((k % kBK) >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

template <int kStages>
__global__ void __launch_bounds__(kBatchThreads, 1) batched_lif_kernel(BatchedNet net)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) uint64_t full[kStages];   // chunk in stage b has landed (loader's expect_tx)
    __shared__ __align__(8) uint64_t empty[kStages];  // MMAs that read stage b have completed (commit)
    __shared__ __align__(8) uint64_t done[kIssuers]; // all of an issuer's MMAs of a step have completed
    __shared__ uint32_t sbits[kBM];
    __shared__ unsigned long long s_events;
    const uint32_t item = blockIdx.x;
    const int layer = net.item_layer[item];  // 1..L
    const uint32_t m_tile = net.item_m[item];
    const uint32_t m0 = m_tile * kBM;
    // The pair's tile is neurons np0 .. np0 + 63 over all K; this CTA multiplies K half kh of it and
    // finalises neurons n0 .. n0 + 31 (half kh of the tile) after adding the partner's partial sums.
    const uint32_t kh = net.item_k[item];
    const uint32_t np0 = net.item_n[item] * kPairN;
    const uint32_t n0 = np0 + kBN * kh;
    const uint32_t K = net.size[layer - 1], Kp = net.kpad[layer], N = net.size[layer];
    const uint32_t wn = net.words[layer];
    const uint32_t n_chunks_all = net.chunks[layer];
    const uint32_t c_mid = (n_chunks_all + 1) / 2;
    const uint32_t c_lo = kh ? c_mid : 0u, c_hi = kh ? n_chunks_all : c_mid;
    const uint32_t n_chunks = c_hi - c_lo;  // this CTA's chunks
    const uint32_t Kw = c_mid * kBK;        // K extent of the weight tile (the larger half)
    // Shared memory: weight tile [kPairN x Kw] (K-major core matrices), kStages chunk stages.
    uint8_t *sW = smem;
    uint8_t *sA = smem + static_cast<size_t>(kPairN) * Kw * 2;
    const uint32_t sbo_w = (Kw / 8) * 128;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // Weight tile rows np0..np0+63 (zero beyond N), inputs c_lo * 128 + [0, Kw) (zero beyond K).
    for (uint32_t u = threadIdx.x; u < kPairN * (Kw / 8); u += blockDim.x)
    {
        const uint32_t r = u / (Kw / 8), g = u % (Kw / 8), n = np0 + r, k = g * 8, kg = c_lo * kBK + k;
        __nv_bfloat16 tmp[8];
#pragma unroll
        for (int e = 0; e < 8; ++e)
            tmp[e] = (n < N && kg + e < K) ? net.w[layer - 1][static_cast<size_t>(n) * K + kg + e]
                                           : __float2bfloat16(0.0f);
        *reinterpret_cast<uint4 *>(sW + tc::core_offset(r, k, 128, sbo_w)) = *reinterpret_cast<uint4 *>(tmp);
    }
    // Tensor memory: issuer q accumulates the 64-column tile into columns [64 q, 64 q + 64).
    if (warp == 0) tc::tmem_alloc(&tmem_slot, kPairN * kIssuers);
    if (threadIdx.x == 0)
    {
        for (int b = 0; b < kStages; ++b)
        {
            tc::mbar_init(&full[b], 1);
            tc::mbar_init(&empty[b], 1);
        }
        for (int q = 0; q < kIssuers; ++q) tc::mbar_init(&done[q], 1);
        s_events = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, kPairN);
    // Matrix descriptors of stage 0 and of the weight tile's first K slice; the others follow by
    // adding byte offsets / 16 to the start-address field.
    const uint64_t dA0 = tc::smem_desc(tc::smem_u32(sA), 128, kSboA);
    const uint64_t dW0 = tc::smem_desc(tc::smem_u32(sW), 128, sbo_w);
    uint32_t seq = 0;        // chunks streamed by this CTA in earlier steps (stage = seq % kStages)
    uint32_t act_steps = 0;  // steps this CTA has computed (phase of done[])
    bool ok = true;
    unsigned long long my_events = 0;

    // Epilogue ownership, fixed for the run: thread (warp, lane) owns row 32 (warp % 4) + lane of the
    // tile and columns 16 (warp / 4) .. +15, so it keeps their LIF state in registers.
    const uint32_t er = 32u * (warp & 3) + lane;
    const uint32_t erow = m0 + er;
    const uint32_t cb = 16u * (warp >> 2);
    float V[16];
    uint32_t RC[16];
    int CNT[16];
#pragma unroll
    for (int i = 0; i < 16; ++i)
    {
        V[i] = 0.f;
        RC[i] = 0u;
        CNT[i] = 0;
    }
    const int li = layer - 1;
    const float leak = net.leak[li], thr = net.thr[li], rst = net.reset[li];
    const uint32_t per = net.refract[li];
    // This thread's sample: its own neuron count and its next layer's (the fan-out of its spikes).
    const uint32_t e_smp = erow < net.batch ? net.perm[erow] : 0u;
    const uint32_t my_n = (net.sample_size[layer] && erow < net.batch) ? net.sample_size[layer][e_smp] : N;
    const uint32_t my_fan_out =
        layer < net.n_layers ? ((net.sample_size[layer + 1] && erow < net.batch) ? net.sample_size[layer + 1][e_smp]
                                                                                  : net.size[layer + 1])
                             : 0u;

    // Input words drawn by this warp every step (drawing warps only: u = draw warp id + j * draw
    // warps in grid) and, for the first kInCache of them, this lane's threshold and sample.
    const uint32_t n_in = net.size[0], w0 = net.words[0];
    const uint64_t in_total = static_cast<uint64_t>(net.batch) * w0;
    const uint32_t dpb = (blockDim.x >> 5) - kFirstDrawWarp;
    const bool drawer = warp >= kFirstDrawWarp;
    const uint64_t gw = static_cast<uint64_t>(blockIdx.x) * dpb + (warp - kFirstDrawWarp),
                   nw = static_cast<uint64_t>(gridDim.x) * dpb;
    unsigned long long in_thr[kInCache];
    uint32_t in_smp[kInCache];
#pragma unroll
    for (int j = 0; j < kInCache; ++j)
    {
        const uint64_t u = gw + j * nw;
        in_thr[j] = 0;
        in_smp[j] = 0;
        if (drawer && u < in_total)
        {
            const uint32_t slot = static_cast<uint32_t>(u / w0), i = static_cast<uint32_t>(u % w0) * 32 + lane;
            in_smp[j] = net.perm[slot];
            if (i < n_in && (!net.sample_size[0] || i < net.sample_size[0][in_smp[j]]))
                in_thr[j] = net.rate_thr[static_cast<size_t>(in_smp[j]) * n_in + i];
        }
    }
    const size_t spk0_tile = static_cast<size_t>(net.chunks[1]) * kChunkBytes;
    const uint32_t kpad1 = net.kpad[1];
    // This warp's input words: gw, gw + nw, ... below in_total (as (slot, word) pairs).
    const uint32_t dr_items = (drawer && gw < in_total) ? static_cast<uint32_t>((in_total - 1 - gw) / nw + 1) : 0u;
    const uint32_t dr_slot0 = drawer ? static_cast<uint32_t>(gw / w0) : 0u;
    const uint32_t dr_wi0 = drawer ? static_cast<uint32_t>(gw % w0) : 0u;
    const uint32_t dr_step_q = static_cast<uint32_t>(nw / w0), dr_step_r = static_cast<uint32_t>(nw % w0);

    uint32_t b_next = net.act[0];
    for (uint32_t t = 0; t < net.t_max && ok; ++t)
    {
        const uint32_t b_act = b_next;
        if (t + 1 < net.t_max) b_next = net.act[t + 1];  // used next step; the load overlaps this one
        const bool active = m0 < b_act;
        if (threadIdx.x < kBM) sbits[threadIdx.x] = 0;
        if (active)
        {
            const uint8_t *src = net.spk[layer - 1][(t + 1) & 1] +
                                 (static_cast<size_t>(m_tile) * n_chunks_all + c_lo) * kChunkBytes;
            if (warp == kLoaderWarp && lane == 0)
            {
                // Loader: the chunks were written by other CTAs before the grid barrier (generic
                // proxy); the bulk copies read them through the async proxy.
                asm volatile("fence.proxy.async.global;" ::: "memory");
                for (uint32_t c = 0; c < n_chunks; ++c)
                {
                    const uint32_t sq = seq + c, b = sq % kStages;
                    if (sq >= kStages && !tc::mbar_wait(&empty[b], (sq / kStages - 1) & 1u, kWaitLimit)) ok = false;
                    mbar_arrive_expect_tx(&full[b], kChunkBytes);
                    bulk_load(sA + static_cast<size_t>(b) * kChunkBytes, src + static_cast<size_t>(c) * kChunkBytes,
                              kChunkBytes, &full[b]);
                }
            }
            else if (warp < kIssuers && lane == 0)
            {
                // Issuer q: chunks q, q + 2, ... of this half into its accumulator, then one commit
                // for the step.
                for (uint32_t c = warp; c < n_chunks; c += kIssuers)
                {
                    const uint32_t sq = seq + c, b = sq % kStages;
                    if (!tc::mbar_wait(&full[b], (sq / kStages) & 1u, kWaitLimit)) ok = false;
                    tc::fence_after_sync();
                    const uint64_t da = dA0 + b * (kChunkBytes >> 4);
                    const uint64_t db = dW0 + c * ((kBK / 8 * 128) >> 4);
                    const uint32_t kc = min(static_cast<uint32_t>(kBK), Kp - (c_lo + c) * kBK);
                    for (uint32_t j = 0; j < kc / 16; ++j)
                        tc::mma_bf16(tmem + kPairN * warp, da + j * 16, db + j * 16, idesc,
                                     (c >= static_cast<uint32_t>(kIssuers) || j > 0) ? 1u : 0u);
                    tc::commit(&empty[b]);
                }
                tc::commit(&done[warp]);
            }
        }
        // Input spikes of step t (layer 0), drawn by the drawing warps of every CTA: a warp makes one
        // 32-input word per item, one draw per lane. Each lane writes its BF16 0/1 into layer 1's A
        // layout; the ballot gives the word for the record and the event count.
        if (drawer)
        {
            uint8_t *d0 = net.spk[0][t & 1];
            const unsigned long long ctr_t = static_cast<unsigned long long>(t) * net.batch;
            const unsigned long long rec_t = net.record ? t * net.rec_stride + net.rec_off[0] : 0ull;
            auto emit = [&](uint32_t slot, uint32_t wi, bool bit, uint32_t smp)
            {
                const uint32_t i = wi * 32 + lane;
                if (i < kpad1)
                    *reinterpret_cast<uint16_t *>(d0 + (slot / kBM) * spk0_tile + spk_offset(slot % kBM, i)) =
                        bit ? 0x3F80u : 0u;
                const uint32_t word = __ballot_sync(0xffffffffu, bit);
                if (lane == 0 && slot < b_act)
                {
                    if (net.record) net.record[rec_t + static_cast<size_t>(smp) * w0 + wi] = word;
                    my_events += static_cast<unsigned long long>(__popc(word)) *
                                 (net.sample_size[1] ? net.sample_size[1][smp] : net.size[1]);
                }
            };
            auto draw = [&](uint32_t slot, uint32_t wi, unsigned long long thr64, uint32_t smp) -> bool
            {
                const uint32_t i = wi * 32 + lane;
                return slot < b_act && i < n_in && (rand64(net.key, (ctr_t + smp) * n_in + i) >> 11) < thr64;
            };
            // Word u = slot * w0 + wi advances by nw each item; (slot, wi) follow without division.
            // The cached items' draws are independent: all drawn first, then written.
            uint32_t slot = dr_slot0, wi = dr_wi0;
            bool bits[kInCache];
            uint32_t slots[kInCache], wis[kInCache];
#pragma unroll
            for (int j = 0; j < kInCache; ++j)
            {
                slots[j] = slot;
                wis[j] = wi;
                bits[j] = static_cast<uint32_t>(j) < dr_items && draw(slot, wi, in_thr[j], in_smp[j]);
                wi += dr_step_r;
                slot += dr_step_q;
                if (wi >= w0)
                {
                    wi -= w0;
                    ++slot;
                }
            }
#pragma unroll
            for (int j = 0; j < kInCache; ++j)
                if (static_cast<uint32_t>(j) < dr_items) emit(slots[j], wis[j], bits[j], in_smp[j]);
            for (uint32_t j = kInCache; j < dr_items; ++j)
            {
                const uint32_t i = wi * 32 + lane;
                const uint32_t smp = net.perm[slot];
                const bool exists = i < n_in && (!net.sample_size[0] || i < net.sample_size[0][smp]);
                emit(slot, wi, draw(slot, wi, exists ? net.rate_thr[static_cast<size_t>(smp) * n_in + i] : 0ull, smp),
                     smp);
                wi += dr_step_r;
                slot += dr_step_q;
                if (wi >= w0)
                {
                    wi -= w0;
                    ++slot;
                }
            }
        }
        if (active)
        {
            // Every issuer commits done[] once per computed step; waiting for both means no MMA of
            // this step is in flight.
            bool waited = true;
            for (int q = 0; q < kIssuers; ++q)
                waited = tc::mbar_wait(&done[q], act_steps & 1u, kWaitLimit) && waited;
            tc::fence_after_sync();
            ok = __syncthreads_and((waited && ok) ? 1 : 0) != 0;
            ++act_steps;
            seq += n_chunks;
            uint32_t mask = 0;
            // This half's partial sums of 16 columns at tile column `col` (issuer 0 + issuer 1).
            const uint32_t lane_base = (32u * (warp & 3)) << 16;
            auto partial = [&](uint32_t col, float *v)
            {
                if (n_chunks == 0)
                {
#pragma unroll
                    for (int i = 0; i < 16; ++i) v[i] = 0.0f;
                    return;
                }
                tc::tmem_ld16(tmem + lane_base + col, v);
                for (int q = 1; q < kIssuers; ++q)
                {
                    if (static_cast<uint32_t>(q) >= n_chunks) break;
                    float part[16];
                    tc::tmem_ld16(tmem + lane_base + kPairN * q + col, part);
#pragma unroll
                    for (int i = 0; i < 16; ++i) v[i] = __fadd_rn(v[i], part[i]);
                }
            };
            float acc[16];
            // Hand the partner the columns it finalises, then add its partial to ours: the total is
            // (K half 0) + (K half 1) on both sides.
            if (ok)
            {
                partial(kBN * (1u - kh) + cb, acc);
                float4 *xo = reinterpret_cast<float4 *>(net.xbuf + (static_cast<size_t>(item) * kBM + er) * kBN + cb);
#pragma unroll
                for (int i = 0; i < 4; ++i) xo[i] = make_float4(acc[4 * i], acc[4 * i + 1], acc[4 * i + 2], acc[4 * i + 3]);
            }
            ok = pair_sync(net.pair_flag + item / 2, 2u * (act_steps - 1u), 1u << 26) && ok;
            if (ok)
            {
                partial(kBN * kh + cb, acc);
                const float4 *xi =
                    reinterpret_cast<const float4 *>(net.xbuf + (static_cast<size_t>(item ^ 1u) * kBM + er) * kBN + cb);
#pragma unroll
                for (int i = 0; i < 4; ++i)
                {
                    const float4 p4 = __ldcg(xi + i);
                    const float pv[4] = {p4.x, p4.y, p4.z, p4.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        acc[4 * i + e] = kh ? __fadd_rn(pv[e], acc[4 * i + e]) : __fadd_rn(acc[4 * i + e], pv[e]);
                }
                if (erow < b_act)
                {
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                    {
                        if (n0 + cb + i >= my_n) break;
                        // lif_impl.h:33-86: leak and input only outside the refractory period;
                        // strict '>'; reset to a value.
                        if (RC[i] == 0u)
                        {
                            const float v = __fadd_rn(__fmul_rn(V[i], leak), acc[i]);
                            if (v > thr)
                            {
                                V[i] = rst;
                                RC[i] = per;
                                mask |= 1u << (cb + i);
                                ++CNT[i];
                            }
                            else
                            {
                                V[i] = v;
                            }
                        }
                        else
                        {
                            --RC[i];
                        }
                    }
                }
            }
            // This thread's 16 spikes as the next layer's A operand (two 16-byte stores).
            if (layer < net.n_layers && erow < net.batch)
            {
                uint8_t *d = net.spk[layer][t & 1] + static_cast<size_t>(m_tile) * net.chunks[layer + 1] * kChunkBytes;
                const uint32_t k = n0 + cb;
                *reinterpret_cast<uint4 *>(d + spk_offset(er, k)) = bf16_bits(mask >> cb);
                *reinterpret_cast<uint4 *>(d + spk_offset(er, k + 8)) = bf16_bits(mask >> (cb + 8));
            }
            if (mask) atomicOr(&sbits[er], mask);
            my_events += static_cast<unsigned long long>(__popc(mask)) * my_fan_out;
            tc::fence_before_sync();
            __syncthreads();
            if (net.record && threadIdx.x < kBM && (n0 >> 5) < wn)  // the second half of a tile may lie past N
            {
                const uint32_t rr = threadIdx.x, rw = m0 + rr;
                if (rw < b_act)
                    net.record[t * net.rec_stride + net.rec_off[layer] + static_cast<size_t>(net.perm[rw]) * wn +
                               (n0 >> 5)] = sbits[rr];
            }
        }
        if (!grid_sync(net.barrier, gridDim.x, 1u << 26)) ok = false;
        tc::fence_after_sync();
    }
    // Output spike counts of the last layer: each (sample, neuron) is owned by one thread.
    if (layer == net.n_layers && erow < net.batch)
    {
        const uint32_t smp = net.perm[erow];
#pragma unroll
        for (int i = 0; i < 16; ++i)
            if (n0 + cb + i < N) net.counts[static_cast<size_t>(smp) * N + n0 + cb + i] = CNT[i];
    }
    if (my_events) atomicAdd(&s_events, my_events);
    if (!ok)
    {
        if (threadIdx.x == 0) atomicOr(net.err, 1u);
        // After a failed wait: let any MMA and bulk copy still in flight finish (bounded) before the
        // tensor memory and shared memory are released.
        if (threadIdx.x == 0)
            for (int q = 0; q < kIssuers; ++q) tc::mbar_wait(&done[q], (act_steps + 1) & 1u, kWaitLimit);
        if (warp == kLoaderWarp && lane == 0)
            for (uint32_t sq = (seq > kStages ? seq - kStages : 0); sq < seq; ++sq)
                tc::mbar_wait(&full[sq % kStages], (sq / kStages) & 1u, kWaitLimit);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0 && s_events) atomicAdd(net.events, s_events);
    if (warp == 0) tc::tmem_dealloc(tmem, kPairN * kIssuers);
}

}  // namespace

// A batch prepared once and run as one CUDA-graph launch (memsets of the run's state, the input
// threshold kernel and the cooperative persistent kernel). Reusable: every run starts from zero
// state, so repeated runs of the same plan give identical results.
struct BatchedPlan
{
    BatchedNet net{};
    cudaStream_t caller = nullptr;  // the caller's stream: a run starts after its queued work
    cudaStream_t stream = nullptr;  // the plan's own stream (graphs cannot be captured on the legacy stream)
    cudaEvent_t ready = nullptr;
    std::vector<void *> allocs;
    std::vector<std::pair<void *, size_t>> zero;  // cleared at the start of every run
    const float *rates = nullptr;
    unsigned long long *d_thr = nullptr;
    size_t n_thr = 0;
    size_t w_bytes = 0;  // largest weight tile (shared memory besides the ring)
    uint32_t n_items = 0;
    cudaGraphExec_t exec = nullptr;
    int stages = 0;
    float tune_ms[kMaxStages + 1] = {};

    ~BatchedPlan()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (stream) cudaStreamSynchronize(stream);
        for (void *p : allocs) cudaFree(p);
        if (ready) cudaEventDestroy(ready);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace
{

const void *kernel_for(int stages)
{
    switch (stages)
    {
        case 3:
            return reinterpret_cast<const void *>(batched_lif_kernel<3>);
        case 4:
            return reinterpret_cast<const void *>(batched_lif_kernel<4>);
        default:
            return reinterpret_cast<const void *>(batched_lif_kernel<5>);
    }
}

// Whether a ring of `stages` chunks fits (shared memory, every CTA resident at once).
bool variant_fits(const BatchedPlan &p, int stages)
{
    int device = 0, sms = 0, smem_max = 0, per_sm = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    const size_t smem = p.w_bytes + static_cast<size_t>(stages) * kChunkBytes;
    if (smem + 2048 > static_cast<size_t>(smem_max)) return false;  // 2 KB: the kernel's static shared memory
    const void *k = kernel_for(stages);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess)
        return false;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kBatchThreads, smem) != cudaSuccess) return false;
    return static_cast<long long>(per_sm) * sms >= p.n_items;
}

// Captures one run with a ring of `stages` chunks into p.exec.
cudaError_t capture(BatchedPlan &p, int stages)
{
    if (p.exec)
    {
        cudaGraphExecDestroy(p.exec);
        p.exec = nullptr;
    }
    cudaStream_t s = p.stream;
    cudaError_t err = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (err != cudaSuccess) return err;
    for (auto &z : p.zero) cudaMemsetAsync(z.first, 0, z.second, s);
    rate_threshold_kernel<<<static_cast<unsigned>((p.n_thr + 255) / 256), 256, 0, s>>>(p.rates, p.d_thr, p.n_thr);
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(p.n_items);
    cfg.blockDim = dim3(kBatchThreads);
    cfg.dynamicSmemBytes = p.w_bytes + static_cast<size_t>(stages) * kChunkBytes;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void *args[] = {&p.net};
    const cudaError_t lerr = cudaLaunchKernelExC(&cfg, kernel_for(stages), args);
    cudaGraph_t g = nullptr;
    err = cudaStreamEndCapture(s, &g);
    if (lerr != cudaSuccess) err = lerr;
    if (err == cudaSuccess) err = cudaGraphInstantiate(&p.exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (err == cudaSuccess) p.stages = stages;
    return err;
}

cudaError_t launch_timed(BatchedPlan &p, float *ms)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    // Order the run after the caller's queued work (weights, rates written on its stream).
    cudaEventRecord(p.ready, p.caller);
    cudaStreamWaitEvent(p.stream, p.ready, 0);
    cudaEventRecord(e0, p.stream);
    cudaError_t err = cudaGraphLaunch(p.exec, p.stream);
    cudaEventRecord(e1, p.stream);
    if (err == cudaSuccess) err = cudaEventSynchronize(e1);
    float t = 0.f;
    if (err == cudaSuccess) cudaEventElapsedTime(&t, e0, e1);
    if (ms) *ms = t;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return err;
}

}  // namespace

// Prepares a batch. Host arrays: sizes[n_layers + 1], leak/threshold/reset/refract[n_layers],
// steps[batch], sample_sizes[(n_layers + 1) * batch] (layer-major, optional); device arrays:
// weights[l] (BF16 [sizes[l + 1]][sizes[l]]), rates [batch][sizes[0]], counts [batch][sizes[n_layers]]
// and record (optional; layouts in knp_gb300.h). With `autotune`, each operand ring depth that fits
// is run twice and the fastest kept; every depth computes the same results.
int batched_plan_create(
    int n_layers, const uint32_t *sizes, const void *const *weights, const float *leak, const float *threshold,
    const float *reset, const uint32_t *refract, uint32_t batch, const uint32_t *steps, const uint32_t *sample_sizes,
    const float *rates, unsigned long long key, int *counts, uint32_t *record, int autotune, cudaStream_t s,
    BatchedPlan **out, const char **why)
{
    *out = nullptr;
    if (n_layers < 1 || n_layers > kMaxLayers || batch == 0 || !sizes || !weights || !steps || !rates || !counts)
    {
        *why = "bad arguments";
        return -1;
    }
    std::unique_ptr<BatchedPlan> plan(new BatchedPlan());
    BatchedPlan &p = *plan;
    BatchedNet &net = p.net;
    p.caller = s;
    if (cudaStreamCreateWithFlags(&p.stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&p.ready, cudaEventDisableTiming) != cudaSuccess)
    {
        *why = "could not create the plan's stream";
        return -3;
    }
    net.n_layers = n_layers;
    for (int l = 0; l <= n_layers; ++l)
    {
        if (sizes[l] == 0 || sizes[l] > 4096)
        {
            *why = "layer sizes must be in [1, 4096]";
            return -1;
        }
        net.size[l] = sizes[l];
        net.words[l] = (sizes[l] + 31) / 32;
        if (l > 0)
        {
            net.kpad[l] = (sizes[l - 1] + 15) / 16 * 16;
            net.chunks[l] = (net.kpad[l] + kBK - 1) / kBK;
        }
    }
    for (uint32_t b = 0; b < batch; ++b)
    {
        if (steps[b] == 0 || steps[b] > 1000000)
        {
            *why = "per-sample step counts must be in [1, 1000000]";
            return -1;
        }
        if (sample_sizes)
            for (int l = 0; l <= n_layers; ++l)
                if (sample_sizes[static_cast<size_t>(l) * batch + b] > sizes[l])
                {
                    *why = "a sample's layer size exceeds the layer size";
                    return -1;
                }
    }
    // Work items: (layer, 128-sample tile, 64-neuron tile, K half), the two halves of a tile adjacent.
    const uint32_t m_tiles = (batch + kBM - 1) / kBM;
    for (int l = 1; l <= n_layers; ++l)
    {
        const uint32_t n_tiles = (net.size[l] + kPairN - 1) / kPairN;
        for (uint32_t m = 0; m < m_tiles; ++m)
            for (uint32_t n = 0; n < n_tiles; ++n)
                for (uint32_t h = 0; h < 2; ++h)
                {
                    if (p.n_items >= kMaxItems)
                    {
                        *why = "too many (layer, sample tile, neuron tile) work items";
                        return -1;
                    }
                    net.item_layer[p.n_items] = static_cast<uint16_t>(l);
                    net.item_m[p.n_items] = static_cast<uint16_t>(m);
                    net.item_n[p.n_items] = static_cast<uint16_t>(n);
                    net.item_k[p.n_items] = static_cast<uint8_t>(h);
                    ++p.n_items;
                }
        const uint32_t c_mid = (net.chunks[l] + 1) / 2;
        p.w_bytes = std::max<size_t>(p.w_bytes, static_cast<size_t>(kPairN) * c_mid * kBK * 2);
    }
    net.n_items = p.n_items;
    int best = 0;
    for (int st = kMaxStages; st >= kMinStages && !best; --st)
        if (variant_fits(p, st)) best = st;
    if (!best)
    {
        *why = "the batch does not fit: a layer's weight tile and operand ring exceed one CTA's shared memory "
               "(fan-in too large) or the work items exceed the resident CTAs";
        return -1;
    }
    // Samples sorted by decreasing length.
    std::vector<uint32_t> perm(batch), st(batch);
    for (uint32_t b = 0; b < batch; ++b) perm[b] = b;
    std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) { return steps[a] > steps[b]; });
    for (uint32_t i = 0; i < batch; ++i) st[i] = steps[perm[i]];
    net.t_max = st[0];
    net.batch = batch;
    net.key = key;
    net.counts = counts;
    net.record = record;
    for (int l = 0; l < n_layers; ++l)
    {
        net.w[l] = static_cast<const __nv_bfloat16 *>(weights[l]);
        net.leak[l] = leak ? leak[l] : 1.0f;
        net.thr[l] = threshold ? threshold[l] : 1.0f;
        net.reset[l] = reset ? reset[l] : 0.0f;
        net.refract[l] = refract ? refract[l] : 0u;
    }
    auto dalloc = [&](size_t bytes) -> void *
    {
        void *q = nullptr;
        if (cudaMalloc(&q, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        p.allocs.push_back(q);
        return q;
    };
    auto upload = [&](const void *src, size_t bytes) -> void *
    {
        void *q = dalloc(bytes);
        if (q && cudaMemcpy(q, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
        return q;
    };
    // act[t] = slots with T > t (slots are sorted by decreasing T).
    std::vector<uint32_t> act(net.t_max);
    for (uint32_t t = 0, a = batch; t < net.t_max; ++t)
    {
        while (a > 0 && st[a - 1] <= t) --a;
        act[t] = a;
    }
    bool ok = (net.perm = static_cast<const uint32_t *>(upload(perm.data(), batch * 4))) != nullptr;
    ok = ok && (net.act = static_cast<const uint32_t *>(upload(act.data(), act.size() * 4))) != nullptr;
    if (sample_sizes)
        for (int l = 0; l <= n_layers && ok; ++l)
            ok = (net.sample_size[l] = static_cast<const uint32_t *>(
                      upload(sample_sizes + static_cast<size_t>(l) * batch, batch * 4))) != nullptr;
    for (int l = 0; l < n_layers && ok; ++l)
        for (int q = 0; q < 2 && ok; ++q)
        {
            const size_t bytes = static_cast<size_t>(m_tiles) * net.chunks[l + 1] * kChunkBytes;
            ok = (net.spk[l][q] = static_cast<uint8_t *>(dalloc(bytes))) != nullptr;
            p.zero.emplace_back(net.spk[l][q], bytes);
        }
    p.n_thr = static_cast<size_t>(batch) * sizes[0];
    ok = ok && (p.d_thr = static_cast<unsigned long long *>(dalloc(p.n_thr * 8))) != nullptr;
    net.rate_thr = p.d_thr;
    p.rates = rates;
    ok = ok && (net.events = static_cast<unsigned long long *>(dalloc(8))) != nullptr;
    ok = ok && (net.err = static_cast<unsigned int *>(dalloc(4))) != nullptr;
    ok = ok && (net.barrier = static_cast<unsigned int *>(dalloc(8))) != nullptr;
    ok = ok && (net.xbuf = static_cast<float *>(dalloc(static_cast<size_t>(p.n_items) * kBM * kBN * 4))) != nullptr;
    ok = ok && (net.pair_flag = static_cast<unsigned int *>(dalloc(static_cast<size_t>(p.n_items / 2 + 1) * 4))) !=
                   nullptr;
    if (!ok)
    {
        *why = "device allocation failed";
        return -5;
    }
    p.zero.emplace_back(counts, static_cast<size_t>(batch) * net.size[n_layers] * 4);
    p.zero.emplace_back(net.events, 8);
    p.zero.emplace_back(net.err, 4);
    p.zero.emplace_back(net.barrier, 8);
    p.zero.emplace_back(net.pair_flag, static_cast<size_t>(p.n_items / 2 + 1) * 4);
    unsigned long long off = 0;
    for (int l = 0; l <= n_layers; ++l)
    {
        net.rec_off[l] = off;
        off += static_cast<unsigned long long>(batch) * net.words[l];
    }
    net.rec_stride = off;
    if (record) p.zero.emplace_back(record, static_cast<size_t>(net.t_max) * off * 4);

    cudaError_t err = cudaSuccess;
    if (autotune)
    {
        float best_ms = 0.f;
        for (int stg = kMinStages; stg <= kMaxStages; ++stg)
        {
            if (!variant_fits(p, stg)) continue;
            err = capture(p, stg);
            float t = 0.f;
            for (int rep = 0; rep < 2 && err == cudaSuccess; ++rep) err = launch_timed(p, &t);
            if (err != cudaSuccess) break;
            p.tune_ms[stg] = t;
            if (!best_ms || t < best_ms)
            {
                best_ms = t;
                best = stg;
            }
        }
    }
    if (err == cudaSuccess && p.stages != best) err = capture(p, best);
    if (err != cudaSuccess)
    {
        *why = cudaGetErrorString(err);
        return -3;
    }
    *out = plan.release();
    return 0;
}

int batched_plan_run(BatchedPlan *p, unsigned long long *events_out, float *ms, const char **why)
{
    cudaError_t err = launch_timed(*p, ms);
    unsigned long long ev = 0;
    unsigned int kerr = 0;
    if (err == cudaSuccess) err = cudaMemcpy(&ev, p->net.events, 8, cudaMemcpyDeviceToHost);
    if (err == cudaSuccess) err = cudaMemcpy(&kerr, p->net.err, 4, cudaMemcpyDeviceToHost);
    if (events_out) *events_out = ev;
    if (err != cudaSuccess)
    {
        *why = cudaGetErrorString(err);
        return -3;
    }
    if (kerr)
    {
        *why = "a tensor-core completion wait, a bulk copy wait or the grid barrier timed out";
        return -4;
    }
    return 0;
}

void batched_plan_info(const BatchedPlan *p, int *stages, float *tune_ms)
{
    if (stages) *stages = p->stages;
    if (tune_ms)
        for (int i = kMinStages; i <= kMaxStages; ++i) tune_ms[i - kMinStages] = p->tune_ms[i];
}

void batched_plan_destroy(BatchedPlan *p) { delete p; }

// One-shot form: prepare, run once, release.
int batched_lif_run(
    int n_layers, const uint32_t *sizes, const void *const *weights, const float *leak, const float *threshold,
    const float *reset, const uint32_t *refract, uint32_t batch, const uint32_t *steps, const float *rates,
    unsigned long long key, int *counts, uint32_t *record, unsigned long long *events_out, float *ms,
    cudaStream_t s, const char **why)
{
    BatchedPlan *p = nullptr;
    int rc = batched_plan_create(n_layers, sizes, weights, leak, threshold, reset, refract, batch, steps, nullptr,
                                 rates, key, counts, record, 0, s, &p, why);
    if (rc == 0) rc = batched_plan_run(p, events_out, ms, why);
    if (p) batched_plan_destroy(p);
    return rc;
}

}  // namespace knp_gb300
