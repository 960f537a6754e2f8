// Batched form on 5th-generation tensor cores.
//
// bf16_gemm_tn_simple: D[M x N] (FP32) = A[M x K] * B[N x K]^T with BF16 operands (row-major, K
// contiguous), tcgen05.mma kind::f16 with the accumulator in tensor memory, single stage; the
// pipelined GEMM is gemm.cu.
#include <algorithm>
#include <cstdlib>
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
constexpr uint32_t kWaitLimit = 1u << 22;  // try_wait calls of up to kSuspendNs each

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

// The single-stage GEMM: any K and alignment (bf16_gemm_tn in gemm.cu takes it for shapes the
// pipelined kernel does not).
int bf16_gemm_tn_simple(const void *A, const void *B, float *D, int M, int N, int K, unsigned int *d_err, cudaStream_t s)
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
// Each step of a layer is a BF16 GEMM of the 0/1 spike matrix (exact in BF16) against BF16 weights
// with FP32 accumulation in tensor memory. A CTA pair (a cluster of two) owns (layer, 128-sample
// tile, 64-neuron tile): each CTA multiplies one half of the K range against its half of the weight
// tile (resident in shared memory for the whole run), sends the partner the partial sums of the 32
// neurons the partner finalises (st.async into the partner's shared memory) and finalises its own
// 32 neurons, whose LIF state stays in registers.
//
// Spikes travel between layers as bitmaps (one 32-bit word per sample and 32 neurons) in a ring of
// R steps per layer (R tuned, at most kMaxRing). A consumer expands its K half chunk by chunk into BF16 operand chunks in
// tensor memory (one sample row per lane) while the tensor cores multiply the previous chunk. There
// is no grid-wide barrier: per (layer, sample tile, ring slot) counters record how
// many times the layer's CTAs have written the slot (`ready`) and how many times consumer CTAs have
// read it (`consumed`), so a layer starts step t as soon as every CTA of the layer below has
// published step t - 1, and overwrites a slot only after every consumer has read it (a layer runs
// at most R - 2 steps ahead of its consumers). Counting per slot matters: CTAs of one layer are
// not in lockstep, and a sum over all slots would let a fast CTA stand in for a slow one. Input spikes do not depend on the network, so
// a separate kernel draws them ahead of the run (layer 0's slots hold every step of a segment; long
// runs are cut into segments, the LIF state saved and restored between them). Samples are processed
// sorted by decreasing T, so finished samples leave whole sample tiles idle. Every wait is bounded.
namespace knp_gb300
{
namespace
{

constexpr int kBM = 128, kBN = 32, kBK = 128, kMaxLayers = 4, kMaxItems = 512;
constexpr int kPairN = 2 * kBN;                 // neurons of a CTA pair's tile; each CTA finalises kBN
constexpr int kMinStages = 2, kMaxStages = 4;  // operand ring depths the autotuner tries
constexpr uint32_t kAccCols = 2 * kPairN;        // tensor-memory columns of the two accumulators
constexpr uint32_t kStageCols = kBK / 2;         // tensor-memory columns of one 128 x 128 BF16 operand chunk
constexpr uint32_t kTmemCols = 512;              // the whole tensor memory (one CTA per SM)
constexpr size_t kMinDynSmem = size_t(120) << 10;  // keeps a second CTA off the SM (it would wait for tensor memory)
static_assert(kAccCols + kMaxStages * kStageCols <= kTmemCols, "operand stages exceed tensor memory");
constexpr uint32_t kChunkWords = kBK / 32;       // bitmap words per sample row and chunk
constexpr uint32_t kMaxHalfChunks = 8;           // chunks of a K half (bounded by shared memory)
constexpr uint32_t kMaxRing = 16;                // bitmap steps kept per layer at most (counter stride)
constexpr uint32_t kRingChoices[3] = {4, 8, 16};   // ring lengths the autotuner tries
constexpr uint32_t kDefaultRing = 8;
constexpr uint32_t kXchBytes = kBM * kBN * 4;    // one exchange buffer: [kBM][kBN] FP32 partial sums
constexpr uint32_t kPollLimit = 1u << 22;        // polls of a cross-CTA counter before giving up
constexpr int kExpandWarps = 4, kEpilogueWarps = 8;  // warps 0-3 expand, 4-11 epilogue, 12 issues
constexpr int kIssuerWarp = kExpandWarps + kEpilogueWarps;
constexpr int kExpandThreads = 32 * kExpandWarps, kEpilogueThreads = 32 * kEpilogueWarps;
constexpr int kBatchThreads = kExpandThreads + kEpilogueThreads + 32;
constexpr int kEN = 16;                  // neurons per epilogue thread (two threads per sample row)
constexpr int kStateWords = 3 * kEN;  // V, refractory counter, spike count of an epilogue thread's neurons
constexpr uint32_t kCntBytes = kBM * kBN * 4;  // last layer's spike counts of a tile, [kBN][kBM] int
constexpr size_t kInputSlotBudget = size_t(256) << 20;  // bytes of layer 0's slots per segment

struct BatchedNet
{
    int n_layers;
    uint32_t size[kMaxLayers + 1];
    uint32_t words[kMaxLayers + 1];   // ceil(size / 32)
    uint32_t kpad[kMaxLayers + 1];    // kpad[l] = size[l - 1] rounded up to 16 (layer l's K)
    uint32_t chunks[kMaxLayers + 1];  // chunks[l] = ceil(kpad[l] / 128)
    uint32_t wpad[kMaxLayers + 1];    // wpad[l] = 4 * chunks[l + 1]: words per sample row of layer l's slots
    uint32_t n_cta[kMaxLayers + 1];   // CTAs of layer l per sample tile
    const __nv_bfloat16 *w[kMaxLayers];
    float leak[kMaxLayers], thr[kMaxLayers], reset[kMaxLayers];
    uint32_t refract[kMaxLayers];
    uint32_t batch, m_tiles;
    const uint32_t *perm;  // slot -> sample
    const uint32_t *act;   // [t_max]: slots still running at step t (slots sorted by decreasing T)
    const unsigned long long *rate_thr;  // [batch][size[0]] by sample: rate * 2^53, the draw's threshold
    // Optional per-sample layer sizes ([batch] by sample, <= size[l]); neurons and inputs beyond a
    // sample's size do not exist for it (never spike). Null: every sample has the full sizes.
    const uint32_t *sample_size[kMaxLayers + 1];
    unsigned long long key;
    uint32_t t_max;
    // bits[l]: spikes of layer l as layer l + 1's input, [slot][m tile][kBM][wpad[l]] words (bit j of
    // word w = neuron 32 w + j, words past words[l] zero). Layer 0: slot j of a segment starting at
    // step t0 = input drawn at step t0 + j - 1 (nothing before step 0). Layers >= 1: ring slots,
    // slot (t + 1) % ring written at step t.
    uint32_t *bits[kMaxLayers];
    uint32_t ring;           // steps kept per layer ring (3 .. kMaxRing)
    unsigned int *ready;     // [kMaxLayers + 1][m_tiles][kMaxRing]: writes of layer l's slot by its CTAs
    unsigned int *consumed;  // [kMaxLayers + 1][m_tiles][kMaxRing]: reads of layer l's slot by layer l + 1's CTAs
    uint32_t *state;         // [n_items][kEpilogueThreads][kStateWords]: LIF state between segments
    int *counts;             // [batch][size[L]] by sample
    uint32_t *record;        // [t_max][sum_l batch * words[l]] by sample, or null
    unsigned long long rec_off[kMaxLayers + 1];
    unsigned long long rec_stride;
    unsigned long long *events;
    unsigned int *err;       // bit 0: a wait gave up; bit 1: launched without the 2-CTA cluster shape
    uint32_t poll_limit;     // polls of a cross-CTA ring counter before a wait gives up
    uint32_t stall;          // failure test: consumers wait for this many more producer CTAs than exist
    uint32_t n_items;
    uint16_t item_layer[kMaxItems];
    uint16_t item_m[kMaxItems];
    uint16_t item_n[kMaxItems];  // kPairN-neuron tile index
    uint8_t item_k[kMaxItems];   // K half = rank in the cluster: items 2i and 2i + 1 are one tile
};

// Per (sample, input): the 53-bit threshold that the input draw is compared with, rate * 2^53
// truncated, computed exactly from the FP32 rate's fields (no FP64 on the device): m * 2^(e - 97)
// for a normal rate in (0, 1) with 24-bit significand m and biased exponent e; 0 for rates <= 0,
// subnormal or NaN; 2^53 (every draw is below it) for rates >= 1.
__global__ void rate_threshold_kernel(const float *rates, unsigned long long *thr, size_t n)
{
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t bits = __float_as_uint(rates[i]);
    const uint32_t e = (bits >> 23) & 0xFFu;
    unsigned long long v = 0;
    if ((bits >> 31) == 0u && e != 0u && e != 0xFFu)
    {
        const unsigned long long m = (bits & 0x7FFFFFu) | 0x800000u;
        if (e >= 127u)
            v = 1ull << 53;
        else if (e >= 97u)
            v = m << (e - 97u);
        else if (97u - e < 64u)
            v = m >> (97u - e);
    }
    else if ((bits >> 31) == 0u && e == 0xFFu && (bits & 0x7FFFFFu) == 0u)
    {
        v = 1ull << 53;  // +infinity
    }
    thr[i] = v;
}

// Layer 0's slots of the segment [t0, t1): slot j = the input spikes drawn at step t0 + j - 1, one
// thread per bitmap word (32 draws). Also writes layer 0's record and adds the synaptic events of
// each step drawn; the last segment has one extra row of words (j = t1 - t0, the draws of step
// t_max - 1) that no layer reads.
__global__ void input_bits_kernel(BatchedNet net, uint32_t t0, uint32_t t1)
{
    const uint32_t wp = net.wpad[0], w0 = net.words[0], n_in = net.size[0];
    const uint32_t span = t1 - t0 + (t1 == net.t_max ? 1u : 0u);
    const size_t per_slot = static_cast<size_t>(net.m_tiles) * kBM * wp;
    const size_t total = span * per_slot;
    unsigned long long ev = 0;
    for (size_t u = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x; u < total;
         u += static_cast<size_t>(gridDim.x) * blockDim.x)
    {
        const uint32_t j = static_cast<uint32_t>(u / per_slot);
        const uint32_t rem = static_cast<uint32_t>(u - static_cast<size_t>(j) * per_slot);
        const uint32_t row = rem / wp, w = rem - row * wp;  // row = m tile * kBM + slot row
        const uint32_t t = t0 + j;                           // the step that consumes the draws of t - 1
        uint32_t word = 0;
        if (t >= 1 && w < w0 && row < net.act[t - 1])
        {
            const uint32_t s = t - 1, smp = net.perm[row];
            const uint32_t lim = net.sample_size[0] ? min(n_in, net.sample_size[0][smp]) : n_in;
            const unsigned long long base = (static_cast<unsigned long long>(s) * net.batch + smp) * n_in;
            const unsigned long long *thr = net.rate_thr + static_cast<size_t>(smp) * n_in;
            const uint32_t i0 = w * 32;
            for (uint32_t b = 0; b < 32 && i0 + b < lim; ++b)
                if ((rand64(net.key, base + i0 + b) >> 11) < thr[i0 + b]) word |= 1u << b;
            if (net.record)
                net.record[s * net.rec_stride + net.rec_off[0] + static_cast<size_t>(smp) * w0 + w] = word;
            ev += static_cast<unsigned long long>(__popc(word)) *
                  (net.sample_size[1] ? net.sample_size[1][smp] : net.size[1]);
        }
        if (j < t1 - t0) net.bits[0][u] = word;
    }
    for (int o = 16; o > 0; o >>= 1) ev += __shfl_down_sync(0xffffffffu, ev, o);
    if ((threadIdx.x & 31) == 0 && ev) atomicAdd(net.events, ev);
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *mbar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(mbar)),
                 "r"(bytes)
                 : "memory");
}

// Whether this CTA (its shared failure flag) or any CTA of the launch (the error word) has given up.
__device__ __forceinline__ bool failed(const volatile int *flag, const unsigned int *gerr)
{
    return *flag != 0 || *reinterpret_cast<const volatile unsigned int *>(gerr) != 0u;
}

// Polls (acquire, bounded) until *counter >= target; false after `limit` polls or once a failure has
// been reported (checked every 64 polls).
__device__ __forceinline__ bool poll_at_least(const unsigned int *counter, unsigned int target, uint32_t limit,
                                              const volatile int *flag, const unsigned int *gerr)
{
    for (uint32_t i = 0; i < limit; ++i)
    {
        unsigned int cur;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(counter) : "memory");
        if (static_cast<int>(cur - target) >= 0) return true;
        if ((i & 63u) == 63u && failed(flag, gerr)) return false;
    }
    return false;
}

// mbar_wait that also gives up as soon as a failure has been reported (checked after each poll).
__device__ __forceinline__ bool wait_or_fail(uint64_t *mbar, uint32_t parity, const volatile int *flag,
                                             const unsigned int *gerr)
{
    for (uint32_t i = 0; i < kWaitLimit; ++i)
    {
        if (tc::mbar_try_wait(mbar, parity)) return true;
        if (failed(flag, gerr)) return false;
    }
    return false;
}

__device__ __forceinline__ bool wait_cluster_or_fail(uint64_t *mbar, uint32_t parity, const volatile int *flag,
                                                     const unsigned int *gerr)
{
    for (uint32_t i = 0; i < kWaitLimit; ++i)
    {
        if (tc::mbar_try_wait_cluster(mbar, parity)) return true;
        if (failed(flag, gerr)) return false;
    }
    return false;
}

// A counter read ahead of need (relaxed: later memory operations do not wait for it). A value
// found sufficient is followed by fence_acquire() before the data it guards is touched.
__device__ __forceinline__ unsigned int load_relaxed(const unsigned int *counter)
{
    unsigned int v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(counter) : "memory");
    return v;
}

__device__ __forceinline__ void fence_acquire() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// Whether *counter >= target: from a value read ahead if that suffices, else by polling.
__device__ __forceinline__ bool reached(const unsigned int *counter, unsigned int target, unsigned int seen,
                                        uint32_t limit, const volatile int *flag, const unsigned int *gerr)
{
    if (static_cast<int>(seen - target) >= 0)
    {
        fence_acquire();
        return true;
    }
    return poll_at_least(counter, target, limit, flag, gerr);
}

__device__ __forceinline__ void release_add(unsigned int *counter)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(counter) : "memory");
}

// Roles of the 13 warps: warps 0-3 expand the input bitmaps into the operand ring (one sample row
// per thread), warps 4-11 run the epilogue (one sample row and 16 of the CTA's 32 neurons per
// thread), lane 0 of warp 12 issues the MMAs. Two accumulators in tensor memory let the MMAs of
// step s + 1 run while the epilogue of step s exchanges partial sums and updates the neurons.
template <int kStages>
__global__ void __launch_bounds__(kBatchThreads, 1) batched_lif_kernel(BatchedNet net, uint32_t t0, uint32_t t1)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) uint64_t full[kStages];   // operand stage b written (kExpandThreads arrivals)
    __shared__ __align__(8) uint64_t empty[kStages];  // the MMAs that read stage b have completed (commit)
    __shared__ __align__(8) uint64_t acc_full[2];     // every MMA into accumulator a has completed (commit)
    __shared__ __align__(8) uint64_t acc_empty[2];    // the epilogue has read accumulator a (kEpilogueThreads)
    __shared__ __align__(8) uint64_t xfull[2];        // the partner's partial sums of a step have landed
    __shared__ __align__(8) uint64_t drain;           // every MMA this CTA issued has completed (teardown)
    __shared__ unsigned long long s_events;
    __shared__ int s_fail;  // some role gave up on a wait (each group reads it through one thread)
    __shared__ uint32_t s_half[2][2][kBM];  // [step parity][neuron half][row]: epilogue spike masks
    // Exchange bookkeeping for the teardown: steps whose partial sums this CTA sent to its partner,
    // exchange phases it received, phases it armed; the partner's sent count (written by the partner).
    __shared__ uint32_t s_sent, s_recv, s_armed, s_peer_sent;
    // A launch without the two-CTA cluster shape (every CTA sees the same count) stops here, before
    // any access to a partner's shared memory.
    if (tc::cluster_nctarank() != 2u)
    {
        if (threadIdx.x == 0) atomicOr(net.err, 2u);
        return;
    }
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
    const uint32_t n_chunks = c_hi - c_lo;  // this CTA's chunks (<= kMaxHalfChunks)
    const uint32_t Kw = c_mid * kBK;        // K extent of the weight tile (the larger half)
    // Shared memory: weight tile [kPairN x Kw] (K-major core matrices), two exchange buffers, the
    // last layer's spike counts. Tensor
    // memory: two accumulators (columns [0, kAccCols)), then kStages operand stages of kStageCols.
    uint8_t *sW = smem;
    uint8_t *sX = smem + static_cast<size_t>(kPairN) * Kw * 2;
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
    if (warp == kIssuerWarp) tc::tmem_alloc(&tmem_slot, kTmemCols);
    if (threadIdx.x == 0)
    {
        for (int b = 0; b < kStages; ++b)
        {
            tc::mbar_init(&full[b], kExpandThreads);
            tc::mbar_init(&empty[b], 1);
        }
        for (int a = 0; a < 2; ++a)
        {
            tc::mbar_init(&acc_full[a], 1);
            tc::mbar_init(&acc_empty[a], kEpilogueThreads);
            tc::mbar_init(&xfull[a], 1);
        }
        tc::mbar_init(&drain, 1);
        s_events = 0;
        // A failure reported by an earlier segment of the run: this launch steps nothing (but keeps
        // the teardown protocol with its partner).
        s_fail = *reinterpret_cast<volatile unsigned int *>(net.err) != 0u ? 1 : 0;
        s_sent = s_recv = s_armed = s_peer_sent = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::cluster_sync();  // the partner's barriers are initialised before any st.async reaches them
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    const uint32_t m_tiles = net.m_tiles;
    const uint32_t R = net.ring;
    const size_t ctr_in = (static_cast<size_t>(layer - 1) * m_tiles + m_tile) * kMaxRing;
    const size_t ctr_out = (static_cast<size_t>(layer) * m_tiles + m_tile) * kMaxRing;
    const bool producer = layer < net.n_layers;
    unsigned long long my_events = 0;

    if (warp < kExpandWarps)
    {
        // Expanders: per step, wait until every CTA of layer - 1 (this sample tile) has published
        // step t - 1, load this row's words of the K half, and write each chunk as BF16 0/1 into a
        // free operand stage in tensor memory (thread = sample row = tensor-memory lane).
        const uint32_t xr = threadIdx.x;
        const uint32_t wp_in = net.wpad[layer - 1];
        const unsigned int *ready_in = layer > 1 ? net.ready + ctr_in : nullptr;
        const uint32_t need_in = layer > 1 ? net.n_cta[layer - 1] + net.stall : 0u;
        const uint32_t x_lane = (32u * warp) << 16;
        uint32_t seq = 0;
        bool ok = true;
        unsigned int ready_seen = 0;  // the next step's counter, read early in this step
        auto row_words = [&](uint32_t t) -> const uint4 *
        {
            const uint32_t slot = layer == 1 ? t - t0 : t % R;
            return reinterpret_cast<const uint4 *>(
                net.bits[layer - 1] + (static_cast<size_t>(slot) * m_tiles + m_tile) * kBM * wp_in +
                static_cast<size_t>(xr) * wp_in + c_lo * kChunkWords);
        };
        uint4 wv[kMaxHalfChunks];  // this step's words
        uint4 wn[kMaxHalfChunks];  // the next step's words, when they could be loaded during this step
        bool have_next = false;
        for (uint32_t t = t0; t < t1; ++t)
        {
            if (m0 >= net.act[t]) break;  // sample tiles finish in order: no steps left
            bool go = ok;
            if (threadIdx.x == 0)
                go = go && !s_fail &&
                     (have_next || !ready_in || t == 0 ||
                      reached(ready_in + t % R, need_in * ((t - 1) / R + 1), ready_seen, net.poll_limit, &s_fail,
                              net.err));
            if (!tc::named_sync_and(1, kExpandThreads, go))  // the group's decision is uniform
            {
                s_fail = 1;
                atomicOr(net.err, 1u);
                break;
            }
            if (have_next)
            {
#pragma unroll
                for (uint32_t c = 0; c < kMaxHalfChunks; ++c) wv[c] = wn[c];
            }
            else
            {
                const uint4 *rowp = row_words(t);
#pragma unroll
                for (uint32_t c = 0; c < kMaxHalfChunks; ++c)
                    wv[c] = c < n_chunks ? __ldcg(rowp + c) : make_uint4(0, 0, 0, 0);
            }
            have_next = false;
            const bool can_next = t + 1 < t1 && m0 < net.act[t + 1];  // uniform
            if (threadIdx.x == 0 && ready_in && can_next) ready_seen = load_relaxed(ready_in + (t + 1) % R);
            // After chunk `c_ask`, the next step's words are loaded (to be used next step) if layer - 1
            // has already published that step, so their L2 round trip overlaps this step's chunks.
            const uint32_t c_ask = n_chunks > 1 ? 1u : 0u;
            // One copy of the chunk body (kept small for the instruction cache); the loaded words
            // shift down by one chunk per iteration so that every register index stays static.
#pragma unroll 1
            for (uint32_t c = 0; c < n_chunks; ++c)
            {
                const uint32_t u = seq + c, b = u % kStages;
                if (ok && u >= kStages && !wait_or_fail(&empty[b], ((u / kStages) - 1u) & 1u, &s_fail, net.err))
                {
                    // The stage may still be read by MMAs: it is not written, and the failure stops
                    // the issuer (which waits on this stage) and, at the next step, this group.
                    ok = false;
                    s_fail = 1;
                    atomicOr(net.err, 1u);
                }
                tc::fence_after_sync();
                const uint32_t w4[4] = {wv[0].x, wv[0].y, wv[0].z, wv[0].w};
#pragma unroll
                for (uint32_t k = 0; k + 1 < kMaxHalfChunks; ++k) wv[k] = wv[k + 1];
                // tcgen05.st is warp-collective: a warp writes only if all its lanes may.
                if (__all_sync(0xffffffffu, ok))
                {
#pragma unroll
                    for (uint32_t q = 0; q < 4; ++q)
                    {
                        // Word q holds inputs 32 q .. 32 q + 31 of the chunk: 16 columns of two BF16
                        // each, bits (2 i, 2 i + 1) -> column i = 1.0 or 0 in its low and high halves.
                        uint32_t v[16];
#pragma unroll
                        for (uint32_t i = 0; i < 16; ++i)
                            v[i] = (((w4[q] >> (2u * i) & 3u) * 0x8001u) & 0x10001u) * 0x3F80u;
                        tc::tmem_st16(tmem + x_lane + kAccCols + b * kStageCols + 16u * q, v);
                    }
                    tc::tmem_wait_st();
                    tc::fence_before_sync();
                    tc::mbar_arrive(&full[b]);
                }
                if (c == c_ask && can_next)
                {
                    bool nx = true;
                    if (threadIdx.x == 0 && ready_in)
                    {
                        const unsigned int target = need_in * (t / R + 1);
                        nx = static_cast<int>(ready_seen - target) >= 0;
                        if (nx) fence_acquire();
                    }
                    have_next = tc::named_sync_and(1, kExpandThreads, nx);
                    if (have_next)
                    {
                        const uint4 *rown = row_words(t + 1);
#pragma unroll
                        for (uint32_t c2 = 0; c2 < kMaxHalfChunks; ++c2)
                            wn[c2] = c2 < n_chunks ? __ldcg(rown + c2) : make_uint4(0, 0, 0, 0);
                    }
                }
            }
            seq += n_chunks;
        }
    }
    else if (warp < kExpandWarps + kEpilogueWarps)
    {
        // Epilogue: thread (warp 4 + w, lane) owns sample row er = 32 (w % 4) + lane of the tile and
        // the CTA's neurons cb .. cb + 15 (cb = 16 (w / 4)), keeping their LIF state in registers;
        // warp 4 + w reads tensor-memory lanes 32 (w % 4) .. + 31.
        const uint32_t et = threadIdx.x - kExpandThreads, ew = et >> 5;
        const uint32_t er = 32u * (ew & 3u) + lane, erow = m0 + er;
        const uint32_t cb = kEN * (ew >> 2);
        const uint32_t lane_base = (32u * (warp & 3)) << 16;
        float V[kEN];
        uint32_t RC[kEN];
        uint32_t *saved = net.state + (static_cast<size_t>(item) * kEpilogueThreads + et) * kStateWords;
#pragma unroll
        for (int i = 0; i < kEN; ++i)
        {
            V[i] = t0 ? __uint_as_float(saved[i]) : 0.f;
            RC[i] = t0 ? saved[kEN + i] : 0u;
        }
        const int li = layer - 1;
        const float leak = net.leak[li], thr = net.thr[li], rst = net.reset[li];
        const uint32_t per = net.refract[li];
        // This row's sample: its own neuron count and its next layer's (the fan-out of its spikes).
        const uint32_t e_smp = erow < net.batch ? net.perm[erow] : 0u;
        const uint32_t my_n = (net.sample_size[layer] && erow < net.batch) ? net.sample_size[layer][e_smp] : N;
        const uint32_t my_fan_out =
            producer ? ((net.sample_size[layer + 1] && erow < net.batch) ? net.sample_size[layer + 1][e_smp]
                                                                          : net.size[layer + 1])
                     : 0u;
        uint32_t *out_bits = producer ? net.bits[layer] : nullptr;
        const uint32_t wp_out = producer ? net.wpad[layer] : 0u;
        unsigned int *ready_out = producer ? net.ready + ctr_out : nullptr;
        const unsigned int *consumed_out = producer ? net.consumed + ctr_out : nullptr;
        const uint32_t need_out = producer ? net.n_cta[layer + 1] : 0u;
        // Last layer: spike counts in shared memory, neuron-major so that a warp's 32 rows hit 32 banks.
        int *cnt = layer == net.n_layers ? reinterpret_cast<int *>(sX + 2 * kXchBytes) + cb * kBM + er : nullptr;
        if (cnt)
#pragma unroll
            for (int i = 0; i < kEN; ++i) cnt[i * kBM] = t0 ? static_cast<int>(saved[2 * kEN + i]) : 0;
        const uint32_t peer = tc::cluster_rank() ^ 1u;
        // Neurons at or past this sample's size do not exist (never updated, never spike).
        const uint32_t n_here = my_n > n0 + cb ? my_n - n0 - cb : 0u;
        const uint32_t exists = n_here >= 16u ? 0xFFFFu : (1u << n_here) - 1u;
        uint32_t s = 0, sent = 0, armed = 0;
        for (uint32_t t = t0; t < t1; ++t)
        {
            const uint32_t b_act = net.act[t];
            if (m0 >= b_act) break;
            // Ring slot (t + 1) % R was read at steps t + 1 - R, t + 1 - 2 R, ...: every
            // consumer must have read it that many times before it is overwritten below (the count
            // is read now and checked after the update).
            const bool check_room = et == 0 && producer && t + 1 >= R;
            const unsigned int room_seen = check_room ? load_relaxed(consumed_out + (t + 1) % R) : 0u;
            const uint32_t a = s & 1u, ph = (s >> 1) & 1u;
            // A failed accumulator wait stops the group before it reads tensor memory that MMAs may
            // still write, and before it sends its partner anything for this step.
            if (!tc::named_sync_and(2, kEpilogueThreads, wait_or_fail(&acc_full[a], ph, &s_fail, net.err)))
            {
                s_fail = 1;
                atomicOr(net.err, 1u);
                break;
            }
            bool ok = true;
            tc::fence_after_sync();
            // Read the accumulator while the tensor cores are idle (the issuer starts the next step's
            // MMAs once it is released): the partner's columns go straight to the partner (row er,
            // 16-byte slot q of the row stored at q ^ (er % 8), so that 8 consecutive rows hit
            // different banks), ours stay in registers. Then our partial + the partner's ((K half 0)
            // + (K half 1) on both sides) and the LIF update.
            if (et == 0) mbar_arrive_expect_tx(&xfull[a], kXchBytes);
            armed = s + 1;
            const uint32_t row_peer = tc::mapa(tc::smem_u32(sX), peer) + a * kXchBytes + er * (kBN * 4u);
            const uint32_t xfull_peer = tc::mapa(tc::smem_u32(&xfull[a]), peer);
            float acc[kEN];
            if (n_chunks)
                tc::tmem_ld16(tmem + lane_base + a * kPairN + kBN * (1u - kh) + cb, acc);
            else
#pragma unroll
                for (int i = 0; i < kEN; ++i) acc[i] = 0.0f;
#pragma unroll
            for (uint32_t q = 0; q < kEN / 4; ++q)
                tc::st_async_v4(row_peer + ((((cb >> 2) + q) ^ (er & 7u)) << 4), acc[4 * q], acc[4 * q + 1],
                                acc[4 * q + 2], acc[4 * q + 3], xfull_peer);
            sent = s + 1;
            if (n_chunks)
                tc::tmem_ld16(tmem + lane_base + a * kPairN + kBN * kh + cb, acc);
            tc::fence_before_sync();
            tc::mbar_arrive(&acc_empty[a]);
            ok = wait_cluster_or_fail(&xfull[a], ph, &s_fail, net.err) && ok;
            const uint8_t *row_own = sX + a * kXchBytes + er * (kBN * 4u);
#pragma unroll
            for (uint32_t q = 0; q < kEN / 4; ++q)
            {
                const float4 p4 = *reinterpret_cast<const float4 *>(row_own + ((((cb >> 2) + q) ^ (er & 7u)) << 4));
                const float pv[4] = {p4.x, p4.y, p4.z, p4.w};
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    acc[4 * q + e] = kh ? __fadd_rn(pv[e], acc[4 * q + e]) : __fadd_rn(acc[4 * q + e], pv[e]);
            }
            const uint32_t live = (ok && erow < b_act) ? exists : 0u;
            uint32_t mask = 0;  // this thread's spikes, bit i = neuron cb + i
#pragma unroll
            for (int i = 0; i < kEN; ++i)
            {
                // lif_impl.h:33-86: leak and input only outside the refractory period; strict '>';
                // reset to a value. Branch-free: the lanes are different samples.
                const bool here = (live >> i) & 1u;
                const bool free_ = RC[i] == 0u;
                const float v = __fadd_rn(__fmul_rn(V[i], leak), acc[i]);
                const bool spike = here && free_ && v > thr;
                V[i] = spike ? rst : ((here && free_) ? v : V[i]);
                RC[i] = spike ? per : ((here && !free_) ? RC[i] - 1u : RC[i]);
                mask |= static_cast<uint32_t>(spike) << i;
            }
            if (cnt)
                for (uint32_t m = mask; m; m &= m - 1u) ++cnt[(__ffs(m) - 1) * kBM];
            s_half[a][ew >> 2][er] = mask;
            const bool room = !check_room || reached(consumed_out + (t + 1) % R, need_out * ((t + 1 - R) / R + 1),
                                                     room_seen, net.poll_limit, &s_fail, net.err);
            const bool go = ok && room && (et != 0 || !s_fail);
            if (!tc::named_sync_and(2, kEpilogueThreads, go))  // the group's decision is uniform
            {
                s_fail = 1;
                atomicOr(net.err, 1u);
                if (ok) ++s;  // this step's exchange phase completed in every thread
                break;
            }
            ++s;
            my_events += static_cast<unsigned long long>(__popc(mask)) * my_fan_out;
            // The row's word (both halves) is written by the thread of the first half.
            if (cb == 0 && (n0 >> 5) < wn)  // the second half of a tile may lie past N
            {
                const uint32_t word = s_half[a][0][er] | (s_half[a][1][er] << kEN);
                if (producer)
                    out_bits[((static_cast<size_t>((t + 1) % R) * m_tiles + m_tile) * kBM + er) * wp_out +
                             (n0 >> 5)] = word;
                if (net.record && erow < b_act)
                    net.record[t * net.rec_stride + net.rec_off[layer] + static_cast<size_t>(e_smp) * wn + (n0 >> 5)] =
                        word;
            }
            if (producer)
            {
                tc::named_sync_and(2, kEpilogueThreads, true);
                if (et == 0) release_add(ready_out + (t + 1) % R);
            }
        }
        if (t1 < net.t_max)
        {
#pragma unroll
            for (int i = 0; i < kEN; ++i)
            {
                saved[i] = __float_as_uint(V[i]);
                saved[kEN + i] = RC[i];
                if (cnt) saved[2 * kEN + i] = static_cast<uint32_t>(cnt[i * kBM]);
            }
        }
        else if (cnt && erow < net.batch)
        {
            // Output spike counts of the last layer: each (sample, neuron) is owned by one thread.
            for (int i = 0; i < kEN; ++i)
                if (n0 + cb + i < N) net.counts[static_cast<size_t>(e_smp) * N + n0 + cb + i] = cnt[i * kBM];
        }
        if (et == 0)
        {
            s_sent = sent;
            s_recv = s;
            s_armed = armed;
        }
    }
    else if (lane == 0)
    {
        // Issuer: per step, once the epilogue has read the previous step's accumulator, the MMAs of
        // each expanded stage into accumulator s % 2, then one commit for it. The input slot has been read
        // once every stage of the step is expanded.
        constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, kPairN);
        // Matrix descriptor of the weight tile's first K slice; the others follow by adding byte
        // offsets / 16 to the start-address field. The A operand is read from tensor memory.
        const uint64_t dW0 = tc::smem_desc(tc::smem_u32(sW), 128, sbo_w);
        unsigned int *consumed_in = layer > 1 ? net.consumed + ctr_in : nullptr;
        uint32_t seq = 0, s = 0;
        bool stop = false;
        for (uint32_t t = t0; t < t1 && !stop; ++t)
        {
            if (m0 >= net.act[t] || s_fail) break;
            const uint32_t a = s & 1u;
            // The epilogue has read the previous step's accumulator (no tensor-memory reads run
            // beside these MMAs).
            if (s >= 1 && !wait_or_fail(&acc_empty[(s - 1) & 1u], ((s - 1) >> 1) & 1u, &s_fail, net.err))
            {
                stop = true;
                break;
            }
            tc::fence_after_sync();
            for (uint32_t c = 0; c < n_chunks; ++c)
            {
                const uint32_t u = seq + c, b = u % kStages;
                // A stage that was not written is not multiplied: the run stops here.
                if (!wait_or_fail(&full[b], (u / kStages) & 1u, &s_fail, net.err))
                {
                    stop = true;
                    break;
                }
                tc::fence_after_sync();
                const uint32_t ta = tmem + kAccCols + b * kStageCols;
                const uint64_t db = dW0 + c * ((kBK / 8 * 128) >> 4);
                const uint32_t kc = min(static_cast<uint32_t>(kBK), Kp - (c_lo + c) * kBK);
                for (uint32_t j = 0; j < kc / 16; ++j)
                    tc::mma_bf16_ta(tmem + a * kPairN, ta + j * 8, db + j * 16, idesc, (c > 0 || j > 0) ? 1u : 0u);
                tc::commit(&empty[b]);
            }
            if (stop) break;
            seq += n_chunks;
            tc::commit(&acc_full[a]);
            if (consumed_in) release_add(consumed_in + t % R);
            ++s;
        }
        if (stop)
        {
            s_fail = 1;
            atomicOr(net.err, 1u);
        }
        // Every MMA this thread issued completes (bounded wait) before the tensor memory is released;
        // a drain that does not finish is reported too.
        tc::commit(&drain);
        if (!tc::mbar_wait(&drain, 0, kWaitLimit))
        {
            s_fail = 1;
            atomicOr(net.err, 1u);
        }
    }
    if (my_events) atomicAdd(&s_events, my_events);
    tc::fence_before_sync();
    __syncthreads();
    // Exchange drain: each CTA tells its partner how many steps of partial sums it sent, then waits
    // (bounded) until every one of them has landed in its own shared memory, so that no store of the
    // partner is in flight into this CTA when it leaves (after a failure the loops end at different
    // steps).
    const bool xthread = threadIdx.x == static_cast<unsigned>(kExpandThreads);  // the first epilogue thread
    if (xthread) tc::st_cluster_u32(tc::mapa(tc::smem_u32(&s_peer_sent), tc::cluster_rank() ^ 1u), s_sent);
    tc::cluster_sync();
    if (xthread)
    {
        const uint32_t peer_sent = s_peer_sent;
        for (uint32_t q = s_recv; q < peer_sent; ++q)
        {
            if (q >= s_armed) mbar_arrive_expect_tx(&xfull[q & 1u], kXchBytes);
            if (!tc::mbar_wait_cluster(&xfull[q & 1u], (q >> 1) & 1u, kWaitLimit))
            {
                s_fail = 1;
                atomicOr(net.err, 1u);
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        if (s_fail) atomicOr(net.err, 1u);
        if (s_events) atomicAdd(net.events, s_events);
    }
    tc::cluster_sync();  // neither CTA leaves while the other may still write into its shared memory
    if (warp == kIssuerWarp) tc::tmem_dealloc(tmem, kTmemCols);
}

}  // namespace

// A batch prepared once and run as one CUDA-graph launch: memsets of the run's state, the input
// threshold kernel, then per segment of steps the input-drawing kernel and the persistent kernel
// (cluster launch of CTA pairs, every CTA resident). Reusable: every run starts from zero state, so
// repeated runs of the same plan give identical results.
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
    size_t w_bytes = 0;  // largest weight tile (shared memory besides the ring and the exchange buffers)
    uint32_t n_items = 0;
    uint32_t seg_steps = 0;  // steps per segment
    cudaGraphExec_t exec = nullptr;
    int stages = 0;
    bool cooperative = true;  // cluster launch with the cooperative attribute (cleared if refused)
    float tune_ms[3][kMaxStages + 1] = {};  // [ring choice][operand ring depth] of the autotuning runs

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
        case 2:
            return reinterpret_cast<const void *>(batched_lif_kernel<2>);
        case 3:
            return reinterpret_cast<const void *>(batched_lif_kernel<3>);
        default:
            return reinterpret_cast<const void *>(batched_lif_kernel<4>);
    }
}

size_t smem_bytes(const BatchedPlan &p, int stages)
{
    (void)stages;  // operand stages live in tensor memory
    return std::max(p.w_bytes + 2 * kXchBytes + kCntBytes, kMinDynSmem);
}

// Whether a ring of `stages` chunks fits (shared memory, every CTA pair resident at once).
bool variant_fits(const BatchedPlan &p, int stages)
{
    int device = 0, smem_max = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    const size_t smem = smem_bytes(p, stages);
    if (smem + 4096 > static_cast<size_t>(smem_max)) return false;  // 4 KB: the kernel's static shared memory
    const void *k = kernel_for(stages);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess)
        return false;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(p.n_items);
    cfg.blockDim = dim3(kBatchThreads);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, k, &cfg) != cudaSuccess)
    {
        cudaGetLastError();
        return false;
    }
    return 2ll * clusters >= p.n_items;
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
    int device = 0, sms = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaError_t lerr = cudaSuccess;
    for (uint32_t t0 = 0; t0 < p.net.t_max && lerr == cudaSuccess; t0 += p.seg_steps)
    {
        uint32_t t1 = std::min(p.net.t_max, t0 + p.seg_steps);
        const size_t words = (static_cast<size_t>(t1 - t0) + 1) * p.net.m_tiles * kBM * p.net.wpad[0];
        const unsigned blocks = static_cast<unsigned>(std::min<size_t>((words + 255) / 256, static_cast<size_t>(sms) * 8));
        input_bits_kernel<<<blocks, 256, 0, s>>>(p.net, t0, t1);
        cudaLaunchConfig_t cfg{};
        cfg.gridDim = dim3(p.n_items);
        cfg.blockDim = dim3(kBatchThreads);
        cfg.dynamicSmemBytes = smem_bytes(p, stages);
        cfg.stream = s;
        cudaLaunchAttribute attr[2];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = 2;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        attr[1].id = cudaLaunchAttributeCooperative;
        attr[1].val.cooperative = 1;
        cfg.attrs = attr;
        cfg.numAttrs = p.cooperative ? 2 : 1;
        void *args[] = {&p.net, &t0, &t1};
        lerr = cudaLaunchKernelExC(&cfg, kernel_for(stages), args);
    }
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

// Whether this process's device accepted a cooperative cluster launch (-1: not tried yet).
int g_coop_cluster = -1;

// Captures the plan with `stages` and, if `timed` (or to find out whether the cooperative cluster
// launch is accepted), runs it once. A refused cooperative launch is captured again as a plain
// cluster launch; co-residency of every CTA pair is still checked by variant_fits.
cudaError_t prepare(BatchedPlan &p, int stages, bool timed, float *ms)
{
    p.cooperative = g_coop_cluster != 0;
    cudaError_t err = capture(p, stages);
    if (err == cudaSuccess && (timed || g_coop_cluster < 0)) err = launch_timed(p, ms);
    if (err == cudaSuccess)
    {
        if (p.cooperative) g_coop_cluster = 1;
        return err;
    }
    if (p.cooperative && g_coop_cluster < 0 &&
        (err == cudaErrorInvalidValue || err == cudaErrorNotSupported || err == cudaErrorInvalidConfiguration ||
         err == cudaErrorCooperativeLaunchTooLarge))
    {
        cudaGetLastError();
        g_coop_cluster = 0;
        p.cooperative = false;
        err = capture(p, stages);
        if (err == cudaSuccess && timed) err = launch_timed(p, ms);
    }
    return err;
}

}  // namespace

// Prepares a batch. Host arrays: sizes[n_layers + 1], leak/threshold/reset/refract[n_layers],
// steps[batch], sample_sizes[(n_layers + 1) * batch] (layer-major, optional); device arrays:
// weights[l] (BF16 [sizes[l + 1]][sizes[l]]), rates [batch][sizes[0]], counts [batch][sizes[n_layers]]
// and record (optional; layouts in knp_gb300.h). With `autotune` > 0, each operand ring depth that
// fits is run twice and the fastest kept; < 0 uses depth -autotune; 0 the deepest that fits. Every
// depth computes the same results. `segment_steps` > 0
// caps the steps per persistent launch (0: as many as layer 0's slot budget allows).
int batched_plan_create(
    int n_layers, const uint32_t *sizes, const void *const *weights, const float *leak, const float *threshold,
    const float *reset, const uint32_t *refract, uint32_t batch, const uint32_t *steps, const uint32_t *sample_sizes,
    const float *rates, unsigned long long key, int *counts, uint32_t *record, int autotune, uint32_t segment_steps,
    cudaStream_t s, BatchedPlan **out, const char **why)
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
    // Failure test (KNP_GB300_BATCHED_STALL=1): every consumer layer waits for one producer CTA more
    // than exists, so its first ring wait runs out (after a short poll limit) and the run ends with
    // the error word set instead of results.
    const char *stall = std::getenv("KNP_GB300_BATCHED_STALL");
    net.stall = (stall && stall[0] == '1') ? 1u : 0u;
    net.poll_limit = net.stall ? (1u << 16) : kPollLimit;
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
            net.wpad[l - 1] = net.chunks[l] * kChunkWords;
            if ((net.chunks[l] + 1) / 2 > kMaxHalfChunks)
            {
                *why = "a layer's fan-in exceeds 2048";
                return -1;
            }
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
    // Work items: (layer, 128-sample tile, 64-neuron tile, K half), the two halves of a tile adjacent
    // (one cluster).
    const uint32_t m_tiles = (batch + kBM - 1) / kBM;
    net.m_tiles = m_tiles;
    for (int l = 1; l <= n_layers; ++l)
    {
        const uint32_t n_tiles = (net.size[l] + kPairN - 1) / kPairN;
        net.n_cta[l] = 2 * n_tiles;
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
               "(fan-in too large) or the CTA pairs exceed the resident clusters";
        return -1;
    }
    if (autotune < 0)
    {
        // A fixed ring depth (-autotune).
        if (-autotune < kMinStages || -autotune > kMaxStages || !variant_fits(p, -autotune))
        {
            *why = "the requested operand ring depth is out of range or does not fit";
            return -1;
        }
        best = -autotune;
        autotune = 0;
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
    // Segments: layer 0's slots of one segment stay within the budget.
    const size_t slot_bytes = static_cast<size_t>(m_tiles) * kBM * net.wpad[0] * 4;
    p.seg_steps = static_cast<uint32_t>(std::max<size_t>(1, std::min<size_t>(net.t_max, kInputSlotBudget / slot_bytes)));
    if (segment_steps) p.seg_steps = std::min(p.seg_steps, segment_steps);
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
    ok = ok && (net.bits[0] = static_cast<uint32_t *>(dalloc(p.seg_steps * slot_bytes))) != nullptr;
    for (int l = 1; l < n_layers && ok; ++l)
    {
        const size_t bytes = static_cast<size_t>(kMaxRing) * m_tiles * kBM * net.wpad[l] * 4;
        ok = (net.bits[l] = static_cast<uint32_t *>(dalloc(bytes))) != nullptr;
        p.zero.emplace_back(net.bits[l], bytes);
    }
    const size_t n_counters = static_cast<size_t>(kMaxLayers + 1) * m_tiles * kMaxRing;
    ok = ok && (net.ready = static_cast<unsigned int *>(dalloc(n_counters * 4))) != nullptr;
    ok = ok && (net.consumed = static_cast<unsigned int *>(dalloc(n_counters * 4))) != nullptr;
    ok = ok && (net.state = static_cast<uint32_t *>(
                    dalloc(static_cast<size_t>(p.n_items) * kEpilogueThreads * kStateWords * 4))) != nullptr;
    p.n_thr = static_cast<size_t>(batch) * sizes[0];
    ok = ok && (p.d_thr = static_cast<unsigned long long *>(dalloc(p.n_thr * 8))) != nullptr;
    net.rate_thr = p.d_thr;
    p.rates = rates;
    ok = ok && (net.events = static_cast<unsigned long long *>(dalloc(8))) != nullptr;
    ok = ok && (net.err = static_cast<unsigned int *>(dalloc(4))) != nullptr;
    if (!ok)
    {
        *why = "device allocation failed";
        return -5;
    }
    p.zero.emplace_back(counts, static_cast<size_t>(batch) * net.size[n_layers] * 4);
    p.zero.emplace_back(net.events, 8);
    p.zero.emplace_back(net.err, 4);
    p.zero.emplace_back(net.ready, n_counters * 4);
    p.zero.emplace_back(net.consumed, n_counters * 4);
    unsigned long long off = 0;
    for (int l = 0; l <= n_layers; ++l)
    {
        net.rec_off[l] = off;
        off += static_cast<unsigned long long>(batch) * net.words[l];
    }
    net.rec_stride = off;
    if (record) p.zero.emplace_back(record, static_cast<size_t>(net.t_max) * off * 4);

    cudaError_t err = cudaSuccess;
    net.ring = kDefaultRing;
    if (autotune)
    {
        // Schedule choices that leave every result bit-identical: the operand ring depth and the
        // length of the layer rings (how far a layer may run ahead of the next).
        float best_ms = 0.f;
        uint32_t best_ring = kDefaultRing;
        for (int ri = 0; ri < 3 && err == cudaSuccess; ++ri)
            for (int stg = kMinStages; stg <= kMaxStages; ++stg)
            {
                if (!variant_fits(p, stg)) continue;
                net.ring = kRingChoices[ri];
                float t = 0.f;
                err = prepare(p, stg, true, &t);
                if (err == cudaSuccess) err = launch_timed(p, &t);
                if (err != cudaSuccess) break;
                p.tune_ms[ri][stg] = t;
                if (!best_ms || t < best_ms)
                {
                    best_ms = t;
                    best = stg;
                    best_ring = kRingChoices[ri];
                }
            }
        net.ring = best_ring;
        if (err == cudaSuccess) err = capture(p, best);
    }
    else
    {
        err = prepare(p, best, false, nullptr);
    }
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
        *why = (kerr & 2u) ? "the batched kernel ran without its two-CTA cluster shape"
                           : "a tensor-core completion wait, the pair exchange or a layer's step counter wait timed out";
        return -4;
    }
    return 0;
}

void batched_plan_info(const BatchedPlan *p, int *stages, int *ring_steps, float *tune_ms)
{
    if (stages) *stages = p->stages;
    if (ring_steps) *ring_steps = static_cast<int>(p->net.ring);
    if (tune_ms)
        for (int ri = 0; ri < 3; ++ri)
            for (int i = kMinStages; i <= kMaxStages; ++i)
                tune_ms[ri * (kMaxStages - kMinStages + 1) + (i - kMinStages)] = p->tune_ms[ri][i];
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
                                 rates, key, counts, record, 0, 0, s, &p, why);
    if (rc == 0) rc = batched_plan_run(p, events_out, ms, why);
    if (p) batched_plan_destroy(p);
    return rc;
}

}  // namespace knp_gb300
