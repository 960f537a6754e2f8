// Batched form on 5th-generation tensor cores.
//
// bf16_gemm_tn: D[M x N] (FP32) = A[M x K] * B[N x K]^T with BF16 operands (row-major, K
// contiguous), tcgen05.mma kind::f16 with the accumulator in tensor memory. Used to validate the
// tcgen05 encodings and as a library GEMM of spike matrices.
#include <algorithm>
#include <cstdint>
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
// tile stays in shared memory for the whole run. Spike matrices live in global memory as bitmaps
// (double-buffered by step parity) and are expanded to BF16 0/1 in shared memory, 128 inputs at a
// time. Samples are processed sorted by decreasing T, so finished samples leave whole M-tiles idle
// ("compaction" by order). Steps are separated by a grid barrier; the kernel is launched
// cooperatively (every CTA resident) and every wait is bounded.
namespace knp_gb300
{
namespace
{

constexpr int kBM = 128, kBN = 32, kBK = 128, kMaxLayers = 4, kMaxItems = 512;
constexpr int kRoundChunks = 2;                   // K chunks expanded between two block barriers
constexpr int kABufs = 2 * kRoundChunks;          // A chunk buffers: two rounds in flight
constexpr int kInCache = 8;                       // input words per warp whose draw thresholds stay in registers
constexpr int kBatchThreads = 256;

struct BatchedNet
{
    int n_layers;
    uint32_t size[kMaxLayers + 1];
    uint32_t words[kMaxLayers + 1];  // ceil(size / 32)
    uint32_t kpad[kMaxLayers + 1];   // kpad[l] = size[l - 1] rounded up to 16
    const __nv_bfloat16 *w[kMaxLayers];
    float leak[kMaxLayers], thr[kMaxLayers], reset[kMaxLayers];
    uint32_t refract[kMaxLayers];
    uint32_t batch;
    const uint32_t *perm;  // slot -> sample
    const uint32_t *act;   // [t_max]: slots still running at step t (slots sorted by decreasing T)
    const unsigned long long *rate_thr;  // [batch][size[0]] by sample: rate * 2^53, the draw's threshold
    unsigned long long key;
    uint32_t t_max;
    uint32_t *bits[kMaxLayers + 1][2];  // [batch][words[l]] per step parity
    int *counts;                         // [batch][size[L]] by sample
    uint32_t *record;                    // [t_max][sum_l batch * words[l]] by sample, or null
    unsigned long long rec_off[kMaxLayers + 1];
    unsigned long long rec_stride;
    unsigned long long *events;
    unsigned int *err;
    unsigned int *barrier;  // [0] arrivals, [1] generation
    uint32_t n_items;
    uint16_t item_layer[kMaxItems];
    uint16_t item_m[kMaxItems];
    uint16_t item_n[kMaxItems];  // 32-neuron tile index
};

__device__ __forceinline__ bool grid_sync(unsigned int *bar, unsigned int n_blocks, uint32_t limit)
{
    __shared__ int ok_s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        volatile unsigned int *gen = bar + 1;
        const unsigned int g = *gen;
        __threadfence();
        const unsigned int arrived = atomicAdd(bar, 1u) + 1u;
        int ok = 1;
        if (arrived == n_blocks)
        {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        }
        else
        {
            uint32_t i = 0;
            while (*gen == g && i < limit) ++i;
            ok = *gen != g;
        }
        __threadfence();
        ok_s = ok;
    }
    __syncthreads();
    return ok_s != 0;
}

// Per (sample, input): the 53-bit threshold that the input draw is compared with.
__global__ void rate_threshold_kernel(const float *rates, unsigned long long *thr, size_t n)
{
    const size_t i = static_cast<size_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) thr[i] = static_cast<unsigned long long>(static_cast<double>(rates[i]) * 9007199254740992.0);
}

__device__ __forceinline__ void cp_async4(uint32_t *dst, const uint32_t *src)
{
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(tc::smem_u32(dst)), "l"(src) : "memory");
}

__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__global__ void __launch_bounds__(kBatchThreads, 1) batched_lif_kernel(BatchedNet net)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint32_t tmem_slot;
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t sbits[kBM];
    __shared__ unsigned long long s_events;
    const uint32_t item = blockIdx.x;
    const int layer = net.item_layer[item];  // 1..L
    const uint32_t m0 = net.item_m[item] * kBM;
    const uint32_t n0 = net.item_n[item] * kBN;
    const uint32_t K = net.size[layer - 1], Kp = net.kpad[layer], N = net.size[layer];
    const uint32_t wk = net.words[layer - 1], wn = net.words[layer];
    const uint32_t bm_stride = wk | 1u;  // odd row stride: 32 consecutive rows hit 32 banks
    // Shared memory: weight tile [kBN x Kp], kABufs A chunks [kBM x kBK], spike bitmap rows [kBM x bm_stride].
    uint8_t *sW = smem;
    uint8_t *sA = smem + static_cast<size_t>(kBN) * Kp * 2;
    uint32_t *sBM = reinterpret_cast<uint32_t *>(sA + static_cast<size_t>(kABufs) * kBM * kBK * 2);
    const uint32_t sbo_w = (Kp / 8) * 128, sbo_a = (kBK / 8) * 128;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // Weight tile rows n0..n0+31 (zero beyond N), inputs 0..Kp (zero beyond K).
    for (uint32_t u = threadIdx.x; u < kBN * (Kp / 8); u += blockDim.x)
    {
        const uint32_t r = u / (Kp / 8), g = u % (Kp / 8), n = n0 + r, k = g * 8;
        __nv_bfloat16 tmp[8];
#pragma unroll
        for (int e = 0; e < 8; ++e)
            tmp[e] = (n < N && k + e < K) ? net.w[layer - 1][static_cast<size_t>(n) * K + k + e] : __float2bfloat16(0.0f);
        *reinterpret_cast<uint4 *>(sW + tc::core_offset(r, k, 128, sbo_w)) = *reinterpret_cast<uint4 *>(tmp);
    }
    if (warp == 0) tc::tmem_alloc(&tmem_slot, 32);
    if (threadIdx.x == 0)
    {
        tc::mbar_init(&mbar[0], 1);
        tc::mbar_init(&mbar[1], 1);
        s_events = 0;
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = tmem_slot;
    constexpr uint32_t idesc = tc::idesc_bf16_f32(kBM, kBN);
    const uint32_t fan_out = layer < net.n_layers ? net.size[layer + 1] : 0u;
    const uint32_t n_chunks = (Kp + kBK - 1) / kBK;
    uint32_t uses[2] = {0, 0};  // commits made on each round mbarrier so far
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

    // Input words this warp draws every step (u = warp id + j * warps in grid) and, for the first
    // kInCache of them, this lane's draw threshold and sample, kept in registers for the run.
    const uint32_t n_in = net.size[0], w0 = net.words[0];
    const uint64_t in_total = static_cast<uint64_t>(net.batch) * w0;
    const uint32_t wpb = blockDim.x >> 5;
    const uint64_t gw = static_cast<uint64_t>(blockIdx.x) * wpb + warp, nw = static_cast<uint64_t>(gridDim.x) * wpb;
    unsigned long long in_thr[kInCache];
    uint32_t in_smp[kInCache];
#pragma unroll
    for (int j = 0; j < kInCache; ++j)
    {
        const uint64_t u = gw + j * nw;
        in_thr[j] = 0;
        in_smp[j] = 0;
        if (u < in_total)
        {
            const uint32_t slot = static_cast<uint32_t>(u / w0), i = static_cast<uint32_t>(u % w0) * 32 + lane;
            in_smp[j] = net.perm[slot];
            if (i < n_in) in_thr[j] = net.rate_thr[static_cast<size_t>(in_smp[j]) * n_in + i];
        }
    }

    uint32_t b_next = net.act[0];
    for (uint32_t t = 0; t < net.t_max && ok; ++t)
    {
        const uint32_t b_act = b_next;
        if (t + 1 < net.t_max) b_next = net.act[t + 1];  // used next step; the load overlaps this one
        const uint32_t *src = net.bits[layer - 1][(t + 1) & 1];
        uint32_t *dst = net.bits[layer][t & 1];
        if (threadIdx.x < kBM) sbits[threadIdx.x] = 0;
        if (m0 < b_act)
        {
            // This tile's rows of the previous layer's spike bitmap (step t - 1): asynchronous 4-byte
            // copies, all in flight at once.
            for (uint32_t u = threadIdx.x; u < kBM * wk; u += blockDim.x)
            {
                const uint32_t r = u / wk, w = u % wk, row = m0 + r;
                if (row < net.batch)
                    cp_async4(sBM + r * bm_stride + w, src + static_cast<size_t>(row) * wk + w);
                else
                    sBM[r * bm_stride + w] = 0u;
            }
            cp_async_wait_all();
            __syncthreads();
            uint32_t rounds = 0;
            for (uint32_t c0 = 0; c0 < n_chunks && ok; c0 += kRoundChunks, ++rounds)
            {
                const uint32_t c1 = min(c0 + kRoundChunks, n_chunks);
                const uint32_t pr = rounds & 1u;
                if (rounds >= 2)
                {
                    // The MMAs of round `rounds - 2` read these buffers; they must have completed.
                    const bool waited = tc::mbar_wait(&mbar[pr], (uses[pr] - 1) & 1u, kWaitLimit);
                    tc::fence_after_sync();
                    if (!waited) ok = false;
                }
                // Expand 0/1 bits to BF16 (1.0 = 0x3F80): unit (row r, 8-input group g of the round);
                // rows vary fastest so that 8 consecutive lanes fill one 128-byte core matrix.
                const uint32_t groups = (min(c1 * kBK, Kp) - c0 * kBK) / 8;
                for (uint32_t u = threadIdx.x; u < kBM * groups; u += blockDim.x)
                {
                    const uint32_t r = u % kBM, gg = u / kBM;
                    const uint32_t k = c0 * kBK + gg * 8;
                    const uint32_t c = k / kBK, g = (k % kBK) / 8;
                    uint8_t *a = sA + static_cast<size_t>(c % kABufs) * kBM * kBK * 2;
                    const uint32_t byte = (sBM[r * bm_stride + (k >> 5)] >> (k & 31)) & 0xFFu;
                    uint32_t h[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        h[e] = (((byte >> (2 * e)) & 1u) ? 0x3F80u : 0u) |
                               (((byte >> (2 * e + 1)) & 1u) ? 0x3F800000u : 0u);
                    *reinterpret_cast<uint4 *>(a + tc::core_offset(r, g * 8, 128, sbo_a)) =
                        make_uint4(h[0], h[1], h[2], h[3]);
                }
                tc::fence_async_smem();
                ok = __syncthreads_and(ok ? 1 : 0) != 0;
                if (!ok) break;
                if (threadIdx.x == 0)
                {
                    tc::fence_after_sync();
                    for (uint32_t c = c0; c < c1; ++c)
                    {
                        const uint8_t *a = sA + static_cast<size_t>(c % kABufs) * kBM * kBK * 2;
                        const uint32_t k0 = c * kBK, kc = min(static_cast<uint32_t>(kBK), Kp - k0);
                        for (uint32_t j = 0; j < kc / 16; ++j)
                        {
                            const uint64_t da = tc::smem_desc(tc::smem_u32(a) + j * 256, 128, sbo_a);
                            const uint64_t db = tc::smem_desc(tc::smem_u32(sW) + (k0 / 8 + 2 * j) * 128, 128, sbo_w);
                            tc::mma_bf16(tmem, da, db, idesc, (c > 0 || j > 0) ? 1u : 0u);
                        }
                    }
                    tc::commit(&mbar[pr]);
                }
                ++uses[pr];
            }
            // Wait for the commits not waited for yet (the last min(rounds, 2) rounds), also after a
            // failed wait, so that no MMA is in flight when the kernel leaves.
            {
                bool waited = true;
                for (uint32_t q = (rounds > 2 ? rounds - 2 : 0); q < rounds; ++q)
                    waited = tc::mbar_wait(&mbar[q & 1u], (uses[q & 1u] - 1) & 1u, kWaitLimit) && waited;
                tc::fence_after_sync();
                ok = waited && ok;
            }
            ok = __syncthreads_and(ok ? 1 : 0) != 0;
            uint32_t mask = 0;
            if (ok)
            {
                float acc[16];
                tc::tmem_ld16(tmem + ((32u * (warp & 3)) << 16) + cb, acc);
                if (erow < b_act)
                {
#pragma unroll
                    for (int i = 0; i < 16; ++i)
                    {
                        if (n0 + cb + i >= N) break;
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
            if (mask) atomicOr(&sbits[er], mask);
            tc::fence_before_sync();
            __syncthreads();
            if (threadIdx.x < kBM)
            {
                const uint32_t rr = threadIdx.x, rw = m0 + rr;
                if (rw < net.batch)
                {
                    const uint32_t bw = sbits[rr];
                    dst[static_cast<size_t>(rw) * wn + (n0 >> 5)] = bw;
                    if (net.record && rw < b_act)
                        net.record[t * net.rec_stride + net.rec_off[layer] + static_cast<size_t>(net.perm[rw]) * wn +
                                   (n0 >> 5)] = bw;
                    my_events += static_cast<unsigned long long>(__popc(bw)) * fan_out;
                }
            }
        }
        // Input spikes of step t (layer 0), spread over every warp of the grid: a warp makes one
        // 32-input word per iteration, one draw per lane, combined by a ballot.
        {
            uint32_t *d0 = net.bits[0][t & 1];
            uint32_t j = 0;
            for (uint64_t u = gw; u < in_total; u += nw, ++j)
            {
                const uint32_t slot = static_cast<uint32_t>(u / w0), wi = static_cast<uint32_t>(u % w0);
                const uint32_t i = wi * 32 + lane;
                bool bit = false;
                uint32_t smp = 0;
                if (slot < b_act)
                {
                    unsigned long long thr64;
                    if (j < kInCache)
                    {
                        // Registers indexed by a loop counter: select with a fixed unrolled scan.
                        thr64 = 0;
#pragma unroll
                        for (int q = 0; q < kInCache; ++q)
                            if (q == static_cast<int>(j))
                            {
                                thr64 = in_thr[q];
                                smp = in_smp[q];
                            }
                    }
                    else
                    {
                        smp = net.perm[slot];
                        thr64 = i < n_in ? net.rate_thr[static_cast<size_t>(smp) * n_in + i] : 0ull;
                    }
                    if (i < n_in)
                    {
                        const unsigned long long ctr = (static_cast<unsigned long long>(t) * net.batch + smp) * n_in + i;
                        bit = (rand64(net.key, ctr) >> 11) < thr64;
                    }
                }
                const uint32_t word = __ballot_sync(0xffffffffu, bit);
                if (lane == 0)
                {
                    d0[u] = word;
                    if (slot < b_act)
                    {
                        if (net.record)
                            net.record[t * net.rec_stride + net.rec_off[0] + static_cast<size_t>(smp) * w0 + wi] = word;
                        my_events += static_cast<unsigned long long>(__popc(word)) * net.size[1];
                    }
                }
            }
        }
        __threadfence();
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
    if (!ok && threadIdx.x == 0) atomicOr(net.err, 1u);
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0 && s_events) atomicAdd(net.events, s_events);
    if (warp == 0) tc::tmem_dealloc(tmem, 32);
}

}  // namespace

// Runs a whole batch. Host arrays: sizes[n_layers + 1], leak/threshold/reset/refract[n_layers],
// steps[batch]; device arrays: weights[l] (BF16 [sizes[l + 1]][sizes[l]]), rates [batch][sizes[0]],
// counts [batch][sizes[n_layers]] (zeroed here), record (optional, see knp_gb300.h).
int batched_lif_run(
    int n_layers, const uint32_t *sizes, const void *const *weights, const float *leak, const float *threshold,
    const float *reset, const uint32_t *refract, uint32_t batch, const uint32_t *steps, const float *rates,
    unsigned long long key, int *counts, uint32_t *record, unsigned long long *events_out, float *ms,
    cudaStream_t s, const char **why)
{
    if (n_layers < 1 || n_layers > kMaxLayers || batch == 0 || !sizes || !weights || !steps || !rates || !counts)
    {
        *why = "bad arguments";
        return -1;
    }
    BatchedNet net{};
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
        if (l > 0) net.kpad[l] = (sizes[l - 1] + 15) / 16 * 16;
    }
    // Work items: (layer, 128-sample tile, 32-neuron tile).
    const uint32_t m_tiles = (batch + kBM - 1) / kBM;
    uint32_t n_items = 0;
    size_t smem = 0;
    for (int l = 1; l <= n_layers; ++l)
    {
        for (uint32_t m = 0; m < m_tiles; ++m)
            for (uint32_t n = 0; n < net.words[l]; ++n)
            {
                if (n_items >= kMaxItems)
                {
                    *why = "too many (layer, sample tile, neuron tile) work items";
                    return -1;
                }
                net.item_layer[n_items] = static_cast<uint16_t>(l);
                net.item_m[n_items] = static_cast<uint16_t>(m);
                net.item_n[n_items] = static_cast<uint16_t>(n);
                ++n_items;
            }
        smem = std::max<size_t>(smem, static_cast<size_t>(kBN) * net.kpad[l] * 2 + kABufs * kBM * kBK * 2 +
                                          kBM * (net.words[l - 1] | 1u) * 4);
    }
    net.n_items = n_items;
    int device = 0, sms = 0, per_sm = 0, smem_max = 0;
    cudaGetDevice(&device);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (smem > static_cast<size_t>(smem_max))
    {
        *why = "a layer's weight tile and staging buffers exceed the shared memory of one CTA (fan-in too large)";
        return -1;
    }
    cudaError_t err = cudaFuncSetAttribute(batched_lif_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(smem));
    if (err == cudaSuccess)
        err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_lif_kernel, kBatchThreads, smem);
    if (err != cudaSuccess)
    {
        *why = cudaGetErrorString(err);
        return -3;
    }
    if (static_cast<long long>(per_sm) * sms < n_items)
    {
        *why = "the batch needs more resident CTAs than the device holds";
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
    for (int l = 0; l < n_layers; ++l)
    {
        net.w[l] = static_cast<const __nv_bfloat16 *>(weights[l]);
        net.leak[l] = leak ? leak[l] : 1.0f;
        net.thr[l] = threshold ? threshold[l] : 1.0f;
        net.reset[l] = reset ? reset[l] : 0.0f;
        net.refract[l] = refract ? refract[l] : 0u;
    }
    std::vector<void *> allocs;
    auto dalloc = [&](size_t bytes) -> void *
    {
        void *p = nullptr;
        if (cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        allocs.push_back(p);
        cudaMemsetAsync(p, 0, bytes ? bytes : 16, s);
        return p;
    };
    bool ok = true;
    uint32_t *d_perm = static_cast<uint32_t *>(dalloc(batch * 4));
    uint32_t *d_act = static_cast<uint32_t *>(dalloc(static_cast<size_t>(net.t_max) * 4));
    ok = ok && d_perm && d_act;
    for (int l = 0; l <= n_layers && ok; ++l)
        for (int p = 0; p < 2 && ok; ++p)
            ok = (net.bits[l][p] = static_cast<uint32_t *>(dalloc(static_cast<size_t>(batch) * net.words[l] * 4)));
    unsigned long long *d_thr =
        static_cast<unsigned long long *>(dalloc(static_cast<size_t>(batch) * sizes[0] * sizeof(unsigned long long)));
    ok = ok && d_thr;
    net.rate_thr = d_thr;
    net.events = static_cast<unsigned long long *>(dalloc(8));
    net.err = static_cast<unsigned int *>(dalloc(4));
    net.barrier = static_cast<unsigned int *>(dalloc(8));
    ok = ok && net.events && net.err && net.barrier;
    int rc = 0;
    if (!ok)
    {
        *why = "device allocation failed";
        rc = -5;
    }
    else
    {
        cudaMemcpyAsync(d_perm, perm.data(), batch * 4, cudaMemcpyHostToDevice, s);
        // act[t] = slots with T > t (slots are sorted by decreasing T).
        std::vector<uint32_t> act(net.t_max);
        for (uint32_t t = 0, a = batch; t < net.t_max; ++t)
        {
            while (a > 0 && st[a - 1] <= t) --a;
            act[t] = a;
        }
        cudaMemcpyAsync(d_act, act.data(), act.size() * 4, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(counts, 0, static_cast<size_t>(batch) * net.size[n_layers] * 4, s);
        net.perm = d_perm;
        net.act = d_act;
        net.record = record;
        unsigned long long off = 0;
        for (int l = 0; l <= n_layers; ++l)
        {
            net.rec_off[l] = off;
            off += static_cast<unsigned long long>(batch) * net.words[l];
        }
        net.rec_stride = off;
        if (record) cudaMemsetAsync(record, 0, static_cast<size_t>(net.t_max) * off * 4, s);
        const size_t n_thr = static_cast<size_t>(batch) * sizes[0];
        rate_threshold_kernel<<<static_cast<unsigned>((n_thr + 255) / 256), 256, 0, s>>>(rates, d_thr, n_thr);
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, s);
        void *args[] = {&net};
        err = cudaLaunchCooperativeKernel(reinterpret_cast<void *>(batched_lif_kernel), dim3(n_items),
                                          dim3(kBatchThreads), args, smem, s);
        cudaEventRecord(e1, s);
        if (err == cudaSuccess) err = cudaEventSynchronize(e1);
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        if (ms) *ms = t;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        unsigned long long ev = 0;
        unsigned int kerr = 0;
        if (err == cudaSuccess) err = cudaMemcpy(&ev, net.events, 8, cudaMemcpyDeviceToHost);
        if (err == cudaSuccess) err = cudaMemcpy(&kerr, net.err, 4, cudaMemcpyDeviceToHost);
        if (events_out) *events_out = ev;
        if (err != cudaSuccess)
        {
            *why = cudaGetErrorString(err);
            rc = -3;
        }
        else if (kerr)
        {
            *why = "a tensor-core completion wait or the grid barrier timed out";
            rc = -4;
        }
    }
    cudaStreamSynchronize(s);
    for (void *p : allocs) cudaFree(p);
    return rc;
}

}  // namespace knp_gb300
