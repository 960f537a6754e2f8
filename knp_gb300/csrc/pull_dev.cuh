// Device code of the gather ("pull") form of a delta projection, shared by the per-step gather
// kernel (pull.cu) and the persistent grid step kernel (grid_net.cu).
//
// For the step tn whose input it completes, a block walks, for every delay d whose step tn - d was
// recorded in the projection's spike bitmap, the slices of its range of 256-target windows in the
// sliced ELL layout of kernels.h: each lane owns one target of a slice and sums, down its list, the
// weights of the synapses whose presynaptic bit is set (bitmap staged in shared memory), then adds
// the sum to the target's accumulator; the accumulators are added once to the targets' input-ring
// slot of step tn. The sums are the impacts the scatter would have delivered at step tn (delay
// convention of delta_impl.h:78-79 of the reference CPU library), added in another order, which is
// exact for the FP32 ring (dyadic weights); populations with the fixed-point ring never use this form.
#pragma once

#include <cstdint>
#include <type_traits>

#include <cuda_fp16.h>

#include "kernels.h"

namespace knp_gb300
{
namespace
{

constexpr int kGatherThreads = 1024;
constexpr int kDepth = 16;  // list entries per lane in flight

// Hint: bring [p, p + bytes) into L2 (16-byte aligned address and size; no completion to wait for).
__device__ __forceinline__ void prefetch_l2(const void *p, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Slices ahead of the one a warp takes whose entries it asks L2 to fetch: by the time a warp takes
// that slice its loads hit L2 instead of DRAM (full-size step: 8 and 16 give 0.80 ms, 32 0.81 ms,
// 64 0.84 ms).
constexpr uint32_t kPrefetchAhead = 16;

enum WeightForm
{
    kDict = 0,  // 8-bit dictionary index in the top bits of the packed entry
    kHalf = 1,  // FP16
    kFull = 2,  // FP32
};


// Shared memory of one gather block: the step's spike bitmap, the accumulators of the block's
// windows and (dictionary weights) 32 replicas of the dictionary.
__host__ __device__ inline size_t gather_smem_for(const PullDev &p, uint32_t G)
{
    const uint64_t windows_per_block = (p.n_windows + G - 1) / G;
    return static_cast<size_t>(p.words) * 4 + windows_per_block * kPullWindow * 4 +
           (p.tab_rep ? static_cast<size_t>(p.n_tab) * 32 * 4 : 0);
}

// Whether the gather of step tn has work: some delay d in 1..max_delay whose step tn - d was pulled.
__device__ __forceinline__ bool gather_needed(const PullDev &g, unsigned long long tn)
{
    for (uint32_t d = 1; d <= g.max_delay && d <= tn; ++d)
        if (g.pulled[static_cast<uint32_t>((tn - d) % g.hist_slots)]) return true;
    return false;
}

// Clears block `block`'s share (of G) of the bitmap slot that the scatter kernel of step tn will
// fill; it holds step tn - hist_slots, which no gather reads any more.
__device__ __forceinline__ void clear_bitmap_slot(const PullDev &g, unsigned long long tn, uint32_t block, uint32_t G)
{
    const uint32_t sl_next = static_cast<uint32_t>(tn % g.hist_slots);
    uint32_t *dst = g.bitmap + static_cast<size_t>(sl_next) * g.words;
    const uint32_t b0 = static_cast<uint32_t>(static_cast<uint64_t>(block) * g.words / G);
    const uint32_t b1 = static_cast<uint32_t>(static_cast<uint64_t>(block + 1) * g.words / G);
    for (uint32_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) dst[i] = 0u;
}

// Block `block` of G gather blocks completes the input of step tn (every thread of the block calls
// it; it contains block barriers), and clears its share of the bitmap slot that step tn's spikes
// will be recorded in. smem_u4: gather_smem_for(p.pull, G) bytes of dynamic shared memory.
template <int kForm>
__device__ __forceinline__ void gather_block(const ProjectionDev &p, unsigned long long tn, uint32_t block, uint32_t G,
                                             uint4 *smem_u4)
{
    __shared__ uint32_t s_next;  // next slice of the current delay to hand out
    __shared__ float s_tab[256];
    __shared__ uint8_t s_pflag[256];  // pulled flag of step tn - d, d = 1 .. max_delay (max_delay <= 255)
    const PullDev &g = p.pull;
    uint32_t *bm = reinterpret_cast<uint32_t *>(smem_u4);
    float *acc = reinterpret_cast<float *>(bm + g.words);
    float *rep = acc + static_cast<size_t>((g.n_windows + G - 1) / G) * kPullWindow;  // after the largest acc
    if (kForm == kDict)
    {
        if (g.tab_rep)
            for (uint32_t i = threadIdx.x; i < g.n_tab * 32u; i += blockDim.x) rep[i] = g.wtab[i >> 5];
        else
            for (uint32_t i = threadIdx.x; i < 256; i += blockDim.x) s_tab[i] = g.wtab[i];
    }
    const uint32_t w0 = static_cast<uint32_t>(static_cast<uint64_t>(block) * g.n_windows / G);
    const uint32_t w1 = static_cast<uint32_t>(static_cast<uint64_t>(block + 1) * g.n_windows / G);
    const uint32_t n_acc = (w1 - w0) * kPullWindow;
    const int lane = threadIdx.x & 31;
    for (uint32_t d = 1 + threadIdx.x; d <= g.max_delay; d += blockDim.x)
        s_pflag[d] = d <= tn ? static_cast<uint8_t>(g.pulled[static_cast<uint32_t>((tn - d) % g.hist_slots)]) : 0;
    __syncthreads();

    bool any = false;
    for (uint32_t d = 1; d <= g.max_delay && d <= tn; ++d)
    {
        const unsigned long long s = tn - d;
        const uint32_t sl = static_cast<uint32_t>(s % g.hist_slots);
        const uint32_t pflag = s_pflag[d];
        if (!pflag) continue;
        const bool all = pflag == 2u;  // every presynaptic neuron fired at step s: no bitmap needed
        if (!any)
        {
            for (uint32_t i = threadIdx.x; i < n_acc; i += blockDim.x) acc[i] = 0.0f;
            any = true;
        }
        __syncthreads();  // the previous bitmap is no longer read
        if (!all)
        {
            const uint4 *src = reinterpret_cast<const uint4 *>(g.bitmap + static_cast<size_t>(sl) * g.words);
            for (uint32_t i = threadIdx.x; i < g.words / 4; i += blockDim.x) smem_u4[i] = src[i];
        }
        if (threadIdx.x == 0) s_next = 0;
        __syncthreads();
        const size_t q0 = (static_cast<size_t>(d - 1) * g.n_windows + w0) * kPullSlicesPerWindow;
        const uint32_t n_q = (w1 - w0) * kPullSlicesPerWindow;
        // Slices are handed out one at a time (lists differ in length: longest first within a window).
        for (;;)
        {
            uint32_t qi = 0;
            if (lane == 0) qi = atomicAdd(&s_next, 1u);
            qi = __shfl_sync(0xffffffffu, qi, 0);
            if (qi >= n_q)
            {
                // The first kPrefetchAhead warps to run out prefetch the first slices of the next
                // delay (those no earlier slice's prefetch covered).
                const uint32_t r = qi - n_q;
                if (lane == 0 && r < kPrefetchAhead && r < n_q && d < g.max_delay && d < tn &&
                    g.pulled[static_cast<uint32_t>((tn - d - 1) % g.hist_slots)])
                {
                    const size_t qa = (static_cast<size_t>(d) * g.n_windows + w0) * kPullSlicesPerWindow + r;
                    const uint32_t la = g.slice_len[qa];
                    if (la)
                    {
                        prefetch_l2(g.packed + g.slice_ptr[qa], la * kPullSlice * 4u);
                        if (kForm == kHalf) prefetch_l2(g.w16 + g.slice_ptr[qa], la * kPullSlice * 2u);
                        if (kForm == kFull) prefetch_l2(g.w + g.slice_ptr[qa], la * kPullSlice * 4u);
                    }
                }
                break;
            }
            if (lane == 0 && qi + kPrefetchAhead < n_q)
            {
                const size_t qa = q0 + qi + kPrefetchAhead;
                const uint32_t la = g.slice_len[qa];
                if (la)
                {
                    // Slices start on 32-entry boundaries; one slice is len x 32 entries.
                    prefetch_l2(g.packed + g.slice_ptr[qa], la * kPullSlice * 4u);
                    if (kForm == kHalf) prefetch_l2(g.w16 + g.slice_ptr[qa], la * kPullSlice * 2u);
                    if (kForm == kFull) prefetch_l2(g.w + g.slice_ptr[qa], la * kPullSlice * 4u);
                }
            }
            const size_t q = q0 + qi;
            const uint32_t len = g.slice_len[q];
            if (len == 0) continue;
            // Entry k of this lane's list is at slice_ptr + 32 k + lane (a warp load reads 128
            // consecutive bytes). Full rounds of kDepth entries run without bounds checks; an absent
            // spike adds +0.0, which leaves the sum unchanged (the sum is never -0.0: it starts at
            // +0.0 and a round-to-nearest sum is -0.0 only if both terms are).
            const long long off = g.slice_ptr[q] + lane;
            const uint32_t *pk = g.packed + off;
            const uint16_t *ph = kForm == kHalf ? g.w16 + off : nullptr;
            const float *pf = kForm == kFull ? g.w + off : nullptr;
            // Two copies of the walk: with the bit test, and without it for a step in which every
            // presynaptic neuron fired (the test would always pass).
            auto walk = [&](auto all_tag) -> float
            {
                constexpr bool kAll = decltype(all_tag)::value;
                auto value = [&](uint32_t pn, float wi) -> float
                {
                    if (kForm == kDict)
                    {
                        wi = g.tab_rep ? rep[((pn >> 24) << 5) + lane] : s_tab[pn >> 24];
                        pn &= 0xFFFFFFu;
                    }
                    if (kAll) return wi;
                    return ((bm[pn >> 5] >> (pn & 31)) & 1u) ? wi : 0.0f;
                };
                float sum = 0.0f;
                uint32_t k0 = 0;
                for (; k0 + kDepth <= len; k0 += kDepth)
                {
                    const size_t o = static_cast<size_t>(k0) * kPullSlice;
                    uint32_t pre[kDepth];
                    float w[kDepth];
#pragma unroll
                    for (int i = 0; i < kDepth; ++i)
                    {
                        pre[i] = __ldcs(pk + o + i * kPullSlice);
                        w[i] = 0.0f;
                        if (kForm == kHalf) w[i] = __half2float(__ushort_as_half(__ldcs(ph + o + i * kPullSlice)));
                        if (kForm == kFull) w[i] = __ldcs(pf + o + i * kPullSlice);
                    }
#pragma unroll
                    for (int i = 0; i < kDepth; ++i) sum = __fadd_rn(sum, value(pre[i], w[i]));
                }
                if (k0 < len)
                {
                    const size_t o = static_cast<size_t>(k0) * kPullSlice;
                    uint32_t pre[kDepth];
                    float w[kDepth];
#pragma unroll
                    for (int i = 0; i < kDepth; ++i)
                    {
                        pre[i] = 0u;
                        w[i] = 0.0f;
                        if (k0 + i < len)
                        {
                            pre[i] = __ldcs(pk + o + i * kPullSlice);
                            if (kForm == kHalf) w[i] = __half2float(__ushort_as_half(__ldcs(ph + o + i * kPullSlice)));
                            if (kForm == kFull) w[i] = __ldcs(pf + o + i * kPullSlice);
                        }
                    }
#pragma unroll
                    for (int i = 0; i < kDepth; ++i)
                        if (k0 + i < len) sum = __fadd_rn(sum, value(pre[i], w[i]));
                }
                return sum;
            };
            const float sum = all ? walk(std::true_type{}) : walk(std::false_type{});
            // This lane's target: one owner per (delay, target), so a plain add.
            const uint32_t t = g.perm[q * kPullSlice + lane];
            if (sum != 0.0f) acc[(qi / kPullSlicesPerWindow) * kPullWindow + t] += sum;
        }
    }
    __syncthreads();
    if (any)
    {
        const uint32_t slot = static_cast<uint32_t>(tn % p.ring.slots);
        float *ring = p.ring.v32 + static_cast<size_t>(slot) * p.ring.pitch;
        for (uint32_t i = threadIdx.x; i < n_acc; i += blockDim.x)
        {
            const uint32_t j = w0 * kPullWindow + i;
            if (j < g.n_post && acc[i] != 0.0f) ring[j] = __fadd_rn(ring[j], acc[i]);
        }
    }
    clear_bitmap_slot(g, tn, block, G);
}

}  // namespace
}  // namespace knp_gb300
