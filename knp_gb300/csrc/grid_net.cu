// Persistent step kernel for large networks: one cooperative launch of one 1024-thread CTA per SM
// runs whole steps of every population, projection (scatter or gather direction) and STDP rule of a
// backend, `n_steps` steps per launch, with the phases of a step separated by grid barriers instead
// of kernel boundaries.
//
// A step of the per-phase path is five to six dependent launches; at the large sparse
// configuration's low firing rates (a few thousand spikes of 10^6 neurons per step) a step is tens
// of microseconds of work, and the launches and the gaps between them are a large share of it. Here
// a step is two or three phases of one resident grid:
//   A: the populations of step t beside the STDP rules of step t - 1;
//   B: the projections of step t (scatter of the spike rows into the input rings, or, for a step
//      whose spike count reaches a projection's pull threshold, its spike bitmap), beside the
//      retirement of step t - 1's per-step counters and the clearing of the bitmap slot step t + 1
//      will fill;
//   C: only when a step of a gather's delay window was pulled (every CTA takes the same decision in
//      phase B), the gathers that complete step t + 1's input from the bitmaps of earlier steps.
// A grid barrier follows phase A and phase B, and phase C when it runs (its ring writes are the next
// step's input). This keeps the order of the
// single-threaded backend's step (backend.cpp:89-141 of the reference) for every datum, as the
// per-phase kernels do. The per-neuron, per-synapse and per-column code is theirs
// (population_dev.cuh, projection_dev.cuh, pull_dev.cuh, stdp_dev.cuh) over the same device layout
// and the same two parity-indexed descriptor sets as the fused cluster kernel (small_net.cu), so
// results equal those of the per-phase path.
//
// Grid barrier: an arrival counter in global memory (zeroed before each launch), thread 0 of every
// CTA adds one and polls it (acquire) until all CTAs of this barrier have arrived. The cooperative
// launch guarantees that every CTA is resident. Every wait is bounded by the global timer: a CTA
// that waits longer than kBarrierNs sets kErrGridBarrier in the control block and leaves the step
// loop; a CTA that finds the bit set while polling leaves too, so a stuck grid ends within about
// one limit and the host reads the error.
#include <cstdint>

#include "kernels.h"
#include "population_dev.cuh"
#include "projection_dev.cuh"
#include "pull_dev.cuh"
#include "stdp_dev.cuh"

namespace knp_gb300
{
namespace
{

constexpr int kGridThreads = kGatherThreads;  // the gather phase is tuned for 32 warps per SM
constexpr uint32_t kGridWarps = kGridThreads / 32;
// Longest wait at a barrier: above the longest phase a legitimate step can have (a saturated
// scatter-only step of 10^9 events takes a few seconds).
constexpr unsigned long long kBarrierNs = 30000000000ull;  // 30 s

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long v;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(v));
    return v;
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Every thread of every CTA calls it with the same `target` sequence (G, 2G, 3G, ...). Returns
// false in every thread of the block when the barrier gave up (timeout, or another CTA reported one).
__device__ __forceinline__ bool grid_sync(unsigned long long *bar, Control *ctl, unsigned long long target)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        int ok = 1;
        __threadfence();
        atomicAdd(bar, 1ull);
        const unsigned long long t0 = global_ns();
        for (uint32_t i = 0;; ++i)
        {
            if (ld_acquire_u64(bar) >= target) break;
            if ((i & 63u) == 63u)
            {
                if (*reinterpret_cast<volatile unsigned int *>(&ctl->error) & kErrGridBarrier)
                {
                    ok = 0;
                    break;
                }
                if (global_ns() - t0 > kBarrierNs)
                {
                    atomicOr(&ctl->error, kErrGridBarrier);
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Whether a step of the gather's delay window for step t + 1 (t + 1 - d, d = 1 .. max_delay) was
// pulled: step t from its spike count (the rule of project()), earlier steps from their flags.
// Every thread of the CTA may call it; threads share the flag reads.
__device__ __forceinline__ bool pull_window_active(const ProjectionDev &p, unsigned long long t)
{
    const PullDev &g = p.pull;
    if (threadIdx.x == 0 && p.n_src != 0)
    {
        const uint32_t *idx[kMaxSources];
        uint32_t cnt[kMaxSources];
        if (resolve_sources(p, t, idx, cnt) >= g.threshold) return true;
    }
    bool need = false;
    for (uint32_t d = 2 + threadIdx.x; d <= g.max_delay && d <= t + 1; d += blockDim.x)
        need = need || g.pulled[static_cast<uint32_t>((t + 1 - d) % g.hist_slots)] != 0u;
    return need;
}

// One projection's work of step t over the whole grid: the pull decision and bitmap (gather form),
// or the scatter of its spike rows. Returns the synaptic events this warp accounted for (the same
// value in every lane).
template <bool kFixed, bool kUniformExc>
__device__ __forceinline__ unsigned long long project(const ProjectionDev &p, unsigned long long t, uint32_t gthread,
                                                      uint32_t n_threads, uint32_t gwarp, uint32_t n_warps, int lane)
{
    const uint32_t *idx[kMaxSources];
    uint32_t cnt[kMaxSources];
    const uint32_t total = resolve_sources(p, t, idx, cnt);
    if (p.pull.bitmap)
    {
        // As projection_kernel (projection.cu): a step at or above the threshold is only recorded.
        const bool pull = total >= p.pull.threshold;
        const bool full = pull && p.n_src == 1 && !p.src[0].channel && p.src[0].n && total >= p.src[0].n;
        const uint32_t sl = static_cast<uint32_t>(t % p.pull.hist_slots);
        if (gthread == 0) p.pull.pulled[sl] = pull ? (full ? 2u : 1u) : 0u;
        if (pull)
        {
            unsigned long long ev = 0;
            if (full)
            {
                if (gthread == 0) ev = static_cast<unsigned long long>(p.row_ptr[p.n_rows] - p.row_ptr[0]);
            }
            else
            {
                uint32_t *bm = p.pull.bitmap + static_cast<size_t>(sl) * p.pull.words;
                for (uint32_t j = gthread; j < total; j += n_threads)
                {
                    uint32_t jj = j;
                    int k = 0;
                    while (jj >= cnt[k])
                    {
                        jj -= cnt[k];
                        ++k;
                    }
                    const uint32_t pre = idx[k][jj];
                    if (pre >= p.n_rows) continue;
                    atomicOr(bm + (pre >> 5), 1u << (pre & 31));
                    ev += static_cast<unsigned long long>(p.row_ptr[pre + 1] - p.row_ptr[pre]);
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) ev += __shfl_xor_sync(0xffffffffu, ev, o);
            return ev;
        }
    }
    const uint32_t slot_base = static_cast<uint32_t>(t % p.ring.slots);
    return scatter_rows<kFixed, kUniformExc>(p, slot_base, idx, cnt, total, gwarp, n_warps, lane);
}

__device__ __forceinline__ void retire(const StepEnd &e, uint32_t gthread, uint32_t n_threads, unsigned long long *spikes)
{
    for (uint32_t k = gthread; k < e.n_zero_u32; k += n_threads)
    {
        const uint32_t v = e.zero_u32[k];
        if (k < e.n_spike_counts && v) atomicAdd(spikes, static_cast<unsigned long long>(v));
        if (v) e.zero_u32[k] = 0;
    }
}

// The STDP rules of step t (descriptor set of step t), as small_net.cu runs them, with grid
// barriers between the appends of a multi-source rule. Returns false if a barrier gave up.
__device__ __forceinline__ bool grid_stdp_rules(const SmallStdp *rules, uint32_t n_rules, unsigned long long t,
                                                uint32_t thread, uint32_t n_threads, int lane, unsigned long long *bar,
                                                Control *ctl, unsigned long long &target)
{
    const uint32_t warp = thread >> 5, n_warps = n_threads >> 5;
    for (uint32_t k = 0; k < n_rules; ++k)
    {
        const SmallStdp &r = rules[k];
        if (r.n_src == 1 && !r.src[0].channel)
        {
            stdp_append_update_range(r.d, r.src[0], r.both[0], t, thread, n_threads);
            continue;
        }
        for (uint32_t j = 0; j < r.n_src; ++j)
        {
            stdp_append_range(r.d, r.src[j], r.both[j], t, thread, n_threads);
            target += gridDim.x;
            if (!grid_sync(bar, ctl, target)) return false;
        }
        stdp_modify_range(r.d, warp, n_warps, lane);
    }
    return true;
}

__device__ __forceinline__ void grid_gather(const ProjectionDev &p, unsigned long long tn, uint4 *smem)
{
    if (p.pull.wtab)
        gather_block<kDict>(p, tn, blockIdx.x, gridDim.x, smem);
    else if (p.pull.w16)
        gather_block<kHalf>(p, tn, blockIdx.x, gridDim.x, smem);
    else
        gather_block<kFull>(p, tn, blockIdx.x, gridDim.x, smem);
    __syncthreads();  // the next projection's gather reuses the shared memory
}

__global__ void __launch_bounds__(kGridThreads, 1) grid_net_kernel(GridNet g, Control *ctl, uint32_t n_steps)
{
    extern __shared__ uint4 grid_smem[];
    __shared__ unsigned long long s_spikes;
    const SmallNet &net = g.net;
    const int lane = threadIdx.x & 31;
    const uint32_t G = gridDim.x;
    const uint32_t gthread = blockIdx.x * kGridThreads + threadIdx.x, n_threads = G * kGridThreads;
    const uint32_t gwarp = gthread >> 5, n_warps = G * kGridWarps;
    const uint32_t sthread = (gthread + n_threads / 2) % n_threads;
    if (threadIdx.x == 0) s_spikes = 0;
    unsigned long long t = ctl->step;
    unsigned long long events = 0;
    unsigned long long target = 0;
    bool ok = true;
    // Every CTA has read the step number before CTA 0 may advance it (at the end).
    target += G;
    ok = grid_sync(g.barrier, ctl, target);
    // Phase timer state in shared memory (read by one thread), not in registers held across the loop.
    __shared__ unsigned long long ts, acc[3];
    const bool timer = g.phase_ns && blockIdx.x == 0 && threadIdx.x == 0;
    if (timer) ts = acc[0] = acc[1] = acc[2] = 0;
    uint32_t s = 0;
    for (; ok && s < n_steps; ++s, ++t)
    {
        if (timer)
        {
            const unsigned long long now = global_ns();
            if (s > 0) acc[2] += now - ts;  // phase C of the previous step
            ts = now;
        }
        const bool odd = t & 1u;
        const SmallPop *pops = odd ? net.pops[1] : net.pops[0];
        const ProjectionDev *projs = odd ? net.projs[1] : net.projs[0];
        // ---- phase A: populations of step t (a pass covers 4 * n_threads neurons; each CTA compacts
        // its own spikes into the list), STDP rules of step t - 1.
        for (uint32_t k = 0; k < net.n_pops; ++k)
        {
            const SmallPop &q = pops[k];
            if (q.kind == kSmallLif)
            {
                const LifDev &p = q.lif;
                for (uint32_t base = 0; base < p.n; base += 4 * n_threads)
                {
                    const uint32_t i0 = base + 4 * gthread;
                    const uint32_t mask = lif_quad(p, t, i0);
                    emit_spikes<kGridThreads>(mask, i0, p.spikes, p.spike_count,
                                              record_slot(p.rec_bits, p.rec_words, p.rec_slots, t), p.rec_words);
                }
            }
            else
            {
                const BlifatDev &p = q.blifat;
                for (uint32_t base = 0; base < p.n; base += 4 * n_threads)
                {
                    const uint32_t i0 = base + 4 * gthread;
                    const uint32_t mask = blifat_quad_any(p, t, i0);
                    emit_spikes<kGridThreads>(mask, i0, p.spikes, p.spike_count,
                                              record_slot(p.rec_bits, p.rec_words, p.rec_slots, t), p.rec_words);
                }
            }
        }
        if (s > 0 && net.n_stdp &&
            !grid_stdp_rules(odd ? net.stdp[0] : net.stdp[1], net.n_stdp, t - 1, sthread, n_threads, lane, g.barrier,
                             ctl, target))
        {
            ok = false;
            break;
        }
        target += G;
        if (!grid_sync(g.barrier, ctl, target))
        {
            ok = false;
            break;
        }
        if (timer)
        {
            const unsigned long long now = global_ns();
            acc[0] += now - ts;
            ts = now;
        }
        // ---- phase B: step t - 1's counters are no longer read; projections of step t.
        retire(odd ? net.end[0] : net.end[1], gthread, n_threads, &s_spikes);
        for (uint32_t k = 0; k < net.n_projs; ++k)
        {
            const ProjectionDev &p = projs[k];
            if (p.n_src == 0) continue;
            const bool uexc = !p.type && p.uniform_type == 0;
            if (p.ring.fixed)
                events += uexc ? project<true, true>(p, t, gthread, n_threads, gwarp, n_warps, lane)
                               : project<true, false>(p, t, gthread, n_threads, gwarp, n_warps, lane);
            else
                events += uexc ? project<false, true>(p, t, gthread, n_threads, gwarp, n_warps, lane)
                               : project<false, false>(p, t, gthread, n_threads, gwarp, n_warps, lane);
        }
        // Gathers complete step t + 1's input when a step of their delay window was pulled: every CTA
        // takes the same decision from this step's spike counts (the pulled flag of step t is being
        // written in this phase) and the flags of earlier steps. The bitmap slot step t + 1 fills
        // holds step t - max_delay, which the last gathers (of step t - 1) have read.
        bool need = false;
        for (uint32_t k = 0; k < g.n_pull; ++k)
        {
            const ProjectionDev &p = projs[g.pull[k]];
            clear_bitmap_slot(p.pull, t + 1, blockIdx.x, G);
            need = need || pull_window_active(p, t);
        }
        need = __syncthreads_or(need) != 0;
        // The scatter's writes (slots t + 1 .. t + D) are complete before step t + 1's populations
        // read slot t + 1, and the step's bitmaps before the gathers read them.
        target += G;
        if (!grid_sync(g.barrier, ctl, target))
        {
            ok = false;
            break;
        }
        if (timer)
        {
            const unsigned long long now = global_ns();
            acc[1] += now - ts;
            ts = now;
        }
        if (!need) continue;
        // ---- phase C: gathers completing step t + 1's input.
        for (uint32_t k = 0; k < g.n_pull; ++k) grid_gather(projs[g.pull[k]], t + 1, grid_smem);
        target += G;
        if (!grid_sync(g.barrier, ctl, target))
        {
            ok = false;
            break;
        }
    }
    if (!ok)
    {
        // A barrier gave up: the host reads kErrGridBarrier; nothing further is stepped.
        return;
    }
    if (timer)
    {
        if (s > 0) acc[2] += global_ns() - ts;
        for (int k = 0; k < 3; ++k) g.phase_ns[k] += acc[k];
    }
    // The last step's STDP rules, then its counters: both sets are zero between launches.
    const bool last_odd = (t - 1) & 1u;
    if (net.n_stdp)
    {
        if (!grid_stdp_rules(last_odd ? net.stdp[1] : net.stdp[0], net.n_stdp, t - 1, sthread, n_threads, lane,
                             g.barrier, ctl, target))
            return;
        target += G;
        if (!grid_sync(g.barrier, ctl, target)) return;
    }
    retire(last_odd ? net.end[1] : net.end[0], gthread, n_threads, &s_spikes);
    if (lane == 0 && events) atomicAdd(&ctl->events_total, events);
    __syncthreads();
    if (threadIdx.x == 0 && s_spikes) atomicAdd(&ctl->spikes_total, s_spikes);
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->step = t;
}

}  // namespace

// CTAs of the grid kernel (one per SM when the shared memory fits), or 0 if it cannot be launched
// cooperatively with `smem` bytes of dynamic shared memory.
int grid_net_ctas(size_t smem)
{
    int device = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&device) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) return 0;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(grid_net_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) !=
            cudaSuccess)
    {
        cudaGetLastError();
        return 0;
    }
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, grid_net_kernel, kGridThreads, smem) != cudaSuccess)
    {
        cudaGetLastError();
        return 0;
    }
    return per_sm >= 1 ? sms : 0;
}

size_t grid_net_smem(const PullDev &p, int ctas) { return gather_smem_for(p, static_cast<uint32_t>(ctas)); }

cudaError_t launch_grid_net(const GridNet &g, Control *ctl, uint32_t n_steps, int ctas, size_t smem,
                            const cudaAccessPolicyWindow *window, cudaStream_t s)
{
    if (!n_steps) return cudaSuccess;
    cudaError_t err = cudaMemsetAsync(g.barrier, 0, sizeof(unsigned long long), s);
    if (err != cudaSuccess) return err;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(kGridThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    int n_attr = 0;
    attr[n_attr].id = cudaLaunchAttributeCooperative;
    attr[n_attr].val.cooperative = 1;
    ++n_attr;
    if (window && window->num_bytes)
    {
        attr[n_attr].id = cudaLaunchAttributeAccessPolicyWindow;
        attr[n_attr].val.accessPolicyWindow = *window;
        ++n_attr;
    }
    cfg.attrs = attr;
    cfg.numAttrs = n_attr;
    return cudaLaunchKernelEx(&cfg, grid_net_kernel, g, ctl, n_steps);
}

}  // namespace knp_gb300
