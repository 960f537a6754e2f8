// Fused step kernel for small networks: one thread-block cluster runs whole steps of every
// population, projection and STDP rule of a backend, `n_steps` steps per launch, with the phases of
// a step separated by cluster barriers instead of kernel boundaries.
//
// A step of the per-phase path is five to six dependent launches (population, scatter per
// projection, STDP append and modify, end of step); below ~10^4 neurons each phase is a few
// microseconds of latency and the launches, not the work, set the step time. Here a step is two
// phases inside one cluster of up to 8 CTAs on 8 SMs (enough warps to keep the scatter's dependent
// loads of many rows in flight): the populations of step t beside the STDP rules of step t - 1,
// then the projections of step t. That keeps the order of the single-threaded backend's step
// (backend.cpp:89-141 of the reference: populations, projections, then the STDP rules, whose
// weights the next step's projections read) for every datum, and no wait spins: every ordering is a
// hardware cluster barrier (barrier.cluster arrive.release / wait.acquire, which also orders the
// CTAs' global-memory accesses) or a block barrier.
//
// The per-neuron, per-synapse and per-column code is the per-phase kernels' own (population_dev.cuh,
// projection_dev.cuh, stdp_dev.cuh), and the cluster walks the same device layout, so results are
// those of the per-phase path. Only projections without a gather layout take part (the host selects
// this kernel only then).
#include <cstdint>

#include "kernels.h"
#include "population_dev.cuh"
#include "projection_dev.cuh"
#include "stdp_dev.cuh"
#include "tcgen05.cuh"

namespace knp_gb300
{
namespace
{

constexpr int kSmallThreads = 512;
constexpr uint32_t kSmallWarps = kSmallThreads / 32;

template <bool kFixed, bool kUniformExc>
__device__ __forceinline__ unsigned long long scatter_one(const ProjectionDev &p, unsigned long long t, uint32_t warp,
                                                          uint32_t n_warps, int lane)
{
    const uint32_t *idx[kMaxSources];
    uint32_t cnt[kMaxSources];
    const uint32_t total = resolve_sources(p, t, idx, cnt);
    const uint32_t slot_base = static_cast<uint32_t>(t % p.ring.slots);
    return scatter_rows<kFixed, kUniformExc>(p, slot_base, idx, cnt, total, warp, n_warps, lane);
}

// Reads (into the CTA's spike total) and zeroes the per-step counters of one descriptor set.
__device__ __forceinline__ void retire_counters(const StepEnd &e, uint32_t gthread, uint32_t n_threads,
                                                unsigned long long *spikes)
{
    for (uint32_t k = gthread; k < e.n_zero_u32; k += n_threads)
    {
        const uint32_t v = e.zero_u32[k];
        if (k < e.n_spike_counts && v) atomicAdd(spikes, static_cast<unsigned long long>(v));
        if (v) e.zero_u32[k] = 0;
    }
}

// The STDP rules of step t (descriptor set of step t): a one-source rule appends and updates in one
// pass; otherwise the sources' appends in order, then the weight update of the touched columns that
// are full. `thread` / `warp` are this thread's ids rotated by half the cluster, so that the rules'
// work lands on other SMs than the first neurons' population work it runs beside.
__device__ __forceinline__ void stdp_rules(const SmallStdp *rules, uint32_t n_rules, unsigned long long t,
                                           uint32_t thread, uint32_t n_threads, int lane)
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
            tc::cluster_sync();
        }
        stdp_modify_range(r.d, warp, n_warps, lane);
    }
}

// Launched as one cluster of C CTAs (C = cluster size, 1 to 8); every thread of the cluster passes
// the same sequence of cluster barriers (all loop bounds below are the same in every thread).
// Step t is two phases, each closed by a cluster barrier:
//   A: the populations of step t, beside the STDP rules of step t - 1 (they read step t - 1's spike
//      lists and counters, the other descriptor set, and change weights no one reads in phase A);
//   B: the projections of step t (reading the weights after step t - 1's STDP update, as the
//      reference's order requires), beside the retirement of step t - 1's counters.
// A launch ends with the STDP rules of its last step, so both descriptor sets' counters are zero and
// every update is done between launches.
__global__ void __launch_bounds__(kSmallThreads, 1) small_net_kernel(SmallNet net, Control *ctl, uint32_t n_steps)
{
    __shared__ unsigned long long s_spikes;
    const int lane = threadIdx.x & 31;
    const uint32_t C = gridDim.x;
    const uint32_t rank = blockIdx.x;
    const uint32_t gthread = rank * kSmallThreads + threadIdx.x, n_threads = C * kSmallThreads;
    const uint32_t gwarp = gthread >> 5, n_warps = C * kSmallWarps;
    const uint32_t sthread = (gthread + n_threads / 2) % n_threads;
    if (threadIdx.x == 0) s_spikes = 0;
    unsigned long long t = ctl->step;
    unsigned long long events = 0;
    // Every CTA has read the step number before CTA 0 may advance it (at the end).
    tc::cluster_sync();
    for (uint32_t s = 0; s < n_steps; ++s, ++t)
    {
        // Descriptor sets of this step and of the previous one (selects, not a dynamic index into
        // the parameter block).
        const bool odd = t & 1u;
        const SmallPop *pops = odd ? net.pops[1] : net.pops[0];
        const ProjectionDev *projs = odd ? net.projs[1] : net.projs[0];
        // ---- phase A
        // Populations (each pass of the cluster covers 4 * n_threads neurons; each CTA compacts
        // its own spikes into the list).
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
                    emit_spikes<kSmallThreads>(mask, i0, p.spikes, p.spike_count,
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
                    emit_spikes<kSmallThreads>(mask, i0, p.spikes, p.spike_count,
                                               record_slot(p.rec_bits, p.rec_words, p.rec_slots, t), p.rec_words);
                }
            }
        }
        // The STDP rules of step t - 1 (done by the previous launch for its first step).
        if (s > 0 && net.n_stdp) stdp_rules(odd ? net.stdp[0] : net.stdp[1], net.n_stdp, t - 1, sthread, n_threads, lane);
        tc::cluster_sync();
        // ---- phase B
        // Step t - 1's counters are no longer read by anyone.
        retire_counters(odd ? net.end[0] : net.end[1], gthread, n_threads, &s_spikes);
        // Projections: every warp of the cluster walks its share of each projection's spike rows.
        for (uint32_t k = 0; k < net.n_projs; ++k)
        {
            const ProjectionDev &p = projs[k];
            if (p.n_src == 0) continue;
            const bool uexc = !p.type && p.uniform_type == 0;
            unsigned long long ev;
            if (p.ring.fixed)
                ev = uexc ? scatter_one<true, true>(p, t, gwarp, n_warps, lane)
                          : scatter_one<true, false>(p, t, gwarp, n_warps, lane);
            else
                ev = uexc ? scatter_one<false, true>(p, t, gwarp, n_warps, lane)
                          : scatter_one<false, false>(p, t, gwarp, n_warps, lane);
            events += ev;
        }
        tc::cluster_sync();
    }
    // The last step's STDP rules, then its counters: both sets are zero between launches.
    const bool last_odd = (t - 1) & 1u;
    if (net.n_stdp)
    {
        stdp_rules(last_odd ? net.stdp[1] : net.stdp[0], net.n_stdp, t - 1, sthread, n_threads, lane);
        tc::cluster_sync();
    }
    retire_counters(last_odd ? net.end[1] : net.end[0], gthread, n_threads, &s_spikes);
    if (lane == 0 && events) atomicAdd(&ctl->events_total, events);
    __syncthreads();
    if (threadIdx.x == 0 && s_spikes) atomicAdd(&ctl->spikes_total, s_spikes);
    if (rank == 0 && threadIdx.x == 0) ctl->step = t;
}

}  // namespace

int small_net_cluster()
{
    static int c = [] {
        cudaLaunchConfig_t cfg{};
        cfg.blockDim = dim3(kSmallThreads);
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        for (int size = 8; size > 1; size /= 2)
        {
            cfg.gridDim = dim3(size);
            attr[0].val.clusterDim.x = size;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            int n = 0;
            if (cudaOccupancyMaxActiveClusters(&n, small_net_kernel, &cfg) == cudaSuccess && n > 0) return size;
            cudaGetLastError();
        }
        return 1;
    }();
    return c;
}

cudaError_t launch_small_net(const SmallNet &net, Control *ctl, uint32_t n_steps, int cluster, cudaStream_t s)
{
    if (!n_steps) return cudaSuccess;
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(kSmallThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, small_net_kernel, net, ctl, n_steps);
}

}  // namespace knp_gb300
