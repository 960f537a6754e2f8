// Projection kernel: for each presynaptic spike of this step, walk its CSR row and scatter-add the
// impacts into the target population's input ring at slot (step + delay) mod slots.
//
// Semantics (delta_impl.h:54-114 of the reference CPU library) are in projection_dev.cuh.
//
// Work distribution: persistent grid; each warp takes whole spike rows (row-major over the
// concatenated spike lists of all sources) and its 32 lanes stream the row's col / weight / delay
// arrays with coalesced loads, 4 synapses per lane in flight.
#include <cstdint>

#include "kernels.h"
#include "projection_dev.cuh"

namespace knp_gb300
{
namespace
{

template <bool kFixed, bool kUniformExc>
__global__ void __launch_bounds__(256) projection_kernel(ProjectionDev p, Control *ctl)
{
    pdl_begin();
    const unsigned long long t = ctl->step;
    const uint32_t slot_base = static_cast<uint32_t>(t % p.ring.slots);
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;

    const uint32_t *idx[kMaxSources];
    uint32_t cnt[kMaxSources];
    const uint32_t total = resolve_sources(p, t, idx, cnt);
    __shared__ unsigned long long block_events;
    if (threadIdx.x == 0) block_events = 0;
    __syncthreads();
    unsigned long long events = 0;
    if (p.pull.bitmap)
    {
        // Direction choice for this step's spikes (the same in every block: it depends only on the
        // spike count). A pulled step only records its spikes; gather_kernel delivers them.
        const bool pull = total >= p.pull.threshold;
        // Every presynaptic neuron fired (one population source, whose spike indexes are distinct
        // and below its size): the gather then needs no bitmap and tests no bit for this step.
        const bool full = pull && p.n_src == 1 && !p.src[0].channel && p.src[0].n && total >= p.src[0].n;
        const uint32_t sl = static_cast<uint32_t>(t % p.pull.hist_slots);
        if (blockIdx.x == 0 && threadIdx.x == 0) p.pull.pulled[sl] = pull ? (full ? 2u : 1u) : 0u;
        if (full)
        {
            // Every row fired: the step's events are all the synapses, and the bitmap stays unused.
            if (blockIdx.x == 0 && threadIdx.x == 0)
                atomicAdd(&ctl->events_total, static_cast<unsigned long long>(p.row_ptr[p.n_rows] - p.row_ptr[0]));
            return;
        }
        if (pull)
        {
            uint32_t *bm = p.pull.bitmap + static_cast<size_t>(sl) * p.pull.words;
            const uint32_t stride = gridDim.x * blockDim.x;
            for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < total; j += stride)
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
                events += static_cast<unsigned long long>(p.row_ptr[pre + 1] - p.row_ptr[pre]);
            }
            // Per-thread counts: reduce over the warp, then the block.
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) events += __shfl_down_sync(0xffffffffu, events, o);
            if (lane == 0 && events) atomicAdd(&block_events, events);
            __syncthreads();
            if (threadIdx.x == 0 && block_events) atomicAdd(&ctl->events_total, block_events);
            return;
        }
    }
    events = scatter_rows<kFixed, kUniformExc>(p, slot_base, idx, cnt, total, warp, n_warps, lane);
    if (p.last_spike)
    {
        // Resource-STDP synapses: init_synapse (synaptic_resource_stdp.h:36-41, called per synapse of
        // a spiking row in delta_impl.h:75) records the step of the presynaptic spike.
        for (uint32_t j = warp; j < total; j += n_warps)
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
            for (int64_t e = p.row_ptr[pre] + lane; e < p.row_ptr[pre + 1]; e += 32) p.last_spike[e] = t;
        }
    }
    if (lane == 0 && events) atomicAdd(&block_events, events);
    __syncthreads();
    if (threadIdx.x == 0 && block_events) atomicAdd(&ctl->events_total, block_events);
}

}  // namespace

void launch_projection(const ProjectionDev &p, Control *ctl, int grid, cudaStream_t s)
{
    const bool uexc = !p.type && p.uniform_type == 0;
    if (p.ring.fixed)
    {
        if (uexc)
            launch_pdl(projection_kernel<true, true>, dim3(grid), dim3(256), 0, s, p, ctl);
        else
            launch_pdl(projection_kernel<true, false>, dim3(grid), dim3(256), 0, s, p, ctl);
    }
    else
    {
        if (uexc)
            launch_pdl(projection_kernel<false, true>, dim3(grid), dim3(256), 0, s, p, ctl);
        else
            launch_pdl(projection_kernel<false, false>, dim3(grid), dim3(256), 0, s, p, ctl);
    }
}

}  // namespace knp_gb300
