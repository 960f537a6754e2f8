// Projection kernel: for each presynaptic spike of this step, walk its CSR row and scatter-add the
// impacts into the target population's input ring at slot (step + delay) mod slots.
//
// Semantics follow delta::calculate_projection_impl (knp/backends/cpu/cpu-library/include/
// knp/backends/cpu-library/impl/projections/delta/delta_impl.h:54-114): an impact created at step t
// through delay d is sent at step t + d - 1 and applied by the population at step t + d; delay 0
// lands on step t - 1, which has already been sent, so it is counted as an event and never applied.
// Sums of impacts are order-independent (FP32 for dyadic weights, or two-word fixed point), so the
// warp/atomic order of the scatter does not change results.
//
// Work distribution: persistent grid; each warp takes whole spike rows (row-major over the
// concatenated spike lists of all sources) and its 32 lanes stream the row's col / weight / delay
// arrays with coalesced loads, 4 synapses per lane in flight.
#include <cstdint>

#include "kernels.h"

namespace knp_gb300
{
namespace
{


__device__ __forceinline__ void resolve_source(
    const SpikeSource &s, unsigned long long t, const uint32_t *&idx, uint32_t &cnt)
{
    if (s.channel)
    {
        const ChannelDev &c = *s.channel;
        if (t >= c.first_step && t - c.first_step < c.n_steps)
        {
            const unsigned long long k = t - c.first_step;
            const long long a = c.offsets[k];
            idx = c.idx + a;
            cnt = static_cast<uint32_t>(c.offsets[k + 1] - a);
        }
        else
        {
            idx = nullptr;
            cnt = 0;
        }
    }
    else
    {
        idx = s.idx;
        cnt = *s.count;
    }
}

template <bool kFixed, bool kUniformExc>
__device__ __forceinline__ void deliver(
    const ProjectionDev &p, uint32_t slot_base, int64_t e, int32_t c, float w, uint32_t d, int ty)
{
    if (d == 0u) return;  // lost, as in the reference
    uint32_t slot = slot_base + d;
    while (slot >= p.ring.slots) slot -= p.ring.slots;
    const size_t o = static_cast<size_t>(slot) * p.ring.pitch + static_cast<uint32_t>(c);
    if (kUniformExc || ty == 0 || ty == 1)
    {
        if (!kUniformExc && ty == 1) w = -w;
        if (kFixed)
            fx_atomic_add(p.ring.v64, p.ring.v64lo, o, w);
        else
            atomicAdd(p.ring.v32 + o, w);
        if ((kUniformExc || ty == 0) && p.forcing && p.ring.forced)
            atomicOr(p.ring.forced + static_cast<size_t>(slot) * p.ring.words + (static_cast<uint32_t>(c) >> 5),
                     1u << (c & 31));
    }
    else if (ty == 2)
    {
        if (p.ring.g) atomicAdd(p.ring.g + o, w);
    }
    else if (ty == 3)
    {
        if (p.ring.dopa) atomicAdd(p.ring.dopa + o, w);
    }
}

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
    uint32_t total = 0;
#pragma unroll
    for (int k = 0; k < kMaxSources; ++k)
    {
        if (k < p.n_src)
        {
            resolve_source(p.src[k], t, idx[k], cnt[k]);
            total += cnt[k];
        }
        else
        {
            idx[k] = nullptr;
            cnt[k] = 0;
        }
    }
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
    // Few spikes for many warps: each row is split over F warps (warp f of a row takes its 128-synapse
    // rounds f, f + F, ...), so one long row does not serialise the step.
    const uint32_t F = total ? max(1u, min(8u, n_warps / total)) : 1u;
    for (uint32_t it = warp; it < total * F; it += n_warps)
    {
        const uint32_t j = it / F, f = it - j * F;
        uint32_t jj = j;
        int k = 0;
        while (jj >= cnt[k])
        {
            jj -= cnt[k];
            ++k;
        }
        const uint32_t pre = idx[k][jj];
        if (pre >= p.n_rows) continue;  // no synapses from this neuron
        const int64_t a = p.row_ptr[pre];
        const int64_t b = p.row_ptr[pre + 1];
        if (f == 0) events += static_cast<unsigned long long>(b - a);
        int64_t e = a + 128 * static_cast<int64_t>(f) + lane;
        for (; e + 96 < b; e += 128 * static_cast<int64_t>(F))
        {
            int32_t c[4];
            float w[4];
            uint32_t d[4];
            int ty[4] = {0, 0, 0, 0};
#pragma unroll
            for (int u = 0; u < 4; ++u)
            {
                c[u] = __ldg(p.col + e + 32 * u);
                w[u] = p.w[e + 32 * u];
                d[u] = __ldg(p.delay + e + 32 * u);
                if (!kUniformExc) ty[u] = p.type ? __ldg(p.type + e + 32 * u) : p.uniform_type;
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) deliver<kFixed, kUniformExc>(p, slot_base, e + 32 * u, c[u], w[u], d[u], ty[u]);
        }
        // The last, partial round of this warp (the next one would start past b).
        for (; e < b; e += 32)
        {
            const int ty = kUniformExc ? 0 : (p.type ? __ldg(p.type + e) : p.uniform_type);
            deliver<kFixed, kUniformExc>(p, slot_base, e, __ldg(p.col + e), p.w[e], __ldg(p.delay + e), ty);
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
