// Device-side scatter code of the projection kernels, shared by the per-phase kernel
// (projection.cu) and the fused small-network step kernel (small_net.cu).
//
// Semantics follow delta::calculate_projection_impl (knp/backends/cpu/cpu-library/include/
// knp/backends/cpu-library/impl/projections/delta/delta_impl.h:54-114): an impact created at step t
// through delay d is sent at step t + d - 1 and applied by the population at step t + d; delay 0
// lands on step t - 1, which has already been sent, so it is counted as an event and never applied.
// Sums of impacts are order-independent (FP32 for dyadic weights, or two-word fixed point), so the
// warp/atomic order of the scatter does not change results.
#pragma once

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
        if (kFixed && p.ring.nf && !isfinite(w))
        {
            const uint32_t bit = isnan(w) ? 1u : (w > 0.0f ? 2u : 4u);
            atomicOr(p.ring.nf + (o >> 2), bit << (8 * (o & 3)));
            return;
        }
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
    else if (ty == 4)
    {
        if (p.ring.blk)
        {
            atomicMax(p.ring.blk + o, blocking_key(p.order, d, e));
        }
        else if (p.ring.bev_key)
        {
            // AltAI-LIF target: keep the impact as an event of its slot (the overflow is detected by
            // the blocking kernel from the count).
            const uint32_t k = atomicAdd(p.ring.bev_count + slot, 1u);
            if (k < p.ring.bev_cap)
            {
                const size_t q = static_cast<size_t>(slot) * p.ring.bev_cap + k;
                p.ring.bev_key[q] = blocking_key(p.order, d, e);
                p.ring.bev_val[q] = w;
                p.ring.bev_tgt[q] = static_cast<uint32_t>(c);
            }
        }
    }
}

// Sources of projection p at step t: idx[k] / cnt[k] for source k (unused entries empty); returns
// the total spike count.
__device__ __forceinline__ uint32_t resolve_sources(
    const ProjectionDev &p, unsigned long long t, const uint32_t *(&idx)[kMaxSources], uint32_t (&cnt)[kMaxSources])
{
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
    return total;
}

// Scatters the rows of this step's `total` spikes over warps: this is warp `warp` of `n_warps`.
// Returns the events (synapses of the rows) this warp started, the same value in every lane.
template <bool kFixed, bool kUniformExc>
__device__ __forceinline__ unsigned long long scatter_rows(
    const ProjectionDev &p, uint32_t slot_base, const uint32_t *const (&idx)[kMaxSources],
    const uint32_t (&cnt)[kMaxSources], uint32_t total, uint32_t warp, uint32_t n_warps, int lane)
{
    unsigned long long events = 0;
    // Each row is split over F warps (warp f of a row takes its 128-synapse rounds f, f + F, ...), so
    // that one long row does not serialise the step and the rows' parts spread evenly over the warps:
    // about four parts per warp (with whole rows, 1.25 rows per warp would leave a quarter of the warps
    // a second full row while the rest idle).
    const uint32_t F = total ? max(1u, min(8u, (4u * n_warps) / total)) : 1u;
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
    return events;
}

}  // namespace
}  // namespace knp_gb300
