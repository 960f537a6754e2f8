// Population kernels: one thread per 4 consecutive neurons, block-level ballot/popc compaction of
// spike indexes (per-neuron code in population_dev.cuh), and the kernel that applies external
// SynapticImpactMessages to an input ring.
#include <cstdint>

#include "kernels.h"
#include "population_dev.cuh"

namespace knp_gb300
{
namespace
{

constexpr int kBlock = 256;

template <bool kFixed, bool kRS>
__global__ void __launch_bounds__(kBlock, 3) blifat_kernel(BlifatDev p, Control *ctl)
{
    pdl_begin();
    const unsigned long long t = ctl->step;
    const uint32_t i0 = (blockIdx.x * kBlock + threadIdx.x) * 4;
    const uint32_t mask =
        (!kFixed && !kRS && p.flags == 0u) ? blifat_quad_lean(p, t, i0) : blifat_quad<kFixed, kRS>(p, t, i0);
    emit_spikes<kBlock>(mask, i0, p.spikes, p.spike_count, record_slot(p.rec_bits, p.rec_words, p.rec_slots, t),
                        p.rec_words);
}

__global__ void __launch_bounds__(kBlock) lif_kernel(LifDev p, Control *ctl)
{
    pdl_begin();
    const unsigned long long t = ctl->step;
    const uint32_t i0 = (blockIdx.x * kBlock + threadIdx.x) * 4;
    const uint32_t mask = lif_quad(p, t, i0);
    emit_spikes<kBlock>(mask, i0, p.spikes, p.spike_count, record_slot(p.rec_bits, p.rec_words, p.rec_slots, t),
                        p.rec_words);
}

__global__ void apply_impacts_kernel(
    RingView ring, const uint32_t *post, const float *value, const uint8_t *type, int forcing, uint32_t n,
    uint32_t seq_base, Control *ctl)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const uint32_t slot = static_cast<uint32_t>(ctl->step % ring.slots);
    const uint32_t i = post[k];
    const size_t o = static_cast<size_t>(slot) * ring.pitch + i;
    const int ty = type ? type[k] : 0;
    float w = value[k];
    if (ty == 0 || ty == 1)
    {
        if (ty == 1) w = -w;
        if (ring.nf && !isfinite(w))
            atomicOr(ring.nf + (o >> 2), (isnan(w) ? 1u : (w > 0.0f ? 2u : 4u)) << (8 * (o & 3)));
        else if (ring.fixed)
            fx_atomic_add(ring.v64, ring.v64lo, o, w);
        else
            atomicAdd(ring.v32 + o, w);
        if (ty == 0 && forcing && ring.forced)
            atomicOr(ring.forced + static_cast<size_t>(slot) * ring.words + (i >> 5), 1u << (i & 31));
    }
    else if (ty == 2 && ring.g)
        atomicAdd(ring.g + o, w);
    else if (ty == 3 && ring.dopa)
        atomicAdd(ring.dopa + o, w);
    else if (ty == 4 && ring.blk)
    {
        // The host keeps only each target's last external BLOCKING impact of the step.
        ring.blk_ext[i] = static_cast<long long>(w);
        atomicMax(ring.blk + o, kBlkExternal << kBlkOrderShift);
    }
    else if (ty == 4 && ring.bev_key)
    {
        // AltAI-LIF: every external BLOCKING impact is an event, after the projections' ones, in message order.
        const uint32_t e = atomicAdd(ring.bev_count + slot, 1u);
        if (e < ring.bev_cap)
        {
            const size_t q = static_cast<size_t>(slot) * ring.bev_cap + e;
            ring.bev_key[q] = (kBlkExternal << kBlkOrderShift) | (seq_base + k);
            ring.bev_val[q] = w;
            ring.bev_tgt[q] = i;
        }
    }
}

template <bool kFixed>
__global__ void __launch_bounds__(kBlock) altai_kernel(AltaiDev p, Control *ctl)
{
    pdl_begin();
    const unsigned long long t = ctl->step;
    const uint32_t i0 = (blockIdx.x * kBlock + threadIdx.x) * 4;
    const uint32_t mask = altai_quad<kFixed>(p, t, i0);
    emit_spikes<kBlock>(mask, i0, p.spikes, p.spike_count, record_slot(p.rec_bits, p.rec_words, p.rec_slots, t),
                        p.rec_words);
}

// The step's BLOCKING impacts on an AltAI-LIF population, applied to the activity times in the
// reference's message order (altai_impl.h:74-83: an impact replaces the activity time unless it has
// the same sign and a smaller magnitude, so order matters): one CTA sorts the slot's events by
// (target, key) in shared memory (bitonic) and the first event of each target applies that target's
// events in order. More events than kAltaiEvents set kErrBlockingEvents.
constexpr int kAltaiEvents = 2048;
constexpr int kAltaiBlockThreads = 1024;

__global__ void __launch_bounds__(kAltaiBlockThreads) altai_blocking_kernel(AltaiDev p, Control *ctl)
{
    __shared__ unsigned long long s_key[kAltaiEvents];
    __shared__ uint32_t s_tgt[kAltaiEvents];
    __shared__ float s_val[kAltaiEvents];
    pdl_begin();
    const RingView &rg = p.ring;
    const uint32_t slot = static_cast<uint32_t>(ctl->step % rg.slots);
    const uint32_t count = rg.bev_count[slot];
    if (count == 0) return;
    const uint32_t cap = min(rg.bev_cap, static_cast<uint32_t>(kAltaiEvents));
    if (count > cap && threadIdx.x == 0) atomicOr(&ctl->error, kErrBlockingEvents);
    const uint32_t n = min(count, cap);
    uint32_t np2 = 1;
    while (np2 < n) np2 <<= 1;
    const size_t base = static_cast<size_t>(slot) * rg.bev_cap;
    for (uint32_t j = threadIdx.x; j < np2; j += blockDim.x)
    {
        if (j < n)
        {
            s_key[j] = rg.bev_key[base + j];
            s_tgt[j] = rg.bev_tgt[base + j];
            s_val[j] = rg.bev_val[base + j];
        }
        else
        {
            s_key[j] = ~0ull;
            s_tgt[j] = 0xFFFFFFFFu;
            s_val[j] = 0.0f;
        }
    }
    __syncthreads();
    for (uint32_t size = 2; size <= np2; size <<= 1)
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1)
        {
            for (uint32_t j = threadIdx.x; j < np2; j += blockDim.x)
            {
                const uint32_t l = j ^ stride;
                if (l <= j) continue;
                const bool up = (j & size) == 0;
                const bool greater = s_tgt[j] > s_tgt[l] || (s_tgt[j] == s_tgt[l] && s_key[j] > s_key[l]);
                if (greater == up)
                {
                    const unsigned long long k0 = s_key[j];
                    s_key[j] = s_key[l];
                    s_key[l] = k0;
                    const uint32_t t0 = s_tgt[j];
                    s_tgt[j] = s_tgt[l];
                    s_tgt[l] = t0;
                    const float v0 = s_val[j];
                    s_val[j] = s_val[l];
                    s_val[l] = v0;
                }
            }
            __syncthreads();
        }
    for (uint32_t j = threadIdx.x; j < n; j += blockDim.x)
    {
        const uint32_t tg = s_tgt[j];
        if (j > 0 && s_tgt[j - 1] == tg) continue;
        long long a = p.activity[tg];
        for (uint32_t q = j; q < n && s_tgt[q] == tg; ++q)
        {
            const float v = s_val[q];
            if ((a < 0) != (signbit(v) != 0) || static_cast<float>(a < 0 ? -a : a) <= fabsf(v))
                a = static_cast<long long>(v);
        }
        p.activity[tg] = a;
    }
    if (threadIdx.x == 0) rg.bev_count[slot] = 0;
}

}  // namespace

void launch_blifat(const BlifatDev &p, Control *ctl, cudaStream_t s)
{
    const uint32_t quads = (p.n + 3) / 4;
    const uint32_t grid = (quads + kBlock - 1) / kBlock;
    // Resource-STDP synapses always feed a fixed-point ring.
    if (p.flags & kResSyn)
        launch_pdl(blifat_kernel<true, true>, dim3(grid), dim3(kBlock), 0, s, p, ctl);
    else if (p.ring.fixed)
        launch_pdl(blifat_kernel<true, false>, dim3(grid), dim3(kBlock), 0, s, p, ctl);
    else
        launch_pdl(blifat_kernel<false, false>, dim3(grid), dim3(kBlock), 0, s, p, ctl);
}

void launch_altai(const AltaiDev &p, Control *ctl, cudaStream_t s)
{
    const uint32_t quads = (p.n + 3) / 4;
    const uint32_t grid = (quads + kBlock - 1) / kBlock;
    if (p.ring.fixed)
        launch_pdl(altai_kernel<true>, dim3(grid), dim3(kBlock), 0, s, p, ctl);
    else
        launch_pdl(altai_kernel<false>, dim3(grid), dim3(kBlock), 0, s, p, ctl);
}

void launch_altai_blocking(const AltaiDev &p, Control *ctl, cudaStream_t s)
{
    launch_pdl(altai_blocking_kernel, dim3(1), dim3(kAltaiBlockThreads), 0, s, p, ctl);
}

void launch_lif(const LifDev &p, Control *ctl, cudaStream_t s)
{
    const uint32_t quads = (p.n + 3) / 4;
    const uint32_t grid = (quads + kBlock - 1) / kBlock;
    launch_pdl(lif_kernel, dim3(grid), dim3(kBlock), 0, s, p, ctl);
}

void launch_apply_impacts(
    const RingView &ring, const uint32_t *post, const float *value, const uint8_t *type, int forcing, uint32_t n,
    uint32_t seq_base, Control *ctl, cudaStream_t s)
{
    if (!n) return;
    apply_impacts_kernel<<<(n + 255) / 256, 256, 0, s>>>(ring, post, value, type, forcing, n, seq_base, ctl);
}

}  // namespace knp_gb300
