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
    const uint32_t mask = blifat_quad<kFixed, kRS>(p, t, i0);
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
    Control *ctl)
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
        if (ring.fixed)
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

void launch_lif(const LifDev &p, Control *ctl, cudaStream_t s)
{
    const uint32_t quads = (p.n + 3) / 4;
    const uint32_t grid = (quads + kBlock - 1) / kBlock;
    launch_pdl(lif_kernel, dim3(grid), dim3(kBlock), 0, s, p, ctl);
}

void launch_apply_impacts(
    const RingView &ring, const uint32_t *post, const float *value, const uint8_t *type, int forcing, uint32_t n,
    Control *ctl, cudaStream_t s)
{
    if (!n) return;
    apply_impacts_kernel<<<(n + 255) / 256, 256, 0, s>>>(ring, post, value, type, forcing, n, ctl);
}

}  // namespace knp_gb300
