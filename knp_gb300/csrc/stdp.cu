// Additive STDP kernels and the end-of-step kernel.
//
// The reference rule (knp/backends/cpu/cpu-library/include/knp/backends/cpu-library/impl/projections/
// training/stdp/additive_stdp.h) keeps two spike-time lists per synapse and, every step, scans all
// synapses:
//   init_projection (:117-170)  a SpikeMessage from an STDP population appends its send time to the
//       postsynaptic list (and, for STDPAndSpike, the presynaptic list) of every synapse found
//       by_postsynaptic for each spiking index, while the list is shorter than tau+ + tau-;
//   modify_weights (:173-196)   when both lists reach tau+ + tau-, weight += sum over (t_f in pre,
//       t_n in post) of stdp_w(float(t_n - t_f)) with unsigned differences, then both lists clear.
// Every synapse of one postsynaptic column receives the same appends, so the GB300 layout keeps one
// pair of lists per column and touches only the columns appended this step. stdp_w(d) is 1 for
// d = 0, expf(-d / tau+) for d > 0 and 0 for t_n < t_f (the unsigned difference wraps to a huge
// value); its values for d in [0, table_len) come from the host, computed with the same libm call as
// the reference, and the sum is accumulated in the reference's order in FP32.
#include <cstdint>

#include "kernels.h"
#include "stdp_dev.cuh"

namespace knp_gb300
{
namespace
{

__global__ void stdp_append_kernel(StdpDev d, SpikeSource src, int both_lists, Control *ctl)
{
    pdl_begin();
    stdp_append_range(d, src, both_lists, ctl->step, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// One warp per touched column.
__global__ void stdp_modify_kernel(StdpDev d, Control *ctl)
{
    pdl_begin();
    stdp_modify_range(d, (blockIdx.x * blockDim.x + threadIdx.x) >> 5, (gridDim.x * blockDim.x) >> 5,
                      threadIdx.x & 31);
}

__global__ void step_end_kernel(StepEnd e, uint32_t n_spike_counts, Control *ctl)
{
    pdl_begin();
    __shared__ unsigned long long spikes;
    if (threadIdx.x == 0) spikes = 0;
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < e.n_zero_u32; k += blockDim.x)
    {
        if (k < n_spike_counts) atomicAdd(&spikes, static_cast<unsigned long long>(e.zero_u32[k]));
        e.zero_u32[k] = 0;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        ctl->spikes_total += spikes;
        ctl->step += 1;
    }
}

}  // namespace

void launch_stdp_append(const StdpDev &d, SpikeSource src, int both_lists, Control *ctl, cudaStream_t s)
{
    const int threads = 256;
    const int blocks = static_cast<int>((d.n_cols + threads - 1) / threads);
    launch_pdl(stdp_append_kernel, dim3(blocks > 0 ? blocks : 1), dim3(threads), 0, s, d, src, both_lists, ctl);
}

void launch_stdp_modify(const StdpDev &d, Control *ctl, cudaStream_t s)
{
    const int threads = 256;
    int blocks = static_cast<int>((static_cast<uint64_t>(d.n_cols) * 32 + threads - 1) / threads);
    if (blocks > 1216) blocks = 1216;
    launch_pdl(stdp_modify_kernel, dim3(blocks > 0 ? blocks : 1), dim3(threads), 0, s, d, ctl);
}

// Zeroes this step's counters (adding the population spike counts to the spike total) and advances
// the device step number.
void launch_step_end(const StepEnd &e, Control *ctl, cudaStream_t s)
{
    launch_pdl(step_end_kernel, dim3(1), dim3(256), 0, s, e, e.n_spike_counts, ctl);
}

}  // namespace knp_gb300
