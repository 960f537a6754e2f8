// Neuron-side training of resource-STDP BLIFAT and AltAI-LIF populations over their
// SynapticResourceSTDPDeltaSynapse projections, after the population step and before the
// projections (the population's step in populations_old.h:195-217 ends with train_population; the
// AltAI-LIF training of altai/altai_stdp.h is the same computation):
//   process_spiking_neurons_impl (knp/backends/cpu/cpu-library/include/knp/backends/cpu-library/impl/
//     populations/blifat/blifat_stdp.h:35-103) for every neuron that spiked,
//   do_dopamine_plasticity_impl (:106-155) and renormalize_resource (impl/populations/training/
//     stdp.h:152-186) for every neuron, with recalculate_synapse_weights (training/stdp.h:40-52).
//
// Neurons are independent (a neuron's synapses are the ones into it), so one warp trains one neuron
// through all three stages in the reference's order. The work list is this step's spike list
// followed by the non-spiking neurons the population kernel found with dopamine or renormalisation
// work; every other neuron would be left unchanged. A neuron's synapses are its entries of the
// column index, in get_all_connected_synapses order (projection load order, then synapse index),
// skipping locked projections. Per-synapse updates run on the warp's lanes; the two quantities the
// reference accumulates across synapses (the FP64 additional threshold and the FP32 free
// resource) are accumulated in synapse order, so every rounding is the reference's.
#include <cstdint>

#include "kernels.h"
#include "population_dev.cuh"

namespace knp_gb300
{
namespace
{

constexpr int kTrainThreads = 256;
constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr unsigned long long kPosMask = (1ull << kResSlotShift) - 1;

// std::min(static_cast<float>(std::pow(2, -stability)), 1.F): the power in FP64 (CUDA's exp2),
// rounded to FP32.
__device__ __forceinline__ float resource_factor(float stability)
{
    const float v = __double2float_rn(exp2(-static_cast<double>(stability)));
    return 1.0f < v ? 1.0f : v;
}

// recalculate_synapse_weights (training/stdp.h:40-52) for one synapse.
__device__ __forceinline__ float synapse_weight(float resource, float w_min, float w_max)
{
    const float syn_w = resource < 0.0f ? 0.0f : resource;  // std::max(resource, 0.F)
    const float diff = __fsub_rn(w_max, w_min);
    return __fadd_rn(w_min, __fdiv_rn(__fmul_rn(diff, syn_w), __fadd_rn(diff, syn_w)));
}

// is_point_in_interval (training/stdp.h:129-133), unsigned.
__device__ __forceinline__ bool in_interval(unsigned long long a, unsigned long long b, unsigned long long x)
{
    if (a > b)
    {
        const unsigned long long c = a;
        a = b;
        b = c;
    }
    return a <= x && x <= b;
}

// Synapse `e` of the column range [a, b): its position in the concatenated arrays, and whether it
// belongs to an unlocked projection (is in the working list).
__device__ __forceinline__ bool working_synapse(const ResSynDev &y, long long e, long long b, unsigned long long &pos)
{
    if (e >= b) return false;
    const unsigned long long ent = y.col_pos[e];
    pos = ent & kPosMask;
    return y.locked[ent >> kResSlotShift] == 0u;
}

__device__ void train_neuron(const TrainView &p, uint32_t i, unsigned long long t, bool spiked, int lane)
{
    const ResourceDev &r = p.res;
    const ResSynDev &y = p.syn;
    int32_t status = r.isi_status[i];
    const bool forced = r.is_forced[i] != 0;
    const float dopa = p.dopa[i];
    float stab = r.stability[i], fr = r.free_resource[i];
    unsigned long long last_step = r.last_step[i], first = r.first_isi_spike[i], last_spike = r.last_spike_step[i];
    const uint32_t isi_max = pu(r.isi_max, i);
    const long long a = y.col_ptr[i], b = y.col_ptr[i + 1];

    if (spiked)
    {
        // process_spiking_neurons_impl: ISI status, stability at a new ISI period, then one pass over
        // the synapses (additional-threshold term from the weight before this step's change,
        // contribution flag, Hebbian flag reset, resource change, new weight).
        last_spike = t;
        status = update_isi(status, forced, dopa, isi_max, t, last_step, first);
        if (status == 1) stab = __fsub_rn(stab, pf(r.stability_change_at_isi, i));
        const float d_h = __fmul_rn(pf(r.d_h, i), resource_factor(stab));
        double add = 0.0;
        for (long long base = a; base < b; base += 32)
        {
            unsigned long long pos = 0;
            const bool ok = working_synapse(y, base + lane, b, pos);
            float x = 0.0f, du = 0.0f;
            bool hebb = false;
            if (ok)
            {
                const float w = y.w[pos];
                x = __fmul_rn(w, w > 0.0f ? 1.0f : 0.0f);
                const bool had_spike = in_interval(t - y.period[pos], t, y.last_spike[pos] + y.delay[pos] - 1ull);
                uint32_t fl = y.flags[pos];
                if (status != 2 || had_spike) fl = had_spike ? (fl | 2u) : (fl & ~2u);
                if (status != 2) fl &= ~1u;
                float res = y.resource[pos];
                if (status != 0)
                {
                    du = y.d_u[pos];
                    res = __fsub_rn(res, du);
                    if ((fl & 2u) && !(fl & 1u))
                    {
                        res = __fadd_rn(res, d_h);
                        fl |= 1u;
                        hebb = true;
                    }
                }
                y.resource[pos] = res;
                y.flags[pos] = static_cast<uint8_t>(fl);
                y.w[pos] = synapse_weight(res, y.w_min[pos], y.w_max[pos]);
            }
            const unsigned okm = __ballot_sync(kFull, ok), hm = __ballot_sync(kFull, hebb);
            for (int q = 0; q < 32; ++q)
            {
                const float xq = __shfl_sync(kFull, x, q), dq = __shfl_sync(kFull, du, q);
                if (!((okm >> q) & 1u)) continue;
                add = __dadd_rn(add, static_cast<double>(xq));
                if (status != 0)
                {
                    fr = __fadd_rn(fr, dq);
                    if ((hm >> q) & 1u) fr = __fsub_rn(fr, d_h);
                }
            }
        }
        add = __dmul_rn(add, static_cast<double>(pf(r.add_thr_coef, i)));
        if (lane == 0) y.add_thr[i] = add;
    }

    if (dopa > 0.0f || (dopa < 0.0f && status != 0))
    {
        // do_dopamine_plasticity_impl: resource change of contributing synapses while the last spike
        // is recent, stability change, new weights of every synapse.
        const bool recent = t - last_spike <= pu(r.dopamine_time, i);
        const float change = __fmul_rn(dopa, resource_factor(stab));
        for (long long base = a; base < b; base += 32)
        {
            unsigned long long pos = 0;
            const bool ok = working_synapse(y, base + lane, b, pos);
            bool app = false;
            if (ok)
            {
                float res = y.resource[pos];
                if (recent && (y.flags[pos] & 2u))
                {
                    res = __fadd_rn(res, change);
                    y.resource[pos] = res;
                    app = true;
                }
                y.w[pos] = synapse_weight(res, y.w_min[pos], y.w_max[pos]);
            }
            const unsigned am = __ballot_sync(kFull, app);
            for (int q = 0; q < 32; ++q)
                if ((am >> q) & 1u) fr = __fsub_rn(fr, change);
        }
        stab = dopamine_stability(stab, dopa, pf(r.stability_change_param, i), forced, t, first, isi_max);
    }

    if (!(t - last_step <= isi_max && status != 0) && !(fabsf(fr) < pf(r.resource_threshold, i)))
    {
        // renormalize_resource: the free resource divided over the working synapses and the drain.
        unsigned long long n_syn = 0;
        for (long long base = a; base < b; base += 32)
        {
            unsigned long long pos = 0;
            n_syn += __popc(__ballot_sync(kFull, working_synapse(y, base + lane, b, pos)));
        }
        const float add_v = __fdiv_rn(fr, __ull2float_rn(n_syn + pu(r.drain, i)));
        for (long long base = a; base < b; base += 32)
        {
            unsigned long long pos = 0;
            if (working_synapse(y, base + lane, b, pos))
            {
                const float res = __fadd_rn(y.resource[pos], add_v);
                y.resource[pos] = res;
                y.w[pos] = synapse_weight(res, y.w_min[pos], y.w_max[pos]);
            }
        }
        fr = 0.0f;
    }

    if (lane == 0)
    {
        r.isi_status[i] = status;
        r.last_step[i] = last_step;
        r.first_isi_spike[i] = first;
        r.last_spike_step[i] = last_spike;
        r.stability[i] = stab;
        r.free_resource[i] = fr;
    }
}

__global__ void __launch_bounds__(kTrainThreads) resource_train_kernel(TrainView p, Control *ctl)
{
    pdl_begin();
    const unsigned long long t = ctl->step;
    const uint32_t n_spk = *p.spike_count, n_work = *p.syn.work_count;
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t j = warp; j < n_spk + n_work; j += n_warps)
    {
        const bool spiked = j < n_spk;
        train_neuron(p, spiked ? p.spikes[j] : p.syn.work[j - n_spk], t, spiked, lane);
    }
}

}  // namespace

void launch_resource_train(const TrainView &p, int blocks, Control *ctl, cudaStream_t s)
{
    launch_pdl(resource_train_kernel, dim3(blocks > 0 ? blocks : 1), dim3(kTrainThreads), 0, s, p, ctl);
}

}  // namespace knp_gb300
