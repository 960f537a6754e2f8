// Device-side per-neuron code of the population kernels, shared by the per-phase kernels
// (population.cu) and the fused small-network step kernel (small_net.cu). A thread steps 4
// consecutive neurons (float4 / 16-byte loads of state and input-ring slots); a block compacts its
// threads' spike masks into the population's spike list.
//
// BLIFAT arithmetic follows the reference per-neuron functions
//   calculate_pre_impact_single_neuron_state_impl   blifat_impl.h:31-47 (resource-STDP: :50-65)
//   impact_neuron_impl                              blifat_impl.h:68-107 (impacts pre-summed in the ring)
//   calculate_post_impact_single_neuron_state_impl  blifat_impl.h:110-168
//   resource-STDP neuron training without resource synapses  blifat_stdp.h:35-172, training/stdp.h:88-186
// (knp/backends/cpu/cpu-library/include/knp/backends/cpu-library/impl/populations/...), with FP32
// state. LIF follows lif_impl.h:33-86. Every floating-point operation is an explicit
// round-to-nearest intrinsic, so the compiler cannot contract it into an FMA.
#pragma once

#include <cstdint>

#include "kernels.h"

namespace knp_gb300
{
namespace
{

__device__ __forceinline__ float pf(const ParamF &p, uint32_t i) { return p.a ? p.a[i] : p.u; }
__device__ __forceinline__ uint32_t pu(const ParamU &p, uint32_t i) { return p.a ? p.a[i] : p.u; }

__device__ __forceinline__ float4 ld4(const float *p, uint32_t i) { return *reinterpret_cast<const float4 *>(p + i); }
__device__ __forceinline__ void st4(float *p, uint32_t i, float4 v) { *reinterpret_cast<float4 *>(p + i) = v; }
__device__ __forceinline__ uint4 ld4u(const uint32_t *p, uint32_t i) { return *reinterpret_cast<const uint4 *>(p + i); }
__device__ __forceinline__ void st4u(uint32_t *p, uint32_t i, uint4 v) { *reinterpret_cast<uint4 *>(p + i) = v; }
__device__ __forceinline__ float &at(float4 &v, int k) { return reinterpret_cast<float *>(&v)[k]; }
__device__ __forceinline__ uint32_t &at(uint4 &v, int k) { return reinterpret_cast<uint32_t *>(&v)[k]; }

// Append this thread's spikes (bit k of mask = neuron i0 + k) to list[*count ...] with one atomic
// per block; indexes stay ascending within a block. With a recording slot `rec` (rec_words words),
// also writes the step's spike bitmap: the 8 lanes of an aligned lane group cover 32 consecutive
// neurons, so OR-ing their 4-bit masks gives one whole word, stored by the group's first lane.
// Every thread of the block calls this (threads past the population with mask 0).
template <int kThreads>
__device__ __forceinline__ void emit_spikes(
    uint32_t mask, uint32_t i0, uint32_t *list, uint32_t *count, uint32_t *rec, uint32_t rec_words)
{
    __shared__ uint32_t warp_tot[kThreads / 32];
    __shared__ uint32_t block_base;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    if (rec)
    {
        uint32_t v = mask << (4 * (lane & 7));
        v |= __shfl_xor_sync(0xffffffffu, v, 1);
        v |= __shfl_xor_sync(0xffffffffu, v, 2);
        v |= __shfl_xor_sync(0xffffffffu, v, 4);
        const uint32_t word = i0 >> 5;
        if ((lane & 7) == 0 && word < rec_words) rec[word] = v;
    }
    const uint32_t c = __popc(mask);
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) warp_tot[warp] = incl;
    __syncthreads();
    if (warp == 0)
    {
        // Exclusive scan of the warps' totals on warp 0's lanes, one block-wide reservation.
        const uint32_t x = lane < kThreads / 32 ? warp_tot[lane] : 0u;
        uint32_t run = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const uint32_t v = __shfl_up_sync(0xffffffffu, run, o);
            if (lane >= o) run += v;
        }
        const uint32_t all = __shfl_sync(0xffffffffu, run, 31);
        if (lane < kThreads / 32) warp_tot[lane] = run - x;
        if (lane == 0) block_base = all ? atomicAdd(count, all) : 0u;
    }
    __syncthreads();
    if (!c) return;
    uint32_t pos = block_base + warp_tot[warp] + incl - c;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (mask & (1u << k)) list[pos++] = i0 + k;
}

__device__ __forceinline__ uint32_t *record_slot(uint32_t *rec_bits, uint32_t rec_words, uint32_t rec_slots,
                                                 unsigned long long t)
{
    return rec_bits ? rec_bits + static_cast<size_t>(t % rec_slots) * rec_words : nullptr;
}

struct NeuronState
{
    float V, V_pre, thr_dyn, trace, g, dopa, add_thr;
    uint32_t ns, phase;
    long long block;
    double add64;  // kResSyn: the FP64 additional threshold
};

// One BLIFAT neuron for one step. `acc` is this step's summed EXCITATORY - INHIBITORY_CURRENT input
// (FP32 ring) and (acc_hi, acc_lo) the same in two-word fixed point (fixed ring). kRS: a kResSyn
// population (separate instantiation, so that other populations carry none of its code).
template <bool kFixed, bool kRS = false>
__device__ __forceinline__ bool blifat_step(
    const BlifatDev &p, uint32_t i, unsigned long long t, NeuronState &s, float acc, long long acc_hi,
    long long acc_lo, float g_in, float d_in, uint32_t nf = 0)
{
    const uint32_t f = p.flags;
    const bool res = f & kResource;
    // ---- pre-impact (blifat_impl.h:31-65)
    if (f & kLiveRefract) s.ns = (s.ns == 0xFFFFFFFFu) ? 0u : (s.ns >= 0xFFFFFFFEu ? 0xFFFFFFFEu : s.ns + 1u);
    if (f & kLiveThrDyn) s.thr_dyn = __fmul_rn(s.thr_dyn, pf(p.thr_decay, i));
    if (f & kLiveTrace) s.trace = __fmul_rn(s.trace, pf(p.trace_decay, i));
    if (f & kLiveG) s.g = __fmul_rn(s.g, pf(p.g_decay, i));
    if (res) s.dopa = 0.0f;
    if (kRS && !(f & kLiveVRead))
        s.V = isfinite(s.V) ? 0.0f : __int_as_float(0x7FC00000);  // V * 0: NaN for a NaN or infinite V
    else
        s.V = (f & kLiveVRead) ? __fmul_rn(s.V, pf(p.v_decay, i)) : 0.0f;
    if ((f & kLiveBurst) && s.phase == 1u)
    {
        if (!res) s.phase = 0u;
        s.V = __fadd_rn(s.V, pf(p.reflexive, i));
    }
    s.V_pre = s.V;
    // ---- impacts (blifat_impl.h:68-107), pre-summed per channel
    // Fixed point: the exact potential as vh * 2^-8 + vl * 2^-48; the spike test compares it with the
    // threshold exactly, and the stored potential is its correctly rounded FP32 value.
    long long vh = 0, vl = 0;
    bool fx_ok = false;
    if (kFixed)
    {
        vh = acc_hi;
        vl = acc_lo;
        fx_normalize(vh, vl);
        if (s.V_pre != 0.0f)
        {
            long long ph, pl;
            fx_split(s.V_pre, ph, pl);
            vh += ph;
            vl += pl;
            fx_normalize(vh, vl);
        }
        fx_ok = true;
        s.V = fx_to_float(vh, vl);
        if (kRS && (nf || !isfinite(s.V_pre)))
        {
            // A non-finite term makes the FP64 sum non-finite: NaN if any term is NaN or both infinities
            // occur, else the infinity.
            const bool pinf = (nf & 2u) || s.V_pre == __int_as_float(0x7F800000);
            const bool ninf = (nf & 4u) || s.V_pre == __int_as_float(0xFF800000);
            if ((nf & 1u) || isnan(s.V_pre) || (pinf && ninf))
                s.V = __int_as_float(0x7FC00000);
            else
                s.V = pinf ? __int_as_float(0x7F800000) : __int_as_float(0xFF800000);
            fx_ok = false;
        }
    }
    else
    {
        s.V = __fadd_rn(s.V, acc);
    }
    if (f & kLiveG) s.g = __fadd_rn(s.g, g_in);
    if (f & kLiveDopa) s.dopa = __fadd_rn(s.dopa, d_in);
    // ---- post-impact (blifat_impl.h:119-168)
    if (f & kLiveBlock)
    {
        if (s.block <= 0)
        {
            s.V = s.V_pre;
            fx_ok = false;
        }
        if (s.block < 0)
        {
            ++s.block;
            if (s.block == 0) s.block = 0x7FFFFFFFFFFFFFFFll;
        }
        else if (s.block > 0)
        {
            --s.block;
        }
    }
    if (f & kLiveG)
    {
        const float e = pf(p.e_inh, i);
        if (s.g < 1.0f)
            s.V = __fsub_rn(s.V, __fmul_rn(__fsub_rn(s.V, e), s.g));
        else
            s.V = e;
        fx_ok = false;
    }
    const float thr_total = __fadd_rn(__fadd_rn(pf(p.thr, i), s.thr_dyn), s.add_thr);
    const bool ref_ok = (f & kLiveRefract) ? (s.ns > pu(p.t_ref, i)) : (t > 0);
    bool above;
    if (kRS)
    {
        // The additional threshold of trained synapses is an FP64 sum: compare in FP64, exactly
        // against the fixed-point potential.
        const double thr64 =
            __dadd_rn(__dadd_rn(static_cast<double>(pf(p.thr, i)), static_cast<double>(s.thr_dyn)), s.add64);
        if (kFixed && fx_ok)
        {
            long long th, tl;
            fx_ceil64(thr64, th, tl);
            above = vh > th || (vh == th && vl >= tl);
        }
        else
        {
            above = static_cast<double>(s.V) >= thr64;
        }
    }
    else if (kFixed && fx_ok)
    {
        long long th, tl;
        fx_split(thr_total, th, tl);
        above = vh > th || (vh == th && vl >= tl);
    }
    else
    {
        above = s.V >= thr_total;
    }
    const bool spike = ref_ok && above;
    if (spike)
    {
        if (f & kLiveThrDyn) s.thr_dyn = __fadd_rn(s.thr_dyn, pf(p.thr_inc, i));
        if (f & kLiveTrace) s.trace = __fadd_rn(s.trace, pf(p.trace_inc, i));
        s.V = pf(p.v_reset, i);
        if (f & kLiveBurst) s.phase = pu(p.burst_period, i);
        s.ns = (f & kLiveRefract) ? 0u : static_cast<uint32_t>(t);
    }
    const float vmin = pf(p.v_min, i);
    if (s.V < vmin) s.V = vmin;
    return spike;
}

// update_isi (training/stdp.h:88-126) of a neuron that spiked at step t: its new ISI status
// (0 is_forced, 1 period_started, 2 period_continued, 3 not_in_period). The step differences are
// unsigned, as in the reference.
__device__ __forceinline__ int32_t update_isi(
    int32_t status, bool forced, float dopa, uint32_t isi_max, unsigned long long t, unsigned long long &last_step,
    unsigned long long &first_isi_spike)
{
    if (forced) return 0;  // last_step_ is not updated
    switch (status)
    {
        case 3:
        case 0:
            status = 1;
            first_isi_spike = t;
            break;
        case 1:
            if (last_step - t < isi_max) status = 2;
            break;
        default:
            if (last_step - t >= isi_max || dopa != 0.0f)
            {
                status = 1;
                first_isi_spike = t;
            }
            break;
    }
    last_step = t;
    return status;
}

// The dopamine change of stability (blifat_stdp.h:138-150). The reference's dopamine value and
// intermediates are FP64 and the stored stability FP32: the same operations here.
__device__ __noinline__ float dopamine_stability(
    float stability, float dopa, float change_param, bool forced, unsigned long long t,
    unsigned long long first_isi_spike, uint32_t isi_max)
{
    if (forced || dopa < 0.0f)
    {
        const float st = __double2float_rn(
            __dsub_rn(static_cast<double>(stability), __dmul_rn(static_cast<double>(dopa), static_cast<double>(change_param))));
        return st < 0.0f ? 0.0f : st;  // std::max(stability, 0.0F)
    }
    // std::fabs of the unsigned difference, converted to double.
    const double difference = __ull2double_rn(t - first_isi_spike - isi_max);
    const double q = __dsub_rn(2.0, __ddiv_rn(difference, static_cast<double>(isi_max)));
    const double m = q < -1.0 ? -1.0 : q;  // std::max(q, -1.0)
    const double inc = __dmul_rn(__dmul_rn(static_cast<double>(change_param), static_cast<double>(dopa)), m);
    return __double2float_rn(__dadd_rn(static_cast<double>(stability), inc));
}

// Resource-STDP neuron bookkeeping with no resource-STDP synapses (blifat_stdp.h:35-172). Returns
// whether the dopamine change of stability is due; the caller applies it (dopamine_stability) once
// the neuron's other state is stored, which keeps the rare FP64 path off the step's registers.
__device__ __forceinline__ bool resource_step(
    const BlifatDev &p, uint32_t i, unsigned long long t, bool spike, bool forced, float dopa, float &add_thr)
{
    const ResourceDev &r = p.res;
    int32_t status = r.isi_status[i];
    const uint32_t isi_max = pu(r.isi_max, i);
    if (spike)
    {
        // process_spiking_neurons_impl (blifat_stdp.h:43-67) + update_isi.
        r.last_spike_step[i] = t;
        unsigned long long last = r.last_step[i], first = r.first_isi_spike[i];
        status = update_isi(status, forced, dopa, isi_max, t, last, first);
        r.last_step[i] = last;
        r.first_isi_spike[i] = first;
        if (status == 1) r.stability[i] = __fsub_rn(r.stability[i], pf(r.stability_change_at_isi, i));
        add_thr = __fmul_rn(0.0f, pf(r.add_thr_coef, i));
    }
    // do_dopamine_plasticity_impl (blifat_stdp.h:106-155), no connected synapses: only stability
    // changes, and the renormalisation below does not read it.
    const bool dopamine = dopa > 0.0f || (dopa < 0.0f && status != 0);
    // renormalize_resource (training/stdp.h:152-186), no connected synapses.
    if (p.flags & kLiveRenorm)
    {
        if (!(t - r.last_step[i] <= isi_max && status != 0))
        {
            const float fr = r.free_resource[i];
            if (!(fabsf(fr) < pf(r.resource_threshold, i))) r.free_resource[i] = 0.0f;
        }
    }
    r.isi_status[i] = status;
    r.is_forced[i] = forced ? 1 : 0;
    return dopamine;
}

// kResSyn populations: the training kernel (resource.cu) runs the whole neuron-side training after
// the population step. Here the step's forcing flag is stored, and a neuron that did not spike is
// listed for the training kernel when it has dopamine or renormalisation work (the spike list
// holds the others); a neuron with neither is left unchanged by the training.
__device__ __forceinline__ void resource_mark(const BlifatDev &p, uint32_t i, unsigned long long t, bool spike,
                                              bool forced, float dopa)
{
    const ResourceDev &r = p.res;
    r.is_forced[i] = forced ? 1 : 0;
    if (spike) return;
    const int32_t status = r.isi_status[i];
    bool need = dopa > 0.0f || (dopa < 0.0f && status != 0);
    if (!need)
        need = !(t - r.last_step[i] <= pu(r.isi_max, i) && status != 0) &&
               !(fabsf(r.free_resource[i]) < pf(r.resource_threshold, i));
    if (need) p.syn.work[atomicAdd(p.syn.work_count, 1u)] = i;
}

// Steps neurons i0 .. i0 + 3 of a BLIFAT population (those below n) at step t and returns their spike
// mask (bit k = neuron i0 + k fired).
template <bool kFixed, bool kRS = false>
__device__ __forceinline__ uint32_t blifat_quad(const BlifatDev &p, unsigned long long t, uint32_t i0)
{
    const uint32_t f = p.flags;
    uint32_t mask = 0;
    if (i0 < p.n)
    {
        const RingView &rg = p.ring;
        const uint32_t slot = static_cast<uint32_t>(t % rg.slots);
        const size_t ro = static_cast<size_t>(slot) * rg.pitch + i0;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        long long acc_hi[4] = {0, 0, 0, 0}, acc_lo[4] = {0, 0, 0, 0};
        if (kFixed)
        {
            longlong2 *a = reinterpret_cast<longlong2 *>(rg.v64 + ro);
            longlong2 *b = reinterpret_cast<longlong2 *>(rg.v64lo + ro);
            const longlong2 x = a[0], y = a[1], xl = b[0], yl = b[1];
            acc_hi[0] = x.x;
            acc_hi[1] = x.y;
            acc_hi[2] = y.x;
            acc_hi[3] = y.y;
            acc_lo[0] = xl.x;
            acc_lo[1] = xl.y;
            acc_lo[2] = yl.x;
            acc_lo[3] = yl.y;
            a[0] = a[1] = b[0] = b[1] = make_longlong2(0, 0);
        }
        else
        {
            acc = ld4(rg.v32, ro);
            st4(rg.v32, ro, make_float4(0.f, 0.f, 0.f, 0.f));
        }
        float4 gin = make_float4(0.f, 0.f, 0.f, 0.f), din = gin;
        if (rg.g)
        {
            gin = ld4(rg.g, ro);
            st4(rg.g, ro, make_float4(0.f, 0.f, 0.f, 0.f));
        }
        if (rg.dopa)
        {
            din = ld4(rg.dopa, ro);
            st4(rg.dopa, ro, make_float4(0.f, 0.f, 0.f, 0.f));
        }
        uint32_t forced_bits = 0;
        if (rg.forced)
        {
            uint32_t *wp = rg.forced + static_cast<size_t>(slot) * rg.words + (i0 >> 5);
            forced_bits = (*wp >> (i0 & 31)) & 0xFu;
            if (forced_bits) atomicAnd(wp, ~(0xFu << (i0 & 31)));
        }
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        float4 V = (kRS || (f & kLiveVRead)) ? ld4(p.V, i0) : z;
        uint32_t nf_bits = 0;  // kRS: the four neurons' non-finite impact bytes
        if (kRS && rg.nf)
        {
            uint32_t *wp = rg.nf + (ro >> 2);
            nf_bits = *wp;
            if (nf_bits) *wp = 0u;
        }
        float4 thr_dyn = (f & kLiveThrDyn) ? ld4(p.thr_dyn, i0) : z;
        float4 trace = (f & kLiveTrace) ? ld4(p.trace, i0) : z;
        float4 g = (f & kLiveG) ? ld4(p.g, i0) : z;
        float4 dopa = ((f & kLiveDopa) && !(f & kResource)) ? ld4(p.dopa, i0) : z;
        float4 add_thr = (f & kLiveAddThr) ? ld4(p.add_thr, i0) : z;
        uint4 ns = (f & kLiveRefract) ? ld4u(p.n_since, i0) : make_uint4(0, 0, 0, 0);
        uint4 phase = (f & kLiveBurst) ? ld4u(p.burst_phase, i0) : make_uint4(0, 0, 0, 0);
        float4 vpre;
        const uint4 ns_old = ns;
        uint32_t dopamine_due = 0;  // neurons whose dopamine stability change follows the loop
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            const uint32_t i = i0 + k;
            if (i >= p.n) break;
            NeuronState s;
            s.V = at(V, k);
            s.thr_dyn = at(thr_dyn, k);
            s.trace = at(trace, k);
            s.g = at(g, k);
            s.dopa = at(dopa, k);
            s.add_thr = at(add_thr, k);
            s.ns = at(ns, k);
            s.phase = at(phase, k);
            s.block = (f & kLiveBlock) ? p.blocking[i] : 0;
            s.add64 = kRS ? p.syn.add_thr[i] : 0.0;
            if ((f & kLiveBlock) && rg.blk)
            {
                // The step's last BLOCKING impact sets the period (impact phase, blifat_impl.h:86).
                const unsigned long long key = rg.blk[ro + k];
                if (key)
                {
                    rg.blk[ro + k] = 0ull;
                    const unsigned long long order = key >> kBlkOrderShift;
                    s.block = order == kBlkExternal
                                  ? rg.blk_ext[i]
                                  : static_cast<long long>(rg.blk_w[order - 1][key & kBlkPosMask]);
                }
            }
            const bool spike = blifat_step<kFixed, kRS>(p, i, t, s, at(acc, k), acc_hi[k], acc_lo[k], at(gin, k), at(din, k),
                                                        (nf_bits >> (8 * k)) & 0xFFu);
            if (spike) mask |= 1u << k;
            if (kRS)
                resource_mark(p, i, t, spike, (forced_bits >> k) & 1u, s.dopa);
            else if ((f & kResource) && resource_step(p, i, t, spike, (forced_bits >> k) & 1u, s.dopa, s.add_thr))
                dopamine_due |= 1u << k;
            at(V, k) = s.V;
            at(vpre, k) = s.V_pre;
            at(thr_dyn, k) = s.thr_dyn;
            at(trace, k) = s.trace;
            at(g, k) = s.g;
            at(dopa, k) = s.dopa;
            at(add_thr, k) = s.add_thr;
            at(ns, k) = s.ns;
            at(phase, k) = s.phase;
            if (f & kLiveBlock) p.blocking[i] = s.block;
        }
        // Padding lanes beyond n write their (unused) slots too; the arrays are padded to n_pad.
        st4(p.V, i0, V);
        if (f & kLiveVPre) st4(p.V_pre, i0, vpre);
        if (f & kLiveThrDyn) st4(p.thr_dyn, i0, thr_dyn);
        if (f & kLiveTrace) st4(p.trace, i0, trace);
        if (f & kLiveG) st4(p.g, i0, g);
        if ((f & kLiveDopa) || (f & kResource)) st4(p.dopa, i0, dopa);
        if ((f & kLiveAddThr) || (f & kResource)) st4(p.add_thr, i0, add_thr);
        if (f & kLiveRefract)
            st4u(p.n_since, i0, ns);
        else if (mask)
        {
            // Lazy refractory tracking: record the step of the last spike.
#pragma unroll
            for (int k = 0; k < 4; ++k)
                if (mask & (1u << k)) p.n_since[i0 + k] = at(ns, k);
        }
        (void)ns_old;
        if (f & kLiveBurst) st4u(p.burst_phase, i0, phase);
        for (; dopamine_due; dopamine_due &= dopamine_due - 1)
        {
            const uint32_t k = __ffs(dopamine_due) - 1, i = i0 + k;
            const ResourceDev &r = p.res;
            r.stability[i] = dopamine_stability(r.stability[i], at(dopa, k), pf(r.stability_change_param, i),
                                                (forced_bits >> k) & 1u, t, r.first_isi_spike[i], pu(r.isi_max, i));
        }
    }
    return mask;
}

// Steps neurons i0 .. i0 + 3 of a LIF population at step t; returns their spike mask.
// blifat_quad for a population whose every state field is lazy (flags 0: no potential,
// threshold, trace, conductance or dopamine dynamics, no bursting or blocking, refractory period 0
// with the default counter, no additional threshold — the reference's default BLIFAT neuron) and an
// FP32 input ring. blifat_step then reduces to: the potential is +0 plus this step's input sum, a
// spike iff the step is not step 0 and the potential reaches the threshold, the reset, and the
// min-potential clamp; the same operations in the same order, so results are identical.
__device__ __forceinline__ uint32_t blifat_quad_lean(const BlifatDev &p, unsigned long long t, uint32_t i0)
{
    uint32_t mask = 0;
    if (i0 < p.n)
    {
        const RingView &rg = p.ring;
        const uint32_t slot = static_cast<uint32_t>(t % rg.slots);
        const size_t ro = static_cast<size_t>(slot) * rg.pitch + i0;
        float4 acc = ld4(rg.v32, ro);
        st4(rg.v32, ro, make_float4(0.f, 0.f, 0.f, 0.f));
        float4 V = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            const uint32_t i = i0 + k;
            if (i >= p.n) break;
            float v = __fadd_rn(0.0f, at(acc, k));
            const float thr_total = __fadd_rn(__fadd_rn(pf(p.thr, i), 0.0f), 0.0f);
            if (t > 0 && v >= thr_total)
            {
                mask |= 1u << k;
                v = pf(p.v_reset, i);
                p.n_since[i] = static_cast<uint32_t>(t);  // lazy refractory tracking: the step of the spike
            }
            const float vmin = pf(p.v_min, i);
            if (v < vmin) v = vmin;
            at(V, k) = v;
        }
        st4(p.V, i0, V);
    }
    return mask;
}

// The BLIFAT quad step of any plain population (no resource-STDP synapses) for the fused and grid
// kernels.
__device__ __forceinline__ uint32_t blifat_quad_any(const BlifatDev &p, unsigned long long t, uint32_t i0)
{
    if (p.ring.fixed) return blifat_quad<true>(p, t, i0);
    if (p.flags == 0u) return blifat_quad_lean(p, t, i0);
    return blifat_quad<false>(p, t, i0);
}

// AltAI-LIF neurons i0 .. i0 + 3 (altai_impl.h:33-168) at step t; returns their spike mask. The
// impact sum is exact (FP32 ring of dyadic weights or fixed point) and rounded once, which equals the
// reference's FP32 sum taken impact by impact whenever its partial sums are exact (integer weights,
// as AltAI hardware uses, or dyadic ones). BLOCKING impacts were applied to the activity time by
// the population's blocking kernel before this step's kernel.
template <bool kFixed>
__device__ __forceinline__ uint32_t altai_quad(const AltaiDev &p, unsigned long long t, uint32_t i0)
{
    const uint32_t f = p.flags;
    uint32_t mask = 0;
    if (i0 >= p.n) return 0;
    const RingView &rg = p.ring;
    const uint32_t slot = static_cast<uint32_t>(t % rg.slots);
    const size_t ro = static_cast<size_t>(slot) * rg.pitch + i0;
    uint32_t forced_bits = 0;
    if (rg.forced)
    {
        uint32_t *wp = rg.forced + static_cast<size_t>(slot) * rg.words + (i0 >> 5);
        forced_bits = (*wp >> (i0 & 31)) & 0xFu;
        if (forced_bits) atomicAnd(wp, ~(0xFu << (i0 & 31)));
    }
    uint32_t nf_bits = 0;
    if (rg.nf)
    {
        uint32_t *wp = rg.nf + (ro >> 2);
        nf_bits = *wp;
        if (nf_bits) *wp = 0u;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
    {
        const uint32_t i = i0 + k;
        if (i >= p.n) break;
        const uint32_t cfg = pu(p.cfg, i);
        // ---- pre-impact: the potential rounded (std::round: half away from zero) or reset.
        float V = (cfg & kAltaiNoSave) ? static_cast<float>(pu(p.reset, i)) : roundf(p.V[i]);
        const float v_pre = V;
        float dopa = 0.0f;
        // ---- impacts
        bool finite_sum = true;
        if (kFixed)
        {
            long long vh = rg.v64[ro + k], vl = rg.v64lo[ro + k];
            rg.v64[ro + k] = 0;
            rg.v64lo[ro + k] = 0;
            fx_normalize(vh, vl);
            if (isfinite(V))
            {
                if (V != 0.0f)
                {
                    long long ph, pl;
                    fx_split(V, ph, pl);
                    vh += ph;
                    vl += pl;
                    fx_normalize(vh, vl);
                }
                V = fx_to_float(vh, vl);
            }
            else
            {
                finite_sum = false;
            }
        }
        else
        {
            V = __fadd_rn(V, rg.v32[ro + k]);
            rg.v32[ro + k] = 0.0f;
        }
        const uint32_t nf = (nf_bits >> (8 * k)) & 0xFFu;
        if (nf || !finite_sum)
        {
            const bool pinf = (nf & 2u) || v_pre == __int_as_float(0x7F800000);
            const bool ninf = (nf & 4u) || v_pre == __int_as_float(0xFF800000);
            if ((nf & 1u) || isnan(v_pre) || (pinf && ninf))
                V = __int_as_float(0x7FC00000);
            else
                V = pinf ? __int_as_float(0x7F800000) : __int_as_float(0xFF800000);
        }
        if (rg.dopa)
        {
            dopa = rg.dopa[ro + k];
            rg.dopa[ro + k] = 0.0f;
        }
        // The resource-STDP variant clears the dopamine value at pre-impact; the plain one keeps adding.
        if (!(f & kResource) && p.dopa) dopa = __fadd_rn(p.dopa[i], dopa);
        // ---- post-impact
        const int32_t leak = static_cast<int32_t>(pu(p.leak, i));
        const int sign = ((cfg & kAltaiLeakRev) && V < 0.0f) ? -1 : 1;
        V = __fadd_rn(V, static_cast<float>(leak * sign));
        long long act = p.activity[i];
        if (act > 0)
            --act;
        else if (act < 0)
            ++act;
        if (act == 0) act = 0x7FFFFFFFFFFFFFFFll;
        const double thr = __dadd_rn(static_cast<double>(pu(p.thr, i)), p.add_thr[i]);
        bool spike = false, was_reset = false;
        if (static_cast<double>(V) >= thr)
        {
            if (act > 0) spike = true;
            if (cfg & kAltaiDiff) V = __double2float_rn(__dsub_rn(static_cast<double>(V), thr));
            if (cfg & kAltaiReset)
            {
                V = static_cast<float>(pu(p.reset, i));
                was_reset = true;
            }
        }
        const float neg = static_cast<float>(pu(p.neg_thr, i));
        if (V <= -neg && !was_reset)
        {
            if (cfg & kAltaiSaturate)
                V = -neg;
            else if (cfg & kAltaiReset)
                V = static_cast<float>(-static_cast<int32_t>(pu(p.reset, i)));
            else if (cfg & kAltaiDiff)
                V = __fadd_rn(V, neg);
        }
        p.V[i] = V;
        p.V_pre[i] = v_pre;
        p.activity[i] = act;
        if (p.dopa) p.dopa[i] = dopa;
        if (f & kResource)
        {
            // The resource-STDP training kernel runs the neuron-side training; list this neuron for it.
            const ResourceDev &r = p.res;
            const bool forced = (forced_bits >> k) & 1u;
            r.is_forced[i] = forced ? 1 : 0;
            if (!spike)
            {
                const int32_t status = r.isi_status[i];
                bool need = dopa > 0.0f || (dopa < 0.0f && status != 0);
                if (!need)
                    need = !(t - r.last_step[i] <= pu(r.isi_max, i) && status != 0) &&
                           !(fabsf(r.free_resource[i]) < pf(r.resource_threshold, i));
                if (need) p.syn.work[atomicAdd(p.syn.work_count, 1u)] = i;
            }
        }
        if (spike) mask |= 1u << k;
    }
    return mask;
}

__device__ __forceinline__ uint32_t lif_quad(const LifDev &p, unsigned long long t, uint32_t i0)
{
    uint32_t mask = 0;
    if (i0 < p.n)
    {
        const RingView &rg = p.ring;
        const uint32_t slot = static_cast<uint32_t>(t % rg.slots);
        const size_t ro = static_cast<size_t>(slot) * rg.pitch + i0;
        float4 acc = ld4(rg.v32, ro);
        st4(rg.v32, ro, make_float4(0.f, 0.f, 0.f, 0.f));
        float4 V = ld4(p.V, i0);
        uint4 rc = ld4u(p.refract, i0);
#pragma unroll
        for (int k = 0; k < 4; ++k)
        {
            const uint32_t i = i0 + k;
            if (i >= p.n) break;
            float v = at(V, k);
            uint32_t r = at(rc, k);
            // lif_impl.h:33-86: leak and impacts only outside the refractory period; strict '>'.
            if (r == 0u)
            {
                v = __fmul_rn(v, pf(p.leak, i));
                v = __fadd_rn(v, at(acc, k));
                if (v > pf(p.thr, i))
                {
                    v = pf(p.v_reset, i);
                    r = pu(p.refract_period, i);
                    mask |= 1u << k;
                }
            }
            else
            {
                --r;
            }
            at(V, k) = v;
            at(rc, k) = r;
        }
        st4(p.V, i0, V);
        st4u(p.refract, i0, rc);
    }
    return mask;
}

}  // namespace
}  // namespace knp_gb300
