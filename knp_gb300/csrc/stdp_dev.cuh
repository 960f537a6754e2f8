// Device-side additive-STDP code, shared by the per-phase kernels (stdp.cu) and the fused
// small-network step kernel (small_net.cu). The rule and its layout are described in stdp.cu.
#pragma once

#include <cstdint>

#include "kernels.h"

namespace knp_gb300
{
namespace
{

// Appends step t's spikes of one STDP source to the column histories; this thread takes spikes
// thread, thread + n_threads, ...
__device__ __forceinline__ void stdp_append_range(
    const StdpDev &d, const SpikeSource &src, int both_lists, unsigned long long t, uint32_t thread,
    uint32_t n_threads)
{
    const uint32_t *idx;
    uint32_t cnt;
    if (src.channel)
    {
        const ChannelDev &c = *src.channel;
        if (t >= c.first_step && t - c.first_step < c.n_steps)
        {
            const unsigned long long k = t - c.first_step;
            idx = c.idx + c.offsets[k];
            cnt = static_cast<uint32_t>(c.offsets[k + 1] - c.offsets[k]);
        }
        else
        {
            return;
        }
    }
    else
    {
        idx = src.idx;
        cnt = *src.count;
    }
    for (uint32_t k = thread; k < cnt; k += n_threads)
    {
        const uint32_t col = idx[k];
        if (col >= d.n_cols) continue;
        const uint32_t tt = static_cast<uint32_t>(t);
        uint32_t c = d.post_cnt[col];
        if (c < d.period)
        {
            d.post_hist[static_cast<size_t>(col) * d.period + c] = tt;
            d.post_cnt[col] = c + 1;
        }
        if (both_lists)
        {
            c = d.pre_cnt[col];
            if (c < d.period)
            {
                d.pre_hist[static_cast<size_t>(col) * d.period + c] = tt;
                d.pre_cnt[col] = c + 1;
            }
        }
        if (d.touched_stamp[col] != t + 1)
        {
            d.touched_stamp[col] = t + 1;
            d.touched[atomicAdd(d.touched_count, 1u)] = col;
        }
    }
}

// Weight change of a column whose two histories are full: the sum over (t_f in pre, t_n in post) of
// stdp_w(t_n - t_f) in the reference's order (additive_stdp.h:173-196), in FP32.
__device__ __forceinline__ float stdp_column_sum(const StdpDev &d, uint32_t col)
{
    const uint32_t *pre = d.pre_hist + static_cast<size_t>(col) * d.period;
    const uint32_t *post = d.post_hist + static_cast<size_t>(col) * d.period;
    float wj = 0.0f;
    for (uint32_t a = 0; a < d.period; ++a)
    {
        const uint32_t tf = pre[a];
        for (uint32_t b = 0; b < d.period; ++b)
        {
            const uint32_t tn = post[b];
            if (tn < tf) continue;  // term is exactly +0
            const uint32_t diff = tn - tf;
            if (diff < d.table_len) wj = __fadd_rn(wj, d.table[diff]);
        }
    }
    return wj;
}

// Weight update of the columns touched this step whose histories are full: one warp per column
// (warp, warp + n_warps, ...), lane 0 sums the term table in the reference's order.
__device__ __forceinline__ void stdp_modify_range(const StdpDev &d, uint32_t warp, uint32_t n_warps, int lane)
{
    const uint32_t n = *d.touched_count;
    for (uint32_t k = warp; k < n; k += n_warps)
    {
        const uint32_t col = d.touched[k];
        if (d.pre_cnt[col] < d.period || d.post_cnt[col] < d.period) continue;
        float wj = 0.0f;
        if (lane == 0) wj = stdp_column_sum(d, col);
        wj = __shfl_sync(0xffffffffu, wj, 0);
        const long long a = d.col_ptr[col], b = d.col_ptr[col + 1];
        for (long long e = a + lane; e < b; e += 32)
        {
            const uint64_t pos = d.col_pos[e];
            d.w[pos] = __fadd_rn(d.w[pos], wj);
        }
        __syncwarp();
        if (lane == 0)
        {
            d.pre_cnt[col] = 0;
            d.post_cnt[col] = 0;
        }
    }
}

// Append and weight update in one pass, for a rule with one source: that source's spike indexes are
// distinct (a population's spike list), so each column is appended at most once per step and can be
// updated as soon as its own append fills both histories; no touched list is kept. The caller's
// threads are thread, thread + n_threads, ... in whole warps; a warp updates its full columns
// together (lane l of the warp takes synapses l, l + 32, ... of each).
__device__ __forceinline__ void stdp_append_update_range(
    const StdpDev &d, const SpikeSource &src, int both_lists, unsigned long long t, uint32_t thread,
    uint32_t n_threads)
{
    const uint32_t *idx = src.idx;
    const uint32_t cnt = *src.count;
    const int lane = static_cast<int>(thread & 31u);
    const uint32_t tt = static_cast<uint32_t>(t);
    for (uint32_t kb = thread - static_cast<uint32_t>(lane); kb < cnt; kb += n_threads)
    {
        const uint32_t k = kb + static_cast<uint32_t>(lane);
        uint32_t col = 0xFFFFFFFFu;
        bool full = false;
        if (k < cnt)
        {
            col = idx[k];
            if (col < d.n_cols)
            {
                uint32_t c = d.post_cnt[col];
                if (c < d.period)
                {
                    d.post_hist[static_cast<size_t>(col) * d.period + c] = tt;
                    d.post_cnt[col] = ++c;
                }
                uint32_t cp = d.pre_cnt[col];
                if (both_lists && cp < d.period)
                {
                    d.pre_hist[static_cast<size_t>(col) * d.period + cp] = tt;
                    d.pre_cnt[col] = ++cp;
                }
                full = c >= d.period && cp >= d.period;
            }
        }
        uint32_t pending = __ballot_sync(0xffffffffu, full);
        const float mine = full ? stdp_column_sum(d, col) : 0.0f;
        while (pending)
        {
            const int src_lane = __ffs(pending) - 1;
            pending &= pending - 1;
            const uint32_t c = __shfl_sync(0xffffffffu, col, src_lane);
            const float wj = __shfl_sync(0xffffffffu, mine, src_lane);
            const long long a = d.col_ptr[c], b = d.col_ptr[c + 1];
            for (long long e = a + lane; e < b; e += 32)
            {
                const uint64_t pos = d.col_pos[e];
                d.w[pos] = __fadd_rn(d.w[pos], wj);
            }
        }
        if (full)
        {
            d.pre_cnt[col] = 0;
            d.post_cnt[col] = 0;
        }
    }
}

}  // namespace
}  // namespace knp_gb300
