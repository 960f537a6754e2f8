// Gather ("pull") form of a delta projection, used for the steps whose spike count is high.
//
// The scatter kernel costs one global atomic per synaptic event, which limits a step in which a
// large share of the presynaptic neurons fire. For such a step the scatter kernel only records the
// spikes in a bitmap slot; the gather kernel, run at the end of every step for the next step t,
// walks the synapses sorted by (delay d, postsynaptic neuron), and for every delay whose step t - d
// was recorded stages that bitmap in shared memory and adds the weights of the synapses whose
// presynaptic bit is set. Contributions are reduced per target with a warp-segmented scan and one
// shared-memory atomic per run of equal targets, then added once to the target's input-ring slot of
// step t. The sums are the same impacts the scatter would have delivered at step t (delay
// convention of delta_impl.h:78-79), added in another order, which is exact for the FP32 ring
// (dyadic weights); populations with the fixed-point ring never use this form.
#include <cstdint>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cuda_fp16.h>

#include "kernels.h"

namespace knp_gb300
{
namespace
{

constexpr int kGatherThreads = 1024;
constexpr int kLaneRun = 8;   // consecutive synapses per lane (segments are padded to multiples of it)
constexpr int kUnroll = 2;    // groups of kLaneRun synapses in flight per lane

__global__ void row_of_kernel(const long long *row_ptr, uint32_t n_rows, uint32_t *row_of)
{
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (uint32_t r = warp; r < n_rows; r += n_warps)
        for (long long e = row_ptr[r] + lane; e < row_ptr[r + 1]; e += 32) row_of[e] = r;
}

__global__ void pull_key_kernel(
    uint64_t n, const int32_t *col, const uint8_t *delay, uint32_t n_post, uint32_t max_delay, uint32_t *key,
    uint32_t *val)
{
    for (uint64_t e = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        const uint32_t d = delay[e];
        // Delay-0 synapses never deliver; they sort after every segment.
        key[e] = d == 0 ? max_delay * n_post : (d - 1) * n_post + static_cast<uint32_t>(col[e]);
        val[e] = static_cast<uint32_t>(e);
    }
}

// seg[i] for i = (d - 1) * n_tiles + tile: first sorted position whose key >= (d - 1) * n_post + tile * kPullTile.
__global__ void pull_seg_kernel(
    const uint32_t *keys, uint64_t n, uint32_t n_post, uint32_t n_tiles, uint32_t max_delay, long long *seg)
{
    const uint64_t total = static_cast<uint64_t>(max_delay) * n_tiles;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i <= total;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        uint64_t target;
        if (i == total)
            target = static_cast<uint64_t>(max_delay) * n_post;
        else
            target = (i / n_tiles) * static_cast<uint64_t>(n_post) + (i % n_tiles) * kPullTile;
        uint64_t lo = 0, hi = n;
        while (lo < hi)
        {
            const uint64_t mid = (lo + hi) >> 1;
            if (keys[mid] < target)
                lo = mid + 1;
            else
                hi = mid;
        }
        seg[i] = static_cast<long long>(lo);
    }
}

// One warp per segment: copy the segment's synapses (sorted positions [seg[s], seg[s+1])) to
// padded positions [pseg[s], pseg[s+1]) as packed (pre << 9 | post mod 512) + weight, and fill the
// padding (up to 7 entries, so that every segment starts on a 32-byte boundary) with key 0 / weight 0.
__global__ void pull_fill_kernel(
    uint64_t n_seg, const long long *seg, const long long *pseg, const uint32_t *order, const uint32_t *row_of,
    const int32_t *col, const float *w, bool negate, uint32_t *packed, float *w_out)
{
    const uint64_t warp = (blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x) >> 5;
    const uint64_t n_warps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (uint64_t sg = warp; sg < n_seg; sg += n_warps)
    {
        const long long a = seg[sg], b = seg[sg + 1], pa = pseg[sg], pb = pseg[sg + 1];
        for (long long i = lane; i < pb - pa; i += 32)
        {
            if (i < b - a)
            {
                const uint32_t e = order[a + i];
                packed[pa + i] = (row_of[e] << kPullTileBits) | (static_cast<uint32_t>(col[e]) & (kPullTile - 1));
                const float x = w[e];
                w_out[pa + i] = negate ? -x : x;
            }
            else
            {
                packed[pa + i] = 0u;
                w_out[pa + i] = 0.0f;
            }
        }
    }
}

// flag |= 1 if some weight is not exactly an FP16 value.
__global__ void half_exact_kernel(const float *w, uint64_t n, unsigned int *flag)
{
    bool bad = false;
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        bad = bad || !(__half2float(__float2half_rn(w[i])) == w[i]);
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1u);
}

__global__ void to_half_kernel(const float *w, uint64_t n, uint16_t *out)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        out[i] = __half_as_ushort(__float2half_rn(w[i]));
}

__device__ __forceinline__ void reduce_runs(uint32_t jl, float val, float *acc)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t prev = __shfl_up_sync(full, jl, 1);
    const bool head = lane == 0 || jl != prev;
    const unsigned hm = __ballot_sync(full, head);
    const int my_head = 31 - __clz(hm & (full >> (31 - lane)));
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const float v = __shfl_up_sync(full, val, o);
        if (lane - o >= my_head) val = __fadd_rn(val, v);
    }
    const bool tail = lane == 31 || ((hm >> (lane + 1)) & 1u);
    if (tail && jl != 0xFFFFFFFFu && val != 0.0f) atomicAdd(acc + jl, val);
}

// kHalf: weights stored as FP16 (exact); one 16-byte load gives a lane's 8 weights.
template <bool kHalf>
__global__ void __launch_bounds__(kGatherThreads, 1) gather_kernel(ProjectionDev p, Control *ctl)
{
    extern __shared__ uint4 smem_u4[];
    const PullDev &g = p.pull;
    uint32_t *bm = reinterpret_cast<uint32_t *>(smem_u4);
    float *acc = reinterpret_cast<float *>(bm + g.words);
    const uint32_t G = gridDim.x;
    const uint32_t t0 = static_cast<uint32_t>(static_cast<uint64_t>(blockIdx.x) * g.n_tiles / G);
    const uint32_t t1 = static_cast<uint32_t>(static_cast<uint64_t>(blockIdx.x + 1) * g.n_tiles / G);
    const uint32_t n_acc = (t1 - t0) * kPullTile;
    const unsigned long long tn = ctl->step + 1;  // the step whose input this gather completes
    const int lane = threadIdx.x & 31;
    const uint32_t warp_base = threadIdx.x & ~31u;

    bool any = false;
    for (uint32_t d = 1; d <= g.max_delay && d <= tn; ++d)
    {
        const unsigned long long s = tn - d;
        const uint32_t sl = static_cast<uint32_t>(s % g.hist_slots);
        if (!g.pulled[sl]) continue;
        if (!any)
        {
            for (uint32_t i = threadIdx.x; i < n_acc; i += blockDim.x) acc[i] = 0.0f;
            any = true;
        }
        __syncthreads();  // the previous bitmap is no longer read
        const uint4 *src = reinterpret_cast<const uint4 *>(g.bitmap + static_cast<size_t>(sl) * g.words);
        for (uint32_t i = threadIdx.x; i < g.words / 4; i += blockDim.x) smem_u4[i] = src[i];
        __syncthreads();
        for (uint32_t tile = t0; tile < t1; ++tile)
        {
            const size_t si = static_cast<size_t>(d - 1) * g.n_tiles + tile;
            // Segments start and end on 8-entry boundaries: a lane takes 8 consecutive synapses per
            // group (two 16-byte loads of keys; one of FP16 or two of FP32 weights), two groups in
            // flight. Padding entries (and lanes past the segment) are key 0 / weight 0: presynaptic
            // neuron 0, target 0, contributing nothing.
            const long long oa = g.seg_ptr[si] / kLaneRun, ob = g.seg_ptr[si + 1] / kLaneRun;
            float *acc_t = acc + static_cast<size_t>(tile - t0) * kPullTile;
            const uint4 *pk = reinterpret_cast<const uint4 *>(g.packed);
            const float4 *pw = reinterpret_cast<const float4 *>(g.w);
            const uint4 *ph = reinterpret_cast<const uint4 *>(g.w16);
            for (long long base = oa + warp_base; base < ob; base += static_cast<long long>(blockDim.x) * kUnroll)
            {
                uint4 key[kUnroll][2];
                float4 w[kUnroll][2];
#pragma unroll
                for (int u = 0; u < kUnroll; ++u)
                {
                    const long long o = base + static_cast<long long>(u) * blockDim.x + lane;
                    key[u][0] = key[u][1] = make_uint4(0u, 0u, 0u, 0u);
                    w[u][0] = w[u][1] = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (o < ob)
                    {
                        key[u][0] = __ldcs(pk + 2 * o);
                        key[u][1] = __ldcs(pk + 2 * o + 1);
                        if (kHalf)
                        {
                            const uint4 h = __ldcs(ph + o);
                            const __half2 *h2 = reinterpret_cast<const __half2 *>(&h);
                            const float2 a = __half22float2(h2[0]), b = __half22float2(h2[1]);
                            const float2 c = __half22float2(h2[2]), e = __half22float2(h2[3]);
                            w[u][0] = make_float4(a.x, a.y, b.x, b.y);
                            w[u][1] = make_float4(c.x, c.y, e.x, e.y);
                        }
                        else
                        {
                            w[u][0] = __ldcs(pw + 2 * o);
                            w[u][1] = __ldcs(pw + 2 * o + 1);
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < kUnroll; ++u)
                {
                    // Runs of equal targets inside the lane's 8 entries: every run but the last is
                    // added at once; the last joins the warp-wide merge across lanes.
                    const uint32_t kk[8] = {key[u][0].x, key[u][0].y, key[u][0].z, key[u][0].w,
                                            key[u][1].x, key[u][1].y, key[u][1].z, key[u][1].w};
                    const float ww[8] = {w[u][0].x, w[u][0].y, w[u][0].z, w[u][0].w,
                                         w[u][1].x, w[u][1].y, w[u][1].z, w[u][1].w};
                    uint32_t cur = kk[0] & (kPullTile - 1);
                    float sum = 0.0f;
#pragma unroll
                    for (int i = 0; i < 8; ++i)
                    {
                        const uint32_t pre = kk[i] >> kPullTileBits;
                        const uint32_t jl = kk[i] & (kPullTile - 1);
                        const float v = ((bm[pre >> 5] >> (pre & 31)) & 1u) ? ww[i] : 0.0f;
                        if (jl != cur)
                        {
                            if (sum != 0.0f) atomicAdd(acc_t + cur, sum);
                            cur = jl;
                            sum = v;
                        }
                        else
                        {
                            sum = __fadd_rn(sum, v);
                        }
                    }
                    reduce_runs(cur, sum, acc_t);
                }
            }
        }
    }
    __syncthreads();
    if (any)
    {
        const uint32_t slot = static_cast<uint32_t>(tn % p.ring.slots);
        float *ring = p.ring.v32 + static_cast<size_t>(slot) * p.ring.pitch;
        for (uint32_t i = threadIdx.x; i < n_acc; i += blockDim.x)
        {
            const uint32_t j = t0 * kPullTile + i;
            if (j < g.n_post && acc[i] != 0.0f) ring[j] = __fadd_rn(ring[j], acc[i]);
        }
    }
    // Clear the bitmap slot that the scatter kernel of step tn will fill; it holds step
    // tn - hist_slots, which no gather reads any more.
    const uint32_t sl_next = static_cast<uint32_t>(tn % g.hist_slots);
    uint32_t *dst = g.bitmap + static_cast<size_t>(sl_next) * g.words;
    const uint32_t w0 = static_cast<uint32_t>(static_cast<uint64_t>(blockIdx.x) * g.words / G);
    const uint32_t w1 = static_cast<uint32_t>(static_cast<uint64_t>(blockIdx.x + 1) * g.words / G);
    for (uint32_t i = w0 + threadIdx.x; i < w1; i += blockDim.x) dst[i] = 0u;
}

int grid_for(uint64_t n)
{
    const uint64_t b = (n + 255) / 256;
    return static_cast<int>(b < 152ull * 16 ? (b ? b : 1) : 152ull * 16);
}

int bits_for(uint64_t max_key)
{
    int bits = 1;
    while (bits < 32 && (1ull << bits) <= max_key) ++bits;
    return bits;
}

}  // namespace

size_t gather_smem_bytes(const PullDev &p, int grid)
{
    const uint64_t tiles_per_block = (p.n_tiles + grid - 1) / grid;
    return static_cast<size_t>(p.words) * 4 + tiles_per_block * kPullTile * 4;
}

void launch_gather(const ProjectionDev &p, Control *ctl, int grid, cudaStream_t s)
{
    const size_t smem = gather_smem_bytes(p.pull, grid);
    if (p.pull.w16)
        gather_kernel<true><<<grid, kGatherThreads, smem, s>>>(p, ctl);
    else
        gather_kernel<false><<<grid, kGatherThreads, smem, s>>>(p, ctl);
}

cudaError_t set_gather_smem(size_t bytes)
{
    cudaError_t err =
        cudaFuncSetAttribute(gather_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes));
    if (err != cudaSuccess) return err;
    return cudaFuncSetAttribute(gather_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(bytes));
}

// Builds the sorted (delay, postsynaptic) layout from a projection's CSR. Allocates the outputs
// with cudaMalloc (the caller owns them) and its temporaries with cudaMallocAsync.
cudaError_t build_pull_layout(
    uint64_t n_syn, uint32_t n_rows, uint32_t n_post, const long long *row_ptr, const int32_t *col, const float *w,
    const uint8_t *delay, bool negate, PullDev &out, uint32_t **packed_out, float **w_out, uint16_t **w16_out,
    long long **seg_out, cudaStream_t s)
{
    *w16_out = nullptr;
    unsigned int *flag = nullptr;
    const uint32_t D = out.max_delay;
    const uint32_t n_tiles = (n_post + kPullTile - 1) / kPullTile;
    out.n_tiles = n_tiles;
    out.n_post = n_post;
    uint32_t *row_of = nullptr, *k_in = nullptr, *k_out = nullptr, *v_in = nullptr, *v_out = nullptr;
    long long *seg_raw = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    const size_t bytes = n_syn * sizeof(uint32_t) + 16;
    cudaError_t err;
#define KNP_TRY(x)                     \
    do                                 \
    {                                  \
        err = (x);                     \
        if (err != cudaSuccess) goto done; \
    } while (0)
    KNP_TRY(cudaMallocAsync(&row_of, bytes, s));
    KNP_TRY(cudaMallocAsync(&k_in, bytes, s));
    KNP_TRY(cudaMallocAsync(&k_out, bytes, s));
    KNP_TRY(cudaMallocAsync(&v_in, bytes, s));
    KNP_TRY(cudaMallocAsync(&v_out, bytes, s));
    row_of_kernel<<<152 * 8, 256, 0, s>>>(row_ptr, n_rows, row_of);
    pull_key_kernel<<<grid_for(n_syn), 256, 0, s>>>(n_syn, col, delay, n_post, D, k_in, v_in);
    {
        const int bits = bits_for(static_cast<uint64_t>(D) * n_post);
        KNP_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, k_in, k_out, v_in, v_out,
                                                static_cast<int64_t>(n_syn), 0, bits, s));
        KNP_TRY(cudaMallocAsync(&tmp, tmp_bytes, s));
        KNP_TRY(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k_in, k_out, v_in, v_out, static_cast<int64_t>(n_syn),
                                                0, bits, s));
    }
    KNP_TRY(cudaMalloc(seg_out, (static_cast<size_t>(D) * n_tiles + 1) * sizeof(long long)));
    KNP_TRY(cudaMallocAsync(&seg_raw, (static_cast<size_t>(D) * n_tiles + 1) * sizeof(long long), s));
    pull_seg_kernel<<<grid_for(static_cast<uint64_t>(D) * n_tiles + 1), 256, 0, s>>>(k_out, n_syn, n_post, n_tiles, D,
                                                                                   seg_raw);
    KNP_TRY(cudaGetLastError());
    KNP_TRY(cudaStreamSynchronize(s));
    {
        // Pad every segment to a multiple of 8 entries (32-byte aligned starts for vector loads).
        const size_t n_seg = static_cast<size_t>(D) * n_tiles;
        std::vector<long long> raw(n_seg + 1), pad(n_seg + 1, 0);
        err = cudaMemcpy(raw.data(), seg_raw, raw.size() * sizeof(long long), cudaMemcpyDeviceToHost);
        if (err != cudaSuccess) goto done;
        for (size_t i = 0; i < n_seg; ++i)
            pad[i + 1] = pad[i] + ((raw[i + 1] - raw[i] + kLaneRun - 1) / kLaneRun) * kLaneRun;
        err = cudaMemcpy(*seg_out, pad.data(), pad.size() * sizeof(long long), cudaMemcpyHostToDevice);
        if (err != cudaSuccess) goto done;
        const size_t padded = static_cast<size_t>(pad[n_seg]) * sizeof(uint32_t) + 16;
        err = cudaMalloc(packed_out, padded);
        if (err != cudaSuccess) goto done;
        err = cudaMalloc(w_out, padded);
        if (err != cudaSuccess) goto done;
        pull_fill_kernel<<<152 * 8, 256, 0, s>>>(n_seg, seg_raw, *seg_out, v_out, row_of, col, w, negate, *packed_out,
                                                 *w_out);
        out.padded_entries = static_cast<uint64_t>(pad[n_seg]);
    }
    KNP_TRY(cudaGetLastError());
    KNP_TRY(cudaStreamSynchronize(s));
    out.seg_ptr = *seg_out;
    out.packed = *packed_out;
    out.w = *w_out;
    out.w16 = nullptr;
    {
        // Lossless 16-bit weights when every weight is exactly an FP16 value (6 instead of 8 bytes
        // per synapse streamed by the gather).
        const uint64_t n_pad = out.padded_entries;
        KNP_TRY(cudaMallocAsync(&flag, sizeof(unsigned int), s));
        KNP_TRY(cudaMemsetAsync(flag, 0, sizeof(unsigned int), s));
        half_exact_kernel<<<grid_for(n_pad), 256, 0, s>>>(*w_out, n_pad, flag);
        unsigned int h_flag = 1;
        KNP_TRY(cudaMemcpyAsync(&h_flag, flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
        KNP_TRY(cudaStreamSynchronize(s));
        if (h_flag == 0)
        {
            KNP_TRY(cudaMalloc(w16_out, n_pad * sizeof(uint16_t) + 16));
            to_half_kernel<<<grid_for(n_pad), 256, 0, s>>>(*w_out, n_pad, *w16_out);
            KNP_TRY(cudaGetLastError());
            KNP_TRY(cudaStreamSynchronize(s));
            cudaFree(*w_out);
            *w_out = nullptr;
            out.w = nullptr;
            out.w16 = *w16_out;
        }
    }
done:
    if (flag) cudaFreeAsync(flag, s);
    if (seg_raw) cudaFreeAsync(seg_raw, s);
    if (tmp) cudaFreeAsync(tmp, s);
    if (row_of) cudaFreeAsync(row_of, s);
    if (k_in) cudaFreeAsync(k_in, s);
    if (k_out) cudaFreeAsync(k_out, s);
    if (v_in) cudaFreeAsync(v_in, s);
    if (v_out) cudaFreeAsync(v_out, s);
    cudaStreamSynchronize(s);
#undef KNP_TRY
    return err;
}

}  // namespace knp_gb300
