// Gather ("pull") form of a delta projection, used for the steps whose spike count is high.
//
// The scatter kernel costs one global atomic per synaptic event, which limits a step in which a
// large share of the presynaptic neurons fire. For such a step the scatter kernel only records the
// spikes in a bitmap slot; the gather kernel, run at the end of every step for the next step t,
// reads for every delay whose step t - d was recorded the synapses of that delay in the sliced ELL
// layout of kernels.h: each lane owns one target of a slice and sums, down its list, the weights of
// the synapses whose presynaptic bit is set (bitmap staged in shared memory), then adds the sum to
// the target's accumulator; the accumulators are added once to the targets' input-ring slot of step
// t. The sums are the same impacts the scatter would have delivered at step t (delay convention of
// delta_impl.h:78-79), added in another order, which is exact for the FP32 ring (dyadic weights);
// populations with the fixed-point ring never use this form.
#include <cstdint>
#include <type_traits>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>
#include <cub/device/device_select.cuh>
#include <cuda_fp16.h>

#include "kernels.h"
#include "pull_dev.cuh"

namespace knp_gb300
{
namespace
{

__global__ void row_of_kernel(const long long *row_ptr, uint32_t n_rows, uint32_t *row_of)
{
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (uint32_t r = warp; r < n_rows; r += n_warps)
        for (long long e = row_ptr[r] + lane; e < row_ptr[r + 1]; e += 32) row_of[e] = r;
}

// key = (d - 1) * n_post + post, or the sentinel max_delay * n_post for delay 0 (never delivered);
// count[key]++ for the delivered ones.
__global__ void pull_key_kernel(
    uint64_t n, const int32_t *col, const uint8_t *delay, uint32_t n_post, uint32_t max_delay, uint32_t *key,
    uint32_t *val, uint32_t *count)
{
    for (uint64_t e = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        const uint32_t d = delay[e];
        const uint32_t k = d == 0 ? max_delay * n_post : (d - 1) * n_post + static_cast<uint32_t>(col[e]);
        key[e] = k;
        val[e] = static_cast<uint32_t>(e);
        if (d != 0) atomicAdd(count + k, 1u);
    }
}

// One block of kPullWindow threads per (delay, window): order the window's targets by decreasing
// synapse count (ties by target), write perm (sorted position -> target offset), inv (target offset
// -> sorted position) and each slice's longest list.
__global__ void pull_window_kernel(
    const uint32_t *count, uint32_t n_post, uint32_t n_windows, uint8_t *perm, uint8_t *inv, uint32_t *slice_len)
{
    __shared__ uint32_t key[kPullWindow];
    __shared__ uint32_t cnt[kPullWindow];
    const uint32_t dw = blockIdx.x;  // (d - 1) * n_windows + window
    const uint32_t d0 = dw / n_windows, win = dw % n_windows;
    const uint32_t t = threadIdx.x;
    const uint32_t j = win * kPullWindow + t;
    const uint32_t c = j < n_post ? count[static_cast<size_t>(d0) * n_post + j] : 0u;
    cnt[t] = c;
    // Descending by count, then ascending by target: sort (min(c, 2^24 - 1) << 8 | 255 - t) descending.
    key[t] = (min(c, 0xFFFFFFu) << 8) | (kPullWindow - 1 - t);
    __syncthreads();
    // Bitonic sort, descending.
    for (uint32_t size = 2; size <= kPullWindow; size <<= 1)
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1)
        {
            const uint32_t partner = t ^ stride;
            if (partner > t)
            {
                const bool desc = (t & size) == 0;
                const uint32_t a = key[t], b = key[partner];
                if (desc ? a < b : a > b)
                {
                    key[t] = b;
                    key[partner] = a;
                }
            }
            __syncthreads();
        }
    const uint32_t tt = kPullWindow - 1 - (key[t] & 0xFFu);  // target offset at sorted position t
    perm[static_cast<size_t>(dw) * kPullWindow + t] = static_cast<uint8_t>(tt);
    inv[static_cast<size_t>(dw) * kPullWindow + tt] = static_cast<uint8_t>(t);
    // Longest list of each slice (sorted positions [32 s, 32 s + 32)).
    uint32_t m = cnt[tt];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((t & 31) == 0) slice_len[static_cast<size_t>(dw) * kPullSlicesPerWindow + t / 32] = m;
}

__global__ void slice_entries_kernel(const uint32_t *slice_len, uint64_t n, long long *entries)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        entries[i] = static_cast<long long>(slice_len[i]) * kPullSlice;
}

// Places every delivered synapse (sorted by key, so a target's synapses of one delay are
// consecutive from first[key]) at its slice entry.
__global__ void pull_fill_kernel(
    uint64_t n, const uint32_t *keys, const uint32_t *order, const long long *first, const uint8_t *inv,
    const long long *slice_ptr, const uint32_t *row_of, const float *w, bool negate, uint32_t n_post,
    uint32_t n_windows, uint32_t max_delay, uint32_t *packed, float *w_out)
{
    const uint32_t sentinel = max_delay * n_post;
    for (uint64_t p = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; p < n;
         p += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        const uint32_t k = keys[p];
        if (k >= sentinel) continue;
        const uint32_t d0 = k / n_post, j = k % n_post;
        const uint32_t dw = d0 * n_windows + j / kPullWindow;
        const uint32_t pos = inv[static_cast<size_t>(dw) * kPullWindow + j % kPullWindow];
        const size_t q = static_cast<size_t>(dw) * kPullSlicesPerWindow + pos / kPullSlice;
        const long long rank = static_cast<long long>(p) - first[k];
        const long long at = slice_ptr[q] + rank * kPullSlice + (pos % kPullSlice);
        const uint32_t e = order[p];
        packed[at] = row_of[e];
        const float x = w[e];
        w_out[at] = negate ? -x : x;
    }
}

__global__ void float_bits_kernel(const float *w, uint64_t n, uint32_t *bits)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        bits[i] = __float_as_uint(w[i]);
}

// packed[i] |= (position of w[i]'s bit pattern in the ascending table) << 24.
__global__ void dict_pack_kernel(const float *w, uint64_t n, const uint32_t *table, uint32_t n_table, uint32_t *packed)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        const uint32_t b = __float_as_uint(w[i]);
        uint32_t lo = 0, hi = n_table;
        while (lo < hi)
        {
            const uint32_t mid = (lo + hi) >> 1;
            if (table[mid] < b)
                lo = mid + 1;
            else
                hi = mid;
        }
        packed[i] |= lo << 24;
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

template <int kForm>
__global__ void __launch_bounds__(kGatherThreads, 1) gather_kernel(ProjectionDev p, Control *ctl)
{
    pdl_begin();
    extern __shared__ uint4 smem_u4[];
    gather_block<kForm>(p, ctl->step + 1, blockIdx.x, gridDim.x, smem_u4);
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

size_t gather_smem_bytes(const PullDev &p, int grid) { return gather_smem_for(p, static_cast<uint32_t>(grid)); }

void launch_gather(const ProjectionDev &p, Control *ctl, int grid, cudaStream_t s)
{
    const size_t smem = gather_smem_bytes(p.pull, grid);
    if (p.pull.wtab)
        launch_pdl(gather_kernel<kDict>, dim3(grid), dim3(kGatherThreads), smem, s, p, ctl);
    else if (p.pull.w16)
        launch_pdl(gather_kernel<kHalf>, dim3(grid), dim3(kGatherThreads), smem, s, p, ctl);
    else
        launch_pdl(gather_kernel<kFull>, dim3(grid), dim3(kGatherThreads), smem, s, p, ctl);
}

cudaError_t set_gather_smem(size_t bytes)
{
    const int b = static_cast<int>(bytes);
    cudaError_t err = cudaFuncSetAttribute(gather_kernel<kDict>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(gather_kernel<kHalf>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(gather_kernel<kFull>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    return err;
}

// Builds the sliced ELL layout from a projection's CSR: sort synapses by (delay, target), count the
// lists, order each window's targets by list length, size and place the slices, then store the
// weights as FP16 if every one is exactly an FP16 value. Outputs are cudaMalloc'd (the caller owns
// them through `bufs`); temporaries use cudaMallocAsync.
cudaError_t build_pull_layout(
    uint64_t n_syn, uint32_t n_rows, uint32_t n_post, const long long *row_ptr, const int32_t *col, const float *w,
    const uint8_t *delay, bool negate, PullDev &out, PullBuffers &bufs, cudaStream_t s)
{
    const uint32_t D = out.max_delay;
    const uint32_t n_win = (n_post + kPullWindow - 1) / kPullWindow;
    out.n_windows = n_win;
    out.n_post = n_post;
    const uint64_t n_keys = static_cast<uint64_t>(D) * n_post;
    const uint64_t n_dw = static_cast<uint64_t>(D) * n_win;
    const uint64_t n_slices = n_dw * kPullSlicesPerWindow;
    uint32_t *row_of = nullptr, *k_in = nullptr, *k_out = nullptr, *v_in = nullptr, *v_out = nullptr,
             *count = nullptr;
    long long *first = nullptr, *entries = nullptr;
    uint8_t *inv = nullptr;
    unsigned int *flag = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    const size_t bytes = n_syn * sizeof(uint32_t) + 16;
    uint32_t *packed = nullptr, *slice_len = nullptr;
    float *w32 = nullptr;
    uint16_t *w16 = nullptr;
    long long *slice_ptr = nullptr;
    uint8_t *perm = nullptr;
    uint64_t n_entries = 0;
    unsigned int h_flag = 1;
    long long total = 0;
    uint32_t *bits_in = nullptr, *bits_out = nullptr, *uniq = nullptr;
    int64_t *n_uniq = nullptr;
    int64_t h_uniq = 0;
    float *wtab = nullptr;
    cudaError_t err;
#define KNP_TRY(x)                         \
    do                                     \
    {                                      \
        err = (x);                         \
        if (err != cudaSuccess) goto done; \
    } while (0)
    KNP_TRY(cudaMallocAsync(&row_of, bytes, s));
    KNP_TRY(cudaMallocAsync(&k_in, bytes, s));
    KNP_TRY(cudaMallocAsync(&k_out, bytes, s));
    KNP_TRY(cudaMallocAsync(&v_in, bytes, s));
    KNP_TRY(cudaMallocAsync(&v_out, bytes, s));
    KNP_TRY(cudaMallocAsync(&count, (n_keys + 1) * sizeof(uint32_t), s));
    KNP_TRY(cudaMemsetAsync(count, 0, (n_keys + 1) * sizeof(uint32_t), s));
    row_of_kernel<<<152 * 8, 256, 0, s>>>(row_ptr, n_rows, row_of);
    pull_key_kernel<<<grid_for(n_syn), 256, 0, s>>>(n_syn, col, delay, n_post, D, k_in, v_in, count);
    KNP_TRY(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, k_in, k_out, v_in, v_out, static_cast<int64_t>(n_syn),
                                            0, bits_for(n_keys), s));
    KNP_TRY(cudaMallocAsync(&tmp, tmp_bytes, s));
    KNP_TRY(cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, k_in, k_out, v_in, v_out, static_cast<int64_t>(n_syn), 0,
                                            bits_for(n_keys), s));
    KNP_TRY(cudaFreeAsync(tmp, s));
    tmp = nullptr;
    // first[key]: sorted position of the key's first synapse (exclusive scan of the counts).
    KNP_TRY(cudaMallocAsync(&first, (n_keys + 1) * sizeof(long long), s));
    tmp_bytes = 0;
    KNP_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, count, first, static_cast<int64_t>(n_keys + 1), s));
    KNP_TRY(cudaMallocAsync(&tmp, tmp_bytes, s));
    KNP_TRY(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, count, first, static_cast<int64_t>(n_keys + 1), s));
    KNP_TRY(cudaFreeAsync(tmp, s));
    tmp = nullptr;
    // Window orders and slice lengths.
    KNP_TRY(cudaMalloc(&perm, n_dw * kPullWindow + 16));
    KNP_TRY(cudaMallocAsync(&inv, n_dw * kPullWindow + 16, s));
    KNP_TRY(cudaMalloc(&slice_len, n_slices * sizeof(uint32_t) + 16));
    if (n_dw > 0)
        pull_window_kernel<<<static_cast<unsigned>(n_dw), kPullWindow, 0, s>>>(count, n_post, n_win, perm, inv,
                                                                               slice_len);
    KNP_TRY(cudaGetLastError());
    // Slice offsets: exclusive scan of 32 x length.
    KNP_TRY(cudaMallocAsync(&entries, (n_slices + 1) * sizeof(long long), s));
    KNP_TRY(cudaMemsetAsync(entries, 0, (n_slices + 1) * sizeof(long long), s));
    slice_entries_kernel<<<grid_for(n_slices), 256, 0, s>>>(slice_len, n_slices, entries);
    KNP_TRY(cudaMalloc(&slice_ptr, (n_slices + 1) * sizeof(long long)));
    tmp_bytes = 0;
    KNP_TRY(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, entries, slice_ptr, static_cast<int64_t>(n_slices + 1),
                                          s));
    KNP_TRY(cudaMallocAsync(&tmp, tmp_bytes, s));
    KNP_TRY(cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, entries, slice_ptr, static_cast<int64_t>(n_slices + 1), s));
    KNP_TRY(cudaFreeAsync(tmp, s));
    tmp = nullptr;
    KNP_TRY(cudaMemcpyAsync(&total, slice_ptr + n_slices, sizeof(long long), cudaMemcpyDeviceToHost, s));
    KNP_TRY(cudaStreamSynchronize(s));
    n_entries = static_cast<uint64_t>(total);
    // Entries: zero (padding: presynaptic 0, weight 0), then every delivered synapse in place.
    KNP_TRY(cudaMalloc(&packed, n_entries * sizeof(uint32_t) + 16));
    KNP_TRY(cudaMalloc(&w32, n_entries * sizeof(float) + 16));
    KNP_TRY(cudaMemsetAsync(packed, 0, n_entries * sizeof(uint32_t) + 16, s));
    KNP_TRY(cudaMemsetAsync(w32, 0, n_entries * sizeof(float) + 16, s));
    pull_fill_kernel<<<grid_for(n_syn), 256, 0, s>>>(n_syn, k_out, v_out, first, inv, slice_ptr, row_of, w, negate,
                                                    n_post, n_win, D, packed, w32);
    KNP_TRY(cudaGetLastError());
    // The sort and placement temporaries are no longer needed.
    for (void **t : {reinterpret_cast<void **>(&row_of), reinterpret_cast<void **>(&k_in),
                     reinterpret_cast<void **>(&k_out), reinterpret_cast<void **>(&v_in),
                     reinterpret_cast<void **>(&v_out), reinterpret_cast<void **>(&count),
                     reinterpret_cast<void **>(&first), reinterpret_cast<void **>(&entries),
                     reinterpret_cast<void **>(&inv)})
    {
        KNP_TRY(cudaFreeAsync(*t, s));
        *t = nullptr;
    }
    // Dictionary form: at most 256 distinct weight bit patterns (the padding's +0.0, the smallest
    // pattern, becomes entry 0) and presynaptic indexes below 2^24.
    if (n_rows <= (1u << 24) && n_entries > 0)
    {
        KNP_TRY(cudaMallocAsync(&bits_in, n_entries * sizeof(uint32_t), s));
        KNP_TRY(cudaMallocAsync(&bits_out, n_entries * sizeof(uint32_t), s));
        KNP_TRY(cudaMallocAsync(&uniq, n_entries * sizeof(uint32_t), s));
        KNP_TRY(cudaMallocAsync(&n_uniq, sizeof(int64_t), s));
        float_bits_kernel<<<grid_for(n_entries), 256, 0, s>>>(w32, n_entries, bits_in);
        tmp_bytes = 0;
        KNP_TRY(cub::DeviceRadixSort::SortKeys(nullptr, tmp_bytes, bits_in, bits_out, static_cast<int64_t>(n_entries), 0,
                                               32, s));
        KNP_TRY(cudaMallocAsync(&tmp, tmp_bytes, s));
        KNP_TRY(cub::DeviceRadixSort::SortKeys(tmp, tmp_bytes, bits_in, bits_out, static_cast<int64_t>(n_entries), 0,
                                               32, s));
        KNP_TRY(cudaFreeAsync(tmp, s));
        tmp = nullptr;
        tmp_bytes = 0;
        KNP_TRY(cub::DeviceSelect::Unique(nullptr, tmp_bytes, bits_out, uniq, n_uniq, static_cast<int64_t>(n_entries),
                                          s));
        KNP_TRY(cudaMallocAsync(&tmp, tmp_bytes, s));
        KNP_TRY(cub::DeviceSelect::Unique(tmp, tmp_bytes, bits_out, uniq, n_uniq, static_cast<int64_t>(n_entries), s));
        KNP_TRY(cudaFreeAsync(tmp, s));
        tmp = nullptr;
        KNP_TRY(cudaMemcpyAsync(&h_uniq, n_uniq, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        KNP_TRY(cudaStreamSynchronize(s));
        if (h_uniq > 0 && h_uniq <= 256)
        {
            KNP_TRY(cudaMalloc(&wtab, 256 * sizeof(float)));
            KNP_TRY(cudaMemsetAsync(wtab, 0, 256 * sizeof(float), s));
            KNP_TRY(cudaMemcpyAsync(wtab, uniq, static_cast<size_t>(h_uniq) * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                                    s));
            dict_pack_kernel<<<grid_for(n_entries), 256, 0, s>>>(w32, n_entries, uniq, static_cast<uint32_t>(h_uniq),
                                                                packed);
            KNP_TRY(cudaGetLastError());
            KNP_TRY(cudaStreamSynchronize(s));
            cudaFree(w32);
            w32 = nullptr;
        }
    }
    // Lossless 16-bit weights when every weight is exactly an FP16 value.
    if (w32)
    {
        KNP_TRY(cudaMallocAsync(&flag, sizeof(unsigned int), s));
        KNP_TRY(cudaMemsetAsync(flag, 0, sizeof(unsigned int), s));
        half_exact_kernel<<<grid_for(n_entries), 256, 0, s>>>(w32, n_entries, flag);
        KNP_TRY(cudaMemcpyAsync(&h_flag, flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, s));
        KNP_TRY(cudaStreamSynchronize(s));
        if (h_flag == 0)
        {
            KNP_TRY(cudaMalloc(&w16, n_entries * sizeof(uint16_t) + 16));
            to_half_kernel<<<grid_for(n_entries), 256, 0, s>>>(w32, n_entries, w16);
            KNP_TRY(cudaGetLastError());
            KNP_TRY(cudaStreamSynchronize(s));
            cudaFree(w32);
            w32 = nullptr;
        }
    }
    out.slice_ptr = slice_ptr;
    out.slice_len = slice_len;
    out.perm = perm;
    out.packed = packed;
    out.wtab = wtab;
    out.n_tab = wtab ? static_cast<uint32_t>(h_uniq) : 0u;
    out.w = w32;
    out.w16 = w16;
    out.padded_entries = n_entries;
    bufs.ptr[0] = packed;
    bufs.bytes[0] = n_entries * sizeof(uint32_t);
    bufs.ptr[1] = w32;
    bufs.bytes[1] = w32 ? n_entries * sizeof(float) : 0;
    bufs.ptr[2] = w16;
    bufs.bytes[2] = w16 ? n_entries * sizeof(uint16_t) : 0;
    bufs.ptr[3] = slice_ptr;
    bufs.bytes[3] = (n_slices + 1) * sizeof(long long);
    bufs.ptr[4] = slice_len;
    bufs.bytes[4] = n_slices * sizeof(uint32_t);
    bufs.ptr[5] = perm;
    bufs.bytes[5] = n_dw * kPullWindow;
    bufs.ptr[6] = wtab;
    bufs.bytes[6] = wtab ? 256 * sizeof(float) : 0;
    packed = nullptr;
    w32 = nullptr;
    w16 = nullptr;
    slice_ptr = nullptr;
    slice_len = nullptr;
    perm = nullptr;
    wtab = nullptr;
done:
    if (bits_in) cudaFreeAsync(bits_in, s);
    if (bits_out) cudaFreeAsync(bits_out, s);
    if (uniq) cudaFreeAsync(uniq, s);
    if (n_uniq) cudaFreeAsync(n_uniq, s);
    if (flag) cudaFreeAsync(flag, s);
    if (tmp) cudaFreeAsync(tmp, s);
    if (row_of) cudaFreeAsync(row_of, s);
    if (k_in) cudaFreeAsync(k_in, s);
    if (k_out) cudaFreeAsync(k_out, s);
    if (v_in) cudaFreeAsync(v_in, s);
    if (v_out) cudaFreeAsync(v_out, s);
    if (count) cudaFreeAsync(count, s);
    if (first) cudaFreeAsync(first, s);
    if (entries) cudaFreeAsync(entries, s);
    if (inv) cudaFreeAsync(inv, s);
    cudaStreamSynchronize(s);
    // On failure, buffers not handed to the caller are released.
    if (packed) cudaFree(packed);
    if (w32) cudaFree(w32);
    if (w16) cudaFree(w16);
    if (slice_ptr) cudaFree(slice_ptr);
    if (slice_len) cudaFree(slice_len);
    if (perm) cudaFree(perm);
    if (wtab) cudaFree(wtab);
#undef KNP_TRY
    return err;
}

}  // namespace knp_gb300
