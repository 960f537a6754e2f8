// Network construction on the device: presynaptic-major CSR build (stable radix sort of synapse
// indexes by presynaptic neuron, so a row keeps the reference's synapse order) and the counter-based
// generators shared with knp_gb300/network.py (fixed fan-in projection, Bernoulli spike schedule).
#include <algorithm>
#include <cstdint>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "kernels.h"

namespace knp_gb300
{
namespace
{

__global__ void iota_kernel(uint32_t *out, uint64_t n)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        out[i] = static_cast<uint32_t>(i);
}

// row_ptr[r] = first position whose sorted key is >= r.
__global__ void row_ptr_kernel(const uint32_t *sorted_keys, uint64_t n, uint32_t n_rows, long long *row_ptr)
{
    for (uint64_t r = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; r <= n_rows;
         r += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        uint64_t lo = 0, hi = n;
        while (lo < hi)
        {
            const uint64_t mid = (lo + hi) >> 1;
            if (sorted_keys[mid] < r)
                lo = mid + 1;
            else
                hi = mid;
        }
        row_ptr[r] = static_cast<long long>(lo);
    }
}

__global__ void gather_kernel(
    uint64_t n, const uint32_t *perm, const uint32_t *post, const float *w, const uint32_t *delay, const uint8_t *type,
    int32_t *col_out, float *w_out, uint8_t *delay_out, uint8_t *type_out)
{
    for (uint64_t e = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        const uint32_t i = perm[e];
        col_out[e] = static_cast<int32_t>(post[i]);
        w_out[e] = w[i];
        const uint32_t d = delay[i];
        delay_out[e] = static_cast<uint8_t>(d > 255u ? 255u : d);
        if (type_out) type_out[e] = type[i];
    }
}

// Presynaptic and postsynaptic neuron of generated synapse i (synapse_generators.h:59-69 all_to_all,
// :93-120 aligned, :139-154 exclusive, :172-178 one_to_one, :259-300 FixedProbability,
// :352-388 FixedNumberPost, :409-445 FixedNumberPre).
__device__ __forceinline__ void gen_pair(const GenSpec &g, uint64_t i, uint32_t &pre, uint32_t &post)
{
    switch (g.kind)
    {
        case kGenAllToAll:
            pre = static_cast<uint32_t>(i % g.n_pre);
            post = static_cast<uint32_t>(i / g.n_pre);
            break;
        case kGenAligned:
            if (g.n_pre >= g.n_post)
            {
                pre = static_cast<uint32_t>(i);
                post = static_cast<uint32_t>(i / (g.n_pre / g.n_post));
            }
            else
            {
                post = static_cast<uint32_t>(i);
                pre = static_cast<uint32_t>(i / (g.n_post / g.n_pre));
            }
            break;
        case kGenExclusive:
        {
            pre = static_cast<uint32_t>(i / (g.n_pre - 1));
            const uint32_t to = static_cast<uint32_t>(i % (g.n_pre - 1));
            post = to >= pre ? to + 1 : to;
            break;
        }
        case kGenOneToOne:
            pre = post = static_cast<uint32_t>(i);
            break;
        case kGenFixedProbability:
        {
            const unsigned long long c = g.cand[i];
            pre = static_cast<uint32_t>(c % g.n_pre);
            post = static_cast<uint32_t>(c / g.n_pre);
            break;
        }
        case kGenFixedNumberPost:
            pre = static_cast<uint32_t>(i % g.n_pre);
            post = static_cast<uint32_t>(uniform_int(g.key_post, i, 0, static_cast<long long>(g.n_post) - 1));
            break;
        default:  // kGenFixedNumberPre
            pre = static_cast<uint32_t>(uniform_int(g.key_pre, i, 0, static_cast<long long>(g.n_pre) - 1));
            post = static_cast<uint32_t>(i % g.n_post);
            break;
    }
}

__global__ void gen_keys_kernel(GenSpec g, uint64_t n, uint32_t *pre_out)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        uint32_t pre, post;
        gen_pair(g, i, pre, post);
        pre_out[i] = pre;
    }
}

__global__ void gen_gather_kernel(GenSpec g, uint64_t n, const uint32_t *perm, int32_t *col_out, float *w_out,
                                  uint8_t *delay_out)
{
    for (uint64_t e = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; e < n;
         e += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        const uint64_t i = perm[e];
        uint32_t pre, post;
        gen_pair(g, i, pre, post);
        col_out[e] = static_cast<int32_t>(post);
        w_out[e] = static_cast<float>(uniform_int(g.key_w, i, g.k_lo, g.k_hi)) * (1.0f / 256.0f);
        delay_out[e] = static_cast<uint8_t>(uniform_int(g.key_d, i, g.d_lo, g.d_hi));
    }
}

constexpr uint32_t kCandChunk = 8192;  // candidate pairs per chunk

// counts[c] = kept candidates of chunk c; one block per chunk (grid-strided).
__global__ void cand_count_kernel(uint64_t n_cand, unsigned long long threshold, unsigned long long key,
                                  uint64_t chunks, unsigned long long *counts)
{
    __shared__ unsigned int tot;
    for (uint64_t c = blockIdx.x; c < chunks; c += gridDim.x)
    {
        if (threadIdx.x == 0) tot = 0;
        __syncthreads();
        unsigned int mine = 0;
        const uint64_t lo = c * kCandChunk, hi = min(n_cand, lo + kCandChunk);
        for (uint64_t x = lo + threadIdx.x; x < hi; x += blockDim.x) mine += (rand64(key, x) >> 11) < threshold;
        atomicAdd(&tot, mine);
        __syncthreads();
        if (threadIdx.x == 0) counts[c] = tot;
        __syncthreads();
    }
}

// Writes chunk c's kept candidates in ascending order from offs[c] (exclusive prefix of counts).
__global__ void cand_write_kernel(uint64_t n_cand, unsigned long long threshold, unsigned long long key,
                                  uint64_t chunks, const unsigned long long *offs, unsigned long long *out)
{
    __shared__ unsigned int warp_tot[32];
    __shared__ unsigned long long base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
    for (uint64_t c = blockIdx.x; c < chunks; c += gridDim.x)
    {
        if (threadIdx.x == 0) base = offs[c];
        __syncthreads();
        const uint64_t lo = c * kCandChunk, hi = min(n_cand, lo + kCandChunk);
        for (uint64_t x0 = lo; x0 < hi; x0 += blockDim.x)
        {
            const uint64_t x = x0 + threadIdx.x;
            const bool hit = x < hi && (rand64(key, x) >> 11) < threshold;
            const unsigned int b = __ballot_sync(0xffffffffu, hit);
            if (lane == 0) warp_tot[warp] = __popc(b);
            __syncthreads();
            unsigned int before = 0, all = 0;
            for (int w = 0; w < n_warps; ++w)
            {
                if (w < warp) before += warp_tot[w];
                all += warp_tot[w];
            }
            if (hit) out[base + before + __popc(b & ((1u << lane) - 1u))] = x;
            __syncthreads();
            if (threadIdx.x == 0) base += all;
            __syncthreads();
        }
    }
}

constexpr int kSchedChunk = 4096;  // sources per block

// counts[t * chunks + c] = spikes of step t among sources [c * kSchedChunk, ...).
__global__ void bernoulli_count_kernel(
    uint32_t n_sources, unsigned long long threshold, unsigned long long key, unsigned long long first_step,
    uint32_t chunks, long long *counts)
{
    const uint64_t t = blockIdx.y;
    const uint32_t c = blockIdx.x;
    __shared__ uint32_t tot;
    if (threadIdx.x == 0) tot = 0;
    __syncthreads();
    uint32_t mine = 0;
    for (uint32_t s = c * kSchedChunk + threadIdx.x; s < n_sources && s < (c + 1) * kSchedChunk; s += blockDim.x)
    {
        const unsigned long long ctr = (first_step + t) * static_cast<unsigned long long>(n_sources) + s;
        mine += (rand64(key, ctr) >> 11) < threshold;
    }
    atomicAdd(&tot, mine);
    __syncthreads();
    if (threadIdx.x == 0) counts[t * chunks + c] = tot;
}

// Writes the spikes of (step t, chunk c) in ascending source order from offset offs[t * chunks + c].
__global__ void bernoulli_write_kernel(
    uint32_t n_sources, unsigned long long threshold, unsigned long long key, unsigned long long first_step,
    uint32_t chunks, const long long *offs, uint32_t *idx)
{
    const uint64_t t = blockIdx.y;
    const uint32_t c = blockIdx.x;
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    const uint32_t lo = c * kSchedChunk;
    for (uint32_t s0 = lo; s0 < n_sources && s0 < lo + kSchedChunk; s0 += blockDim.x)
    {
        const uint32_t s = s0 + threadIdx.x;
        bool hit = false;
        if (s < n_sources && s < lo + kSchedChunk)
        {
            const unsigned long long ctr = (first_step + t) * static_cast<unsigned long long>(n_sources) + s;
            hit = (rand64(key, ctr) >> 11) < threshold;
        }
        const uint32_t b = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) warp_tot[warp] = __popc(b);
        __syncthreads();
        uint32_t before = 0, all = 0;
        for (int w = 0; w < n_warps; ++w)
        {
            if (w < warp) before += warp_tot[w];
            all += warp_tot[w];
        }
        if (hit) idx[offs[t * chunks + c] + base + before + __popc(b & ((1u << lane) - 1u))] = s;
        __syncthreads();
        if (threadIdx.x == 0) base += all;
        __syncthreads();
    }
}

__global__ void step_offsets_kernel(const long long *chunk_offs, uint32_t chunks, uint64_t n_steps, long long total,
                                    long long *step_offs)
{
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t <= n_steps;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        step_offs[t] = t < n_steps ? chunk_offs[t * chunks] : total;
}

int grid_for(uint64_t n)
{
    const uint64_t b = (n + 255) / 256;
    return static_cast<int>(b < 152ull * 16 ? (b ? b : 1) : 152ull * 16);
}

int bits_for(uint32_t n_rows)
{
    int bits = 1;
    while (bits < 32 && (1ull << bits) < n_rows) ++bits;
    return bits;
}

}  // namespace

void launch_iota_u32(uint32_t *out, uint64_t n, cudaStream_t s) { iota_kernel<<<grid_for(n), 256, 0, s>>>(out, n); }

// Stable sort of synapse indexes 0..n_syn-1 by row key; perm_out receives the sorted indexes and
// row_ptr the CSR row offsets. With d_temp == nullptr only *temp_needed is computed. The key buffer
// is overwritten.
cudaError_t build_csr(
    uint64_t n_syn, uint32_t n_rows, const uint32_t *d_row_key, uint32_t *d_perm_out, long long *d_row_ptr,
    void *d_temp, size_t temp_bytes, size_t *temp_needed, cudaStream_t s)
{
    // Temp layout: [keys_alt n_syn][vals_in n_syn][cub temp]
    const int bits = bits_for(n_rows);
    size_t cub_bytes = 0;
    cudaError_t err = cub::DeviceRadixSort::SortPairs(
        nullptr, cub_bytes, static_cast<const uint32_t *>(nullptr), static_cast<uint32_t *>(nullptr),
        static_cast<const uint32_t *>(nullptr), static_cast<uint32_t *>(nullptr), static_cast<int64_t>(n_syn), 0, bits,
        s);
    if (err != cudaSuccess) return err;
    const size_t arr = ((n_syn * sizeof(uint32_t) + 255) / 256) * 256;
    const size_t need = 2 * arr + cub_bytes;
    if (!d_temp)
    {
        *temp_needed = need;
        return cudaSuccess;
    }
    if (temp_bytes < need) return cudaErrorInvalidValue;
    char *base = static_cast<char *>(d_temp);
    uint32_t *keys_sorted = reinterpret_cast<uint32_t *>(base);
    uint32_t *vals_in = reinterpret_cast<uint32_t *>(base + arr);
    void *cub_tmp = base + 2 * arr;
    iota_kernel<<<grid_for(n_syn), 256, 0, s>>>(vals_in, n_syn);
    err = cub::DeviceRadixSort::SortPairs(
        cub_tmp, cub_bytes, d_row_key, keys_sorted, vals_in, d_perm_out, static_cast<int64_t>(n_syn), 0, bits, s);
    if (err != cudaSuccess) return err;
    row_ptr_kernel<<<grid_for(static_cast<uint64_t>(n_rows) + 1), 256, 0, s>>>(keys_sorted, n_syn, n_rows, d_row_ptr);
    return cudaGetLastError();
}

void launch_gather_synapses(
    uint64_t n_syn, const uint32_t *perm, const uint32_t *post, const float *w, const uint32_t *delay,
    const uint8_t *type, int32_t *col_out, float *w_out, uint8_t *delay_out, uint8_t *type_out, cudaStream_t s)
{
    gather_kernel<<<grid_for(n_syn), 256, 0, s>>>(n_syn, perm, post, w, delay, type, col_out, w_out, delay_out,
                                                  type_out);
}

void launch_gen_keys(const GenSpec &g, uint64_t n_syn, uint32_t *pre_out, cudaStream_t s)
{
    gen_keys_kernel<<<grid_for(n_syn), 256, 0, s>>>(g, n_syn, pre_out);
}

void launch_gen_gather(const GenSpec &g, uint64_t n_syn, const uint32_t *perm, int32_t *col_out, float *w_out,
                       uint8_t *delay_out, cudaStream_t s)
{
    gen_gather_kernel<<<grid_for(n_syn), 256, 0, s>>>(g, n_syn, perm, col_out, w_out, delay_out);
}

cudaError_t gen_candidates(uint64_t n_cand, unsigned long long threshold, unsigned long long key,
                           unsigned long long *out, uint64_t *n_kept, cudaStream_t s)
{
    const uint64_t chunks = (n_cand + kCandChunk - 1) / kCandChunk;
    *n_kept = 0;
    if (!chunks) return cudaSuccess;
    unsigned long long *counts = nullptr, *offs = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    const int blocks = static_cast<int>(std::min<uint64_t>(chunks, 1u << 16));
    cudaError_t err = cudaMallocAsync(&counts, (chunks + 1) * sizeof(unsigned long long), s);
    if (err == cudaSuccess) err = cudaMallocAsync(&offs, (chunks + 1) * sizeof(unsigned long long), s);
    if (err == cudaSuccess) err = cudaMemsetAsync(counts + chunks, 0, sizeof(unsigned long long), s);
    if (err == cudaSuccess)
    {
        cand_count_kernel<<<blocks, 256, 0, s>>>(n_cand, threshold, key, chunks, counts);
        err = cudaGetLastError();
    }
    if (err == cudaSuccess)
        err = cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, counts, offs, static_cast<int64_t>(chunks + 1), s);
    if (err == cudaSuccess) err = cudaMallocAsync(&tmp, tmp_bytes, s);
    if (err == cudaSuccess)
        err = cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, counts, offs, static_cast<int64_t>(chunks + 1), s);
    unsigned long long total = 0;
    if (err == cudaSuccess) err = cudaMemcpyAsync(&total, offs + chunks, sizeof(total), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err == cudaSuccess && out && total)
    {
        cand_write_kernel<<<blocks, 256, 0, s>>>(n_cand, threshold, key, chunks, offs, out);
        err = cudaGetLastError();
    }
    if (tmp) cudaFreeAsync(tmp, s);
    if (offs) cudaFreeAsync(offs, s);
    if (counts) cudaFreeAsync(counts, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    *n_kept = total;
    return err;
}

// Bernoulli schedule on the device; allocates *d_idx (caller frees with cudaFree) and fills
// d_offsets[n_steps + 1].
cudaError_t gen_bernoulli_schedule(
    uint32_t n_sources, unsigned long long threshold, unsigned long long key, unsigned long long first_step,
    uint64_t n_steps, long long *d_offsets, uint32_t **d_idx, uint64_t *n_idx, cudaStream_t s)
{
    const uint32_t chunks = (n_sources + kSchedChunk - 1) / kSchedChunk;
    const uint64_t cells = n_steps * chunks;
    long long *counts = nullptr, *offs = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    cudaError_t err = cudaMallocAsync(&counts, (cells + 1) * sizeof(long long), s);
    if (err) return err;
    err = cudaMallocAsync(&offs, (cells + 1) * sizeof(long long), s);
    if (err) return err;
    dim3 grid(chunks ? chunks : 1, static_cast<unsigned>(n_steps));
    if (n_steps && chunks)
        bernoulli_count_kernel<<<grid, 256, 0, s>>>(n_sources, threshold, key, first_step, chunks, counts);
    cudaMemsetAsync(counts + cells, 0, sizeof(long long), s);
    cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, counts, offs, static_cast<int64_t>(cells + 1), s);
    err = cudaMallocAsync(&tmp, tmp_bytes, s);
    if (err) return err;
    cub::DeviceScan::ExclusiveSum(tmp, tmp_bytes, counts, offs, static_cast<int64_t>(cells + 1), s);
    long long total = 0;
    cudaMemcpyAsync(&total, offs + cells, sizeof(long long), cudaMemcpyDeviceToHost, s);
    err = cudaStreamSynchronize(s);
    if (err) return err;
    err = cudaMalloc(reinterpret_cast<void **>(d_idx), (total ? total : 1) * sizeof(uint32_t));
    if (err) return err;
    if (n_steps && chunks)
        bernoulli_write_kernel<<<grid, 256, 0, s>>>(n_sources, threshold, key, first_step, chunks, offs, *d_idx);
    step_offsets_kernel<<<grid_for(n_steps + 1), 256, 0, s>>>(offs, chunks, n_steps, total, d_offsets);
    cudaFreeAsync(tmp, s);
    cudaFreeAsync(counts, s);
    cudaFreeAsync(offs, s);
    *n_idx = static_cast<uint64_t>(total);
    return cudaGetLastError();
}

}  // namespace knp_gb300
