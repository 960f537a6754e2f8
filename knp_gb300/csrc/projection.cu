// Projection kernel: for each presynaptic spike of this step, walk its CSR row and scatter-add the
// impacts into the target population's input ring at slot (step + delay) mod slots.
//
// Semantics (delta_impl.h:54-114 of the reference CPU library) are in projection_dev.cuh.
//
// Work distribution: persistent grid; each warp takes whole spike rows (row-major over the
// concatenated spike lists of all sources) and its 32 lanes stream the row's col / weight / delay
// arrays with coalesced loads, 4 synapses per lane in flight.
#include <algorithm>
#include <cstdint>

#include "kernels.h"
#include "projection_dev.cuh"

namespace knp_gb300
{
namespace
{

template <bool kFixed, bool kUniformExc>
__global__ void __launch_bounds__(256) projection_kernel(ProjectionDev p, Control *ctl)
{
    pdl_begin();
    const unsigned long long t = ctl->step;
    const uint32_t slot_base = static_cast<uint32_t>(t % p.ring.slots);
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;

    const uint32_t *idx[kMaxSources];
    uint32_t cnt[kMaxSources];
    const uint32_t total = resolve_sources(p, t, idx, cnt);
    __shared__ unsigned long long block_events;
    if (threadIdx.x == 0) block_events = 0;
    __syncthreads();
    unsigned long long events = 0;
    if (p.pull.bitmap)
    {
        // Direction choice for this step's spikes (the same in every block: it depends only on the
        // spike count). A pulled step only records its spikes; gather_kernel delivers them.
        const bool pull = total >= p.pull.threshold;
        // Every presynaptic neuron fired (one population source, whose spike indexes are distinct
        // and below its size): the gather then needs no bitmap and tests no bit for this step.
        const bool full = pull && p.n_src == 1 && !p.src[0].channel && p.src[0].n && total >= p.src[0].n;
        const uint32_t sl = static_cast<uint32_t>(t % p.pull.hist_slots);
        if (blockIdx.x == 0 && threadIdx.x == 0) p.pull.pulled[sl] = pull ? (full ? 2u : 1u) : 0u;
        if (full)
        {
            // Every row fired: the step's events are all the synapses, and the bitmap stays unused.
            if (blockIdx.x == 0 && threadIdx.x == 0)
                atomicAdd(&ctl->events_total, static_cast<unsigned long long>(p.row_ptr[p.n_rows] - p.row_ptr[0]));
            return;
        }
        if (pull)
        {
            uint32_t *bm = p.pull.bitmap + static_cast<size_t>(sl) * p.pull.words;
            const uint32_t stride = gridDim.x * blockDim.x;
            for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < total; j += stride)
            {
                uint32_t jj = j;
                int k = 0;
                while (jj >= cnt[k])
                {
                    jj -= cnt[k];
                    ++k;
                }
                const uint32_t pre = idx[k][jj];
                if (pre >= p.n_rows) continue;
                atomicOr(bm + (pre >> 5), 1u << (pre & 31));
                events += static_cast<unsigned long long>(p.row_ptr[pre + 1] - p.row_ptr[pre]);
            }
            // Per-thread counts: reduce over the warp, then the block.
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) events += __shfl_down_sync(0xffffffffu, events, o);
            if (lane == 0 && events) atomicAdd(&block_events, events);
            __syncthreads();
            if (threadIdx.x == 0 && block_events) atomicAdd(&ctl->events_total, block_events);
            return;
        }
    }
    events = scatter_rows<kFixed, kUniformExc>(p, slot_base, idx, cnt, total, warp, n_warps, lane);
    if (p.last_spike)
    {
        // Resource-STDP synapses: init_synapse (synaptic_resource_stdp.h:36-41, called per synapse of
        // a spiking row in delta_impl.h:75) records the step of the presynaptic spike.
        for (uint32_t j = warp; j < total; j += n_warps)
        {
            uint32_t jj = j;
            int k = 0;
            while (jj >= cnt[k])
            {
                jj -= cnt[k];
                ++k;
            }
            const uint32_t pre = idx[k][jj];
            if (pre >= p.n_rows) continue;
            for (int64_t e = p.row_ptr[pre] + lane; e < p.row_ptr[pre + 1]; e += 32) p.last_spike[e] = t;
        }
    }
    if (lane == 0 && events) atomicAdd(&block_events, events);
    __syncthreads();
    if (threadIdx.x == 0 && block_events) atomicAdd(&ctl->events_total, block_events);
}

// Random FP32 adds of 1/256 into buf[0, n), n < 2^32: thread g's i-th add goes to position
// floor(h * n / 2^32) of the 32-bit hash h = mix64(seed, g, i) (a multiply, not a division).
__global__ void add_rate_kernel(float *buf, uint32_t n, uint32_t per, unsigned long long seed)
{
    const unsigned long long g = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x;
    for (uint32_t i = 0; i < per; ++i)
    {
        const uint32_t h = static_cast<uint32_t>(mix64(seed ^ (g * 0x9E3779B97F4A7C15ull + i)));
        atomicAdd(buf + __umulhi(h, n), 1.0f / 256.0f);
    }
}

}  // namespace

int measure_add_rate(uint64_t n, uint64_t adds, double *rate, const char **why)
{
    int device = 0, sms = 0;
    cudaError_t err = cudaGetDevice(&device);
    if (err == cudaSuccess) err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (err != cudaSuccess)
    {
        *why = cudaGetErrorString(err);
        return -3;
    }
    const uint32_t threads = 512, blocks = 4u * static_cast<uint32_t>(sms);
    const uint64_t all = static_cast<uint64_t>(threads) * blocks;
    const uint32_t per = static_cast<uint32_t>(std::max<uint64_t>(1, std::min<uint64_t>(adds / all, 1u << 20)));
    float *buf = nullptr;
    cudaEvent_t a = nullptr, b = nullptr;
    float ms = 0.f;
    err = cudaMalloc(&buf, n * sizeof(float));
    if (err == cudaSuccess) err = cudaMemset(buf, 0, n * sizeof(float));
    if (err == cudaSuccess) err = cudaEventCreate(&a);
    if (err == cudaSuccess) err = cudaEventCreate(&b);
    if (err == cudaSuccess)
    {
        const uint32_t n32 = static_cast<uint32_t>(n);
        add_rate_kernel<<<blocks, threads>>>(buf, n32, per, 1);  // warm-up: the buffer's lines in L2
        cudaEventRecord(a);
        for (int r = 0; r < 3; ++r) add_rate_kernel<<<blocks, threads>>>(buf, n32, per, 2 + r);
        cudaEventRecord(b);
        err = cudaEventSynchronize(b);
        if (err == cudaSuccess) err = cudaGetLastError();
        if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, a, b);
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (buf) cudaFree(buf);
    if (err != cudaSuccess)
    {
        *why = cudaGetErrorString(err);
        return -3;
    }
    *rate = 3.0 * static_cast<double>(all) * per / (static_cast<double>(ms) * 1e-3);
    return 0;
}

void launch_projection(const ProjectionDev &p, Control *ctl, int grid, cudaStream_t s)
{
    const bool uexc = !p.type && p.uniform_type == 0;
    if (p.ring.fixed)
    {
        if (uexc)
            launch_pdl(projection_kernel<true, true>, dim3(grid), dim3(256), 0, s, p, ctl);
        else
            launch_pdl(projection_kernel<true, false>, dim3(grid), dim3(256), 0, s, p, ctl);
    }
    else
    {
        if (uexc)
            launch_pdl(projection_kernel<false, true>, dim3(grid), dim3(256), 0, s, p, ctl);
        else
            launch_pdl(projection_kernel<false, false>, dim3(grid), dim3(256), 0, s, p, ctl);
    }
}

}  // namespace knp_gb300
