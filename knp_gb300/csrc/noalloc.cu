// Allocation-free variant of the device Bernoulli spike-schedule generator.
//
// Some callers of this library cannot allocate GPU memory at the time they need a schedule: code
// that runs while a memory pool is locked by another component, allocators that forbid
// cudaMalloc/cudaFree from a given thread or phase, or hosts (such as a plugin loaded into a
// framework that owns all device memory) that hand over only the buffers they manage themselves.
// The regular generator (knp_gb300_generate_bernoulli_schedule) allocates its per-(step, chunk)
// counts, their prefix sums, the scan's temporary storage and the output schedule. This variant
// writes into the caller's output buffers and keeps its scratch in one fixed, file-scope device
// array, so it calls no cudaMalloc, cudaFree or allocating library routine.
//
// Scratch: kMaxCells + 1 int64 counters (2 MiB + 8 B) per device that loads the library, held until
// the process exits. Every call shares it and finds the last call's contents there; the kernels
// rewrite every cell they read before reading it. Calls that overlap on the GPU (two streams, or
// two threads) race on the scratch and must be serialised by the caller.
//
// Set-up: the CUDA runtime loads a module's device code and its __device__ arrays lazily, on first
// use, and that load allocates device memory. So the first call in a CUDA context (per device, and
// again after cudaDeviceReset, which replaces the context) loads this file's kernels and scratch array
// and looks up the array's device address, with that device current; a caller makes that first call
// during its own set-up, outside stream capture. Later calls in the same context reuse the address
// and allocate nothing.
#include <cmath>
#include <cstdint>
#include <mutex>

#include <cuda.h>
#include <cuda_runtime.h>

#include "kernels.h"

namespace knp_gb300
{
namespace
{

constexpr uint64_t kMaxCells = 1ull << 18;  // (steps x 4096-source chunks) per call
constexpr int kChunk = 4096;

__device__ __align__(256) long long g_schedule_scratch[kMaxCells + 1];

// counts[t * chunks + c] = spikes of step t among sources [c * kChunk, (c + 1) * kChunk).
__global__ void na_count_kernel(
    uint32_t n_sources, unsigned long long threshold, unsigned long long key, unsigned long long first_step,
    uint32_t chunks, long long *counts)
{
    const uint64_t t = blockIdx.y;
    const uint32_t c = blockIdx.x;
    __shared__ unsigned int tot;
    if (threadIdx.x == 0) tot = 0;
    __syncthreads();
    unsigned int mine = 0;
    for (uint32_t s = c * kChunk + threadIdx.x; s < n_sources && s < (c + 1) * kChunk; s += blockDim.x)
    {
        const unsigned long long ctr = (first_step + t) * static_cast<unsigned long long>(n_sources) + s;
        mine += (rand64(key, ctr) >> 11) < threshold;
    }
    atomicAdd(&tot, mine);
    __syncthreads();
    if (threadIdx.x == 0) counts[t * chunks + c] = tot;
}

// In-place exclusive scan of counts[0..n) with counts[n] = total, one block.
__global__ void na_scan_kernel(long long *counts, uint64_t n)
{
    __shared__ long long part[1024];
    const uint64_t per = (n + blockDim.x - 1) / blockDim.x;
    const uint64_t lo = threadIdx.x * per;
    const uint64_t hi = lo + per < n ? lo + per : n;
    long long sum = 0;
    for (uint64_t i = lo; i < hi; ++i) sum += counts[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        long long run = 0;
        for (unsigned i = 0; i < blockDim.x; ++i)
        {
            const long long x = part[i];
            part[i] = run;
            run += x;
        }
        counts[n] = run;
    }
    __syncthreads();
    long long run = part[threadIdx.x];
    for (uint64_t i = lo; i < hi; ++i)
    {
        const long long x = counts[i];
        counts[i] = run;
        run += x;
    }
}

// Writes the spikes of (step t, chunk c) in ascending source order at offsets[t * chunks + c].
__global__ void na_write_kernel(
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
    const uint32_t lo = c * kChunk;
    for (uint32_t s0 = lo; s0 < n_sources && s0 < lo + kChunk; s0 += blockDim.x)
    {
        const uint32_t s = s0 + threadIdx.x;
        bool hit = false;
        if (s < n_sources && s < lo + kChunk)
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

__global__ void na_step_offsets_kernel(const long long *chunk_offs, uint32_t chunks, uint64_t n_steps,
                                       long long *step_offs)
{
    for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t <= n_steps;
         t += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        step_offs[t] = chunk_offs[t * chunks];  // t == n_steps reads the total at counts[n_cells]
}

// Identity of the current CUDA context (unique in the process, never reused), through the driver
// entry point cuCtxGetId; 0 if it cannot be read (the set-up then runs on every call, which stays
// correct: a lookup in a loaded context allocates nothing).
unsigned long long current_context_id()
{
    using GetCurrent = CUresult (*)(CUcontext *);
    using GetId = CUresult (*)(CUcontext, unsigned long long *);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *a = nullptr, *b = nullptr;
        cudaDriverEntryPointQueryResult qa{}, qb{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
            qa == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
            qb == cudaDriverEntryPointSuccess)
        {
            get_current = reinterpret_cast<GetCurrent>(a);
            get_id = reinterpret_cast<GetId>(b);
        }
        cudaGetLastError();
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS)
        return 0;
    return id;
}

// Device address of the scratch array in the current context of `device` (which is current). The
// first call in a context loads this file's kernels (cudaFuncGetAttributes makes the runtime load
// them now rather than at their first launch) and the array, and looks up its address.
long long *scratch_address(int device, cudaError_t &err)
{
    struct Slot
    {
        unsigned long long ctx = 0;
        long long *addr = nullptr;
    };
    static std::mutex m;
    static Slot slots[64];
    std::lock_guard<std::mutex> l(m);
    err = cudaSuccess;
    if (device < 0 || device >= 64)
    {
        err = cudaErrorInvalidDevice;
        return nullptr;
    }
    // Before the runtime's first use of the device no context is current (id 0): the set-up below
    // then runs and makes the primary context current.
    const unsigned long long ctx = current_context_id();
    Slot &s = slots[device];
    if (s.addr && ctx != 0 && s.ctx == ctx) return s.addr;
    cudaFuncAttributes fa{};
    const void *kernels[] = {reinterpret_cast<const void *>(na_count_kernel), reinterpret_cast<const void *>(na_scan_kernel),
                             reinterpret_cast<const void *>(na_write_kernel),
                             reinterpret_cast<const void *>(na_step_offsets_kernel)};
    for (const void *k : kernels)
    {
        err = cudaFuncGetAttributes(&fa, k);
        if (err != cudaSuccess) return nullptr;
    }
    void *p = nullptr;
    err = cudaGetSymbolAddress(&p, g_schedule_scratch);
    if (err != cudaSuccess) return nullptr;
    s.ctx = current_context_id();
    s.addr = static_cast<long long *>(p);
    return s.addr;
}

}  // namespace

// Returns 0, -1 (bad arguments / sizes beyond the scratch), -2 (output capacity too small: *n_idx
// holds the count needed, nothing is written to idx) or -3 (CUDA error).
int bernoulli_schedule_noalloc(
    uint32_t n_sources, double p, uint64_t first_step, uint64_t n_steps, uint64_t seed, uint64_t stream,
    long long *d_offsets, uint32_t *d_idx, uint64_t capacity, uint64_t *n_idx, cudaStream_t s, const char **why)
{
    if (!n_idx)
    {
        *why = "null n_idx";
        return -1;
    }
    *n_idx = 0;  // every argument error leaves 0 here; only the capacity error reports a count
    if (!d_offsets || (capacity && !d_idx))
    {
        *why = "null buffer";
        return -1;
    }
    if (n_steps == 0 || n_sources == 0)
    {
        *why = "n_steps and n_sources must be positive";
        return -1;
    }
    if (!std::isfinite(p))
    {
        *why = "p must be a finite number";
        return -1;
    }
    if (n_steps > 65535)
    {
        *why = "at most 65535 steps per call";
        return -1;
    }
    const uint64_t chunks = (n_sources + kChunk - 1) / kChunk;
    const uint64_t cells = n_steps * chunks;
    if (cells > kMaxCells)
    {
        *why = "n_steps x ceil(n_sources / 4096) exceeds the scratch limit of 262144 cells";
        return -1;
    }
    int device = 0;
    cudaError_t err = cudaGetDevice(&device);
    long long *scratch = err == cudaSuccess ? scratch_address(device, err) : nullptr;
    if (!scratch)
    {
        *why = cudaGetErrorString(err);
        return -3;
    }
    const double pc = p < 0.0 ? 0.0 : (p > 1.0 ? 1.0 : p);
    const unsigned long long thr = static_cast<unsigned long long>(pc * 9007199254740992.0);
    const unsigned long long key = stream_key(seed, stream);
    dim3 grid(static_cast<unsigned>(chunks), static_cast<unsigned>(n_steps));
    na_count_kernel<<<grid, 256, 0, s>>>(n_sources, thr, key, first_step, static_cast<uint32_t>(chunks), scratch);
    na_scan_kernel<<<1, 1024, 0, s>>>(scratch, cells);
    long long total = 0;
    err = cudaMemcpyAsync(&total, scratch + cells, sizeof(long long), cudaMemcpyDeviceToHost, s);
    if (err == cudaSuccess) err = cudaStreamSynchronize(s);
    if (err != cudaSuccess)
    {
        *why = cudaGetErrorString(err);
        return -3;
    }
    *n_idx = static_cast<uint64_t>(total);
    if (static_cast<uint64_t>(total) > capacity)
    {
        *why = "output capacity too small (the required count is in *n_idx)";
        return -2;
    }
    if (total) na_write_kernel<<<grid, 256, 0, s>>>(n_sources, thr, key, first_step, static_cast<uint32_t>(chunks),
                                                    scratch, d_idx);
    na_step_offsets_kernel<<<static_cast<unsigned>((n_steps + 256) / 256), 256, 0, s>>>(
        scratch, static_cast<uint32_t>(chunks), n_steps, d_offsets);
    err = cudaGetLastError();
    if (err != cudaSuccess)
    {
        *why = cudaGetErrorString(err);
        return -3;
    }
    return 0;
}

}  // namespace knp_gb300
