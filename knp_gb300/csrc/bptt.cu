// Differentiation form: the LIF recurrence of a layer over T steps, forward and hand-written
// backward (surrogate-gradient BPTT), one thread per (sample, neuron).
//
//   U_t = beta * V_{t-1} + I_t            (V_{-1} = 0; I_t = this step's synaptic input)
//   S_t = H(U_t - theta)                  (strict '>' as the reference LIF, lif_impl.h:71-78)
//   V_t = U_t - theta * S_t               (reset by subtraction)
//
// Backward uses the fast-sigmoid surrogate dS/dU = g(U - theta), g(x) = (k/2) / (1 + k|x|)^2,
// which is the exact derivative of the relaxed forward S = f(U - theta), f(x) = (1 + kx/(1+k|x|)) / 2.
// With `relaxed` set the forward itself uses f, so finite differences of the forward check the
// backward. The reset term is differentiated (dV_t/dU_t = 1 - theta * g).
//
// Memory: the forward stores V only at every K-th step (checkpoint c holds the state entering
// step c*K); the backward recomputes U inside each K-step segment from its checkpoint and I.
#include <algorithm>
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace knp_gb300
{
namespace
{

constexpr int kMaxSeg = 16;

__device__ __forceinline__ float fast_sigmoid(float x, float k)
{
    return 0.5f * (1.0f + __fdiv_rn(k * x, 1.0f + k * fabsf(x)));
}

__device__ __forceinline__ float surrogate(float x, float k)
{
    const float d = 1.0f + k * fabsf(x);
    return __fdiv_rn(0.5f * k, d * d);
}

// One thread per (sample, neuron). A thread's chain of steps is short of parallelism (BN threads, a
// few warps per SM), so each K-step segment's inputs (and, backward, output gradients) are loaded
// before the segment's recurrence: up to kMaxSeg independent loads in flight instead of one.
__global__ void lif_scan_forward_kernel(
    const float *__restrict__ I, float *__restrict__ S, float *__restrict__ ckpt, int T, long long BN, float beta,
    float theta, int K, int relaxed, float k)
{
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= BN) return;
    float V = 0.0f;
    const int n_seg = (T + K - 1) / K;
    for (int c = 0; c < n_seg; ++c)
    {
        const int t0 = c * K;
        const int t1 = min(T, t0 + K);
        ckpt[static_cast<long long>(c) * BN + i] = V;
        float x[kMaxSeg];
#pragma unroll
        for (int u = 0; u < kMaxSeg; ++u)
            if (t0 + u < t1) x[u] = I[static_cast<long long>(t0 + u) * BN + i];
#pragma unroll
        for (int u = 0; u < kMaxSeg; ++u)
        {
            const int t = t0 + u;
            if (t < t1)
            {
                const float U = beta * V + x[u];
                const float s = relaxed ? fast_sigmoid(U - theta, k) : (U > theta ? 1.0f : 0.0f);
                S[static_cast<long long>(t) * BN + i] = s;
                V = U - theta * s;
            }
        }
    }
}

__global__ void lif_scan_backward_kernel(
    const float *__restrict__ I, const float *__restrict__ ckpt, const float *__restrict__ dS, float *__restrict__ dI,
    int T, long long BN, float beta, float theta, int K, int relaxed, float k)
{
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= BN) return;
    float dV = 0.0f;  // dL/dV_t flowing back from step t + 1
    const int n_seg = (T + K - 1) / K;
    for (int c = n_seg - 1; c >= 0; --c)
    {
        const int t0 = c * K;
        const int t1 = min(T, t0 + K);
        float U[kMaxSeg], g_out[kMaxSeg];
        float V = ckpt[static_cast<long long>(c) * BN + i];
#pragma unroll
        for (int u = 0; u < kMaxSeg; ++u)
            if (t0 + u < t1)
            {
                U[u] = I[static_cast<long long>(t0 + u) * BN + i];
                g_out[u] = dS[static_cast<long long>(t0 + u) * BN + i];
            }
#pragma unroll
        for (int u = 0; u < kMaxSeg; ++u)
        {
            if (t0 + u < t1)
            {
                U[u] = beta * V + U[u];
                const float s = relaxed ? fast_sigmoid(U[u] - theta, k) : (U[u] > theta ? 1.0f : 0.0f);
                V = U[u] - theta * s;
            }
        }
#pragma unroll
        for (int u = kMaxSeg - 1; u >= 0; --u)
        {
            const int t = t0 + u;
            if (t < t1)
            {
                const float g = surrogate(U[u] - theta, k);
                const float dU = g_out[u] * g + dV * (1.0f - theta * g);
                dI[static_cast<long long>(t) * BN + i] = dU;
                dV = beta * dU;
            }
        }
    }
}

// ---- GEMM operand layouts (BF16, K contiguous) built in one pass from an FP32 or BF16 matrix
// X[R][C]. Each output row holds H halves of width P (P >= the copied extent, the rest zero):
// mode 0: one half, bf16(x); mode 1: two equal halves, bf16(x); mode 2: two halves hi = bf16(x),
// lo = bf16(x - hi) (round to nearest even, as torch's conversion), so hi + lo holds x to 2^-17.
// Row form: out[r][h P + c]; transposed form: out[c][h P + r] (a 32 x 32 tile through shared memory,
// reads and writes coalesced).
__device__ __forceinline__ float load_x(const void *X, int x_bf16, long long i)
{
    return x_bf16 ? __bfloat162float(static_cast<const __nv_bfloat16 *>(X)[i]) : static_cast<const float *>(X)[i];
}

__device__ __forceinline__ void halves(float x, int mode, __nv_bfloat16 &h0, __nv_bfloat16 &h1)
{
    h0 = __float2bfloat16_rn(x);
    h1 = mode == 2 ? __float2bfloat16_rn(x - __bfloat162float(h0)) : h0;
}

// Row form: block (x, y) covers columns [2 (256 x + t), +2) of rows y, y + gridDim.y, ...; a thread
// stores its two columns as one bf16 pair (P even, so pairs are 4-byte aligned).
__global__ void operand_rows_kernel(const void *X, int x_bf16, long long R, long long C, int mode, long long P,
                                    __nv_bfloat16 *out)
{
    const int H = mode == 0 ? 1 : 2;
    const long long c = 2 * (static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x);
    if (c >= P) return;
    for (long long r = blockIdx.y; r < R; r += gridDim.y)
    {
        const __nv_bfloat16 z = __float2bfloat16_rn(0.0f);
        __nv_bfloat16 a0 = z, a1 = z, b0 = z, b1 = z;
        if (c < C) halves(load_x(X, x_bf16, r * C + c), mode, a0, a1);
        if (c + 1 < C) halves(load_x(X, x_bf16, r * C + c + 1), mode, b0, b1);
        __nv_bfloat16 *o = out + r * H * P + c;
        *reinterpret_cast<__nv_bfloat162 *>(o) = __halves2bfloat162(a0, b0);
        if (H == 2) *reinterpret_cast<__nv_bfloat162 *>(o + P) = __halves2bfloat162(a1, b1);
    }
}

__global__ void operand_transposed_kernel(const void *X, int x_bf16, long long R, long long C, int mode, long long P,
                                          __nv_bfloat16 *out)
{
    __shared__ float tile[32][33];
    const int H = mode == 0 ? 1 : 2;
    const long long r0 = static_cast<long long>(blockIdx.x) * 32, c0 = static_cast<long long>(blockIdx.y) * 32;
    // Read X[r0 + y][c0 + x] (coalesced along c); rows past R read as zero (the padding).
    for (int y = threadIdx.y; y < 32; y += blockDim.y)
    {
        const long long r = r0 + y, c = c0 + threadIdx.x;
        tile[y][threadIdx.x] = (r < R && c < C) ? load_x(X, x_bf16, r * C + c) : 0.0f;
    }
    __syncthreads();
    // Write out[c0 + y][h P + r0 + x] (coalesced along r).
    for (int y = threadIdx.y; y < 32; y += blockDim.y)
    {
        const long long c = c0 + y, r = r0 + threadIdx.x;
        if (c >= C || r >= P) continue;
        __nv_bfloat16 h0, h1;
        halves(tile[threadIdx.x][y], mode, h0, h1);
        out[c * H * P + r] = h0;
        if (H == 2) out[c * H * P + P + r] = h1;
    }
}

}  // namespace

int bf16_operand(const void *X, int x_bf16, long long R, long long C, int mode, int transpose, long long P, void *out,
                 cudaStream_t s)
{
    if (!X || !out || R < 1 || C < 1 || mode < 0 || mode > 2 || P < (transpose ? R : C)) return -1;
    auto *o = static_cast<__nv_bfloat16 *>(out);
    if (transpose)
    {
        const long long gx = (P + 31) / 32, gy = (C + 31) / 32;
        if (gx > 0x7FFFFFFFll || gy > 65535) return -1;
        operand_transposed_kernel<<<dim3(static_cast<unsigned>(gx), static_cast<unsigned>(gy)), dim3(32, 8), 0, s>>>(
            X, x_bf16, R, C, mode, P, o);
    }
    else
    {
        if (P % 2) return -1;  // pairs of columns
        const long long gx = (P / 2 + 255) / 256;
        const unsigned gy = static_cast<unsigned>(std::min<long long>(R, 4096));
        if (gx > 0x7FFFFFFFll) return -1;
        operand_rows_kernel<<<dim3(static_cast<unsigned>(gx), gy), 256, 0, s>>>(X, x_bf16, R, C, mode, P, o);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int lif_scan_forward(
    const float *I, float *S, float *ckpt, int T, long long BN, float beta, float theta, int K, int relaxed, float k,
    cudaStream_t s)
{
    if (K < 1 || K > kMaxSeg || T < 1 || BN < 1) return -1;
    const int threads = 256;
    const long long blocks = (BN + threads - 1) / threads;
    lif_scan_forward_kernel<<<static_cast<unsigned>(blocks), threads, 0, s>>>(I, S, ckpt, T, BN, beta, theta, K, relaxed,
                                                                             k);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int lif_scan_backward(
    const float *I, const float *ckpt, const float *dS, float *dI, int T, long long BN, float beta, float theta, int K,
    int relaxed, float k, cudaStream_t s)
{
    if (K < 1 || K > kMaxSeg || T < 1 || BN < 1) return -1;
    const int threads = 256;
    const long long blocks = (BN + threads - 1) / threads;
    lif_scan_backward_kernel<<<static_cast<unsigned>(blocks), threads, 0, s>>>(I, ckpt, dS, dI, T, BN, beta, theta, K,
                                                                              relaxed, k);
    return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // namespace knp_gb300
