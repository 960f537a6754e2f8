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
#include <cstdint>

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

__global__ void lif_scan_forward_kernel(
    const float *__restrict__ I, float *__restrict__ S, float *__restrict__ ckpt, int T, long long BN, float beta,
    float theta, int K, int relaxed, float k)
{
    const long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
    if (i >= BN) return;
    float V = 0.0f;
    for (int t = 0; t < T; ++t)
    {
        if (t % K == 0) ckpt[static_cast<long long>(t / K) * BN + i] = V;
        const float U = beta * V + I[static_cast<long long>(t) * BN + i];
        const float s = relaxed ? fast_sigmoid(U - theta, k) : (U > theta ? 1.0f : 0.0f);
        S[static_cast<long long>(t) * BN + i] = s;
        V = U - theta * s;
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
        float U[kMaxSeg];
        float V = ckpt[static_cast<long long>(c) * BN + i];
#pragma unroll
        for (int u = 0; u < kMaxSeg; ++u)
        {
            const int t = t0 + u;
            if (t < t1)
            {
                U[u] = beta * V + I[static_cast<long long>(t) * BN + i];
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
                const float dU = dS[static_cast<long long>(t) * BN + i] * g + dV * (1.0f - theta * g);
                dI[static_cast<long long>(t) * BN + i] = dU;
                dV = beta * dU;
            }
        }
    }
}

}  // namespace

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
