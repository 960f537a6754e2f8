"""Differentiation form: surrogate-gradient BPTT through LIF layers.

A feed-forward LIF network (all-to-all layers, membrane decay beta, threshold theta, reset by
subtraction) is trained on spike counts. Per layer the synaptic input of all T steps is one GEMM of
the previous layer's spikes with the layer's weights (BF16 values of the FP32 master weights,
products exact in FP32, FP32 accumulation); the LIF recurrence over T and its backward are the
hand-written kernels of knp_gb300/csrc/bptt.cu behind ``LIFLayerFn`` (torch.autograd.Function).
The forward keeps the membrane state only every ``checkpoint`` steps; the backward recomputes each
segment. The reference has no gradient-based training; this form has no counterpart there.
"""
from __future__ import annotations

import ctypes

import torch

from . import _capi

K_SLOPE = 25.0


def _p(t: torch.Tensor):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def bf16_values(w: torch.Tensor) -> torch.Tensor:
    """The BF16 value of each master weight, as FP32 (exact)."""
    return w.to(torch.bfloat16).to(torch.float32)


def _mm(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """FP32 GEMM with IEEE FP32 arithmetic (no TF32 rounding of the operands)."""
    cm = torch.backends.cuda.matmul
    prev = cm.allow_tf32
    prev_p = getattr(cm, "fp32_precision", None)
    cm.allow_tf32 = False
    if prev_p is not None:
        cm.fp32_precision = "ieee"
    try:
        return a @ b
    finally:
        if prev_p is not None:
            cm.fp32_precision = prev_p
        cm.allow_tf32 = prev


class LIFLayerFn(torch.autograd.Function):
    """S_out[T, B, N_out] = LIF(S_in[T, B, N_in] @ W) with surrogate-gradient backward."""

    @staticmethod
    def forward(ctx, s_in, w_master, beta: float, theta: float, checkpoint: int, relaxed: bool, k: float):
        T, B, n_in = s_in.shape
        n_out = w_master.shape[1]
        wb = bf16_values(w_master)
        s_in = s_in.contiguous()
        I = _mm(s_in.reshape(T * B, n_in), wb).reshape(T, B, n_out).contiguous()
        S = torch.empty_like(I)
        ckpt = torch.empty(((T + checkpoint - 1) // checkpoint, B, n_out), device=I.device, dtype=torch.float32)
        _capi.check(_capi.lib().knp_gb300_lif_scan_forward(
            _p(I), _p(S), _p(ckpt), T, B * n_out, beta, theta, checkpoint, int(relaxed), k, _stream()))
        ctx.save_for_backward(s_in, wb, ckpt)
        ctx.cfg = (beta, theta, checkpoint, relaxed, k)
        return S

    @staticmethod
    def backward(ctx, dS):
        s_in, wb, ckpt = ctx.saved_tensors
        beta, theta, checkpoint, relaxed, k = ctx.cfg
        T, B, n_in = s_in.shape
        n_out = wb.shape[1]
        flat_in = s_in.reshape(T * B, n_in)
        I = _mm(flat_in, wb).reshape(T, B, n_out).contiguous()  # recomputed, not stored
        dS = dS.contiguous()
        dI = torch.empty_like(I)
        _capi.check(_capi.lib().knp_gb300_lif_scan_backward(
            _p(I), _p(ckpt), _p(dS), _p(dI), T, B * n_out, beta, theta, checkpoint, int(relaxed), k, _stream()))
        flat_dI = dI.reshape(T * B, n_out)
        dW = _mm(flat_in.t(), flat_dI)
        ds_in = _mm(flat_dI, wb.t()).reshape(T, B, n_in) if ctx.needs_input_grad[0] else None
        return ds_in, dW, None, None, None, None, None


class SpikingMLP(torch.nn.Module):
    """LIF layers with FP32 master weights; forward returns output spike counts [B, N_last]."""

    def __init__(self, sizes=(784, 512, 512, 10), beta: float = 0.9, theta: float = 1.0, checkpoint: int = 8,
                 relaxed: bool = False, k: float = K_SLOPE, seed: int = 0, device="cuda"):
        super().__init__()
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.weights = torch.nn.ParameterList(
            [torch.nn.Parameter((torch.randn(a, b, generator=g) * (2.0 / a) ** 0.5).to(device))
             for a, b in zip(sizes[:-1], sizes[1:])])
        self.beta, self.theta, self.checkpoint, self.relaxed, self.k = beta, theta, checkpoint, relaxed, k

    def forward(self, x):
        s = x
        for w in self.weights:
            s = LIFLayerFn.apply(s, w, self.beta, self.theta, self.checkpoint, self.relaxed, self.k)
        return s.sum(0)


def loss_fn(counts, labels):
    return torch.nn.functional.cross_entropy(counts, labels)


def make_batch(T=32, B=128, n_in=784, n_classes=10, max_rate=0.3, seed=0, device="cuda"):
    """Bernoulli input spikes with per-(sample, input) rate uniform in [0, max_rate]; random labels."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    rates = torch.rand(B, n_in, generator=g) * max_rate
    x = (torch.rand(T, B, n_in, generator=g) < rates).to(torch.float32)
    labels = torch.randint(0, n_classes, (B,), generator=g)
    return x.to(device), labels.to(device)


# ------------------------------------------------------------------ FP64 reference (test oracle)


class _SpikeFn64(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, relaxed, k):
        ctx.save_for_backward(x)
        ctx.k = k
        if relaxed:
            return 0.5 * (1.0 + k * x / (1.0 + k * x.abs()))
        return (x > 0).to(x.dtype)

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        d = 1.0 + ctx.k * x.abs()
        return g * (0.5 * ctx.k) / (d * d), None, None


def reference_forward(x, weights, beta=0.9, theta=1.0, relaxed=False, k=K_SLOPE):
    """The same network with torch autograd (loop over steps, no checkpointing), computed in the
    dtype of ``weights[0]``: float64 for the reference answer, float32 for a plain FP32
    implementation whose error against float64 calibrates the tolerance of the relaxed form."""
    dt = weights[0].dtype
    s_all = x.to(dt)
    T = s_all.shape[0]
    for w in weights:
        wb = w.to(dt)
        outs = []
        V = torch.zeros(s_all.shape[1], wb.shape[1], dtype=dt, device=x.device)
        for t in range(T):
            U = beta * V + s_all[t] @ wb
            s = _SpikeFn64.apply(U - theta, relaxed, k)
            V = U - theta * s
            outs.append(s)
        s_all = torch.stack(outs)
    return s_all.sum(0)
