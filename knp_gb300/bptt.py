"""Differentiation form: surrogate-gradient BPTT through LIF layers.

A feed-forward LIF network (all-to-all layers, membrane decay beta, threshold theta, reset by
subtraction) is trained on spike counts. Per layer the synaptic input of all T steps is one GEMM of
the previous layer's spikes with the layer's weights (BF16 values of the FP32 master weights,
products exact in FP32, FP32 accumulation); the LIF recurrence over T and its backward are the
hand-written kernels of knp_gb300/csrc/bptt.cu behind ``LIFLayerFn`` (torch.autograd.Function).
The forward keeps the membrane state only every ``checkpoint`` steps; the backward recomputes each
segment. The reference has no gradient-based training; this form has no counterpart there.

Every contraction runs on the library's tcgen05 BF16 GEMM (knp_gb300_bf16_gemm_tn, FP32 accumulation
in tensor memory): the forward and recomputed inputs take the 0/1 spikes and the BF16 weights
directly (exact operands); the weight and input gradients carry the FP32 surrogate gradients dI as
two BF16 terms, dI = hi + lo with hi = bf16(dI) and lo = bf16(dI - hi), concatenated along K, so
each product is exact in FP32 and dI is represented to 2^-17 relative. The sigmoid-relaxed forward
(a verification mode whose recurrence amplifies input errors about 1e5-fold) has continuous layer
outputs: there every layer input and dI are split into three BF16 terms, which hold every normal
FP32 value exactly (8 + 8 + 8 significand bits), so each contraction equals an FP32 GEMM with exact
products.
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


_ERR = {}


def _err_word(device) -> torch.Tensor:
    """Device error word of the GEMMs on `device` (bit 0: a tensor-core completion wait timed out)."""
    key = str(device)
    if key not in _ERR:
        _ERR[key] = torch.zeros(1, dtype=torch.int32, device=device)
    return _ERR[key]


def check_gemm_errors(device="cuda"):
    """Raises if a GEMM of this module reported a timeout on `device` (one device-to-host read)."""
    e = _err_word(torch.device(device))
    if int(e.item()) != 0:
        e.zero_()
        raise RuntimeError("a tcgen05 GEMM completion wait timed out")


def _pad_k(x: torch.Tensor, mult: int = 8) -> torch.Tensor:
    """Zero columns up to a multiple of `mult` (the pipelined GEMM wants 16-byte rows)."""
    k = x.shape[1]
    kp = (k + mult - 1) // mult * mult
    return x if kp == k else torch.nn.functional.pad(x, (0, kp - k))


def gemm_tn(a: torch.Tensor, b: torch.Tensor) -> torch.Tensor:
    """D[M, N] = A[M, K] @ B[N, K]^T (FP32) on the tcgen05 tensor cores; a and b are BF16, row-major."""
    assert a.dtype == torch.bfloat16 and b.dtype == torch.bfloat16 and a.shape[1] == b.shape[1]
    a = _pad_k(a.contiguous())
    b = _pad_k(b.contiguous())
    M, K = a.shape
    N = b.shape[0]
    d = torch.empty((M, N), device=a.device, dtype=torch.float32)
    _capi.check(_capi.lib().knp_gb300_bf16_gemm_tn(_p(a), _p(b), _p(d), M, N, K, _p(_err_word(a.device)), _stream()))
    return d


def bf16_terms(x: torch.Tensor, n: int):
    """n BF16 tensors whose FP32 sum is x: term k is bf16 of x minus the terms before it. n = 1 for
    values that are BF16 already (0/1 spikes, BF16 weights); n = 2 leaves O(2^-17 |x|); n = 3 is exact
    for normal FP32 values."""
    terms, rest = [], x.float()
    for k in range(n):
        t = rest.to(torch.bfloat16)
        terms.append(t)
        if k + 1 < n:
            rest = rest - t.to(torch.float32)
    return terms


def gemm_terms(a_terms, b_terms) -> torch.Tensor:
    """(sum a_i) @ (sum b_j)^T as one GEMM: every pair (a_i, b_j) concatenated along K, each part padded
    to 16-byte rows."""
    pairs = [(a, b) for a in a_terms for b in b_terms]
    if len(pairs) == 1:
        return gemm_tn(*pairs[0])
    return gemm_tn(torch.cat([_pad_k(a.contiguous()) for a, _ in pairs], 1),
                   torch.cat([_pad_k(b.contiguous()) for _, b in pairs], 1))


def _round8(n: int) -> int:
    return (n + 7) // 8 * 8


def operand(x: torch.Tensor, mode: int, transpose: bool, width: int) -> torch.Tensor:
    """BF16 GEMM operand from x[R, C] (FP32 or BF16) by knp_gb300_bf16_operand: rows of one (mode 0)
    or two (1: the value twice; 2: hi, lo) halves of `width` (zero-padded), from x's rows or, with
    transpose, from its columns."""
    x = x.contiguous()
    R, C = x.shape
    H = 1 if mode == 0 else 2
    out = torch.empty((C if transpose else R, H * width), device=x.device, dtype=torch.bfloat16)
    _capi.check(_capi.lib().knp_gb300_bf16_operand(_p(x), int(x.dtype == torch.bfloat16), R, C, mode, int(transpose),
                                                   width, _p(out), _stream()))
    return out


# The hard-threshold path builds its GEMM operands with knp_gb300_bf16_operand (one pass per
# operand: cast, hi/lo split, transpose, concatenation along K and padding); the relaxed path (three
# BF16 terms of continuous values) keeps the torch composition of bf16_terms / gemm_terms.
FUSED_OPERANDS = True


class LIFLayerFn(torch.autograd.Function):
    """S_out[T, B, N_out] = LIF(S_in[T, B, N_in] @ W) with surrogate-gradient backward."""

    @staticmethod
    def forward(ctx, s_in, w_master, beta: float, theta: float, checkpoint: int, relaxed: bool, k: float):
        T, B, n_in = s_in.shape
        n_out = w_master.shape[1]
        s_in = s_in.contiguous()
        fused = FUSED_OPERANDS and not relaxed
        if fused:
            s2d = s_in.reshape(T * B, n_in)
            a = operand(s2d, 0, False, _round8(n_in))            # [TB, n_in]: 0/1 spikes, exact in BF16
            wt = operand(w_master, 0, True, _round8(n_in))       # [n_out, n_in]: W^T
            I = gemm_tn(a, wt).reshape(T, B, n_out)
            saved = (w_master, s2d, a, wt)
        else:
            wb = w_master.to(torch.bfloat16)  # [n_in, n_out]
            s_terms = bf16_terms(s_in.reshape(T * B, n_in), 3 if relaxed else 1)  # 0/1 spikes are exact
            I = gemm_terms(s_terms, [wb.t().contiguous()]).reshape(T, B, n_out).contiguous()
            saved = (wb, *s_terms)
        S = torch.empty_like(I)
        ckpt = torch.empty(((T + checkpoint - 1) // checkpoint, B, n_out), device=I.device, dtype=torch.float32)
        _capi.check(_capi.lib().knp_gb300_lif_scan_forward(
            _p(I), _p(S), _p(ckpt), T, B * n_out, beta, theta, checkpoint, int(relaxed), k, _stream()))
        ctx.save_for_backward(ckpt, *saved)
        ctx.cfg = (T, B, beta, theta, checkpoint, relaxed, k, fused, n_in, n_out)
        return S

    @staticmethod
    def backward(ctx, dS):
        ckpt, *saved = ctx.saved_tensors
        T, B, beta, theta, checkpoint, relaxed, k, fused, n_in, n_out = ctx.cfg
        if fused:
            w_master, s2d, a, wt = saved
            I = gemm_tn(a, wt).reshape(T, B, n_out)  # recomputed, not stored
        else:
            wb, *s_terms = saved
            I = gemm_terms(s_terms, [wb.t().contiguous()]).reshape(T, B, n_out).contiguous()
        dS = dS.contiguous()
        dI = torch.empty_like(I)
        _capi.check(_capi.lib().knp_gb300_lif_scan_backward(
            _p(I), _p(ckpt), _p(dS), _p(dI), T, B * n_out, beta, theta, checkpoint, int(relaxed), k, _stream()))
        ds_in = None
        if fused:
            dI2 = dI.reshape(T * B, n_out)
            tb = _round8(T * B)
            # dW[n_in, n_out] = S^T (hi + lo): K = 2 T B, [S^T | S^T] against [hi^T | lo^T].
            dW = gemm_tn(operand(s2d, 1, True, tb), operand(dI2, 2, True, tb))
            if ctx.needs_input_grad[0]:
                # ds_in[TB, n_in] = (hi + lo) W^T: K = 2 n_out, [hi | lo] against [W | W].
                w2 = _round8(n_out)
                ds_in = gemm_tn(operand(dI2, 2, False, w2), operand(w_master, 1, False, w2)).reshape(T, B, n_in)
            return ds_in, dW, None, None, None, None, None
        d_terms = bf16_terms(dI.reshape(T * B, n_out), 3 if relaxed else 2)
        # dW[n_in, n_out] = S^T dI: K = T B per (S term, dI term) pair.
        dW = gemm_terms([s.t() for s in s_terms], [d.t() for d in d_terms])
        if ctx.needs_input_grad[0]:
            # ds_in[TB, n_in] = dI W^T, W as [n_in, n_out]: K = n_out per dI term.
            ds_in = gemm_terms(d_terms, [wb]).reshape(T, B, n_in)
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


class GraphedTrainStep:
    """One training iteration (forward, loss, backward, optimizer step) on the static tensors ``x`` and
    ``labels``, captured once as a CUDA graph and replayed by ``__call__``; the iteration's ~70
    kernels then cost one launch. New data is copied into ``x`` / ``labels`` in place. The optimizer
    must be graph-safe (SGD; Adam with ``capturable=True``). Warm-up iterations run on a side stream
    first, as torch's graph capture asks."""

    def __init__(self, model: torch.nn.Module, opt: torch.optim.Optimizer, x: torch.Tensor, labels: torch.Tensor,
                 warmup: int = 3):
        self.x, self.labels = x, labels
        side = torch.cuda.Stream(device=x.device)
        side.wait_stream(torch.cuda.current_stream(x.device))
        with torch.cuda.stream(side):
            for _ in range(warmup):
                opt.zero_grad(set_to_none=True)
                loss_fn(model(x), labels).backward()
                opt.step()
        torch.cuda.current_stream(x.device).wait_stream(side)
        opt.zero_grad(set_to_none=True)
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.loss = loss_fn(model(x), labels)
            self.loss.backward()
            opt.step()

    def __call__(self) -> torch.Tensor:
        """Replays the iteration on torch's current stream; returns the (static) loss tensor."""
        self.graph.replay()
        return self.loss


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
