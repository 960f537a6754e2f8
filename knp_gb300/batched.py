"""Batched / precision form: many independent LIF network samples on the tcgen05 tensor cores.

``BatchedPlan`` drives ``knp_gb300_batched_plan_*`` (knp_gb300/csrc/batched.cu): B samples of a
feed-forward LIF network with all-to-all delay-1 layers, uneven lengths T_b and optionally uneven
layer sizes per sample, Bernoulli inputs with per-(sample, input) rates, BF16 weights (FP32 master
values rounded to BF16), FP32 accumulation; prepared once and run as one CUDA-graph launch. ``run``
is the one-shot form.
``plain_network`` builds the same computation as one block-diagonal network for the plain backend
(FP32 input rings, the same BF16-valued weights), which is what the batched form is compared with.
The reference has no batched execution; these forms have no counterpart there.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _capi
from . import network as N
from . import types as T


@dataclass
class BatchedConfig:
    sizes: tuple
    weights: list  # float32 arrays [n_out, n_in], BF16-representable values
    rates: np.ndarray  # float32 [B, n_0]
    steps: np.ndarray  # uint32 [B]
    seed: int
    leak: tuple = None
    threshold: tuple = None
    reset: tuple = None
    refract: tuple = None
    sample_sizes: np.ndarray = None  # uint32 [n_layers + 1, B]: sample b's size of layer l (<= sizes[l])

    @property
    def batch(self) -> int:
        return int(self.steps.shape[0])


def bf16_round(x: np.ndarray) -> np.ndarray:
    """Round FP32 values to the nearest BF16 (ties to even), returned as FP32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16 << 16
    return u.astype(np.uint32).view(np.float32)


def dense_config(seed: int = 4, batch: int = 256, sizes=(784, 1000, 1000, 10), t_lo: int = 50, t_hi: int = 200,
                 rate_max: float = 0.2) -> BatchedConfig:
    """Batched dense config: weights N(0, 1/fan_in) rounded to BF16, threshold 1, per-input rates
    uniform in [0, rate_max], per-sample lengths uniform in [t_lo, t_hi]."""
    rng = np.random.default_rng(seed)
    ws = [bf16_round(rng.normal(0.0, 1.0 / np.sqrt(a), size=(b, a)).astype(np.float32))
          for a, b in zip(sizes[:-1], sizes[1:])]
    rates = (rng.random((batch, sizes[0])) * rate_max).astype(np.float32)
    steps = rng.integers(t_lo, t_hi + 1, size=batch).astype(np.uint32)
    return BatchedConfig(tuple(sizes), ws, rates, steps, seed)


def input_spikes(cfg: BatchedConfig, b: int, t: int) -> np.ndarray:
    """Input indexes of sample b at step t: the counter-based draw the kernel makes (inputs beyond the
    sample's input width never spike)."""
    n0 = cfg.sizes[0]
    key = N.stream_key(cfg.seed, N.S_INPUT)
    ctr = (np.uint64(t) * np.uint64(cfg.batch) + np.uint64(b)) * np.uint64(n0) + np.arange(n0, dtype=np.uint64)
    # A rate is a probability: below 0 (or NaN) never, 1 or above always.
    r = np.clip(np.nan_to_num(cfg.rates[b].astype(np.float64), nan=0.0), 0.0, 1.0)
    thr = (r * float(1 << 53)).astype(np.uint64)
    idx = np.nonzero((N.rand64(key, ctr) >> np.uint64(11)) < thr)[0].astype(np.uint32)
    if cfg.sample_sizes is not None:
        idx = idx[idx < cfg.sample_sizes[0][b]]
    return idx


def uneven_config(seed: int = 8, batch: int = 40, sizes=(96, 128, 64, 10), t_lo: int = 10, t_hi: int = 30,
                  rate_max: float = 0.3) -> BatchedConfig:
    """Dense config whose samples are network instances of uneven size: sample b keeps a random
    prefix of every layer (at least half of it, the output layer whole) over shared weights."""
    cfg = dense_config(seed=seed, batch=batch, sizes=sizes, t_lo=t_lo, t_hi=t_hi, rate_max=rate_max)
    rng = np.random.default_rng(seed + 1000)
    ss = np.zeros((len(sizes), batch), np.uint32)
    for layer, n in enumerate(sizes):
        ss[layer] = n if layer == len(sizes) - 1 else rng.integers(n // 2, n + 1, size=batch)
    cfg.sample_sizes = ss
    return cfg


class BatchedPlan:
    """A batch prepared on the device (knp_gb300_batched_plan_create) and run as one CUDA-graph
    launch per ``run()``; with ``autotune`` the operand ring depth and the layer ring length are
    chosen by timing each pair, ``stages`` fixes the depth (0: the deepest that fits)."""

    def __init__(self, cfg: BatchedConfig, record: bool = False, autotune: bool = False, device: int = 0,
                 segment_steps: int = 0, stages: int = 0):
        import torch

        self.cfg = cfg
        self._lib = _capi.lib()
        dev = torch.device(f"cuda:{device}")
        L = len(cfg.sizes) - 1
        self._w = [torch.from_numpy(np.ascontiguousarray(w)).to(dev).to(torch.bfloat16).contiguous()
                   for w in cfg.weights]
        self._rates = torch.from_numpy(np.ascontiguousarray(cfg.rates, np.float32)).to(dev)
        self._counts = torch.zeros((cfg.batch, cfg.sizes[-1]), dtype=torch.int32, device=dev)
        self._words = [(n + 31) // 32 for n in cfg.sizes]
        self._t_max = int(cfg.steps.max())
        self._stride = sum(cfg.batch * w for w in self._words)
        self._rec = torch.zeros(self._t_max * self._stride, dtype=torch.int32, device=dev) if record else None
        self._stream = torch.cuda.current_stream(dev)

        def fl(v, default):
            return (ctypes.c_float * L)(*(v if v is not None else [default] * L))

        sizes = (ctypes.c_uint32 * (L + 1))(*cfg.sizes)
        wptr = (ctypes.c_void_p * L)(*[w.data_ptr() for w in self._w])
        refract = (ctypes.c_uint32 * L)(*(cfg.refract if cfg.refract is not None else [0] * L))
        steps = (ctypes.c_uint32 * cfg.batch)(*[int(x) for x in cfg.steps])
        ss = None
        if cfg.sample_sizes is not None:
            flat = np.ascontiguousarray(cfg.sample_sizes, np.uint32).ravel()
            ss = (ctypes.c_uint32 * flat.size)(*flat.tolist())
        self._h = ctypes.c_void_p()
        _capi.check(self._lib.knp_gb300_batched_plan_create(
            L, sizes, wptr, fl(cfg.leak, 1.0), fl(cfg.threshold, 1.0), fl(cfg.reset, 0.0), refract, cfg.batch, steps,
            ss, ctypes.c_void_p(self._rates.data_ptr()), cfg.seed, ctypes.c_void_p(self._counts.data_ptr()),
            ctypes.c_void_p(self._rec.data_ptr()) if self._rec is not None else None,
            -int(stages) if stages else int(bool(autotune)),
            int(segment_steps), ctypes.c_void_p(self._stream.cuda_stream), ctypes.byref(self._h)))

    def run(self):
        """One graph launch; returns (synaptic events, device ms)."""
        events = ctypes.c_uint64(0)
        ms = ctypes.c_float(0)
        _capi.check(self._lib.knp_gb300_batched_plan_run(self._h, ctypes.byref(events), ctypes.byref(ms)))
        return int(events.value), float(ms.value)

    def info(self):
        """(operand ring depth, layer ring length, {(depth, ring length): ms of the autotuning run})."""
        st = ctypes.c_int(0)
        ring = ctypes.c_int(0)
        t = (ctypes.c_float * 9)()
        _capi.check(self._lib.knp_gb300_batched_plan_info(self._h, ctypes.byref(st), ctypes.byref(ring), t))
        tuned = {(d, r): float(t[3 * ri + d - 2]) for ri, r in enumerate((4, 8, 16)) for d in (2, 3, 4)
                 if t[3 * ri + d - 2] > 0}
        return st.value, ring.value, tuned

    def counts(self) -> np.ndarray:
        return self._counts.cpu().numpy()

    def record(self):
        """Per-step spike bitmaps of every layer: {layer: uint32 [T_max, B, words]}."""
        r = self._rec.cpu().numpy().view(np.uint32).reshape(self._t_max, self._stride)
        out, off = {}, 0
        for layer, w in enumerate(self._words):
            out[layer] = r[:, off:off + self.cfg.batch * w].reshape(self._t_max, self.cfg.batch, w)
            off += self.cfg.batch * w
        return out

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.knp_gb300_batched_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run(cfg: BatchedConfig, record: bool = False, device: int = 0, autotune: bool = False, segment_steps: int = 0):
    """Run the batch once on the GPU. Returns (counts [B, n_L], record or None, events, ms). With
    ``record`` the per-step spike bitmaps of every layer come back as a dict
    {layer: uint32 [T_max, B, words]}; ``segment_steps`` caps the steps per persistent launch."""
    plan = BatchedPlan(cfg, record=record, autotune=autotune, device=device, segment_steps=segment_steps)
    try:
        events, ms = plan.run()
        return plan.counts(), (plan.record() if record else None), events, ms
    finally:
        plan.close()


def spikes_from_bits(words_row: np.ndarray, n: int) -> np.ndarray:
    """Ascending indexes of the set bits of one bitmap row."""
    bits = np.unpackbits(words_row.astype("<u4").view(np.uint8), bitorder="little")[:n]
    return np.nonzero(bits)[0].astype(np.uint32)


def plain_network(cfg: BatchedConfig, samples=None):
    """The same samples as one block-diagonal network for the plain backend (LIF populations,
    delay-1 projections with the same weights as FP32, inputs as one external channel). Sample s of
    the selection occupies neurons [s * n_l, (s + 1) * n_l) of layer l. Returns (network, schedule)."""
    samples = list(range(cfg.batch)) if samples is None else list(samples)
    S = len(samples)
    L = len(cfg.sizes) - 1
    pops = []
    for l in range(1, L + 1):
        a = T.lif_defaults(S * cfg.sizes[l])
        if cfg.leak is not None:
            a["leak_coefficient"] = cfg.leak[l - 1]
        if cfg.threshold is not None:
            a["activation_threshold"] = cfg.threshold[l - 1]
        if cfg.reset is not None:
            a["potential_reset_value"] = cfg.reset[l - 1]
        if cfg.refract is not None:
            a["refract_period"] = cfg.refract[l - 1]
        if cfg.sample_sizes is not None:
            # Neurons beyond a sample's layer size do not exist for it: they never fire.
            pos = np.arange(S * cfg.sizes[l]) % cfg.sizes[l]
            own = np.repeat(np.asarray([cfg.sample_sizes[l][b] for b in samples]), cfg.sizes[l])
            a["activation_threshold"] = np.where(pos < own, a["activation_threshold"], np.float32(np.inf))
        pops.append(N.Population(T.uid_from_int(800 + l), T.LIF, a))
    chan = T.uid_from_int(899)
    projs = []
    for l in range(1, L + 1):
        n_in, n_out = cfg.sizes[l - 1], cfg.sizes[l]
        w = cfg.weights[l - 1]  # [n_out, n_in]
        jj, ii = np.meshgrid(np.arange(n_out, dtype=np.uint32), np.arange(n_in, dtype=np.uint32), indexing="ij")
        pre = np.concatenate([s * n_in + ii.ravel() for s in range(S)]).astype(np.uint32)
        post = np.concatenate([s * n_out + jj.ravel() for s in range(S)]).astype(np.uint32)
        wt = np.tile(w.ravel(), S).astype(np.float32)
        pre_uid = T.NULL_UID if l == 1 else pops[l - 2].uid
        projs.append(N.Projection(T.uid_from_int(850 + l), T.DELTA, pre_uid, pops[l - 1].uid, pre, post, wt,
                                  np.ones(pre.size, np.uint32)))
    net = N.Network(pops, projs, [(projs[0].uid, chan)])
    t_max = int(cfg.steps[samples].max())
    offs = np.zeros(t_max + 1, np.int64)
    chunks = []
    for t in range(t_max):
        parts = [s * cfg.sizes[0] + input_spikes(cfg, b, t) for s, b in enumerate(samples) if t < cfg.steps[b]]
        idx = np.concatenate(parts).astype(np.uint32) if parts else np.zeros(0, np.uint32)
        chunks.append(idx)
        offs[t + 1] = offs[t] + idx.size
    return net, N.SpikeSchedule(chan, offs, np.concatenate(chunks) if chunks else np.zeros(0, np.uint32))
