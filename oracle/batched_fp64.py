"""TEST INFRASTRUCTURE — FP64 oracle of the batched form's samples.

Only tests/ and bench.py's checks import this; the GB300 product path never calls it.

Each sample of a batched configuration (knp_gb300.batched.BatchedConfig) is an independent
feed-forward network of LIF populations joined by all-to-all delay-1 delta projections, driven by
the sample's Bernoulli input spikes. This module steps every sample with the reference LIF
semantics (knp/backends/cpu/cpu-library/include/knp/backends/cpu-library/impl/populations/lif/
lif_impl.h:33-86: outside the refractory period the potential is multiplied by the leak and the
impacts are added; spike iff potential > threshold (strict); then the potential is set to the reset
value and the refractory counter to the period; inside the period the counter counts down and
impacts are ignored) and the delay convention of the delta projection (delta_impl.h:54-114: a spike
at step t reaches the next layer at step t + 1), keeping the potentials in FP64. With BF16 weights
(8 significant bits) and 0/1 spikes every input sum of a layer is exact in FP64, so this is the
exact-arithmetic answer that the FP32 forms (the reference's own FP32 LIF, the plain GPU path and
the tensor-core batched form) are compared with.

Vectorised over samples with numpy: step t of layer l takes the spike matrix of layer l - 1 at step
t - 1 (samples x inputs, 0/1) times the layer's weights in FP64.
"""
from __future__ import annotations

import numpy as np


def input_bits(cfg, t: int) -> np.ndarray:
    """Input spikes of every sample at step t as a bool matrix [batch, n_0] (the counter-based draws
    of knp_gb300.batched.input_spikes, all samples at once)."""
    from knp_gb300 import network as N

    B, n0 = cfg.batch, cfg.sizes[0]
    key = N.stream_key(cfg.seed, N.S_INPUT)
    ctr = (np.uint64(t) * np.uint64(B) + np.arange(B, dtype=np.uint64))[:, None] * np.uint64(n0) + \
        np.arange(n0, dtype=np.uint64)[None, :]
    r = np.clip(np.nan_to_num(cfg.rates.astype(np.float64), nan=0.0), 0.0, 1.0)
    thr = (r * float(1 << 53)).astype(np.uint64)
    bits = (N.rand64(key, ctr) >> np.uint64(11)) < thr
    if cfg.sample_sizes is not None:
        bits &= np.arange(n0)[None, :] < np.asarray(cfg.sample_sizes[0], np.int64)[:, None]
    return bits


def run_fp64(cfg, samples=None):
    """Spikes of every layer at every step: {layer: bool [T_max, S, n_layer]} for the selected samples
    (default: all), layer 0 being the inputs; steps at or beyond a sample's own length are False."""
    samples = np.arange(cfg.batch) if samples is None else np.asarray(samples)
    S = samples.size
    L = len(cfg.sizes) - 1
    t_max = int(cfg.steps[samples].max())
    T_b = cfg.steps[samples].astype(np.int64)
    leak = [1.0 if cfg.leak is None else float(cfg.leak[l]) for l in range(L)]
    thr = [1.0 if cfg.threshold is None else float(cfg.threshold[l]) for l in range(L)]
    rst = [0.0 if cfg.reset is None else float(cfg.reset[l]) for l in range(L)]
    per = [0 if cfg.refract is None else int(cfg.refract[l]) for l in range(L)]
    W = [np.asarray(w, np.float64).T for w in cfg.weights]  # [n_in, n_out]
    exists = []
    for l in range(L + 1):
        n = cfg.sizes[l]
        if cfg.sample_sizes is None:
            exists.append(np.ones((S, n), bool))
        else:
            exists.append(np.arange(n)[None, :] < np.asarray(cfg.sample_sizes[l], np.int64)[samples][:, None])
    V = [np.zeros((S, cfg.sizes[l + 1])) for l in range(L)]
    RC = [np.zeros((S, cfg.sizes[l + 1]), np.int64) for l in range(L)]
    out = {l: np.zeros((t_max, S, cfg.sizes[l]), bool) for l in range(L + 1)}
    for t in range(t_max):
        live = (t < T_b)[:, None]
        out[0][t] = input_bits(cfg, t)[samples] & live
        for l in range(1, L + 1):
            prev = out[l - 1][t - 1] if t > 0 else np.zeros((S, cfg.sizes[l - 1]), bool)
            I = prev.astype(np.float64) @ W[l - 1]
            v, rc = V[l - 1], RC[l - 1]
            free = rc == 0
            here = live & exists[l]
            cand = np.where(free, v * leak[l - 1] + I, v)
            spike = here & free & (cand > thr[l - 1])
            v_new = np.where(spike, rst[l - 1], np.where(here & free, cand, v))
            rc_new = np.where(spike, per[l - 1], np.where(here & ~free, rc - 1, rc))
            V[l - 1], RC[l - 1] = v_new, rc_new
            out[l][t] = spike
    return out


def mismatch(fp64, record_bits, cfg, samples=None, layers=None):
    """(mismatched, compared) over (sample, neuron, step) of the given layers (default 1..L) between
    the FP64 oracle's spikes and a batched record ({layer: uint32 words [T_max, batch, words]}), each
    sample over its own steps."""
    samples = np.arange(cfg.batch) if samples is None else np.asarray(samples)
    L = len(cfg.sizes) - 1
    layers = range(1, L + 1) if layers is None else layers
    T_b = cfg.steps[samples].astype(np.int64)
    mism = total = 0
    for l in layers:
        n = cfg.sizes[l]
        words = record_bits[l][:, samples, :]  # [T, S, w]
        bits = np.unpackbits(words.astype("<u4").view(np.uint8), axis=-1, bitorder="little")[..., :n].astype(bool)
        ref = fp64[l]
        tm = min(ref.shape[0], bits.shape[0])
        live = (np.arange(tm)[:, None] < T_b[None, :])[:, :, None]
        mism += int(((bits[:tm] != ref[:tm]) & live).sum())
        total += int(live.sum()) * n
    return mism, total
