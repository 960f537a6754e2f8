"""Network description and seeded network / input generators.

The description mirrors what a KNP user hands to ``Backend::load_populations`` /
``load_projections`` (knp/core-library/include/knp/core/population.h, projection.h): populations of
neuron-parameter structs and projections given as synapse lists ``(params, pre, post)``, plus the
backend-level subscriptions of ``Backend::subscribe`` (backend.h:222-226) and the STDP populations
map of an STDP projection (projection.h:133-164).

The generators are counter-based (SplitMix64 of (seed, stream, counter)) so that the host, the CPU
oracle and the device-side generator (knp_gb300/csrc/generate.cu) produce the same synapses and input
spikes at any scale. The reference's own generators seed ``std::mt19937`` from ``std::random_device``
(knp/base-framework/include/knp/framework/projection/synapse_generators.h:279,370,427) and are not
reproducible, so they cannot be shared with an oracle; index order follows them (``all_to_all``:
pre = i % N_pre, post = i / N_pre, :59-69; ``FixedNumberPre``: post = i % N_post, :410-457).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import types as T

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)
_G = np.uint64(0x9E3779B97F4A7C15)
_C = np.uint64(0x632BE59BD9B4E019)


def mix64(x):
    """SplitMix64 finaliser on uint64 (scalars or arrays; arithmetic wraps mod 2^64)."""
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def stream_key(seed: int, stream: int) -> np.uint64:
    with np.errstate(over="ignore"):
        return mix64(np.uint64(seed) * _G + np.uint64(stream))[()]


def rand64(key, ctr):
    """64 random bits for counter(s) ``ctr`` of stream ``key``."""
    ctr = np.asarray(ctr, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return mix64(np.uint64(key) ^ (ctr * _G + _C))


def uniform_int(key, ctr, lo: int, hi: int):
    """Integers uniform in [lo, hi] (multiply-shift on the top 32 bits)."""
    r = rand64(key, ctr) >> np.uint64(32)
    span = np.uint64(hi - lo + 1)
    return (r * span >> np.uint64(32)).astype(np.int64) + lo


def bernoulli_threshold(p: float) -> int:
    """Integer threshold t with P[(rand >> 11) < t] = p (p quantised to 2^-53)."""
    return int(min(max(p, 0.0), 1.0) * float(1 << 53))


def bernoulli(key, ctr, p: float):
    return (rand64(key, ctr) >> np.uint64(11)) < np.uint64(bernoulli_threshold(p))


# Stream ids: one per generated quantity, so that changing one does not shift the others.
S_PRE, S_WEIGHT, S_DELAY, S_EXISTS, S_INPUT, S_IMAGE = range(1, 7)


@dataclass
class Population:
    uid: bytes
    kind: int
    neurons: np.ndarray  # BLIFAT_DTYPE, LIF_DTYPE or ALTAI_DTYPE
    resource: np.ndarray | None = None  # RESOURCE_DTYPE for the resource-STDP kinds

    @property
    def size(self) -> int:
        return int(self.neurons.shape[0])


@dataclass
class Projection:
    uid: bytes
    kind: int
    pre_uid: bytes
    post_uid: bytes
    pre: np.ndarray  # uint32
    post: np.ndarray  # uint32
    weight: np.ndarray  # float32
    delay: np.ndarray  # uint32
    out_type: np.ndarray | None = None  # uint8; None = all EXCITATORY
    tau_plus: np.ndarray | None = None  # float32, additive STDP only
    tau_minus: np.ndarray | None = None
    stdp_populations: dict = field(default_factory=dict)  # uid -> STDP_ONLY / STDP_AND_SPIKE
    rule: np.ndarray | None = None  # RESOURCE_SYNAPSE_DTYPE, resource-STDP synapses only
    locked: bool = True  # resource-STDP: weights start locked (projection.h:384-396)

    @property
    def size(self) -> int:
        return int(self.pre.shape[0])


@dataclass
class Network:
    populations: list = field(default_factory=list)
    projections: list = field(default_factory=list)
    subscriptions: list = field(default_factory=list)  # (receiver uid, sender uid)


@dataclass
class SpikeSchedule:
    """External spike messages of one sender channel: step t sends indexes[offsets[t]:offsets[t+1]]."""

    sender: bytes
    offsets: np.ndarray  # int64, n_steps + 1
    indexes: np.ndarray  # uint32

    @property
    def n_steps(self) -> int:
        return int(self.offsets.shape[0] - 1)

    def at(self, t: int) -> np.ndarray:
        if t >= self.n_steps:
            return self.indexes[:0]
        return self.indexes[self.offsets[t] : self.offsets[t + 1]]


def bernoulli_schedule(sender: bytes, seed: int, n_sources: int, n_steps: int, p, stream: int = S_INPUT,
                       step0: int = 0) -> SpikeSchedule:
    """Source s spikes at step t iff bernoulli(seed, stream, t * n_sources + s) < p[s]."""
    key = stream_key(seed, stream)
    p = np.broadcast_to(np.asarray(p, dtype=np.float64), (n_sources,))
    thr = (np.clip(p, 0.0, 1.0) * float(1 << 53)).astype(np.uint64)
    offs = np.zeros(n_steps + 1, dtype=np.int64)
    chunks = []
    src = np.arange(n_sources, dtype=np.uint64)
    for t in range(n_steps):
        r = rand64(key, np.uint64(step0 + t) * np.uint64(n_sources) + src) >> np.uint64(11)
        idx = np.nonzero(r < thr)[0].astype(np.uint32)
        chunks.append(idx)
        offs[t + 1] = offs[t] + idx.size
    return SpikeSchedule(sender, offs, np.concatenate(chunks) if chunks else np.zeros(0, np.uint32))


def dyadic_weights(key, ctr, k_lo: int, k_hi: int) -> np.ndarray:
    return (uniform_int(key, ctr, k_lo, k_hi).astype(np.float64) / 256.0).astype(np.float32)


# ----------------------------------------------------------------------------- configurations


def small_network(seed: int = 1, n: int = 1000, n_in: int = 100, p_rec: float = 0.1, steps: int = 1000,
                  p_in: float = 0.05):
    """Plain method, small: n BLIFAT (defaults), n_in Bernoulli(p_in) sources through an all-to-all
    input projection (w = k/256, k in [0, 64], delay 1..4) and a recurrent projection with connection
    probability p_rec (w = k/256, k in [-32, 32], delay 1..5)."""
    pop_uid, in_uid, rec_uid, chan_uid = (T.uid_from_int(seed * 100 + i) for i in (1, 2, 3, 4))
    pop = Population(pop_uid, T.BLIFAT, T.blifat_defaults(n))
    i = np.arange(n_in * n, dtype=np.uint64)
    proj_in = Projection(
        in_uid, T.DELTA, T.NULL_UID, pop_uid,
        pre=(i % np.uint64(n_in)).astype(np.uint32), post=(i // np.uint64(n_in)).astype(np.uint32),
        weight=dyadic_weights(stream_key(seed, 10 + S_WEIGHT), i, 0, 64),
        delay=uniform_int(stream_key(seed, 10 + S_DELAY), i, 1, 4).astype(np.uint32))
    j = np.arange(n * n, dtype=np.uint64)
    keep = bernoulli(stream_key(seed, 20 + S_EXISTS), j, p_rec)
    j = j[keep]
    proj_rec = Projection(
        rec_uid, T.DELTA, pop_uid, pop_uid,
        pre=(j % np.uint64(n)).astype(np.uint32), post=(j // np.uint64(n)).astype(np.uint32),
        weight=dyadic_weights(stream_key(seed, 20 + S_WEIGHT), j, -32, 32),
        delay=uniform_int(stream_key(seed, 20 + S_DELAY), j, 1, 5).astype(np.uint32))
    net = Network([pop], [proj_in, proj_rec], [(in_uid, chan_uid)])
    sched = bernoulli_schedule(chan_uid, seed, n_in, steps, p_in)
    return net, [sched]


def fixed_fan_in_pre(key_pre, key_w, key_d, n_pre: int, n_post: int, fan_in: int, k_lo: int, k_hi: int,
                     d_lo: int, d_hi: int, start: int = 0, count: int | None = None):
    """Synapses [start, start+count) of a FixedNumberPre-style projection: synapse i has
    post = i % n_post, pre uniform in [0, n_pre), w = k/256 with k uniform in [k_lo, k_hi], delay
    uniform in [d_lo, d_hi]."""
    total = n_post * fan_in
    count = total - start if count is None else count
    i = np.arange(start, start + count, dtype=np.uint64)
    pre = uniform_int(key_pre, i, 0, n_pre - 1).astype(np.uint32)
    post = (i % np.uint64(n_post)).astype(np.uint32)
    w = dyadic_weights(key_w, i, k_lo, k_hi)
    d = uniform_int(key_d, i, d_lo, d_hi).astype(np.uint32)
    return pre, post, w, d


def generated_synapses(kind: int, n_pre: int, n_post: int, k_lo: int, k_hi: int, d_lo: int, d_hi: int, seed: int,
                       stream: int, count: int = 0, probability: float = 0.0):
    """The synapses (pre, post, weight, delay), in synapse order, of knp_gb300_generate_projection:
    synapse i connects the pair of the generator's index rule (synapse_generators.h:58-457), with
    weight k/256 (k uniform in [k_lo, k_hi]) and delay uniform in [d_lo, d_hi] drawn for i."""
    key_pre, key_w, key_d = (stream_key(seed, stream + k) for k in (1, 2, 3))
    key_post, key_prob = stream_key(seed, stream + 4), stream_key(seed, stream + 5)
    if kind == T.GEN_ALL_TO_ALL:
        i = np.arange(n_pre * n_post, dtype=np.uint64)
        pre, post = i % np.uint64(n_pre), i // np.uint64(n_pre)
    elif kind == T.GEN_ALIGNED:
        i = np.arange(max(n_pre, n_post), dtype=np.uint64)
        if n_pre >= n_post:
            pre, post = i, i // np.uint64(n_pre // n_post)
        else:
            pre, post = i // np.uint64(n_post // n_pre), i
    elif kind == T.GEN_EXCLUSIVE:
        i = np.arange(n_pre * (n_pre - 1), dtype=np.uint64)
        pre, to = i // np.uint64(n_pre - 1), i % np.uint64(n_pre - 1)
        post = np.where(to >= pre, to + np.uint64(1), to)
    elif kind == T.GEN_ONE_TO_ONE:
        i = np.arange(n_pre, dtype=np.uint64)
        pre = post = i
    elif kind == T.GEN_FIXED_PROBABILITY:
        c = np.arange(n_pre * n_post, dtype=np.uint64)
        kept = c[(rand64(key_prob, c) >> np.uint64(11)) < np.uint64(bernoulli_threshold(probability))]
        i = np.arange(kept.size, dtype=np.uint64)
        pre, post = kept % np.uint64(n_pre), kept // np.uint64(n_pre)
    elif kind == T.GEN_FIXED_NUMBER_POST:
        i = np.arange(count, dtype=np.uint64)
        pre, post = i % np.uint64(n_pre), uniform_int(key_post, i, 0, n_post - 1)
    elif kind == T.GEN_FIXED_NUMBER_PRE:
        i = np.arange(count, dtype=np.uint64)
        pre, post = uniform_int(key_pre, i, 0, n_pre - 1), i % np.uint64(n_post)
    else:
        raise ValueError(f"unknown generator kind {kind}")
    w = dyadic_weights(key_w, i, k_lo, k_hi)
    d = uniform_int(key_d, i, d_lo, d_hi).astype(np.uint32)
    return (np.asarray(pre).astype(np.uint32), np.asarray(post).astype(np.uint32), w, d)


LARGE_SEED_STREAM = 30


def large_sparse_network(seed: int = 2, n: int = 1_000_000, fan_in: int = 1000, p_bg: float = 0.005,
                         steps: int = 500, with_schedule: bool = True):
    """Large sparse plain method: n BLIFAT (defaults), fixed fan-in from uniform random presynaptic
    sources (w = k/256, k in [-16, 48], delay 1..20), and Bernoulli(p_bg) background drive per neuron
    through a one-to-one projection (w = 1.0, delay 1)."""
    pop_uid, rec_uid, bg_uid, chan_uid = (T.uid_from_int(seed * 100 + i) for i in (1, 2, 3, 4))
    pop = Population(pop_uid, T.BLIFAT, T.blifat_defaults(n))
    s = LARGE_SEED_STREAM
    pre, post, w, d = fixed_fan_in_pre(stream_key(seed, s + S_PRE), stream_key(seed, s + S_WEIGHT),
                                       stream_key(seed, s + S_DELAY), n, n, fan_in, -16, 48, 1, 20)
    rec = Projection(rec_uid, T.DELTA, pop_uid, pop_uid, pre, post, w, d)
    ar = np.arange(n, dtype=np.uint32)
    bg = Projection(bg_uid, T.DELTA, T.NULL_UID, pop_uid, ar, ar.copy(), np.ones(n, np.float32),
                    np.ones(n, np.uint32))
    net = Network([pop], [bg, rec], [(bg_uid, chan_uid)])
    scheds = [bernoulli_schedule(chan_uid, seed, n, steps, p_bg)] if with_schedule else []
    return net, scheds


def blob_images(seed: int, n_images: int, side: int = 28) -> np.ndarray:
    """Seeded synthetic images: 1-4 Gaussian blobs each, intensities in [0, 1], shape (n, side*side)."""
    key = stream_key(seed, S_IMAGE)
    yy, xx = np.mgrid[0:side, 0:side].astype(np.float64)
    out = np.zeros((n_images, side * side), dtype=np.float64)
    for m in range(n_images):
        base = np.uint64(m * 64)
        nb = int(uniform_int(key, base, 1, 4))
        img = np.zeros((side, side))
        for b in range(nb):
            c = base + np.uint64(1 + 4 * b)
            cy = float(uniform_int(key, c, 4, side - 5))
            cx = float(uniform_int(key, c + np.uint64(1), 4, side - 5))
            sg = 1.5 + float(uniform_int(key, c + np.uint64(2), 0, 300)) / 100.0
            amp = 0.5 + float(uniform_int(key, c + np.uint64(3), 0, 50)) / 100.0
            img += amp * np.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2 * sg * sg))
        out[m] = np.clip(img, 0.0, 1.0).reshape(-1)
    return out


def stdp_network(seed: int = 3, n_in: int = 784, n: int = 800, samples: int = 200, steps_per_sample: int = 100,
                 tau: float = 20.0, w_max: float = 0.1):
    """STDP learning: rate-coded synthetic 28x28 blob images (p = 0.1 * intensity per step) into an
    all-to-all additive-STDP projection (784 -> 800, w uniform in [0, w_max], tau+ = tau- = tau,
    delay 1) onto resource-STDP BLIFAT neurons (defaults), with all-to-all lateral weight -1.0
    (delay 1). The post population is an STDP population of the plastic projection (STDPAndSpike),
    as in knp/tests/backend/single_thread_cpu_test.cpp:123-124."""
    pop_uid, in_uid, lat_uid, chan_uid = (T.uid_from_int(seed * 100 + i) for i in (1, 2, 3, 4))
    pop = Population(pop_uid, T.RESOURCE_STDP_BLIFAT, T.blifat_defaults(n), T.resource_defaults(n))
    i = np.arange(n_in * n, dtype=np.uint64)
    # w = k * 2^-27, k uniform in [0, w_max * 2^27]: uniform on [0, w_max] at FP32 resolution.
    k = uniform_int(stream_key(seed, 40 + S_WEIGHT), i, 0, int(w_max * (1 << 27)))
    w = (k.astype(np.float64) * 2.0 ** -27).astype(np.float32)
    plastic = Projection(
        in_uid, T.ADDITIVE_STDP_DELTA, T.NULL_UID, pop_uid,
        pre=(i % np.uint64(n_in)).astype(np.uint32), post=(i // np.uint64(n_in)).astype(np.uint32),
        weight=w, delay=np.ones(i.size, np.uint32),
        tau_plus=np.full(i.size, tau, np.float32), tau_minus=np.full(i.size, tau, np.float32),
        stdp_populations={pop_uid: T.STDP_AND_SPIKE})
    j = np.arange(n * n, dtype=np.uint64)
    lateral = Projection(
        lat_uid, T.DELTA, pop_uid, pop_uid,
        pre=(j % np.uint64(n)).astype(np.uint32), post=(j // np.uint64(n)).astype(np.uint32),
        weight=np.full(j.size, -1.0, np.float32), delay=np.ones(j.size, np.uint32))
    net = Network([pop], [plastic, lateral], [(in_uid, chan_uid)])
    images = blob_images(seed, samples)[:, :n_in]  # 28x28 pixels; smaller test networks use the first n_in
    key = stream_key(seed, S_INPUT)
    total = samples * steps_per_sample
    offs = np.zeros(total + 1, np.int64)
    chunks = []
    src = np.arange(n_in, dtype=np.uint64)
    for t in range(total):
        p = 0.1 * images[t // steps_per_sample]
        thr = (p * float(1 << 53)).astype(np.uint64)
        r = rand64(key, np.uint64(t) * np.uint64(n_in) + src) >> np.uint64(11)
        idx = np.nonzero(r < thr)[0].astype(np.uint32)
        chunks.append(idx)
        offs[t + 1] = offs[t] + idx.size
    return net, [SpikeSchedule(chan_uid, offs, np.concatenate(chunks))]


def smallest_network(kind: str = "delta"):
    """The reference's one-neuron test network (knp/tests/backend/single_thread_cpu_test.cpp:54-176,
    fixtures knp/tests/common/generators.h:48-57): input -> input projection (w 1.0, delay 1) ->
    population <-> loop projection (w 1.1, delay 6 for delta; w 1.0, delay 6, tau {1,1} for the
    additive-STDP variant, whose input projection has tau {2,2}). Input spikes on steps 0, 5, 10, 15
    (tests_messaging_common.h:34-44)."""
    pop_uid, in_uid, loop_uid, chan_uid = (T.uid_from_int(900 + i) for i in (1, 2, 3, 4))
    one = np.zeros(1, np.uint32)
    if kind == "delta":
        pop = Population(pop_uid, T.BLIFAT, T.blifat_defaults(1))
        inp = Projection(in_uid, T.DELTA, T.NULL_UID, pop_uid, one, one, np.ones(1, np.float32), np.ones(1, np.uint32))
        loop = Projection(loop_uid, T.DELTA, pop_uid, pop_uid, one, one, np.full(1, 1.1, np.float32),
                          np.full(1, 6, np.uint32))
    elif kind in ("stdp", "stdp_resource_neuron"):
        if kind == "stdp":
            pop = Population(pop_uid, T.BLIFAT, T.blifat_defaults(1))
        else:
            pop = Population(pop_uid, T.RESOURCE_STDP_BLIFAT, T.blifat_defaults(1), T.resource_defaults(1))
        inp = Projection(in_uid, T.ADDITIVE_STDP_DELTA, T.NULL_UID, pop_uid, one, one, np.ones(1, np.float32),
                         np.ones(1, np.uint32), tau_plus=np.full(1, 2, np.float32), tau_minus=np.full(1, 2, np.float32))
        loop = Projection(loop_uid, T.ADDITIVE_STDP_DELTA, pop_uid, pop_uid, one, one, np.ones(1, np.float32),
                          np.full(1, 6, np.uint32), tau_plus=np.ones(1, np.float32), tau_minus=np.ones(1, np.float32),
                          stdp_populations={pop_uid: T.STDP_AND_SPIKE})
    elif kind in ("resource_stdp", "resource_stdp_altai"):
        # single_thread_cpu_test.cpp:179-355: synaptic-resource STDP synapses (input rule {resource 0,
        # w_min 1, w_max 2, d_u 0.1}, loop rule {0, 1, 2}) onto one resource-STDP neuron (BLIFAT or
        # AltAI-LIF; synaptic resource threshold 1, free resource 2, isi_max 0), learning started.
        res = T.resource_defaults(1)
        res["synaptic_resource_threshold"] = 1.0
        res["free_synaptic_resource"] = 2.0
        res["isi_max"] = 0
        if kind == "resource_stdp":
            pop = Population(pop_uid, T.RESOURCE_STDP_BLIFAT, T.blifat_defaults(1), res)
        else:
            pop = Population(pop_uid, T.RESOURCE_STDP_ALTAI_LIF, T.altai_defaults(1), res)
        rule_in = T.resource_synapse_defaults(1)
        rule_in["w_min"], rule_in["w_max"], rule_in["d_u"] = 1.0, 2.0, np.float32(0.1)
        rule_loop = T.resource_synapse_defaults(1)
        rule_loop["w_min"], rule_loop["w_max"] = 1.0, 2.0
        inp = Projection(in_uid, T.RESOURCE_STDP_DELTA, T.NULL_UID, pop_uid, one, one, np.ones(1, np.float32),
                         np.ones(1, np.uint32), rule=rule_in, locked=False)
        loop = Projection(loop_uid, T.RESOURCE_STDP_DELTA, pop_uid, pop_uid, one, one, np.ones(1, np.float32),
                          np.full(1, 6, np.uint32), rule=rule_loop, locked=False)
    else:
        raise ValueError(kind)
    net = Network([pop], [inp, loop], [(in_uid, chan_uid)])
    offs = np.zeros(21, np.int64)
    idx = []
    for t in range(20):
        if t % 5 == 0:
            idx.append(0)
        offs[t + 1] = len(idx)
    return net, [SpikeSchedule(chan_uid, offs, np.array(idx, np.uint32))]


def blocking_network(seed: int = 12, n: int = 400, n_in: int = 100, steps: int = 300):
    """BLOCKING synapses (blifat_impl.h:86: the step's last BLOCKING impact in message order sets the
    neuron's total blocking period) beside excitatory drive: n BLIFAT neurons (defaults); channel A ->
    excitatory projection (p 0.2, w k/256 with k in [0, 96], delays 1..3); channel B -> BLOCKING
    projection (p 0.05 plus repeated (pre, post) pairs, weights from {-3, -1.5, 2, 4.7, -6.2, 1}, delays
    1..4); a recurrent excitatory projection (p 0.05, k in [-32, 64], delays 1..5) and a recurrent
    BLOCKING projection (p 0.01, weights -2 or 3, delays 1..2). Inputs: A Bernoulli 0.1, B 0.05. The
    population also takes external impact messages from channel uid_from_int(1203)."""
    rng = np.random.default_rng(seed)
    pop_uid = T.uid_from_int(1200)
    pop = Population(pop_uid, T.BLIFAT, T.blifat_defaults(n))
    chan_a, chan_b, chan_ext = T.uid_from_int(1201), T.uid_from_int(1202), T.uid_from_int(1203)

    def rand_proj(uid, pre_uid, n_pre, p, weights_fn, d_lo, d_hi, out, extra_pairs=0):
        pre, post = np.nonzero(rng.random((n_pre, n)) < p)
        if extra_pairs:
            k = rng.integers(0, pre.size, extra_pairs)
            pre = np.concatenate([pre, pre[k]])
            post = np.concatenate([post, post[k]])
        w = np.asarray(weights_fn(pre.size), np.float32)
        d = rng.integers(d_lo, d_hi + 1, pre.size).astype(np.uint32)
        return Projection(uid, T.DELTA, pre_uid, pop_uid, pre.astype(np.uint32), post.astype(np.uint32), w, d,
                          out_type=np.full(pre.size, out, np.uint8))

    blk_w = np.float32([-3, -1.5, 2, 4.7, -6.2, 1])
    projs = [
        rand_proj(T.uid_from_int(1210), T.NULL_UID, n_in, 0.2, lambda s: rng.integers(0, 97, s) / 256.0, 1, 3,
                  T.EXCITATORY),
        rand_proj(T.uid_from_int(1211), T.NULL_UID, n_in, 0.05, lambda s: blk_w[rng.integers(0, blk_w.size, s)], 1, 4,
                  T.BLOCKING, extra_pairs=200),
        rand_proj(T.uid_from_int(1212), pop_uid, n, 0.05, lambda s: rng.integers(-32, 65, s) / 256.0, 1, 5,
                  T.EXCITATORY),
        rand_proj(T.uid_from_int(1213), pop_uid, n, 0.01, lambda s: np.where(rng.random(s) < 0.5, -2.0, 3.0), 1, 2,
                  T.BLOCKING),
    ]
    net = Network([pop], projs, [(T.uid_from_int(1210), chan_a), (T.uid_from_int(1211), chan_b),
                                 (pop_uid, chan_ext)])
    return net, [bernoulli_schedule(chan_a, seed, n_in, steps, 0.1),
                 bernoulli_schedule(chan_b, seed, n_in, steps, 0.05, stream=S_INPUT + 50)]


def _aligned(n_pre: int, n_post: int):
    """The reference's aligned synapse generator (synapse_generators.h:94-120): max(n_pre, n_post)
    synapses; the larger side is indexed by the synapse index, the other by index / pack size."""
    i = np.arange(max(n_pre, n_post), dtype=np.uint32)
    if n_pre >= n_post:
        return i, i // np.uint32(n_pre // n_post)
    return i // np.uint32(n_post // n_pre), i


def resource_stdp_network(seed: int = 21, samples: int = 20, n_in: int = 784, per_column: int = 20,
                          classes: int = 10, potential_decay: float = 0.0, steps_per_sample: int = 15,
                          active_steps: int = 10, label_step: int = 11):
    """A network shaped like the reference's mnist-learn BLIFAT model (examples/mnist-learn/models/
    blifat/construct_network.cpp:64-223, hyperparameters.h:35-117) on synthetic blob images: an
    image channel (n_in) -> all-to-all SynapticResourceSTDPDeltaSynapse projection (w_min -0.253, w_max
    0.0924, dopamine plasticity period 10, resource from weight 0) -> INPUT (classes * per_column
    resource-STDP BLIFAT neurons: threshold 8.571, d_h -0.177, dopamine plasticity time 10, threshold
    coefficient 0.218, isi_max 10, min potential 0, stability change 0.05, drain 27) -> OUTPUT (classes)
    -> GATE (classes) by aligned delta projections (w 10; BLOCKING -10 output -> gate), the label
    channel -> INPUT (DOPAMINE 0.18, delay 3; EXCITATORY -30, delay 4) and -> GATE (10), GATE -> INPUT
    (10). Image pixels spike with p = 0.2 * intensity on the first `active_steps` steps of each
    `steps_per_sample`-step sample; the label neuron (sample index mod classes) spikes at step
    `label_step` of the sample (spike_generators.cpp: the 11th of 15 steps). The input neurons'
    potential decay is a parameter (mnist-learn uses 2/3; the default 0 keeps every FP32 potential
    exact). The framework-level winner-take-all is not part of the backend and not modelled.
    Learning is on (every projection unlocked)."""
    n = classes * per_column
    uid = lambda k: T.uid_from_int(seed * 1000 + k)
    in_uid, out_uid, gate_uid = uid(1), uid(2), uid(3)
    raster_chan, label_chan = uid(10), uid(11)
    nn = T.blifat_defaults(n)
    nn["activation_threshold"] = np.float32(8.571)
    nn["potential_decay"] = potential_decay
    nn["min_potential"] = 0.0
    res = T.resource_defaults(n)
    res["d_h"] = np.float32(-0.177)
    res["dopamine_plasticity_time"] = 10
    res["synapse_sum_threshold_coefficient"] = np.float32(0.218)
    res["isi_max"] = 10
    res["stability_change_parameter"] = np.float32(0.05)
    res["resource_drain_coefficient"] = 27
    default = T.blifat_defaults(classes)
    default["activation_threshold"] = np.float32(8.571)
    pops = [Population(in_uid, T.RESOURCE_STDP_BLIFAT, nn, res),
            Population(out_uid, T.RESOURCE_STDP_BLIFAT, default, T.resource_defaults(classes)),
            Population(gate_uid, T.RESOURCE_STDP_BLIFAT, default.copy(), T.resource_defaults(classes))]
    w_min, w_max = np.float32(-0.253), np.float32(0.0924)
    diff, over = np.float32(w_max - w_min), np.float32(np.float32(0.0) - w_min)
    r0 = np.float32(float(over) * float(diff) / (float(diff) - float(over)))  # resource_from_weight(0, ...)
    i = np.arange(n_in * n, dtype=np.uint64)
    rule = T.resource_synapse_defaults(i.size)
    rule["synaptic_resource"] = r0
    rule["w_min"], rule["w_max"] = w_min, w_max
    rule["dopamine_plasticity_period"] = 10
    projs = [Projection(uid(20), T.RESOURCE_STDP_DELTA, T.NULL_UID, in_uid,
                        pre=(i % np.uint64(n_in)).astype(np.uint32), post=(i // np.uint64(n_in)).astype(np.uint32),
                        weight=np.zeros(i.size, np.float32), delay=np.ones(i.size, np.uint32), rule=rule, locked=False)]

    def aligned(k, pre_uid, n_pre, post_uid, n_post, w, d, ty):
        pre, post = _aligned(n_pre, n_post)
        return Projection(uid(k), T.DELTA, pre_uid, post_uid, pre, post, np.full(pre.size, w, np.float32),
                          np.full(pre.size, d, np.uint32), out_type=np.full(pre.size, ty, np.uint8))

    projs += [aligned(21, T.NULL_UID, classes, in_uid, n, 0.18, 3, T.DOPAMINE),
              aligned(22, in_uid, n, out_uid, classes, 10.0, 1, T.EXCITATORY),
              aligned(23, out_uid, classes, gate_uid, classes, -10.0, 1, T.BLOCKING),
              aligned(24, T.NULL_UID, classes, gate_uid, classes, 10.0, 1, T.EXCITATORY),
              aligned(25, gate_uid, classes, in_uid, n, 10.0, 1, T.EXCITATORY),
              aligned(26, T.NULL_UID, classes, in_uid, n, -30.0, 4, T.EXCITATORY)]
    subs = [(uid(20), raster_chan)] + [(uid(k), label_chan) for k in (21, 24, 26)]
    net = Network(pops, projs, subs)
    images = blob_images(seed, samples)[:, :n_in]
    key = stream_key(seed, S_INPUT)
    total = samples * steps_per_sample
    offs, loffs = np.zeros(total + 1, np.int64), np.zeros(total + 1, np.int64)
    chunks, labels = [], []
    src = np.arange(n_in, dtype=np.uint64)
    for t in range(total):
        m, local = divmod(t, steps_per_sample)
        idx = np.zeros(0, np.uint32)
        if local < active_steps:
            thr = (0.2 * images[m] * float(1 << 53)).astype(np.uint64)
            r = rand64(key, np.uint64(t) * np.uint64(n_in) + src) >> np.uint64(11)
            idx = np.nonzero(r < thr)[0].astype(np.uint32)
        chunks.append(idx)
        offs[t + 1] = offs[t] + idx.size
        if local == label_step:
            labels.append(m % classes)
        loffs[t + 1] = len(labels)
    return net, [SpikeSchedule(raster_chan, offs, np.concatenate(chunks)),
                 SpikeSchedule(label_chan, loffs, np.array(labels, np.uint32))]


def resource_stdp_mixed_network(seed: int = 23, n: int = 300, n_in: int = 100, n_plain: int = 50, steps: int = 300):
    """Every path of the resource-STDP training on one network: n resource-STDP BLIFAT neurons with
    per-neuron ISI, Hebbian, dopamine, threshold-coefficient, drain and renormalisation parameters;
    channel X (n_in) -> resource-STDP projection (p 0.2, per-synapse resource, weight bounds, d_u,
    dopamine period, delays 1..4; unlocked); a recurrent resource-STDP projection (p 0.03, delays
    1..3; loaded locked); channel F -> forcing delta projection (EXCITATORY 2.0, aligned); channel D ->
    DOPAMINE delta projection (+-0.3, aligned); and channel X -> a resource-STDP projection into a
    plain BLIFAT population (not trained; its synapses still record spike steps). Inputs: X
    Bernoulli 0.05, F 0.01, D 0.02 per source and step."""
    rng = np.random.default_rng(seed)
    uid = lambda k: T.uid_from_int(seed * 1000 + k)
    a_uid, b_uid = uid(1), uid(2)
    cx, cf, cd = uid(10), uid(11), uid(12)
    res = T.resource_defaults(n)
    pick = lambda vals: np.asarray(vals)[rng.integers(0, len(vals), n)]
    res["isi_max"] = pick([0, 1, 3, 8])
    res["d_h"] = pick(np.float32([0.5, 1.0, -0.2]))
    res["stability_change_at_isi"] = np.float32(0.25)
    res["stability_change_parameter"] = np.float32(0.1)
    res["dopamine_plasticity_time"] = pick([1, 5])
    res["synapse_sum_threshold_coefficient"] = pick(np.float32([0.0, 0.01, 0.05]))
    res["resource_drain_coefficient"] = pick([0, 3])
    res["synaptic_resource_threshold"] = pick(np.float32([T.FLT_MAX, 0.5, 2.0]))
    res["free_synaptic_resource"] = pick(np.float32([1.0, 0.0, 3.0]))
    pops = [Population(a_uid, T.RESOURCE_STDP_BLIFAT, T.blifat_defaults(n), res),
            Population(b_uid, T.BLIFAT, T.blifat_defaults(n_plain))]

    def rule_for(size, lo_choices, hi_choices):
        r = T.resource_synapse_defaults(size)
        r["synaptic_resource"] = (rng.integers(0, 64, size) / 32.0).astype(np.float32)
        r["w_min"] = np.asarray(lo_choices, np.float32)[rng.integers(0, len(lo_choices), size)]
        r["w_max"] = np.asarray(hi_choices, np.float32)[rng.integers(0, len(hi_choices), size)]
        r["d_u"] = np.float32([0.0, 0.01])[rng.integers(0, 2, size)]
        r["dopamine_plasticity_period"] = np.array([0, 2, 5])[rng.integers(0, 3, size)]
        return r

    def random_proj(k, pre_uid, n_pre, post_uid, n_post, p, d_hi, lo, hi, locked):
        pre, post = np.nonzero(rng.random((n_pre, n_post)) < p)
        rule = rule_for(pre.size, lo, hi)
        w = (rng.integers(-64, 64, pre.size) / 64.0).astype(np.float32)
        return Projection(uid(k), T.RESOURCE_STDP_DELTA, pre_uid, post_uid, pre.astype(np.uint32),
                          post.astype(np.uint32), w, rng.integers(1, d_hi + 1, pre.size).astype(np.uint32), rule=rule,
                          locked=locked)

    x_proj = random_proj(20, T.NULL_UID, n_in, a_uid, n, 0.2, 4, [0.0, -0.5], [1.0, 2.0], False)
    rec = random_proj(21, a_uid, n, a_uid, n, 0.03, 3, [-0.5], [0.5], True)
    one = np.arange(n, dtype=np.uint32)
    force = Projection(uid(22), T.DELTA, T.NULL_UID, a_uid, one, one, np.full(n, 2.0, np.float32), np.ones(n, np.uint32))
    dopa = Projection(uid(23), T.DELTA, T.NULL_UID, a_uid, one, one,
                      np.where(one % 3 == 0, -0.3, 0.3).astype(np.float32), np.ones(n, np.uint32),
                      out_type=np.full(n, T.DOPAMINE, np.uint8))
    plain = random_proj(24, T.NULL_UID, n_in, b_uid, n_plain, 0.2, 2, [0.0], [1.0], False)
    net = Network(pops, [x_proj, rec, force, dopa, plain],
                  [(uid(20), cx), (uid(24), cx), (uid(22), cf), (uid(23), cd)])
    return net, [bernoulli_schedule(cx, seed, n_in, steps, 0.05, stream=S_INPUT),
                 bernoulli_schedule(cf, seed, n, steps, 0.01, stream=S_INPUT + 100),
                 bernoulli_schedule(cd, seed, n, steps, 0.02, stream=S_INPUT + 200)]


def altai_network(seed: int = 31, n: int = 200, n_in: int = 80, steps: int = 200):
    """AltAI-LIF neurons (altai_impl.h:33-168) with every option: per-neuron is_diff / is_reset /
    leak_rev / saturate / do_not_save, thresholds 20..60, negative thresholds 10..100, leaks -3..3,
    resets 0..5. Channel A -> excitatory/inhibitory delta projection (p 0.3, integer weights -8..16,
    delays 1..4); a recurrent delta projection (p 0.05, integer weights -6..10, delays 1..3); channel B
    -> BLOCKING projection (p 0.05 plus repeated pairs, weights from {-3, -1, 2, 4, 5, -6}, delays
    1..2); channel D -> DOPAMINE (aligned, 0.5). Integer weights keep every FP32 partial sum exact, so
    the order of the reference's impact-by-impact sum does not matter. External impacts may be sent
    from channel uid 3103. Inputs: A Bernoulli 0.1, B 0.03, D 0.02."""
    rng = np.random.default_rng(seed)
    uid = lambda k: T.uid_from_int(3100 + k)
    pop_uid = uid(0)
    a = T.altai_defaults(n)
    for f in ("is_diff", "is_reset", "leak_rev", "saturate", "do_not_save"):
        a[f] = rng.random(n) < (0.1 if f == "do_not_save" else 0.5)
    a["activation_threshold"] = rng.integers(20, 61, n)
    a["negative_activation_threshold"] = rng.integers(10, 101, n)
    a["potential_leak"] = rng.integers(-3, 4, n)
    a["potential_reset_value"] = rng.integers(0, 6, n)
    pop = Population(pop_uid, T.ALTAI_LIF, a)

    def rand_proj(k, pre_uid, n_pre, p, wfn, d_lo, d_hi, types, extra=0):
        pre, post = np.nonzero(rng.random((n_pre, n)) < p)
        if extra:
            j = rng.integers(0, pre.size, extra)
            pre, post = np.concatenate([pre, pre[j]]), np.concatenate([post, post[j]])
        ty = np.asarray(types, np.uint8)[rng.integers(0, len(types), pre.size)]
        return Projection(uid(k), T.DELTA, pre_uid, pop_uid, pre.astype(np.uint32), post.astype(np.uint32),
                          np.asarray(wfn(pre.size), np.float32), rng.integers(d_lo, d_hi + 1, pre.size).astype(np.uint32),
                          out_type=ty)

    blk = np.float32([-3, -1, 2, 4, 5, -6])
    one = np.arange(n, dtype=np.uint32)
    projs = [
        rand_proj(10, T.NULL_UID, n_in, 0.3, lambda s: rng.integers(-8, 17, s), 1, 4, [T.EXCITATORY, T.INHIBITORY_CURRENT]),
        rand_proj(11, pop_uid, n, 0.05, lambda s: rng.integers(-6, 11, s), 1, 3, [T.EXCITATORY]),
        rand_proj(12, T.NULL_UID, n_in, 0.05, lambda s: blk[rng.integers(0, blk.size, s)], 1, 2, [T.BLOCKING], extra=100),
        Projection(uid(13), T.DELTA, T.NULL_UID, pop_uid, one, one, np.full(n, 0.5, np.float32), np.ones(n, np.uint32),
                   out_type=np.full(n, T.DOPAMINE, np.uint8)),
    ]
    net = Network([pop], projs, [(uid(10), uid(20)), (uid(12), uid(21)), (uid(13), uid(22)), (pop_uid, uid(3))])
    return net, [bernoulli_schedule(uid(20), seed, n_in, steps, 0.1),
                 bernoulli_schedule(uid(21), seed, n_in, steps, 0.03, stream=S_INPUT + 60),
                 bernoulli_schedule(uid(22), seed, n, steps, 0.02, stream=S_INPUT + 70)]

