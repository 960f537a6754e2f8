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
    neurons: np.ndarray  # BLIFAT_DTYPE or LIF_DTYPE
    resource: np.ndarray | None = None  # RESOURCE_DTYPE for RESOURCE_STDP_BLIFAT

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

