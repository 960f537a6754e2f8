"""Parity of the GB300 backend (through the C ABI) with the CPU oracle on the same seeded inputs.

Bar: spike trains bit-exact per step (as ascending index sets) and weights bit-exact wherever the
arithmetic is exact (dyadic weights, default neuron parameters, additive STDP); potentials of
non-default dynamics within the FP32-vs-FP64 tolerance written in each test.
"""
import numpy as np
import pytest

from knp_gb300 import network as N
from knp_gb300 import types as T

pytestmark = pytest.mark.gpu

GOLDEN = [1, 6, 7, 11, 12, 13, 16, 17, 18, 19]


def _gpu():
    from knp_gb300 import backend as B

    return B


# Step modes: AUTO takes the fused step kernel (one CTA cluster) for the small networks of these tests
# and the persistent grid kernel for the larger ones; PHASES keeps the per-phase kernels (population,
# scatter, STDP, end of step); GRID forces the persistent grid kernel (one CTA per SM).
MODES = {"auto": T.STEP_AUTO, "phases": T.STEP_PHASES, "grid": T.STEP_GRID}


def run_both(net, scheds, steps, record=None, device_schedule=False, on_step=None, step_mode=None):
    from oracle import oracle as orc

    B = _gpu()
    g, b = B.run(net, scheds, steps, record=record, device_schedule=device_schedule,
                 on_step=None if on_step is None else (lambda be, t: on_step(be, t, "gpu")),
                 step_mode=None if step_mode is None else MODES[step_mode])
    o, oo = orc.run(net, scheds, steps, record=record,
                    on_step=None if on_step is None else (lambda be, t: on_step(be, t, "oracle")))
    return g, b, o, oo


def assert_same_spikes(g, o):
    for uid in o:
        for t, (a, e) in enumerate(zip(g[uid], o[uid])):
            assert np.array_equal(a, e), f"step {t}: gpu {a[:10]}... ({a.size}) vs oracle {e[:10]}... ({e.size})"


def assert_same_state(b, oo, pop, rtol=0.0):
    gs, gext = b.read_population(pop)
    os_, oext = oo.blifat(pop)
    for f in ("potential", "dynamic_threshold", "postsynaptic_trace", "inhibitory_conductance",
              "additional_threshold", "dopamine_value"):
        exp = os_[f].astype(np.float32).astype(np.float64)
        if rtol == 0.0:
            np.testing.assert_array_equal(gs[f], exp, err_msg=f)
        else:
            np.testing.assert_allclose(gs[f], exp, rtol=rtol, atol=1e-6, err_msg=f)
    for f in ("n_time_steps_since_last_firing", "bursting_phase", "total_blocking_period"):
        np.testing.assert_array_equal(gs[f], os_[f], err_msg=f)
    if oext is not None:
        for f in ("isi_status", "last_step", "last_spike_step", "first_isi_spike", "is_being_forced"):
            np.testing.assert_array_equal(gext[f], oext[f], err_msg=f)
        np.testing.assert_array_equal(gext["stability"], oext["stability"])
        np.testing.assert_array_equal(gext["free_synaptic_resource"], oext["free_synaptic_resource"])


@pytest.mark.parametrize("mode", ["auto", "phases", "grid"])
@pytest.mark.parametrize("kind", ["delta", "stdp", "stdp_resource_neuron"])
def test_smallest_network_golden(kind, mode):
    """knp/tests/backend/single_thread_cpu_test.cpp:54-176 through the C ABI."""
    net, sched = N.smallest_network(kind)
    g, b, o, oo = run_both(net, sched, 20, step_mode=mode)
    assert b.fused == (mode == "auto")
    pop = net.populations[0].uid
    assert [t for t, s in enumerate(g[pop]) if s.size] == GOLDEN
    assert_same_spikes(g, o)
    for pr in net.projections:
        np.testing.assert_array_equal(b.read_weights(pr.uid), oo.weights(pr.uid))
    if kind != "delta":
        assert b.read_weights(net.projections[1].uid)[0] != 1.0  # weights changed, as the reference asserts
    assert_same_state(b, oo, pop)


@pytest.mark.parametrize("mode", ["auto", "phases", "grid"])
@pytest.mark.parametrize("device_schedule", [False, True])
def test_small_network_bit_exact(device_schedule, mode):
    """Plain small config: 1000 BLIFAT, 100 Bernoulli inputs, all-to-all input and p=0.1 recurrent
    projections with dyadic weights, 1000 steps: spikes bit-exact every step."""
    net, sched = N.small_network(seed=1, steps=1000)
    g, b, o, oo = run_both(net, sched, 1000, device_schedule=device_schedule, step_mode=mode)
    assert b.fused == (mode == "auto")
    assert_same_spikes(g, o)
    assert_same_state(b, oo, net.populations[0].uid)
    ev, sp, upd = b.counters()
    assert ev == oo.events
    assert sp == sum(s.size for s in o[net.populations[0].uid])
    assert upd == 1000 * 1000


def test_large_sparse_reduced_scale():
    """Large sparse config at 1/100 scale (10k neurons, fan-in 1000, delays 1..20), host-loaded synapses."""
    net, sched = N.large_sparse_network(seed=2, n=10_000, fan_in=1000, steps=120)
    g, b, o, oo = run_both(net, sched, 120)
    assert_same_spikes(g, o)
    assert b.counters()[0] == oo.events


def test_pipelined_spike_reads_and_caps():
    """A step's spikes read while the next step already runs (its input sent first), into a reused
    buffer, equal the oracle's; a read capped below the spike count returns its ascending prefix
    and the full count."""
    from oracle import oracle as orc

    B = _gpu()
    net, scheds = N.large_sparse_network(seed=3, n=10_000, fan_in=1000, steps=50)
    steps = 50
    o, _ = orc.run(net, scheds, steps)
    pop = net.populations[0].uid
    b = B.GB300Backend(0)
    b.load_network(net)
    b._init()
    buf = np.empty(10_000, np.uint32)
    for k in range(steps + 1):
        if k < steps:
            for sc in scheds:
                idx = sc.at(k)
                if idx.size:
                    b.send_spikes(sc.sender, idx, k)
            b.step(1)
        if k > 0:
            t = k - 1
            exp = o[pop][t]
            got = b.spikes(pop, t, out=buf)
            assert np.array_equal(got, exp), f"step {t}"
            if exp.size > 3:
                capped = np.full(3, 0xFFFFFFFF, np.uint32)
                cnt = b.spikes_capped(pop, t, capped)
                assert cnt == exp.size and np.array_equal(capped, exp[:3])
    b.close()


@pytest.mark.parametrize("mode", ["auto", "phases"])
@pytest.mark.parametrize("fraction", [0.0, 0.05, 0.3, -1.0])
def test_gather_direction_bit_exact(fraction, mode):
    """Steps delivered by the gather kernel (spike share >= fraction; 0 = every step with a spike,
    -1 = never) give the same spike trains as the oracle, through the ramp into saturated firing,
    with the persistent grid kernel (AUTO at this size) and with the per-phase kernels."""
    from knp_gb300 import backend as B
    from oracle import oracle as orc

    net, sched = N.large_sparse_network(seed=2, n=5000, fan_in=1000, steps=70)
    rec = net.projections[1]
    b = B.GB300Backend()
    b.load_network(net)
    b.set_pull_threshold(rec.uid, fraction)
    b.set_step_mode(MODES[mode])
    b._init()
    assert b.step_kernel == (T.STEP_GRID if mode == "auto" else T.STEP_PHASES)
    for t in range(70):
        idx = sched[0].at(t)
        if idx.size:
            b.send_spikes(sched[0].sender, idx, t)
        b.step(1)
    o, oo = orc.run(net, sched, 70)
    pop = net.populations[0].uid
    for t in range(70):
        np.testing.assert_array_equal(b.spikes(pop, t), o[pop][t], err_msg=f"step {t}")
    assert b.counters()[0] == oo.events
    assert_same_state(b, oo, pop)


def test_gather_inhibitory_projection():
    """Uniform INHIBITORY_CURRENT projection in gather form (weights negated in the layout)."""
    from knp_gb300 import backend as B
    from oracle import oracle as orc

    n, fan = 2000, 600
    pop = N.Population(T.uid_from_int(41), T.BLIFAT, T.blifat_defaults(n))
    chan = T.uid_from_int(49)
    k = [N.stream_key(9, s) for s in (1, 2, 3)]
    pre, post, w, d = N.fixed_fan_in_pre(*k, n, n, fan, 0, 64, 1, 6)
    exc = N.Projection(T.uid_from_int(42), T.DELTA, pop.uid, pop.uid, pre, post, w, d)
    k2 = [N.stream_key(10, s) for s in (1, 2, 3)]
    pre2, post2, w2, d2 = N.fixed_fan_in_pre(*k2, n, n, fan, 0, 32, 1, 6)
    inh = N.Projection(T.uid_from_int(43), T.DELTA, pop.uid, pop.uid, pre2, post2, w2, d2,
                       out_type=np.full(pre2.size, T.INHIBITORY_CURRENT, np.uint8))
    ar = np.arange(n, dtype=np.uint32)
    bg = N.Projection(T.uid_from_int(44), T.DELTA, T.NULL_UID, pop.uid, ar, ar.copy(), np.ones(n, np.float32),
                      np.ones(n, np.uint32))
    net = N.Network([pop], [bg, exc, inh], [(bg.uid, chan)])
    sched = N.bernoulli_schedule(chan, 6, n, 60, 0.05)
    b = B.GB300Backend()
    b.load_network(net)
    b.set_pull_threshold(exc.uid, 0.0)
    b.set_pull_threshold(inh.uid, 0.0)
    b._init()
    b.load_spike_schedule(sched)
    b.step(60)
    o, oo = orc.run(net, [sched], 60)
    for t in range(60):
        np.testing.assert_array_equal(b.spikes(pop.uid, t), o[pop.uid][t], err_msg=f"step {t}")
    assert b.counters()[0] == oo.events


@pytest.mark.parametrize("k_range", [(-16, 48), (-1000, 1000), (-3001, 3001)])
def test_gather_weight_storage(k_range):
    """The gather layout stores weights in the smallest lossless form: an 8-bit dictionary index
    (65 distinct weights k/256, k in [-16, 48]), FP16 (2001 distinct weights, all exactly FP16) or FP32
    (k/256 up to ~11.7 needs 12 significant bits); each gives the oracle's spike trains bit for bit."""
    from knp_gb300 import backend as B
    from oracle import oracle as orc

    n, fan = 5000, 220  # >= 2^20 synapses: the projection gets a gather layout
    pop = N.Population(T.uid_from_int(61), T.BLIFAT, T.blifat_defaults(n))
    chan = T.uid_from_int(69)
    k = [N.stream_key(12, s) for s in (1, 2, 3)]
    pre, post, w, d = N.fixed_fan_in_pre(*k, n, n, fan, k_range[0], k_range[1], 1, 8)
    rec = N.Projection(T.uid_from_int(62), T.DELTA, pop.uid, pop.uid, pre, post, w, d)
    ar = np.arange(n, dtype=np.uint32)
    bg = N.Projection(T.uid_from_int(63), T.DELTA, T.NULL_UID, pop.uid, ar, ar.copy(), np.ones(n, np.float32),
                      np.ones(n, np.uint32))
    net = N.Network([pop], [bg, rec], [(bg.uid, chan)])
    sched = N.bernoulli_schedule(chan, 13, n, 50, 0.02)
    b = B.GB300Backend()
    b.load_network(net)
    b.set_pull_threshold(rec.uid, 0.0)
    b._init()
    b.load_spike_schedule(sched)
    b.step(50)
    o, oo = orc.run(net, [sched], 50)
    for t in range(50):
        np.testing.assert_array_equal(b.spikes(pop.uid, t), o[pop.uid][t], err_msg=f"step {t}")
    assert b.counters()[0] == oo.events


def test_device_generated_projection_matches_host_arrays():
    """The device-side fixed fan-in generator builds exactly the synapses of network.fixed_fan_in_pre."""
    from knp_gb300 import backend as B

    seed, n, fan = 2, 10_000, 100
    net, sched = N.large_sparse_network(seed=seed, n=n, fan_in=fan, steps=60)
    rec = net.projections[1]
    bg = net.projections[0]
    b = B.GB300Backend()
    b.load_populations(net.populations)
    b.load_projections([bg])
    s = N.LARGE_SEED_STREAM
    b.generate_fixed_fan_in_projection(rec.uid, rec.pre_uid, rec.post_uid, n, n, fan, -16, 48, 1, 20, seed, s)
    for recv, send in net.subscriptions:
        b.subscribe(recv, [send])
    b.record_spikes(net.populations[0].uid)
    b._init()
    b.load_spike_schedule(sched[0])
    b.step(60)
    from oracle import oracle as orc

    o, oo = orc.run(net, sched, 60)
    pop = net.populations[0].uid
    for t in range(60):
        np.testing.assert_array_equal(b.spikes(pop, t), o[pop][t])
    # CSR-order weights of the generated projection are a permutation of the host weights.
    np.testing.assert_array_equal(np.sort(b.read_weights(rec.uid)), np.sort(rec.weight))


GEN_CASES = [  # kind, n_pre, n_post, count, probability, k_lo, k_hi (B fires on some steps)
    (T.GEN_ALL_TO_ALL, 300, 200, 0, 0.0, -8, 40),
    (T.GEN_ALIGNED, 800, 200, 0, 0.0, 200, 300),
    (T.GEN_ALIGNED, 200, 800, 0, 0.0, 200, 300),
    (T.GEN_EXCLUSIVE, 400, 400, 0, 0.0, -4, 32),
    (T.GEN_ONE_TO_ONE, 500, 500, 0, 0.0, 200, 300),
    (T.GEN_FIXED_PROBABILITY, 700, 600, 0, 0.05, 32, 256),
    (T.GEN_FIXED_NUMBER_POST, 600, 500, 30_000, 0.0, 16, 160),
    (T.GEN_FIXED_NUMBER_PRE, 600, 500, 30_000, 0.0, 16, 160),
]


@pytest.mark.parametrize("case", range(len(GEN_CASES)))
def test_device_synapse_generators(case):
    """knp_gb300_generate_projection builds, for every generator kind, the synapses of
    network.generated_synapses: population A (Bernoulli-driven) projects through the generated
    projection into population B; both populations' spikes equal the oracle's (which loads the host
    arrays) step by step, and so does the event count."""
    from knp_gb300 import backend as B
    from oracle import oracle as orc

    kind, n_pre, n_post, count, prob, k_lo, k_hi = GEN_CASES[case]
    seed, stream, steps = 7 + case, 50, 40
    a_uid, b_uid, g_uid, bg_uid, chan_uid = (T.uid_from_int(9000 + 10 * case + i) for i in range(5))
    pre, post, w, d = N.generated_synapses(kind, n_pre, n_post, k_lo, k_hi, 1, 8, seed, stream, count=count,
                                           probability=prob)
    assert pre.size > 0
    pa = N.Population(a_uid, T.BLIFAT, T.blifat_defaults(n_pre))
    pb = N.Population(b_uid, T.BLIFAT, T.blifat_defaults(n_post))
    ar = np.arange(n_pre, dtype=np.uint32)
    bg = N.Projection(bg_uid, T.DELTA, T.NULL_UID, a_uid, ar, ar.copy(), np.ones(n_pre, np.float32),
                      np.ones(n_pre, np.uint32))
    gp = N.Projection(g_uid, T.DELTA, a_uid, b_uid, pre, post, w, d)
    net = N.Network([pa, pb], [bg, gp], [(bg_uid, chan_uid)])
    sched = [N.bernoulli_schedule(chan_uid, seed, n_pre, steps, 0.05)]
    b = B.GB300Backend()
    b.load_populations(net.populations)
    b.load_projections([bg])
    b.generate_projection(g_uid, a_uid, b_uid, kind, n_pre, n_post, k_lo, k_hi, 1, 8, seed, stream, count=count,
                          probability=prob)
    for recv, send in net.subscriptions:
        b.subscribe(recv, [send])
    b.record_spikes(a_uid)
    b.record_spikes(b_uid)
    b._init()
    b.load_spike_schedule(sched[0])
    b.step(steps)
    o, oo = orc.run(net, sched, steps)
    for uid in (a_uid, b_uid):
        for t_ in range(steps):
            np.testing.assert_array_equal(b.spikes(uid, t_), o[uid][t_], err_msg=f"step {t_}")
    assert sum(s.size for s in o[b_uid]) > 0
    assert b.counters()[0] == oo.events
    np.testing.assert_array_equal(np.sort(b.read_weights(g_uid)), np.sort(w))
    b.close()


def test_device_generator_arguments_are_checked():
    """knp_gb300_generate_projection refuses what the reference's generators cannot build: an
    unknown kind, aligned sizes that are not multiples, exclusive and one-to-one with unequal sizes,
    a probability outside [0, 1], bad weight or delay ranges, a duplicate UID."""
    from knp_gb300 import backend as B
    from knp_gb300._capi import KnpGb300Error

    b = B.GB300Backend()
    pop = N.Population(T.uid_from_int(9901), T.BLIFAT, T.blifat_defaults(100))
    b.load_populations([pop])
    u = T.uid_from_int(9902)
    bad = [dict(kind=9, n_pre=10, n_post=10), dict(kind=T.GEN_ALIGNED, n_pre=10, n_post=4),
           dict(kind=T.GEN_EXCLUSIVE, n_pre=10, n_post=9), dict(kind=T.GEN_ONE_TO_ONE, n_pre=10, n_post=11),
           dict(kind=T.GEN_FIXED_PROBABILITY, n_pre=10, n_post=10, probability=1.5),
           dict(kind=T.GEN_ALL_TO_ALL, n_pre=10, n_post=10, k_lo=5, k_hi=1),
           dict(kind=T.GEN_ALL_TO_ALL, n_pre=10, n_post=10, d_hi=300)]
    for a in bad:
        args = dict(k_lo=0, k_hi=4, d_lo=1, d_hi=4, count=0, probability=0.0)
        args.update(a)
        with pytest.raises(KnpGb300Error):
            b.generate_projection(u, pop.uid, pop.uid, args["kind"], args["n_pre"], args["n_post"], args["k_lo"],
                                  args["k_hi"], args["d_lo"], args["d_hi"], 1, 2, count=args["count"],
                                  probability=args["probability"])
    b.generate_projection(u, pop.uid, pop.uid, T.GEN_ALL_TO_ALL, 100, 100, 0, 4, 1, 4, 1, 2)
    with pytest.raises(KnpGb300Error):
        b.generate_projection(u, pop.uid, pop.uid, T.GEN_ALL_TO_ALL, 100, 100, 0, 4, 1, 4, 1, 2)
    b.close()


def _full_size_run(threshold, n, fan, seed, steps, keep):
    """The large sparse config at full size, synapses and background generated on the device, with
    the given gather threshold. Returns (per-step spike digests, spike masks of the last `keep`
    steps, final potentials, event count)."""
    import zlib

    from knp_gb300 import backend as B

    pop_uid, rec_uid, bg_uid, chan_uid = (T.uid_from_int(seed * 100 + i) for i in (1, 2, 3, 4))
    pop = N.Population(pop_uid, T.BLIFAT, T.blifat_defaults(n))
    ar = np.arange(n, dtype=np.uint32)
    bg = N.Projection(bg_uid, T.DELTA, T.NULL_UID, pop_uid, ar, ar.copy(), np.ones(n, np.float32),
                      np.ones(n, np.uint32))
    b = B.GB300Backend()
    b.load_populations([pop])
    b.load_projections([bg])
    b.generate_fixed_fan_in_projection(rec_uid, pop_uid, pop_uid, n, n, fan, -16, 48, 1, 20, seed,
                                       N.LARGE_SEED_STREAM)
    b.subscribe(bg_uid, [chan_uid])
    b.record_spikes(pop_uid)
    b.set_pull_threshold(rec_uid, threshold)
    b._init()
    b.generate_bernoulli_schedule(chan_uid, n, 0.005, 0, steps, seed=seed + 5)
    b.step(steps)
    digests, masks = [], {}
    for t in range(steps):
        s = b.spikes(pop_uid, t)
        digests.append((s.size, zlib.crc32(s.tobytes())))
        if t >= steps - keep:
            m = np.zeros(n, bool)
            m[s] = True
            masks[t] = m
    v = b.read_population(pop_uid)[0]["potential"].copy()
    events = b.counters()[0]
    b.close()
    return digests, masks, v, events


def test_large_sparse_full_size_properties():
    """The large sparse config at its full size (1M neurons, 1e9 synapses), where the oracle cannot
    run, through size-independent properties:
    - the scatter-only and the mixed scatter/gather runs give identical spike trains and event
      counts over the ramp into saturated firing;
    - for 256 sampled neurons and every step, the exact input sum recomputed on the host from the
      counter-based synapse generator and the recorded spikes (every presynaptic spike at t - d
      through each of the neuron's 1000 synapses, plus its background spike at t - 1) decides the
      neuron's spike (sum >= 1.0, step > 0), and at the last step equals its stored potential when
      it did not fire (reset to 0 when it did)."""
    n, fan, seed, steps = 1_000_000, 1000, 2, 40
    d_a, _, _, ev_a = _full_size_run(-1.0, n, fan, seed, steps, 0)
    d_b, masks, v, ev_b = _full_size_run(0.1, n, fan, seed, steps, steps)
    assert d_a == d_b
    assert ev_a == ev_b
    assert d_b[-1][0] > n // 2  # saturated by the last step
    s = N.LARGE_SEED_STREAM
    keys = [N.stream_key(seed, s + k) for k in (N.S_PRE, N.S_WEIGHT, N.S_DELAY)]
    rng = np.random.default_rng(11)
    targets = np.sort(rng.choice(n, 256, replace=False)).astype(np.uint64)
    tg = targets.astype(np.int64)
    i = (targets[:, None] + np.arange(fan, dtype=np.uint64)[None, :] * np.uint64(n)).ravel()
    pre = N.uniform_int(keys[0], i, 0, n - 1).astype(np.int64).reshape(256, fan)
    w = N.dyadic_weights(keys[1], i, -16, 48).astype(np.float64).reshape(256, fan)
    d = N.uniform_int(keys[2], i, 1, 20).astype(np.int64).reshape(256, fan)
    src = N.stream_key(seed + 5, N.S_INPUT)
    bg_thr = np.uint64(int(0.005 * float(1 << 53)))
    hist = np.stack([masks[t] for t in range(steps)])  # [step, neuron]
    mixed = 0
    for t in range(1, steps):
        ts = t - d  # step of each synapse's presynaptic spike
        fired = np.where(ts >= 0, hist[np.maximum(ts, 0), pre], False)
        bg_prev = (N.rand64(src, np.uint64(t - 1) * np.uint64(n) + targets) >> np.uint64(11)) < bg_thr
        total = np.where(fired, w, 0.0).sum(axis=1) + bg_prev.astype(np.float64)
        spiked = hist[t, tg]
        np.testing.assert_array_equal(spiked, total >= 1.0, err_msg=f"step {t}")
        mixed += 0 < spiked.sum() < spiked.size
    assert mixed > 0  # some checked steps had both firing and silent sampled neurons
    vt = v[tg].astype(np.float64)
    np.testing.assert_array_equal(vt[~spiked], total[~spiked])
    np.testing.assert_array_equal(vt[spiked], 0.0)


def test_device_bernoulli_schedule_matches_host():
    from knp_gb300 import backend as B

    net, sched = N.small_network(seed=5, n=200, n_in=300, steps=50, p_in=0.2)
    b1 = B.GB300Backend()
    b1.load_network(net)
    b1._init()
    b1.generate_bernoulli_schedule(sched[0].sender, 300, 0.2, 0, 50, seed=5)
    b1.step(50)
    g, b2, o, oo = run_both(net, sched, 50)
    pop = net.populations[0].uid
    for t in range(50):
        np.testing.assert_array_equal(b1.spikes(pop, t), o[pop][t])


@pytest.mark.parametrize("mode", ["auto", "phases", "grid"])
def test_stdp_reduced(mode):
    """STDP config with 10 samples x 100 steps: spikes bit-exact, weights bit-exact."""
    net, sched = N.stdp_network(seed=3, samples=10, steps_per_sample=100)
    g, b, o, oo = run_both(net, sched, 1000, step_mode=mode)
    assert b.fused == (mode == "auto")
    assert_same_spikes(g, o)
    for pr in net.projections:
        np.testing.assert_array_equal(b.read_weights(pr.uid), oo.weights(pr.uid))
    assert_same_state(b, oo, net.populations[0].uid)


def test_stdp_full_config_against_fixture():
    """The full STDP learning config (200 samples x 100 steps, 784 -> 800 additive STDP + lateral
    inhibition) against tests/golden/stdp_full.json, written from the reference-header oracle: every
    sample's spike digest, the event count, the final plastic weights bit-exact (CRC32) and, as the
    config's stated bar, every sampled weight within 1e-5 relative."""
    import json
    import os
    import zlib

    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "stdp_full.json")) as f:
        case = json.load(f)
    net, sched = N.__dict__[case["builder"]](**case["kwargs"])
    B = _gpu()
    g, b = B.run(net, sched, case["steps"], device_schedule=True)
    pop = net.populations[0].uid
    d = np.asarray([[s.size, zlib.crc32(np.ascontiguousarray(s, np.uint32).tobytes())] for s in g[pop]],
                   np.uint64).astype(np.uint32)
    samples = [[int(d[s:s + 100, 0].sum()), zlib.crc32(np.ascontiguousarray(d[s:s + 100]).tobytes())]
               for s in range(0, case["steps"], 100)]
    assert samples == case["samples"]
    w = b.read_weights(net.projections[0].uid)
    ws = w[::case["weights_stride"]].astype(np.float64)
    ref = np.asarray(case["weights_sampled"], np.float64)
    np.testing.assert_allclose(ws, ref, rtol=1e-5, atol=0)
    assert zlib.crc32(w.tobytes()) == case["weights_crc"]
    assert b.counters()[0] == case["events"]


def test_external_impacts_and_channels():
    """External SynapticImpactMessages of every supported type into a BLIFAT population with
    non-default dynamics; potentials within 1e-5 relative of the FP64 oracle."""
    rng = np.random.default_rng(7)
    n = 257
    pop = N.Population(T.uid_from_int(1), T.BLIFAT, T.blifat_defaults(n))
    pop.neurons["potential_decay"] = 0.5
    pop.neurons["threshold_decay"] = 0.75
    pop.neurons["threshold_increment"] = 0.25
    pop.neurons["inhibitory_conductance_decay"] = 0.5
    pop.neurons["postsynaptic_trace_decay"] = 0.5
    pop.neurons["postsynaptic_trace_increment"] = 1.0
    pop.neurons["absolute_refractory_period"] = 2
    pop.neurons["bursting_period"] = 3
    pop.neurons["reflexive_weight"] = 0.25
    chan = T.uid_from_int(9)
    net = N.Network([pop], [], [(pop.uid, chan)])

    def inject(be, t, who):
        r = np.random.default_rng(1000 + t)
        k = 64
        post = r.integers(0, n, k).astype(np.uint32)
        val = (r.integers(0, 128, k) / 64.0).astype(np.float32)
        ty = r.choice([0, 0, 0, 1, 2, 3], k).astype(np.uint8)
        be.send_impacts(chan, pop.uid, post, val, ty)

    g, b, o, oo = run_both(net, [], 60, on_step=inject)
    # FP32 state against FP64 state with decays 0.5 / 0.75: spike mismatch at most 0.1% of
    # neuron-steps, potentials within 1e-5 relative when every spike agrees.
    mism = 0
    for a, e in zip(g[pop.uid], o[pop.uid]):
        mism += np.setxor1d(a, e).size
    assert mism <= 1e-3 * n * 60
    if mism == 0:
        assert_same_state(b, oo, pop.uid, rtol=1e-5)
    del rng


@pytest.mark.parametrize("mode", ["auto", "phases", "grid"])
def test_delay_zero_and_inhibitory_types(mode):
    """Delay-0 synapses create events that are never delivered; INHIBITORY_CURRENT subtracts."""
    n = 64
    pop = N.Population(T.uid_from_int(11), T.BLIFAT, T.blifat_defaults(n))
    chan = T.uid_from_int(19)
    pre = np.repeat(np.arange(8, dtype=np.uint32), n)
    post = np.tile(np.arange(n, dtype=np.uint32), 8)
    w = np.full(pre.size, 0.5, np.float32)
    d = (np.arange(pre.size) % 4).astype(np.uint32)  # includes delay 0
    ty = np.where(np.arange(pre.size) % 3 == 0, 1, 0).astype(np.uint8)
    pr = N.Projection(T.uid_from_int(12), T.DELTA, T.NULL_UID, pop.uid, pre, post, w, d, ty)
    net = N.Network([pop], [pr], [(pr.uid, chan)])
    sched = N.bernoulli_schedule(chan, 3, 8, 40, 0.5)
    g, b, o, oo = run_both(net, [sched], 40, step_mode=mode)
    assert_same_spikes(g, o)
    assert b.counters()[0] == oo.events
    assert_same_state(b, oo, pop.uid)


@pytest.mark.parametrize("mode", ["auto", "phases", "grid"])
def test_stdp_only_and_multiple_sources(mode):
    """An STDP projection whose presynaptic population is also an STDP-only population: its spikes
    are emptied before propagation (additive_stdp.h:162-166) and never update weights."""
    n = 32
    a = N.Population(T.uid_from_int(21), T.BLIFAT, T.blifat_defaults(n))
    c = N.Population(T.uid_from_int(22), T.BLIFAT, T.blifat_defaults(n))
    chan = T.uid_from_int(29)
    ar = np.arange(n, dtype=np.uint32)
    drive = N.Projection(T.uid_from_int(23), T.DELTA, T.NULL_UID, a.uid, ar, ar, np.ones(n, np.float32),
                         np.ones(n, np.uint32))
    i = np.arange(n * n)
    plastic = N.Projection(T.uid_from_int(24), T.ADDITIVE_STDP_DELTA, a.uid, c.uid, (i % n).astype(np.uint32),
                           (i // n).astype(np.uint32), np.full(i.size, 0.25, np.float32), np.ones(i.size, np.uint32),
                           tau_plus=np.full(i.size, 2, np.float32), tau_minus=np.full(i.size, 2, np.float32),
                           stdp_populations={a.uid: T.STDP_ONLY, c.uid: T.STDP_AND_SPIKE})
    net = N.Network([a, c], [drive, plastic], [(drive.uid, chan)])
    sched = N.bernoulli_schedule(chan, 4, n, 80, 0.3)
    g, b, o, oo = run_both(net, [sched], 80, step_mode=mode)
    assert_same_spikes(g, o)
    np.testing.assert_array_equal(b.read_weights(plastic.uid), oo.weights(plastic.uid))


def _gpu_lif_run(neuron, steps, impacts=()):
    """knp/tests/framework/lif_test.cpp:60-100 through the C ABI: one LIF neuron, one external
    impact per step, potential read before every step."""
    from knp_gb300 import backend as B

    pop_uid, in_uid = T.uid_from_int(601), T.uid_from_int(602)
    b = B.GB300Backend()
    b.load_network(N.Network([N.Population(pop_uid, T.LIF, neuron.copy())], [], [(pop_uid, in_uid)]))
    b._init()
    pots, spikes = [], []
    for t in range(steps):
        if t < len(impacts):
            b.send_impacts(in_uid, pop_uid, [0], [impacts[t]], [T.EXCITATORY])
        pots.append(float(b.read_lif(pop_uid)["potential"][0]))
        b.step(1)
        if b.spikes(pop_uid, t).size:
            spikes.append(t)
    return pots, spikes


def test_lif_known_answers():
    """Expected potentials and spike steps of lif_test.cpp:103-177."""
    n = T.lif_defaults(1)
    n["activation_threshold"] = 101.0
    n["leak_coefficient"] = 0.25
    n["potential"] = 100.0
    assert _gpu_lif_run(n, 10) == ([100.0 * 0.25 ** k for k in range(10)], [])
    n = T.lif_defaults(1)
    n["leak_coefficient"] = 0.5
    n["potential"] = 3.0
    assert _gpu_lif_run(n, 3) == ([3.0, 0.0, 0.0], [0])
    n = T.lif_defaults(1)
    n["leak_coefficient"] = 0.5
    n["activation_threshold"] = 6.0
    assert _gpu_lif_run(n, 6, [5, 5, 2, 3, 8]) == ([0.0, 5.0, 0.0, 2.0, 4.0, 0.0], [1, 4])
    n["refract_period"] = 2
    assert _gpu_lif_run(n, 7, [5, 5, 10, 10, 5, 5]) == ([0.0, 5.0, 0.0, 0.0, 0.0, 5.0, 0.0], [1, 5])


def test_lif_network_against_oracle():
    """Feed-forward LIF layers (dyadic weights, refractory period 1, threshold 2) against the oracle.
    Leak stays 1 (the reference default) so that FP32 sums are exact whatever their order: the
    reference adds impacts one by one, the ring adds their pre-summed value."""
    n_in, n1, n2 = 100, 300, 50
    l1 = T.lif_defaults(n1)
    l1["refract_period"] = 1
    l2 = T.lif_defaults(n2)
    l2["activation_threshold"] = 2.0
    p1 = N.Population(T.uid_from_int(611), T.LIF, l1)
    p2 = N.Population(T.uid_from_int(612), T.LIF, l2)
    chan = T.uid_from_int(619)
    k = [N.stream_key(13, s) for s in (1, 2, 3)]
    i = np.arange(n_in * n1, dtype=np.uint64)
    a = N.Projection(T.uid_from_int(613), T.DELTA, T.NULL_UID, p1.uid, (i % n_in).astype(np.uint32),
                     (i // n_in).astype(np.uint32), N.dyadic_weights(k[1], i, -32, 64), np.ones(i.size, np.uint32))
    j = np.arange(n1 * n2, dtype=np.uint64)
    b_ = N.Projection(T.uid_from_int(614), T.DELTA, p1.uid, p2.uid, (j % n1).astype(np.uint32),
                      (j // n1).astype(np.uint32), N.dyadic_weights(k[2], j, -16, 32),
                      N.uniform_int(k[0], j, 1, 3).astype(np.uint32))
    net = N.Network([p1, p2], [a, b_], [(a.uid, chan)])
    sched = N.bernoulli_schedule(chan, 14, n_in, 80, 0.1)
    g, b, o, oo = run_both(net, [sched], 80)
    assert_same_spikes(g, o)
    for p in (p1, p2):
        np.testing.assert_array_equal(b.read_lif(p.uid), oo.lif(p.uid))


def test_errors_are_reported():
    from knp_gb300 import backend as B
    from knp_gb300._capi import KnpGb300Error

    b = B.GB300Backend()
    pop = N.Population(T.uid_from_int(31), T.BLIFAT, T.blifat_defaults(4))
    b.load_populations([pop])
    # BLOCKING synapses are taken in delta projections only (an STDP weight may change in flight).
    bad = N.Projection(T.uid_from_int(32), T.ADDITIVE_STDP_DELTA, T.NULL_UID, pop.uid, np.zeros(1, np.uint32),
                       np.zeros(1, np.uint32), np.ones(1, np.float32), np.ones(1, np.uint32),
                       out_type=np.array([T.BLOCKING], np.uint8), tau_plus=np.full(1, 2.0, np.float32),
                       tau_minus=np.full(1, 2.0, np.float32))
    with pytest.raises(KnpGb300Error):
        b.load_projections([bad])
    oob = N.Projection(T.uid_from_int(33), T.DELTA, T.NULL_UID, pop.uid, np.zeros(1, np.uint32),
                       np.array([7], np.uint32), np.ones(1, np.float32), np.ones(1, np.uint32))
    b.load_projections([oob])
    with pytest.raises(KnpGb300Error):
        b._init()
    with pytest.raises(KnpGb300Error):
        b.step(1)


def test_step_mode_selection_and_recording_change():
    """Step modes: an unknown mode and a fused mode forced on a network above the fused kernel's
    size are refused; a recording switched on mid-run under the fused kernel or the grid kernel
    (their descriptors uploaded again) gives the oracle's spikes from that step on."""
    from oracle import oracle as orc
    from knp_gb300 import backend as B
    from knp_gb300._capi import KnpGb300Error

    b = B.GB300Backend()
    with pytest.raises(KnpGb300Error):
        b.set_step_mode(7)
    big = N.Population(T.uid_from_int(41), T.BLIFAT, T.blifat_defaults(20_000))
    b.load_populations([big])
    b.set_step_mode(T.STEP_FUSED)
    with pytest.raises(KnpGb300Error):
        b._init()

    net, sched = N.small_network(seed=5, steps=100)
    pop = net.populations[0].uid
    o, _ = orc.run(net, sched, 100)
    b = B.GB300Backend()
    b.load_network(net, record=[])
    b.set_step_mode(T.STEP_FUSED)
    b._init()
    assert b.fused
    with pytest.raises(KnpGb300Error):
        b.set_step_mode(T.STEP_PHASES)
    for s in sched:
        b.load_spike_schedule(s)
    b.step(50)
    b.record_spikes(pop, True)
    b.step(50)
    for t in range(50, 100):
        np.testing.assert_array_equal(b.spikes(pop, t), o[pop][t])
    b.close()
    # The same under the persistent grid kernel (forced at this size).
    b = B.GB300Backend()
    b.load_network(net, record=[])
    b.set_step_mode(T.STEP_GRID)
    b._init()
    assert b.step_kernel == T.STEP_GRID and not b.fused
    for s in sched:
        b.load_spike_schedule(s)
    b.step(50)
    b.record_spikes(pop, True)
    b.step(50)
    for t in range(50, 100):
        np.testing.assert_array_equal(b.spikes(pop, t), o[pop][t])


def test_profile_grid_phases():
    """knp_gb300_profile_grid_phases: normal steps of the persistent grid kernel (the oracle's spikes)
    with a positive time for the population and projection phases; refused on a per-phase backend."""
    from oracle import oracle as orc
    from knp_gb300 import backend as B
    from knp_gb300._capi import KnpGb300Error

    net, sched = N.small_network(seed=5, steps=100)
    pop = net.populations[0].uid
    o, _ = orc.run(net, sched, 100)
    b = B.GB300Backend()
    b.load_network(net)
    b.set_step_mode(T.STEP_GRID)
    b._init()
    for s in sched:
        b.load_spike_schedule(s)
    b.step(10)
    us = b.profile_grid_phases(90)
    assert us[0] > 0 and us[1] > 0 and us[2] >= 0
    for t in range(100):
        np.testing.assert_array_equal(b.spikes(pop, t), o[pop][t])
    b.close()
    b = B.GB300Backend()
    b.load_network(net)
    b.set_step_mode(T.STEP_PHASES)
    b._init()
    with pytest.raises(KnpGb300Error):
        b.profile_grid_phases(1)


def test_measure_add_rate():
    """knp_gb300_measure_add_rate: a positive, finite rate of random FP32 atomic adds (L2-resident
    and DRAM-sized buffers)."""
    import ctypes

    from knp_gb300 import _capi

    lib = _capi.lib()
    rates = []
    for n in (1 << 20, 1 << 26):
        r = ctypes.c_double(0.0)
        assert lib.knp_gb300_measure_add_rate(n, 1 << 24, ctypes.byref(r)) == 0, lib.knp_gb300_last_error()
        assert np.isfinite(r.value) and r.value > 1e9
        rates.append(r.value)


@pytest.mark.parametrize("mode", ["auto", "phases", "grid"])
def test_blocking_synapses_and_impacts(mode):
    """BLOCKING synapses (blifat_impl.h:86): of a step's BLOCKING impacts on a neuron the last in the
    reference's message order sets its total blocking period (projection load order, then larger
    delays first, then spike and synapse order; external messages last). Repeated (pre, post) pairs,
    recurrent BLOCKING synapses and external BLOCKING impacts (two messages in one step, repeated
    targets within a message) against the oracle: spikes every step and the blocking periods."""
    net, scheds = N.blocking_network(seed=12, steps=200)
    pop = net.populations[0].uid
    ext = T.uid_from_int(1203)
    rng = np.random.default_rng(5)
    plan = {}
    for t in range(3, 200, 7):
        post = rng.integers(0, 400, 12).astype(np.uint32)
        post[5] = post[2]  # a repeated target within the message
        vals = rng.choice(np.float32([-4, -1, 2, 3.5, 6, 0.75]), 12).astype(np.float32)
        types = rng.choice(np.uint8([T.BLOCKING, T.EXCITATORY]), 12, p=[0.7, 0.3]).astype(np.uint8)
        plan[t] = [(post, vals, types)]
        if t % 2:
            plan[t].append((post[:4].copy(), np.float32([5, -2, 1, -7]), np.full(4, T.BLOCKING, np.uint8)))

    def on_step(be, t, which):
        for post, vals, types in plan.get(t, []):
            be.send_impacts(ext, pop, post, vals, types, True)

    g, b, o, oo = run_both(net, scheds, 200, on_step=on_step, step_mode=mode)
    assert_same_spikes(g, o)
    gs, _ = b.read_population(pop)
    os_, _ = oo.blifat(pop)
    np.testing.assert_array_equal(gs["total_blocking_period"], os_["total_blocking_period"])
    assert (os_["total_blocking_period"] != np.iinfo(np.int64).max).sum() > 20
    assert b.counters()[0] == oo.events
