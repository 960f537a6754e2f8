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


def run_both(net, scheds, steps, record=None, device_schedule=False, on_step=None):
    from oracle import oracle as orc

    B = _gpu()
    g, b = B.run(net, scheds, steps, record=record, device_schedule=device_schedule,
                 on_step=None if on_step is None else (lambda be, t: on_step(be, t, "gpu")))
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


@pytest.mark.parametrize("kind", ["delta", "stdp", "stdp_resource_neuron"])
def test_smallest_network_golden(kind):
    """knp/tests/backend/single_thread_cpu_test.cpp:54-176 through the C ABI."""
    net, sched = N.smallest_network(kind)
    g, b, o, oo = run_both(net, sched, 20)
    pop = net.populations[0].uid
    assert [t for t, s in enumerate(g[pop]) if s.size] == GOLDEN
    assert_same_spikes(g, o)
    for pr in net.projections:
        np.testing.assert_array_equal(b.read_weights(pr.uid), oo.weights(pr.uid))
    if kind != "delta":
        assert b.read_weights(net.projections[1].uid)[0] != 1.0  # weights changed, as the reference asserts
    assert_same_state(b, oo, pop)


@pytest.mark.parametrize("device_schedule", [False, True])
def test_small_network_bit_exact(device_schedule):
    """Plain small config: 1000 BLIFAT, 100 Bernoulli inputs, all-to-all input and p=0.1 recurrent
    projections with dyadic weights, 1000 steps: spikes bit-exact every step."""
    net, sched = N.small_network(seed=1, steps=1000)
    g, b, o, oo = run_both(net, sched, 1000, device_schedule=device_schedule)
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


def test_stdp_reduced():
    """STDP config with 10 samples x 100 steps: spikes bit-exact, weights bit-exact."""
    net, sched = N.stdp_network(seed=3, samples=10, steps_per_sample=100)
    g, b, o, oo = run_both(net, sched, 1000)
    assert_same_spikes(g, o)
    for pr in net.projections:
        np.testing.assert_array_equal(b.read_weights(pr.uid), oo.weights(pr.uid))
    assert_same_state(b, oo, net.populations[0].uid)


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


def test_delay_zero_and_inhibitory_types():
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
    g, b, o, oo = run_both(net, [sched], 40)
    assert_same_spikes(g, o)
    assert b.counters()[0] == oo.events
    assert_same_state(b, oo, pop.uid)


def test_stdp_only_and_multiple_sources():
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
    g, b, o, oo = run_both(net, [sched], 80)
    assert_same_spikes(g, o)
    np.testing.assert_array_equal(b.read_weights(plastic.uid), oo.weights(plastic.uid))


def test_errors_are_reported():
    from knp_gb300 import backend as B
    from knp_gb300._capi import KnpGb300Error

    b = B.GB300Backend()
    pop = N.Population(T.uid_from_int(31), T.BLIFAT, T.blifat_defaults(4))
    b.load_populations([pop])
    bad = N.Projection(T.uid_from_int(32), T.DELTA, T.NULL_UID, pop.uid, np.zeros(1, np.uint32),
                       np.zeros(1, np.uint32), np.ones(1, np.float32), np.ones(1, np.uint32),
                       out_type=np.array([T.BLOCKING], np.uint8))
    with pytest.raises(KnpGb300Error):
        b.load_projections([bad])
    oob = N.Projection(T.uid_from_int(33), T.DELTA, T.NULL_UID, pop.uid, np.zeros(1, np.uint32),
                       np.array([7], np.uint32), np.ones(1, np.float32), np.ones(1, np.uint32))
    b.load_projections([oob])
    with pytest.raises(KnpGb300Error):
        b._init()
    with pytest.raises(KnpGb300Error):
        b.step(1)
