"""CPU tests: the oracle against the reference's golden vectors and known answers, the restated
oracle against the reference-header oracle (where the KNP sources were available to build it), and
the generators / fixtures that both sides share."""
import json
import os
import zlib

import numpy as np
import pytest

from knp_gb300 import network as N
from knp_gb300 import types as T
from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN_DIR = os.path.join(HERE, "golden")
GOLDEN = [1, 6, 7, 11, 12, 13, 16, 17, 18, 19]


def load_golden(name):
    with open(os.path.join(GOLDEN_DIR, name)) as f:
        return json.load(f)


def spike_digest(trains):
    """Per-step (count, crc32 of the ascending uint32 indexes)."""
    return [[int(s.size), zlib.crc32(np.ascontiguousarray(s, np.uint32).tobytes())] for s in trains]


@pytest.mark.parametrize("kind", ["delta", "stdp", "stdp_resource_neuron"])
def test_oracle_smallest_network_golden(oracle_lib, kind):
    """knp/tests/backend/single_thread_cpu_test.cpp:54-264 expected spike steps."""
    net, sched = N.smallest_network(kind)
    out, o = orc.run(net, sched, 20)
    pop = net.populations[0].uid
    assert [t for t, s in enumerate(out[pop]) if s.size] == GOLDEN
    if kind != "delta":
        assert o.weights(net.projections[1].uid)[0] != 1.0


def _run_lif(neuron, steps, impacts=()):
    """knp/tests/framework/lif_test.cpp:60-100: one LIF neuron, one external impact per step."""
    pop_uid, in_uid = T.uid_from_int(501), T.uid_from_int(502)
    pop = N.Population(pop_uid, T.LIF, neuron.copy())
    net = N.Network([pop], [], [(pop_uid, in_uid)])
    o = orc.OracleNet("restated")
    o.load(net)
    pots, spikes = [], []
    for t in range(steps):
        if t < len(impacts):
            o.send_impacts(in_uid, pop_uid, [0], [impacts[t]], [T.EXCITATORY], True)
        pots.append(float(o.lif(pop_uid)["potential"][0]))
        o.step()
        if o.spikes(pop_uid).size:
            spikes.append(t)
    return pots, spikes


def test_oracle_lif_known_answers(oracle_lib):
    """Expected potentials and spike steps of lif_test.cpp:103-177."""
    n = T.lif_defaults(1)
    n["activation_threshold"] = 101.0
    n["leak_coefficient"] = 0.25
    n["potential"] = 100.0
    pots, spikes = _run_lif(n, 10)
    assert pots == [100.0 * 0.25 ** k for k in range(10)] and spikes == []
    n = T.lif_defaults(1)
    n["leak_coefficient"] = 0.5
    n["potential"] = 3.0
    assert _run_lif(n, 3) == ([3.0, 0.0, 0.0], [0])
    n = T.lif_defaults(1)
    n["leak_coefficient"] = 0.5
    n["activation_threshold"] = 6.0
    assert _run_lif(n, 6, [5, 5, 2, 3, 8]) == ([0.0, 5.0, 0.0, 2.0, 4.0, 0.0], [1, 4])
    n["refract_period"] = 2
    assert _run_lif(n, 7, [5, 5, 10, 10, 5, 5]) == ([0.0, 5.0, 0.0, 0.0, 0.0, 5.0, 0.0], [1, 5])


def test_oracle_against_golden_fixtures(oracle_lib):
    """Spike digests written by tests/golden/make_golden.py from the reference-header oracle."""
    for case in load_golden("spike_digests.json")["cases"]:
        if "rules_crc" in case:
            continue  # resource-STDP cases: test_oracle_resource_stdp_fixtures
        net, sched = N.__dict__[case["builder"]](**case["kwargs"])
        out, o = orc.run(net, sched, case["steps"])
        pop = net.populations[0].uid
        assert spike_digest(out[pop]) == case["digest"], case["name"]
        if "weights_crc" in case:
            for k, crc in case["weights_crc"].items():
                w = o.weights(net.projections[int(k)].uid)
                assert zlib.crc32(w.tobytes()) == crc, (case["name"], k)
        assert o.events == case["events"], case["name"]


def sample_digest(trains, steps_per_sample):
    """Per sample: [spike count, CRC32 of the concatenated per-step (count, CRC32) pairs]."""
    d = np.asarray(spike_digest(trains), np.uint64).astype(np.uint32)
    return [[int(d[s:s + steps_per_sample, 0].sum()), zlib.crc32(np.ascontiguousarray(d[s:s + steps_per_sample]).tobytes())]
            for s in range(0, len(trains), steps_per_sample)]


def test_oracle_against_full_stdp_fixture(oracle_lib):
    """The first 4 samples of the full STDP learning config (fixture written from the
    reference-header oracle over all 200 samples) reproduce with the restated oracle."""
    case = load_golden("stdp_full.json")
    net, sched = N.__dict__[case["builder"]](**case["kwargs"])
    out, _ = orc.run(net, sched, 400)
    assert sample_digest(out[net.populations[0].uid], 100) == case["samples"][:4]


@pytest.mark.skipif(not orc.available("reference"), reason="reference-header oracle not built (no KNP sources)")
@pytest.mark.parametrize("seed", [11, 12])
def test_restated_oracle_matches_reference_headers(oracle_lib, seed):
    net, sched = N.small_network(seed=seed, n=300, n_in=50, steps=300, p_in=0.1)
    a, oa = orc.run(net, sched, 300, which="restated")
    b, ob = orc.run(net, sched, 300, which="reference")
    pop = net.populations[0].uid
    assert spike_digest(a[pop]) == spike_digest(b[pop])
    assert oa.blifat(pop)[0].tobytes() == ob.blifat(pop)[0].tobytes()
    assert oa.events == ob.events


@pytest.mark.skipif(not orc.available("reference"), reason="reference-header oracle not built (no KNP sources)")
def test_restated_oracle_matches_reference_headers_stdp(oracle_lib):
    net, sched = N.stdp_network(seed=3, n_in=100, n=60, samples=6, steps_per_sample=50)
    a, oa = orc.run(net, sched, 300, which="restated")
    b, ob = orc.run(net, sched, 300, which="reference")
    pop = net.populations[0].uid
    assert spike_digest(a[pop]) == spike_digest(b[pop])
    for pr in net.projections:
        assert oa.weights(pr.uid).tobytes() == ob.weights(pr.uid).tobytes()
    sa, ea = oa.blifat(pop)
    sb, eb = ob.blifat(pop)
    assert sa.tobytes() == sb.tobytes() and ea.tobytes() == eb.tobytes()


def test_generator_is_counter_based():
    """Any slice of a generated projection equals the same slice of the whole."""
    k = [N.stream_key(4, s) for s in (1, 2, 3)]
    full = N.fixed_fan_in_pre(*k, 500, 500, 10, -16, 48, 1, 20)
    part = N.fixed_fan_in_pre(*k, 500, 500, 10, -16, 48, 1, 20, start=1234, count=100)
    for a, b in zip(full, part):
        np.testing.assert_array_equal(a[1234:1334], b)
    pre, post, w, d = full
    assert pre.max() < 500 and d.min() >= 1 and d.max() <= 20
    assert np.all((w * 256) == np.round(w * 256)) and w.min() >= -16 / 256 and w.max() <= 48 / 256
    np.testing.assert_array_equal(post, np.arange(5000) % 500)


def test_struct_layouts():
    assert T.BLIFAT_DTYPE.itemsize == 192
    assert T.RESOURCE_DTYPE.itemsize == 72
    assert T.LIF_DTYPE.itemsize == 24
    d = T.blifat_defaults(2)
    assert d["n_time_steps_since_last_firing"][0] == np.iinfo(np.uint64).max
    assert d["total_blocking_period"][0] == np.iinfo(np.int64).max


@pytest.mark.skipif(not orc.available("reference"), reason="reference-header oracle not built (no KNP sources)")
def test_restated_oracle_matches_reference_headers_blocking(oracle_lib):
    """BLOCKING synapses (blifat_impl.h:86, last writer in message order): the restated oracle gives the
    reference headers' spikes and blocking periods."""
    net, scheds = N.blocking_network(seed=12, steps=120)
    pop = net.populations[0].uid
    a, oa = orc.run(net, scheds, 120, which="restated")
    b, ob = orc.run(net, scheds, 120, which="reference")
    for t, (x, y) in enumerate(zip(a[pop], b[pop])):
        np.testing.assert_array_equal(x, y, err_msg=f"step {t}")
    np.testing.assert_array_equal(oa.blifat(pop)[0]["total_blocking_period"], ob.blifat(pop)[0]["total_blocking_period"])
    assert (oa.blifat(pop)[0]["total_blocking_period"] != np.iinfo(np.int64).max).sum() > 20


@pytest.mark.parametrize("kind", ["resource_stdp", "resource_stdp_altai"])
def test_oracle_resource_stdp_golden(oracle_lib, kind):
    """knp/tests/backend/single_thread_cpu_test.cpp:179-355 (SynapticResourceSTDPDeltaSynapse
    projections onto a resource-STDP BLIFAT or AltAI-LIF neuron, learning started): the expected spike
    steps, and the loop projection's weight changes."""
    net, sched = N.smallest_network(kind)
    out, o = orc.run(net, sched, 20)
    pop = net.populations[0].uid
    assert [t for t, s in enumerate(out[pop]) if s.size] == GOLDEN
    assert o.weights(net.projections[1].uid)[0] != 1.0


def test_oracle_resource_stdp_fixtures(oracle_lib):
    """The resource-STDP cases of the fixture (written from the reference-header oracle): weights,
    synapse rule state and neuron state digests, with the learning switches of each case."""
    from tests.golden.make_golden import canonical, learning_switch, population_state

    cases = [c for c in load_golden("spike_digests.json")["cases"] if "rules_crc" in c]
    assert len(cases) == 4
    for case in cases:
        net, sched = N.__dict__[case["builder"]](**case["kwargs"])
        switches = {int(k): v for k, v in case.get("learning", {}).items()}
        out, o = orc.run(net, sched, case["steps"], on_step=learning_switch(switches) if switches else None)
        pop = net.populations[0].uid
        assert spike_digest(out[pop]) == case["digest"], case["name"]
        for k, crc in case["rules_crc"].items():
            assert zlib.crc32(canonical(o.resource_synapses(net.projections[int(k)].uid))) == crc, (case["name"], k)
        for k, crc in case["weights_crc"].items():
            assert zlib.crc32(canonical(o.weights(net.projections[int(k)].uid))) == crc, (case["name"], k)
        neurons, ext = population_state(o, net.populations[0])
        assert zlib.crc32(canonical(neurons) + (b"" if ext is None else canonical(ext))) == case["state_crc"], case["name"]
        assert o.events == case["events"], case["name"]


def _same_runs(net, sched, steps, switches=None):
    from tests.golden.make_golden import canonical, learning_switch, population_state

    cb = learning_switch(switches) if switches else None
    a, oa = orc.run(net, sched, steps, which="restated", on_step=cb)
    b, ob = orc.run(net, sched, steps, which="reference", on_step=cb)
    for p in net.populations:
        assert spike_digest(a[p.uid]) == spike_digest(b[p.uid])
        (sa, ea), (sb, eb) = population_state(oa, p), population_state(ob, p)
        assert canonical(sa) == canonical(sb)
        assert (ea is None and eb is None) or canonical(ea) == canonical(eb)
    for pr in net.projections:
        assert canonical(oa.weights(pr.uid)) == canonical(ob.weights(pr.uid))
        if pr.kind == T.RESOURCE_STDP_DELTA:
            assert canonical(oa.resource_synapses(pr.uid)) == canonical(ob.resource_synapses(pr.uid))
    assert oa.events == ob.events
    return oa


@pytest.mark.skipif(not orc.available("reference"), reason="reference-header oracle not built (no KNP sources)")
def test_restated_oracle_matches_reference_headers_resource_stdp(oracle_lib):
    """Resource-STDP training (blifat_stdp.h:35-172, training/stdp.h:40-186) on the mnist-learn-shaped
    network and on the mixed network with learning switched off and on again: the restated oracle
    gives the reference headers' spikes, neuron state, weights and synapse rule state."""
    net, sched = N.resource_stdp_network(samples=12)
    o = _same_runs(net, sched, 180)
    assert np.count_nonzero(o.weights(net.projections[0].uid)) > 1000
    net, sched = N.resource_stdp_mixed_network(steps=300)
    o = _same_runs(net, sched, 300, {150: False, 200: True})
    rules = o.resource_synapses(net.projections[0].uid)
    assert rules["had_hebbian_update"].sum() > 100 and rules["has_contributed"].sum() > 100



def _run_altai(neuron, steps, impacts=(), n=1, index=0):
    """knp/tests/framework/altai_lif_test.cpp:45-95: AltAI neurons, one external EXCITATORY impact per
    step to neuron `index`; the potential is read before each step."""
    pop_uid, in_uid = T.uid_from_int(601), T.uid_from_int(602)
    neurons = np.repeat(neuron, n)
    net = N.Network([N.Population(pop_uid, T.ALTAI_LIF, neurons)], [], [(pop_uid, in_uid)])
    o = orc.OracleNet("restated")
    o.load(net)
    pots, spikes = [], []
    for t in range(steps):
        if t < len(impacts):
            o.send_impacts(in_uid, pop_uid, [index], [impacts[t]], [T.EXCITATORY], True)
        pots.append(int(np.int16(o.altai(pop_uid)[0]["potential"][index])))
        o.step()
        if index in o.spikes(pop_uid):
            spikes.append(t)
    return pots, spikes


ALTAI_KATS = [
    # altai_lif_test.cpp:97-190: (fields, steps, impacts, n, index, potentials, spikes)
    ({"activation_threshold": 200, "potential_leak": -25, "potential": 100, "leak_rev": 1}, 10, (), 3, 2,
     [100, 75, 50, 25, 0, -25, 0, -25, 0, -25], []),
    ({"activation_threshold": 200, "negative_activation_threshold": (-200) % 65536, "potential_leak": -25,
      "potential": 100, "leak_rev": 0}, 10, (), 1, 0, [100, 75, 50, 25, 0, -25, -50, -75, -100, -125], []),
    ({"potential": 100, "activation_threshold": 200, "negative_activation_threshold": 60, "potential_leak": -50,
      "leak_rev": 0, "saturate": 1}, 10, (), 1, 0, [100, 50, 0, -50, -60, -60, -60, -60, -60, -60], []),
    ({"potential_leak": 50, "activation_threshold": 110}, 10, (), 1, 0, [0, 50, 100, 0, 50, 100, 0, 50, 100, 0], [2, 5, 8]),
    ({"potential_leak": -30, "activation_threshold": 100}, 10, (130, 50, 50, 50, 50, 0, 100, 80, 80, 80), 5, 3,
     [0, 0, 20, 40, 60, 80, 50, 0, 50, 0], [0, 6, 8]),
]


@pytest.mark.parametrize("case", range(len(ALTAI_KATS)))
def test_oracle_altai_known_answers(oracle_lib, case):
    """Expected potentials and spike steps of knp/tests/framework/altai_lif_test.cpp."""
    fields, steps, impacts, n, index, pots, spikes = ALTAI_KATS[case]
    neuron = T.altai_defaults(1)
    for k, v in fields.items():
        neuron[k] = v
    assert _run_altai(neuron, steps, impacts, n, index) == (pots, spikes)


@pytest.mark.skipif(not orc.available("reference"), reason="reference-header oracle not built (no KNP sources)")
def test_restated_oracle_matches_reference_headers_altai(oracle_lib):
    """AltAI-LIF populations (altai_impl.h:33-168, including the order-dependent BLOCKING rule and
    external impacts) and the resource-STDP AltAI golden network: the restated oracle gives the
    reference headers' spikes and neuron state."""
    from tests.golden.make_golden import canonical

    net, scheds = N.altai_network(steps=150)
    pop = net.populations[0].uid
    rng = np.random.default_rng(2)

    def ext(o, t):
        if t % 9 == 4:
            post = rng.integers(0, 200, 10).astype(np.uint32)
            o.send_impacts(T.uid_from_int(3103), pop, post, rng.choice(np.float32([-5, 3, 7, -2]), 10),
                           rng.choice(np.uint8([T.BLOCKING, T.EXCITATORY, T.DOPAMINE]), 10), True)

    rng_state = rng.bit_generator.state
    a, oa = orc.run(net, scheds, 150, which="restated", on_step=ext)
    rng.bit_generator.state = rng_state
    b, ob = orc.run(net, scheds, 150, which="reference", on_step=ext)
    assert spike_digest(a[pop]) == spike_digest(b[pop])
    assert canonical(oa.altai(pop)[0]) == canonical(ob.altai(pop)[0])
    assert sum(s.size for s in a[pop]) > 200
    assert (oa.altai(pop)[0]["activity_time"] != np.iinfo(np.int64).max).sum() > 5


def test_generated_synapses_follow_the_reference_index_rules():
    """network.generated_synapses (the host image of knp_gb300_generate_projection) pairs neurons as
    the reference's generators do for synapse index i (synapse_generators.h: all_to_all :64-69,
    aligned :99-118, exclusive :144-152, one_to_one :177-178, FixedProbability :295-299,
    FixedNumberPost :384-387, FixedNumberPre :442-444), restated here loop by loop."""
    from knp_gb300 import network as N
    from knp_gb300 import types as T

    args = dict(k_lo=-8, k_hi=8, d_lo=1, d_hi=6, seed=4, stream=40)
    pre, post, w, d = N.generated_synapses(T.GEN_ALL_TO_ALL, 7, 5, **args)
    assert list(zip(pre, post)) == [(i % 7, i // 7) for i in range(35)]
    for n_pre, n_post in ((12, 4), (3, 9), (6, 6)):
        pre, post, _, _ = N.generated_synapses(T.GEN_ALIGNED, n_pre, n_post, **args)
        exp = []
        for i in range(max(n_pre, n_post)):
            if n_pre >= n_post:
                exp.append((i, i // (n_pre // n_post)))
            else:
                exp.append((i // (n_post // n_pre), i))
        assert list(zip(pre, post)) == exp
    pre, post, _, _ = N.generated_synapses(T.GEN_EXCLUSIVE, 3, 3, **args)
    assert list(zip(pre, post)) == [(0, 1), (0, 2), (1, 0), (1, 2), (2, 0), (2, 1)]  # the reference's example
    pre, post, _, _ = N.generated_synapses(T.GEN_ONE_TO_ONE, 9, 9, **args)
    assert list(pre) == list(post) == list(range(9))
    pre, post, w, d = N.generated_synapses(T.GEN_FIXED_PROBABILITY, 40, 50, probability=0.1, **args)
    cand = pre.astype(np.int64) + 40 * post.astype(np.int64)
    assert np.all(np.diff(cand) > 0) and 120 < pre.size < 280  # kept pairs in index order, ~200 expected
    pre, post, _, _ = N.generated_synapses(T.GEN_FIXED_NUMBER_POST, 10, 30, count=100, **args)
    assert list(pre) == [i % 10 for i in range(100)] and post.max() < 30
    pre, post, w, d = N.generated_synapses(T.GEN_FIXED_NUMBER_PRE, 30, 10, count=100, **args)
    assert list(post) == [i % 10 for i in range(100)]
    s = args["stream"]
    fp = N.fixed_fan_in_pre(N.stream_key(4, s + 1), N.stream_key(4, s + 2), N.stream_key(4, s + 3), 30, 10, 10,
                            -8, 8, 1, 6)
    for x, y in zip((pre, post, w, d), fp):
        np.testing.assert_array_equal(x, y)
    assert np.all((w * 256 >= -8) & (w * 256 <= 8)) and np.all((d >= 1) & (d <= 6))
