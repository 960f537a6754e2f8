"""AltAI-LIF populations (altai_impl.h:33-168) and their resource-STDP variant (altai_stdp.h) through the
C ABI: the reference's AltAI known answers (knp/tests/framework/altai_lif_test.cpp), the
resource-STDP AltAI golden network (single_thread_cpu_test.cpp:267-355), and a network with every
option, BLOCKING synapses and external impacts against the CPU oracle.

Bar: spikes bit-exact per step, potentials, pre-impact potentials, activity times, dopamine values and
weights bit-exact (integer weights: the reference's impact-by-impact FP32 sum is exact then).
"""
import numpy as np
import pytest

from knp_gb300 import network as N
from knp_gb300 import types as T
from tests.test_oracle import ALTAI_KATS

pytestmark = pytest.mark.gpu

GOLDEN = [1, 6, 7, 11, 12, 13, 16, 17, 18, 19]


def _run_altai_gpu(neuron, steps, impacts=(), n=1, index=0):
    from knp_gb300 import backend as B

    pop_uid, in_uid = T.uid_from_int(601), T.uid_from_int(602)
    net = N.Network([N.Population(pop_uid, T.ALTAI_LIF, np.repeat(neuron, n))], [], [(pop_uid, in_uid)])
    b = B.GB300Backend(0)
    b.load_network(net)
    b._init()
    pots, spikes = [], []
    for t in range(steps):
        if t < len(impacts):
            b.send_impacts(in_uid, pop_uid, [index], [impacts[t]], [T.EXCITATORY], True)
        pots.append(int(np.int16(b.read_population(pop_uid)[0]["potential"][index])))
        b.step(1)
        if index in b.spikes(pop_uid, t):
            spikes.append(t)
    b.close()
    return pots, spikes


@pytest.mark.parametrize("case", range(len(ALTAI_KATS)))
def test_altai_known_answers(case):
    """Expected potentials and spike steps of knp/tests/framework/altai_lif_test.cpp:97-190."""
    fields, steps, impacts, n, index, pots, spikes = ALTAI_KATS[case]
    neuron = T.altai_defaults(1)
    for k, v in fields.items():
        neuron[k] = v
    assert _run_altai_gpu(neuron, steps, impacts, n, index) == (pots, spikes)


def _same_altai_state(b, oo, pop):
    g, gext = b.read_population(pop)
    o, oext = oo.altai(pop)
    for f in ("potential", "pre_impact_potential", "activity_time", "additional_threshold"):
        np.testing.assert_array_equal(g[f], o[f], err_msg=f)
    np.testing.assert_array_equal(g["dopamine_value"], o["dopamine_value"].astype(np.float32).astype(np.float64))
    if oext is not None:
        for f in ("isi_status", "last_step", "last_spike_step", "first_isi_spike", "stability", "free_synaptic_resource"):
            np.testing.assert_array_equal(gext[f], oext[f], err_msg=f)


def test_altai_network_with_blocking_and_external_impacts():
    """Every AltAI option, integer-weight excitatory / inhibitory / recurrent synapses, BLOCKING
    synapses with repeated (pre, post) pairs (applied in the reference's message order), dopamine, and
    external EXCITATORY / BLOCKING / DOPAMINE impact messages, against the oracle step by step."""
    from knp_gb300 import backend as B
    from oracle import oracle as orc

    net, scheds = N.altai_network(steps=200)
    pop = net.populations[0].uid
    plan = {}
    rng = np.random.default_rng(2)
    for t in range(4, 200, 9):
        plan[t] = (rng.integers(0, 200, 10).astype(np.uint32), rng.choice(np.float32([-5, 3, 7, -2]), 10),
                   rng.choice(np.uint8([T.BLOCKING, T.EXCITATORY, T.DOPAMINE]), 10))

    def ext(be, t):
        if t in plan:
            post, vals, types = plan[t]
            be.send_impacts(T.uid_from_int(3103), pop, post, vals, types, True)

    g, b = B.run(net, scheds, 200, on_step=ext)
    o, oo = orc.run(net, scheds, 200, on_step=ext)
    assert b.step_kernel == T.STEP_PHASES
    for t, (x, y) in enumerate(zip(g[pop], o[pop])):
        assert np.array_equal(x, y), f"step {t}: gpu {x[:8]} vs oracle {y[:8]}"
    _same_altai_state(b, oo, pop)
    assert sum(s.size for s in o[pop]) > 200
    assert b.counters()[0] == oo.events


def test_resource_stdp_altai_golden():
    """single_thread_cpu_test.cpp:267-355: resource-STDP synapses onto one resource-STDP AltAI-LIF
    neuron: spikes on {1, 6, 7, 11, 12, 13, 16, 17, 18, 19}, weights, rule and neuron state as the oracle's."""
    from knp_gb300 import backend as B
    from oracle import oracle as orc

    net, sched = N.smallest_network("resource_stdp_altai")
    g, b = B.run(net, sched, 20)
    o, oo = orc.run(net, sched, 20)
    pop = net.populations[0].uid
    assert [t for t, s in enumerate(g[pop]) if s.size] == GOLDEN
    for pr in net.projections:
        np.testing.assert_array_equal(b.read_weights(pr.uid), oo.weights(pr.uid))
        got, exp = b.read_resource_synapses(pr.uid), oo.resource_synapses(pr.uid)
        for f in exp.dtype.names:
            np.testing.assert_array_equal(got[f], exp[f], err_msg=f)
    assert b.read_weights(net.projections[1].uid)[0] != 1.0
    _same_altai_state(b, oo, pop)
