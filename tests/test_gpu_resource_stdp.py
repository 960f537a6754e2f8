"""SynapticResourceSTDPDeltaSynapse projections trained by resource-STDP BLIFAT populations
(blifat_stdp.h:35-172, training/stdp.h:40-186), through the C ABI, against the CPU oracle.

Bar: spikes bit-exact per step; neuron state, weights and synapse rule state bit-exact (NaN equal to
NaN: the reference's arithmetic yields NaN for isi_max 0 under dopamine, and NaN payloads differ
between machines). The FP64 additional threshold is compared as FP64.
"""
import numpy as np
import pytest

from knp_gb300 import network as N
from knp_gb300 import types as T

pytestmark = pytest.mark.gpu

GOLDEN = [1, 6, 7, 11, 12, 13, 16, 17, 18, 19]


def run_both(net, scheds, steps, switches=None, step_mode=None):
    from knp_gb300 import backend as B
    from oracle import oracle as orc

    switches = switches or {}

    def gpu_step(be, t):
        if t in switches:
            be.start_learning() if switches[t] else be.stop_learning()

    def oracle_step(o, t):
        if t in switches:
            o.set_learning(switches[t])

    g, b = B.run(net, scheds, steps, on_step=gpu_step, step_mode=step_mode)
    o, oo = orc.run(net, scheds, steps, on_step=oracle_step)
    return g, b, o, oo


def same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    if a.dtype.names:
        for f in a.dtype.names:
            if not f.startswith("pad"):
                same(a[f], b[f], f"{what}.{f}")
        return
    np.testing.assert_array_equal(a, b, err_msg=what)  # NaN == NaN here


def check_all(net, g, b, o, oo):
    for k, p in enumerate(net.populations):
        for t, (x, y) in enumerate(zip(g[p.uid], o[p.uid])):
            assert np.array_equal(x, y), f"population {k} step {t}: gpu {x[:8]} vs oracle {y[:8]}"
        if p.kind == T.LIF:
            continue
        gs, gext = b.read_population(p.uid)
        os_, oext = oo.blifat(p.uid)
        for f in ("potential", "dynamic_threshold", "dopamine_value"):
            same(gs[f], os_[f].astype(np.float32).astype(np.float64), f)
        if p.kind == T.RESOURCE_STDP_BLIFAT:
            same(gs["additional_threshold"], os_["additional_threshold"], "additional_threshold")
            for f in ("isi_status", "last_step", "last_spike_step", "first_isi_spike", "is_being_forced",
                      "stability", "free_synaptic_resource"):
                same(gext[f], oext[f], f)
        same(gs["n_time_steps_since_last_firing"], os_["n_time_steps_since_last_firing"], "n_since")
    for k, pr in enumerate(net.projections):
        same(b.read_weights(pr.uid), oo.weights(pr.uid), f"weights of projection {k}")
        if pr.kind == T.RESOURCE_STDP_DELTA:
            same(b.read_resource_synapses(pr.uid), oo.resource_synapses(pr.uid), f"rules of projection {k}")
    assert b.counters()[0] == oo.events


def test_resource_stdp_golden():
    """single_thread_cpu_test.cpp:179-264: spikes on {1, 6, 7, 11, 12, 13, 16, 17, 18, 19} and the loop
    projection's weight changes; the per-phase step runs it (AUTO does not take the fused or grid
    kernel for such networks)."""
    net, sched = N.smallest_network("resource_stdp")
    g, b, o, oo = run_both(net, sched, 20)
    assert b.step_kernel == T.STEP_PHASES
    pop = net.populations[0].uid
    assert [t for t, s in enumerate(g[pop]) if s.size] == GOLDEN
    assert b.read_weights(net.projections[1].uid)[0] != 1.0
    check_all(net, g, b, o, oo)


def test_resource_stdp_mixed_network():
    """Every training path (Hebbian with and without forcing, ISI periods, dopamine reward and
    punishment, renormalisation with drain, the FP64 additional threshold, a recurrent projection
    loaded locked, a resource projection into a plain BLIFAT population, weights and potentials that
    the reference's arithmetic turns into NaN), with learning stopped at step 150 and started again
    at step 200."""
    net, sched = N.resource_stdp_mixed_network(steps=300)
    g, b, o, oo = run_both(net, sched, 300, switches={150: False, 200: True})
    check_all(net, g, b, o, oo)
    rules = b.read_resource_synapses(net.projections[0].uid)
    assert rules["had_hebbian_update"].sum() > 100 and rules["has_contributed"].sum() > 100
    assert np.isnan(b.read_population(net.populations[0].uid)[0]["potential"]).any()
    # The plain population's projection is not trained, but its synapses record presynaptic spikes.
    plain = b.read_resource_synapses(net.projections[4].uid)
    assert (plain["last_spike_step"] > 0).sum() > 100
    assert np.array_equal(plain["synaptic_resource"], net.projections[4].rule["synaptic_resource"])


def test_resource_stdp_mnist_shaped():
    """The mnist-learn-shaped network (resource-STDP input layer with dopamine, forcing and BLOCKING
    gates) over 20 samples of 15 steps."""
    net, sched = N.resource_stdp_network(samples=20)
    g, b, o, oo = run_both(net, sched, 300)
    check_all(net, g, b, o, oo)
    assert np.count_nonzero(b.read_weights(net.projections[0].uid)) > 1000


def test_resource_stdp_rejections():
    """A resource-STDP projection goes through its own entry point, carries no BLOCKING synapses,
    and keeps the backend on the per-phase step."""
    from knp_gb300 import backend as B

    net, _ = N.smallest_network("resource_stdp")
    pr = net.projections[1]
    b = B.GB300Backend(0)
    one = np.zeros(1, np.uint32)
    rc = b._lib.knp_gb300_load_projection(b._h, T.to_c_uid(pr.uid), T.RESOURCE_STDP_DELTA, T.to_c_uid(pr.pre_uid),
                                          T.to_c_uid(pr.post_uid), 1, one.ctypes.data, one.ctypes.data,
                                          np.ones(1, np.float32).ctypes.data, np.ones(1, np.uint32).ctypes.data,
                                          None, None, None)
    assert rc == -1  # KNP_GB300_E_INVALID
    blk = N.Projection(T.uid_from_int(77), T.RESOURCE_STDP_DELTA, T.NULL_UID, pr.post_uid, one, one,
                       np.ones(1, np.float32), np.ones(1, np.uint32), out_type=np.full(1, T.BLOCKING, np.uint8),
                       rule=T.resource_synapse_defaults(1))
    with pytest.raises(Exception):
        b.load_projections([blk])
    b.close()
    for mode in (T.STEP_FUSED, T.STEP_GRID):
        b = B.GB300Backend(0)
        b.set_step_mode(mode)
        b.load_network(net)
        with pytest.raises(Exception):
            b._init()
        b.close()
