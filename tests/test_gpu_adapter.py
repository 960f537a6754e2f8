"""The knp::core::Backend adapter (knp_gb300/adapter) on the GPU, driven like the reference's own
backend tests (knp/tests/backend/single_thread_cpu_test.cpp:54-176): through its message bus, with
input SpikeMessages from an external endpoint on steps 0, 5, 10, 15 and the population's
SpikeMessages received there. The one-neuron delta, additive-STDP and resource-STDP-neuron networks
give the reference's golden spike steps, and the weights get_network_data returns equal the oracle's;
external SynapticImpactMessages to a LIF population fire it where the FP32 potentials cross."""
import numpy as np
import pytest

from knp_gb300 import network as N
from tests import adapter_build as AB

pytestmark = pytest.mark.gpu

GOLDEN = [1, 6, 7, 11, 12, 13, 16, 17, 18, 19]


@pytest.fixture(scope="module")
def harness():
    return AB.build_harness()


def _parse(out):
    lines = dict(line.split(":", 1) for line in out.strip().splitlines() if ":" in line)
    steps = [int(x) for x in lines["steps"].split()]
    weights = [float(x) for x in lines["weights"].split()] if "weights" in lines else None
    return steps, weights


@pytest.mark.parametrize("case,kind", [("delta", "delta"), ("stdp", "stdp"), ("resource", "stdp_resource_neuron"),
                                       ("resource_stdp", "resource_stdp")])
def test_adapter_golden_network_through_the_bus(harness, case, kind):
    from oracle import oracle as orc

    r = AB.run_harness(harness, case)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), (r.stdout, r.stderr)
    steps, weights = _parse(r.stdout)
    assert steps == GOLDEN
    net, sched = N.smallest_network(kind)
    _, o = orc.run(net, sched, 20)
    expect = [float(o.weights(net.projections[1].uid)[0]), float(o.weights(net.projections[0].uid)[0])]
    np.testing.assert_array_equal(np.float32(weights), np.float32(expect))


def test_adapter_external_impacts_to_lif_population(harness):
    r = AB.run_harness(harness, "impacts")
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), (r.stdout, r.stderr)
    steps, _ = _parse(r.stdout)
    v, exp = np.float32(0), []
    for t, x in enumerate(np.float32([0.5, 0.6, 0.2, 0.9, 0.1, 1.5])):
        v = np.float32(v + x)
        if v > np.float32(1):
            exp.append(t)
            v = np.float32(0)
    assert steps == exp
