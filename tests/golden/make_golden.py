"""Writes tests/golden/spike_digests.json from the reference-header oracle (oracle/_ref/libknp_ref.so:
the KNP reference's own per-neuron / per-synapse headers, built by `make -C oracle ref` where the
KNP sources are present). Run from the repository root:

    python tests/golden/make_golden.py

Each case stores, per step, the spike count and the CRC32 of the ascending spike indexes of the
network's first population, the total synaptic event count, and CRC32s of final projection weights.

`python tests/golden/make_golden.py --batched` writes tests/golden/batched_oracle.json: per (layer,
sample) spike digests of a small dense batched config run as one block-diagonal LIF network.

`python tests/golden/make_golden.py --full` also writes tests/golden/stdp_full.json for the full STDP
learning config (200 samples x 100 steps; about two minutes of CPU): per sample the spike count and
a CRC32 over that sample's per-step digests, the final plastic weights' CRC32, and every 613th final
weight (for the relative-error check).
"""
import json
import os
import sys
import zlib

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from knp_gb300 import network as N  # noqa: E402
from knp_gb300 import types as T  # noqa: E402
from oracle import oracle as orc  # noqa: E402

CASES = [
    ("smallest_delta", "smallest_network", {"kind": "delta"}, 20, [0, 1]),
    ("smallest_stdp", "smallest_network", {"kind": "stdp"}, 20, [0, 1]),
    ("smallest_stdp_resource", "smallest_network", {"kind": "stdp_resource_neuron"}, 20, [0, 1]),
    ("small_seed1_1000", "small_network", {"seed": 1, "steps": 1000}, 1000, []),
    ("large_sparse_n2000", "large_sparse_network", {"seed": 2, "n": 2000, "fan_in": 200, "steps": 100}, 100, []),
    ("stdp_3samples", "stdp_network", {"seed": 3, "samples": 3, "steps_per_sample": 100}, 300, [0, 1]),
    ("smallest_resource_stdp", "smallest_network", {"kind": "resource_stdp"}, 20, [0, 1]),
    ("smallest_resource_stdp_altai", "smallest_network", {"kind": "resource_stdp_altai"}, 20, [0, 1]),
    ("resource_mnist_shaped", "resource_stdp_network", {"samples": 8}, 120, [0]),
    ("resource_mixed", "resource_stdp_mixed_network", {"steps": 300}, 300, [0, 1, 4]),
]
# Learning switches of a case: {step: on}, applied before that step (stop_learning / start_learning).
LEARNING = {"resource_mixed": {150: False, 200: True}}


def learning_switch(switches):
    """An oracle.run on_step callback that applies {step: on} learning switches."""
    def on_step(o, t):
        if t in switches:
            o.set_learning(switches[t])
    return on_step


def canonical(a):
    """Bytes of an array with every FP32 / FP64 NaN replaced by one quiet NaN, so that digests do not
    depend on the NaN payloads of the machine (x86 and Arm produce different default NaNs)."""
    a = np.array(a, copy=True)
    if a.dtype.names:
        for f in a.dtype.names:
            if a.dtype[f] in (np.float32, np.float64):
                a[f] = np.where(np.isnan(a[f]), a.dtype[f].type(np.nan), a[f])
        return a.tobytes()
    if a.dtype in (np.float32, np.float64):
        a = np.where(np.isnan(a), a.dtype.type(np.nan), a).astype(a.dtype)
    return a.tobytes()


def population_state(o, pop):
    """(neurons, resource extension or None) of a population of any kind from an oracle."""
    kind = o._sizes[pop.uid][0]
    if T.is_altai(kind):
        return o.altai(pop.uid)
    return o.blifat(pop.uid)


def digest(trains):
    return [[int(s.size), zlib.crc32(np.ascontiguousarray(s, np.uint32).tobytes())] for s in trains]


def sample_digest(trains, steps_per_sample):
    """Per sample: [spike count, CRC32 of the concatenated per-step (count, CRC32) pairs]."""
    d = np.asarray(digest(trains), np.uint64).astype(np.uint32)
    out = []
    for s0 in range(0, len(trains), steps_per_sample):
        blk = d[s0:s0 + steps_per_sample]
        out.append([int(blk[:, 0].sum()), zlib.crc32(np.ascontiguousarray(blk).tobytes())])
    return out


def full_stdp():
    kwargs = {"seed": 3, "samples": 200, "steps_per_sample": 100}
    net, sched = N.stdp_network(**kwargs)
    steps = 200 * 100
    res, o = orc.run(net, sched, steps, which="reference")
    pop = net.populations[0].uid
    w = o.weights(net.projections[0].uid)
    case = {"source": "oracle/_ref/libknp_ref.so (KNP reference headers + shim)", "builder": "stdp_network",
            "kwargs": kwargs, "steps": steps, "events": o.events,
            "samples": sample_digest(res[pop], 100), "weights_crc": zlib.crc32(w.tobytes()),
            "weights_stride": 613, "weights_sampled": [float(x) for x in w[::613]]}
    with open(os.path.join(ROOT, "tests", "golden", "stdp_full.json"), "w") as f:
        json.dump(case, f, separators=(",", ":"))
    print("stdp_full", "spikes", sum(s.size for s in res[pop]), "events", o.events)


BATCHED = {"seed": 9, "batch": 8, "sizes": [128, 160, 128, 10], "t_lo": 20, "t_hi": 60, "rate_max": 0.3}


def batched_oracle():
    """Per (layer, sample) of a small dense batched config run as one block-diagonal LIF network by
    the reference-header oracle: each step's spike count and CRC32 of the sample's ascending
    neuron indexes."""
    from knp_gb300 import batched as BT

    cfg = BT.dense_config(**BATCHED)
    net, sched = BT.plain_network(cfg)
    res, _ = orc.run(net, [sched], int(cfg.steps.max()), which="reference")
    layers = []
    for l in range(1, len(cfg.sizes)):
        n = cfg.sizes[l]
        uid = net.populations[l - 1].uid
        for s in range(cfg.batch):
            counts, crcs = [], []
            for t in range(int(cfg.steps[s])):
                idx = res[uid][t].astype(np.int64)
                mine = (idx[(idx // n) == s] % n).astype(np.uint32)
                counts.append(int(mine.size))
                crcs.append(zlib.crc32(np.ascontiguousarray(mine).tobytes()))
            layers.append({"layer": l, "sample": s, "counts": counts, "crcs": crcs})
    out = {"source": "oracle/_ref/libknp_ref.so (KNP reference headers + shim)", "config": BATCHED, "layers": layers}
    with open(os.path.join(ROOT, "tests", "golden", "batched_oracle.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    print("batched_oracle", "spikes", sum(sum(c["counts"]) for c in layers))


def knp_reference_dir():
    """The KNP sources: $KNP_REF, else a `reference` directory beside this repository."""
    return os.environ.get("KNP_REF") or os.path.join(os.path.dirname(ROOT), "reference")


def main():
    orc.build("reference", knp_ref=knp_reference_dir())
    if "--full" in sys.argv:
        full_stdp()
        return
    if "--batched" in sys.argv:
        batched_oracle()
        return
    out = {"source": "oracle/_ref/libknp_ref.so (KNP reference headers + shim)", "cases": []}
    for name, builder, kwargs, steps, wproj in CASES:
        net, sched = getattr(N, builder)(**kwargs)
        switches = LEARNING.get(name, {})
        res, o = orc.run(net, sched, steps, which="reference", on_step=learning_switch(switches) if switches else None)
        pop = net.populations[0].uid
        case = {"name": name, "builder": builder, "kwargs": kwargs, "steps": steps,
                "digest": digest(res[pop]), "events": o.events}
        if switches:
            case["learning"] = {str(k): v for k, v in switches.items()}
        resource = [k for k, pr in enumerate(net.projections) if pr.kind == T.RESOURCE_STDP_DELTA]
        if resource:
            # Digests over NaN-canonical bytes: weights, rule state and the first population's state.
            case["weights_crc"] = {str(k): zlib.crc32(canonical(o.weights(net.projections[k].uid))) for k in wproj}
            case["rules_crc"] = {str(k): zlib.crc32(canonical(o.resource_synapses(net.projections[k].uid)))
                                 for k in resource}
            neurons, ext = population_state(o, net.populations[0])
            case["state_crc"] = zlib.crc32(canonical(neurons) + (b"" if ext is None else canonical(ext)))
        elif wproj:
            case["weights_crc"] = {str(k): zlib.crc32(o.weights(net.projections[k].uid).tobytes()) for k in wproj}
        out["cases"].append(case)
        print(name, "spikes", sum(s.size for s in res[pop]), "events", o.events)
    with open(os.path.join(ROOT, "tests", "golden", "spike_digests.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
