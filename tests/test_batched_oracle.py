"""CPU tests of the batched form's FP64 oracle (oracle/batched_fp64.py) against the reference LIF
arithmetic: the restated single-threaded backend (FP32 potentials, impacts added in message order,
lif_impl.h:33-86 of the reference CPU library) and, where the KNP sources were present to build it,
the reference-header oracle; and against the fixture the reference-header oracle wrote."""
import json
import os
import zlib

import numpy as np
import pytest

from knp_gb300 import batched as BT
from oracle import batched_fp64 as BF
from oracle import oracle as orc

HERE = os.path.dirname(os.path.abspath(__file__))


def _per_sample(out, net, cfg, samples):
    """{layer: bool [T_max, S, n]} from an oracle run of the block-diagonal network."""
    L = len(cfg.sizes) - 1
    t_max = int(cfg.steps[samples].max())
    res = {}
    for l in range(1, L + 1):
        n = cfg.sizes[l]
        uid = net.populations[l - 1].uid
        a = np.zeros((t_max, len(samples), n), bool)
        for t in range(t_max):
            idx = out[uid][t].astype(np.int64)
            a[t, idx // n, idx % n] = True
        res[l] = a
    return res


def _disagreement(a, b, cfg, samples):
    T_b = cfg.steps[samples].astype(np.int64)
    mism = total = 0
    for l in a:
        if l == 0:
            continue
        live = (np.arange(a[l].shape[0])[:, None] < T_b[None, :])[:, :, None]
        mism += int(((a[l] != b[l]) & live).sum())
        total += int(live.sum()) * a[l].shape[2]
    return mism, total


@pytest.mark.parametrize("which", ["restated", "reference"])
def test_fp64_oracle_against_reference_lif_arithmetic(oracle_lib, which):
    """Six samples of a dense batched config (64-96-96-10, N(0, 1/fan_in) BF16 weights): the FP64
    oracle and the reference LIF arithmetic (FP32) on the same block-diagonal network agree on at
    least 99.9% of (sample, neuron, step); they can differ only where an FP32 potential lies within
    rounding of the threshold."""
    if which == "reference" and not orc.available("reference"):
        pytest.skip("reference-header oracle not built (no KNP sources)")
    cfg = BT.dense_config(seed=9, batch=6, sizes=(64, 96, 96, 10), t_lo=10, t_hi=30, rate_max=0.3)
    samples = np.arange(cfg.batch)
    fp = BF.run_fp64(cfg)
    net, sched = BT.plain_network(cfg)
    out, _ = orc.run(net, [sched], int(cfg.steps.max()), which=which)
    ref = _per_sample(out, net, cfg, samples)
    mism, total = _disagreement(fp, ref, cfg, samples)
    assert total > 0 and sum(int(fp[l].sum()) for l in (1, 2, 3)) > 100
    assert mism <= 0.001 * total, (mism, total)


def test_fp64_oracle_inputs_are_the_batched_draws():
    """The oracle's input spikes are the draws of knp_gb300.batched.input_spikes, sample by sample."""
    cfg = BT.dense_config(seed=5, batch=4, sizes=(100, 32, 10), t_lo=5, t_hi=9, rate_max=0.5)
    fp = BF.run_fp64(cfg)
    for b in range(cfg.batch):
        for t in range(int(cfg.steps.max())):
            exp = BT.input_spikes(cfg, b, t) if t < cfg.steps[b] else np.zeros(0, np.uint32)
            np.testing.assert_array_equal(np.nonzero(fp[0][t, b])[0], exp)


def test_fp64_oracle_against_reference_fixture():
    """Per-sample spike digests of the reference-header oracle (tests/golden/batched_oracle.json,
    written by tests/golden/make_golden.py --batched): the FP64 oracle reproduces them on every
    sample/layer whose sums never came within FP32 rounding of the threshold, and differs on at most
    0.1% of (sample, neuron, step) overall."""
    with open(os.path.join(HERE, "golden", "batched_oracle.json")) as f:
        fx = json.load(f)
    cfg = BT.dense_config(**fx["config"])
    samples = np.arange(cfg.batch)
    fp = BF.run_fp64(cfg)
    exact = mism_steps = 0
    for case in fx["layers"]:
        l, s = case["layer"], case["sample"]
        counts = [int(fp[l][t, s].sum()) for t in range(int(cfg.steps[s]))]
        crcs = [zlib.crc32(np.nonzero(fp[l][t, s])[0].astype(np.uint32).tobytes()) for t in range(int(cfg.steps[s]))]
        same = [a == b and c == d for a, b, c, d in zip(counts, case["counts"], crcs, case["crcs"])]
        exact += all(same)
        mism_steps += same.count(False)
    assert exact >= len(fx["layers"]) - 1
    assert mism_steps <= 0.001 * sum(len(c["counts"]) for c in fx["layers"]) + 2
