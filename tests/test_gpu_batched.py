"""Batched / precision form: tcgen05 BF16 GEMM (FP32 accumulation in tensor memory) against a
PyTorch FP32 reference of the same BF16 operands (tolerance: relative 1e-5, FP32 summation order)."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _gemm(a, b):
    from knp_gb300 import _capi

    M, K = a.shape
    N = b.shape[0]
    d = torch.full((M, N), float("nan"), device="cuda", dtype=torch.float32)
    err = torch.zeros(1, device="cuda", dtype=torch.int32)
    rc = _capi.lib().knp_gb300_bf16_gemm_tn(
        ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(d.data_ptr()), M, N, K,
        ctypes.c_void_p(err.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, _capi.lib().knp_gb300_last_error()
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return d


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (128, 64, 16), (200, 100, 784), (256, 1000, 1000), (37, 10, 1000),
                                   (300, 260, 8192), (4096, 512, 784), (129, 129, 72), (512, 10, 8200),
                                   (304, 256, 8192), (512, 64, 4104), (136, 8, 512),
                                   (4864, 1024, 256), (4900, 1000, 200)])  # the last two: 128 x 256 tiles
def test_bf16_gemm_tn(M, N, K):
    g = torch.Generator(device="cpu").manual_seed(M * 7 + N + K)
    a = (torch.rand(M, K, generator=g) < 0.2).to(torch.bfloat16).cuda()  # 0/1 spike matrix
    b = (torch.randn(N, K, generator=g) / K ** 0.5).to(torch.bfloat16).cuda()
    ref = a.float() @ b.float().t()
    d = _gemm(a, b)
    torch.testing.assert_close(d, ref, rtol=1e-5, atol=1e-5)


def test_bf16_gemm_tn_split_k_is_deterministic():
    """Few tiles and a long K take the split-K form; its partial tiles are added in split order, so
    repeated calls give the same bits."""
    g = torch.Generator(device="cpu").manual_seed(11)
    a = torch.randn(256, 8192, generator=g).to(torch.bfloat16).cuda()
    b = torch.randn(128, 8192, generator=g).to(torch.bfloat16).cuda()
    d0 = _gemm(a, b)
    for _ in range(3):
        assert torch.equal(_gemm(a, b), d0)
    torch.testing.assert_close(d0, a.float() @ b.float().t(), rtol=1e-5, atol=1e-3)


def test_bf16_gemm_tn_dense_values():
    g = torch.Generator(device="cpu").manual_seed(5)
    a = torch.randn(130, 96, generator=g).to(torch.bfloat16).cuda()
    b = torch.randn(48, 96, generator=g).to(torch.bfloat16).cuda()
    torch.testing.assert_close(_gemm(a, b), a.float() @ b.float().t(), rtol=1e-5, atol=1e-4)


def _batched_spikes(cfg, rec, layer, b, t):
    from knp_gb300 import batched as BT

    return BT.spikes_from_bits(rec[layer][t, b], cfg.sizes[layer])


def test_batched_lif_matches_plain_fp32_path():
    """Batched tcgen05 form against the FP32 plain path on the same samples (block-diagonal network,
    same BF16-valued weights, FP32 input rings): every layer's spikes agree on at least 99.9% of
    (sample, neuron, step) and the input spikes agree exactly."""
    from knp_gb300 import backend as B
    from knp_gb300 import batched as BT
    from knp_gb300 import types as T

    cfg = BT.dense_config(seed=9, batch=24, sizes=(64, 96, 96, 10), t_lo=10, t_hi=30, rate_max=0.3)
    counts, rec, events, ms = BT.run(cfg, record=True)
    net, sched = BT.plain_network(cfg)
    t_max = int(cfg.steps.max())
    out, b = B.run(net, [sched], t_max, accumulator=T.ACC_FP32)
    # Input layer: identical draws.
    for s in range(cfg.batch):
        for t in range(int(cfg.steps[s])):
            np.testing.assert_array_equal(_batched_spikes(cfg, rec, 0, s, t), BT.input_spikes(cfg, s, t))
    total = mism = 0
    for l in range(1, len(cfg.sizes)):
        n = cfg.sizes[l]
        uid = net.populations[l - 1].uid
        for t in range(t_max):
            plain = out[uid][t]
            for s in range(cfg.batch):
                if t >= cfg.steps[s]:
                    continue
                g = _batched_spikes(cfg, rec, l, s, t)
                p = plain[(plain >= s * n) & (plain < (s + 1) * n)] - s * n
                mism += np.setxor1d(g, p).size
                total += n
    assert mism <= 1e-3 * total, (mism, total)
    # Output counts are the last layer's recorded spikes.
    L = len(cfg.sizes) - 1
    for s in range(cfg.batch):
        c = np.zeros(cfg.sizes[L], np.int64)
        for t in range(int(cfg.steps[s])):
            c[_batched_spikes(cfg, rec, L, s, t)] += 1
        np.testing.assert_array_equal(counts[s], c)
    assert events > 0 and ms > 0


def test_batched_lif_full_config_runs():
    """The full batched dense config (256 samples, 784-1000-1000-10, T in [50, 200])."""
    from knp_gb300 import batched as BT

    cfg = BT.dense_config(seed=4)
    counts, _, events, ms = BT.run(cfg)
    assert counts.shape == (256, 10) and events > 0 and ms > 0


def _compare_with_plain(cfg, rec, counts):
    """Spike mismatch of the batched form against the plain FP32 path on the same samples."""
    from knp_gb300 import backend as B
    from knp_gb300 import batched as BT
    from knp_gb300 import types as T

    net, sched = BT.plain_network(cfg)
    t_max = int(cfg.steps.max())
    out, b = B.run(net, [sched], t_max, accumulator=T.ACC_FP32)
    for s in range(cfg.batch):
        for t in range(int(cfg.steps[s])):
            np.testing.assert_array_equal(_batched_spikes(cfg, rec, 0, s, t), BT.input_spikes(cfg, s, t))
    total = mism = 0
    for layer in range(1, len(cfg.sizes)):
        n = cfg.sizes[layer]
        uid = net.populations[layer - 1].uid
        for t in range(t_max):
            plain = out[uid][t]
            for s in range(cfg.batch):
                if t >= cfg.steps[s]:
                    continue
                g = _batched_spikes(cfg, rec, layer, s, t)
                p = plain[(plain >= s * n) & (plain < (s + 1) * n)] - s * n
                mism += np.setxor1d(g, p).size
                total += n
    return mism, total


def test_batched_plan_graph_runs_repeat_exactly():
    """A plan (one CUDA-graph launch per run, autotuned ring depth) gives identical counts, spike
    records and event counts on every run, and the same results as the one-shot form."""
    from knp_gb300 import batched as BT

    cfg = BT.dense_config(seed=10, batch=130, sizes=(200, 160, 96, 10), t_lo=20, t_hi=40, rate_max=0.3)
    plan = BT.BatchedPlan(cfg, record=True, autotune=True)
    try:
        stages, ring, tuned = plan.info()
        assert stages in (2, 3, 4) and ring in (4, 8, 16) and (stages, ring) in tuned
        ev1, ms1 = plan.run()
        c1, r1 = plan.counts(), plan.record()
        ev2, ms2 = plan.run()
        c2, r2 = plan.counts(), plan.record()
    finally:
        plan.close()
    assert ev1 == ev2 and ev1 > 0 and ms1 > 0 and ms2 > 0
    np.testing.assert_array_equal(c1, c2)
    for layer in r1:
        np.testing.assert_array_equal(r1[layer], r2[layer])
    c3, r3, ev3, _ = BT.run(cfg, record=True)
    assert ev3 == ev1
    np.testing.assert_array_equal(c3, c1)
    for layer in r1:
        np.testing.assert_array_equal(r3[layer], r1[layer])


def test_batched_uneven_instance_sizes_match_plain_fp32_path():
    """Samples that are network instances of uneven size (per-sample layer widths over shared
    weights) against the plain FP32 path with the missing neurons silenced: at most 0.1% mismatch,
    identical inputs, and no spike from a neuron beyond its sample's size."""
    from knp_gb300 import batched as BT

    cfg = BT.uneven_config(seed=8, batch=40)
    counts, rec, events, ms = BT.run(cfg, record=True)
    for layer in range(1, len(cfg.sizes)):
        for s in range(cfg.batch):
            for t in range(int(cfg.steps[s])):
                g = _batched_spikes(cfg, rec, layer, s, t)
                assert g.size == 0 or g.max() < cfg.sample_sizes[layer][s]
    mism, total = _compare_with_plain(cfg, rec, counts)
    assert mism <= 1e-3 * total, (mism, total)
    assert events > 0 and ms > 0


def test_batched_segments_give_identical_results():
    """Cutting the run into persistent launches of a few steps each (LIF state saved and restored
    between launches, layer rings and step counters carried over, input spikes drawn per segment)
    changes no spike, count or event."""
    from knp_gb300 import batched as BT

    cfg = BT.dense_config(seed=12, batch=150, sizes=(120, 200, 64, 10), t_lo=5, t_hi=33, rate_max=0.3)
    c1, r1, e1, _ = BT.run(cfg, record=True)
    assert e1 > 0
    for seg in (1, 7):
        c2, r2, e2, _ = BT.run(cfg, record=True, segment_steps=seg)
        assert e2 == e1
        np.testing.assert_array_equal(c2, c1)
        for layer in r1:
            np.testing.assert_array_equal(r2[layer], r1[layer])


def test_batched_full_config_identical_across_depths_and_repeats():
    """The full dense config (256 samples, 784-1000-1000-10: several chunks per K half, two sample
    tiles, layers running ahead of each other on the ring counters) gives bit-identical spike
    records, counts and event totals at every operand-ring depth and on repeated runs; a counting
    error in the inter-layer step protocol shows up here as run-to-run differences."""
    from knp_gb300 import batched as BT

    cfg = BT.dense_config(seed=4)
    ref = None
    for stages in (2, 3, 4):
        plan = BT.BatchedPlan(cfg, record=True, stages=stages)
        try:
            for _ in range(2):
                ev, _ = plan.run()
                got = (ev, plan.counts(), plan.record())
                if ref is None:
                    ref = got
                    continue
                assert got[0] == ref[0]
                np.testing.assert_array_equal(got[1], ref[1])
                for layer in ref[2]:
                    np.testing.assert_array_equal(got[2][layer], ref[2][layer])
        finally:
            plan.close()


def test_batched_input_rates_at_the_edges():
    """Input draws for rates at and beyond the ends of [0, 1] (negative, NaN, subnormal, 1, above 1,
    infinity) equal the host restatement: never below 0 or for NaN, always at 1 and above."""
    from knp_gb300 import batched as BT

    cfg = BT.dense_config(seed=13, batch=6, sizes=(64, 32, 10), t_lo=5, t_hi=9, rate_max=0.5)
    edge = np.array([0.0, -0.5, np.nan, 1e-40, 1.0, 1.5, np.inf, 0.999999], np.float32)
    cfg.rates[:, :edge.size] = edge
    counts, rec, events, ms = BT.run(cfg, record=True)
    for s in range(cfg.batch):
        for t in range(int(cfg.steps[s])):
            got = BT.spikes_from_bits(rec[0][t, s], cfg.sizes[0])
            np.testing.assert_array_equal(got, BT.input_spikes(cfg, s, t))
            assert {4, 5, 6} <= set(got.tolist()) and not ({0, 1, 2, 3} & set(got.tolist()))


def test_batched_ring_wait_timeout_reports_an_error(monkeypatch):
    """Failure detection: with KNP_GB300_BATCHED_STALL=1 every consumer layer waits for one producer
    CTA more than exists, a step counter that nothing ever raises. Its bounded wait (a short poll
    limit in this mode) gives up, every other wait of the launch stops on the reported failure, the
    CTA pairs drain their in-flight MMAs and partial-sum stores and free their tensor memory, and the
    run returns the device-error status instead of hanging. A plan created afterwards on the same
    device gives the same results as a run before the failure."""
    from knp_gb300 import batched as BT
    from knp_gb300._capi import KnpGb300Error

    cfg = BT.dense_config(seed=10, batch=130, sizes=(200, 160, 96, 10), t_lo=20, t_hi=40, rate_max=0.3)
    c0, r0, ev0, _ = BT.run(cfg, record=True)
    monkeypatch.setenv("KNP_GB300_BATCHED_STALL", "1")
    plan = BT.BatchedPlan(cfg, record=True, stages=2)  # a fixed ring depth: no tuning runs at creation
    try:
        with pytest.raises(KnpGb300Error) as err:
            plan.run()
        assert err.value.code == -4  # KNP_GB300_E_DEVICE_FLAG
    finally:
        plan.close()
    monkeypatch.delenv("KNP_GB300_BATCHED_STALL")
    c1, r1, ev1, _ = BT.run(cfg, record=True)
    assert ev1 == ev0
    np.testing.assert_array_equal(c1, c0)
    for layer in r0:
        np.testing.assert_array_equal(r1[layer], r0[layer])


def test_batched_dense_config_against_fp64_oracle():
    """The full batched dense config (256 samples, 784-1000-1000-10, T in [50, 200], BF16 weights,
    FP32 accumulation on the tensor cores) against the FP64 oracle (oracle/batched_fp64.py: the
    reference LIF semantics of lif_impl.h:33-86 in exact arithmetic, pinned to the reference-header
    oracle on the CPU) over every sample's own steps: the input spikes are identical, and at most
    0.1% of (sample, neuron, step) of layers 1-3 differ."""
    from knp_gb300 import batched as BT
    from oracle import batched_fp64 as BF

    cfg = BT.dense_config(seed=4)
    _, rec, _, _ = BT.run(cfg, record=True)
    fp = BF.run_fp64(cfg)
    m0, t0 = BF.mismatch(fp, rec, cfg, layers=[0])
    assert m0 == 0 and t0 > 0
    m, t = BF.mismatch(fp, rec, cfg)
    print(f"batched tcgen05 form vs FP64 oracle: {m} of {t} (sample, neuron, step) differ ({m / t:.2e})")
    assert m <= 0.001 * t, (m, t)
