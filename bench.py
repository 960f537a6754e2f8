"""Benchmark of the GB300 KNP backend on the large sparse plain configuration.

Workload (one GPU): 1,000,000 BLIFAT neurons (reference defaults), fixed fan-in 1000 from uniform
random presynaptic sources (1e9 delta synapses; int32 index, FP32 weight k/256 with k in [-16, 48],
u8 delay in 1..20), Bernoulli background drive p = 0.005 per neuron per step through a one-to-one
projection (w = 1.0, delay 1). A step is one simulation step of the whole network; the network
ramps up from the background rate and, after about 30 steps, every neuron fires every step. The
synapse arrays (9 GB) are far larger than L2, so no L2 flush is needed between steps.

Every figure of the main line describes the same steps: W untimed warm-up steps, then the K timed
steps W..W+K-1 (with the defaults, the sparse ramp: a few thousand spikes per step, scattered).
value      synaptic events/s of the K steps with the background schedule already in HBM, timed with
           CUDA events on the backend's stream (in grid mode the K steps are one launch).
roofline   the same launch: algorithmic bytes (9 B per synaptic event + 32 B per neuron update + 8 B
           per spike row) over its CUDA-event time, against the measured HBM copy bandwidth.
           roofline.phases: the window re-run with the kernel's own per-phase timer; the population
           phase against HBM, the scatter phase against the rate of random FP32 ring adds measured in
           the same run, and the whole step against the sum of both bounds.
e2e        the same K steps through the C ABI with host buffers, on a fresh backend that ran the W
           warm-up steps first: every step the host sends the step's background spikes (pinned host ->
           device) and reads the population's spikes back (bitmap device -> host, expanded to indexes),
           pipelined one step deep as a caller would; its event count equals value's.
cpu_baseline / --impl reference: the restated CPU backend (single-threaded, and the multi-threaded
           backend's structure on all host threads) on the same step window of the config at 1/100
           scale.
Extra blocks: a saturated window of the same run, the per-phase kernels on the timed window, and the
batched dense, BPTT and STDP forms. `--form NAME` measures one form alone (`--form gemm`: the tcgen05
GEMM on the BPTT shapes and 8192^3).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "synaptic events/s per GB300, plain vs batched BF16 form, at ≤0.1% spike mismatch"
UNIT = "events/s"
SEED = 2
N = 1_000_000
FAN_IN = 1000
P_BG = 0.005
RING_SLOTS = 20  # input ring slots per neuron: the config's largest delay
GATHER_DRAM_BYTES_PER_SYNAPSE = (677.2e6 + 3.05e6) / 2e8


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def bf16_peak():
    """Dense BF16 burst peak (TFLOP/s) measured with cuBLAS on this GPU model, else the fallback."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


class Clocks:
    """nvidia-smi sampler (SM clock, max clock, throttle reasons) running during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax = float(parts[2])
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower() in ("active", "0x1") or v == "1":
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def build_large(b, n=N, fan_in=FAN_IN):
    from knp_gb300 import network as Nw
    from knp_gb300 import types as T

    pop_uid, rec_uid, bg_uid, chan_uid = (T.uid_from_int(SEED * 100 + i) for i in (1, 2, 3, 4))
    pop = Nw.Population(pop_uid, T.BLIFAT, T.blifat_defaults(n))
    ar = np.arange(n, dtype=np.uint32)
    bg = Nw.Projection(bg_uid, T.DELTA, T.NULL_UID, pop_uid, ar, ar.copy(), np.ones(n, np.float32),
                       np.ones(n, np.uint32))
    b.load_populations([pop])
    b.load_projections([bg])
    b.generate_fixed_fan_in_projection(rec_uid, pop_uid, pop_uid, n, n, fan_in, -16, 48, 1, 20, SEED,
                                       Nw.LARGE_SEED_STREAM)
    b.subscribe(bg_uid, [chan_uid])
    return pop_uid, chan_uid


def large_backend(device, n, fan_in, pull_threshold, mode=None):
    """The large sparse network on the GPU backend, initialised (step mode `mode`, default AUTO)."""
    from knp_gb300 import backend as B
    from knp_gb300 import types as T

    b = B.GB300Backend(device)
    pop_uid, chan_uid = build_large(b, n=n, fan_in=fan_in)
    b.set_pull_threshold(T.uid_from_int(SEED * 100 + 2), pull_threshold)
    if mode is not None:
        b.set_step_mode(mode)
    b._init()
    return b, pop_uid, chan_uid


def window_oracle(which_step: str, n: int, warmup: int, steps: int, target_s: float, threads: int = 1):
    """The restated CPU backend (single-threaded step, or the multi-threaded backend's structure on
    `threads` threads) on the large sparse config at 1/100 scale, over the same step window as the
    GPU measurement: `warmup` steps untimed, then the `steps` timed; the window is run again from a
    snapshot of the loaded network until about target_s of timed CPU work (at most 200 times)."""
    from knp_gb300 import network as Nw
    from oracle import oracle as orc

    net, sched = Nw.large_sparse_network(seed=SEED, n=n, fan_in=FAN_IN, steps=warmup + steps)
    o = orc.OracleNet("restated")
    o.load(net)
    o.snapshot()

    def one(t):
        idx = sched[0].at(t)
        if idx.size:
            o.send_spikes(sched[0].sender, idx, t)
        if which_step == "mt":
            o.step_mt(threads)
        else:
            o.step()

    dt, ev, reps = 0.0, 0, 0
    while reps < 200 and (reps == 0 or dt < target_s):
        if reps:
            o.reset()
        for t in range(warmup):
            one(t)
        e0 = o.events
        t0 = time.perf_counter()
        for t in range(warmup, warmup + steps):
            one(t)
        dt += time.perf_counter() - t0
        ev += o.events - e0
        reps += 1
    what = (f"restated multi-threaded backend step on {threads} threads" if which_step == "mt"
            else "restated single-threaded backend step")
    return {"value": ev / dt, "unit": UNIT, "cores": threads if which_step == "mt" else 1, "kind": "port",
            "sample": f"large sparse config at 1/100 scale ({n} neurons, fan-in {FAN_IN}), steps {warmup}.."
                      f"{warmup + steps - 1} (the GPU's timed window; {warmup} untimed before), run {reps} times "
                      f"from a snapshot: {ev} events, {dt:.2f} s, {what}"}


def cpu_baseline_sample(warmup: int, steps: int, target_s: float = 10.0):
    """Restated single-threaded oracle on the GPU's step window, large sparse config at 1/100 scale."""
    return window_oracle("st", 10_000, warmup, steps, target_s)


def reference_mt_sample(warmup: int, steps: int, target_s: float = 30.0):
    """The reference multi-threaded CPU backend's step structure (restated in the oracle library:
    1000-neuron parts, O(S) synapse scan per step in 1000-synapse parts) on all host threads, on the
    GPU's step window of the large sparse config at 1/100 scale."""
    return window_oracle("mt", 10_000, warmup, steps, target_s, threads=os.cpu_count() or 1)


def replica_totals(t_s: float, events: int, device: str = "cpu"):
    """Whole-job numbers of N independent replicas (one per GPU, no data-path collective): the
    slowest replica's time and the events of all replicas. One process: the inputs unchanged."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(t_s), float(events)
    tt = torch.tensor([float(t_s)], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    ee = torch.tensor([float(events)], device=device, dtype=torch.float64)
    dist.all_reduce(ee)
    return float(tt.item()), float(ee.item())


def _flush_l2(dev):
    """Write a buffer larger than L2 (129 MB) so that the next timed run starts with a cold cache."""
    import torch

    buf = torch.empty(64 << 20, dtype=torch.float32, device=dev)
    buf.fill_(1.0)
    del buf


def batched_dense_measure(device: int, reps: int = 5, warmup: int = 3):
    """Batched dense config (256 LIF samples, 784-1000-1000-10, T uniform in [50, 200], delay-1
    all-to-all layers, BF16 weights, FP32 accumulation) on the tcgen05 batched form, beside the
    plain FP32 backend path running the same samples as one block-diagonal network. Both count a
    synaptic event as a spike times the fan-out of its layer. Spike mismatch: share of (sample,
    neuron, step) of layers 1..3 where the two forms disagree, over each sample's own steps."""
    import torch

    from knp_gb300 import backend as B
    from knp_gb300 import batched as BT
    from knp_gb300 import types as T

    dev = torch.device(f"cuda:{device}")
    cfg = BT.dense_config(seed=4)
    # Prepared once (ring depth autotuned), each run one CUDA-graph launch.
    plan = BT.BatchedPlan(cfg, autotune=True, device=device)
    stages, ring, tuned = plan.info()
    for _ in range(warmup):
        plan.run()
    times, events = [], 0
    for _ in range(reps):
        _flush_l2(dev)
        torch.cuda.synchronize(dev)
        events, ms = plan.run()
        times.append(ms)
    plan.close()
    ms_b = statistics.median(times)
    _, rec, _, _ = BT.run(cfg, record=True, device=device)
    # Checker (outside every timed region): the FP64 oracle of every sample (reference LIF semantics
    # in exact arithmetic), against the batched form's record.
    from oracle import batched_fp64 as BF

    fp64 = BF.run_fp64(cfg)
    m64, t64 = BF.mismatch(fp64, rec, cfg)

    # Plain FP32 path on the same samples.
    t_build = time.perf_counter()
    net, sched = BT.plain_network(cfg)
    b = B.GB300Backend(device)
    b.load_network(net)
    for p in net.populations:
        b.set_accumulator(p.uid, T.ACC_FP32)
    b._init()
    b.load_spike_schedule(sched)
    del net
    t_build = time.perf_counter() - t_build
    t_max = int(cfg.steps.max())
    e0, _, _ = b.counters()
    _flush_l2(dev)
    ms_p = b.step_timed(t_max)
    e1, _, _ = b.counters()
    ev_p = e1 - e0

    # Spike mismatch between the two forms, and of the plain path against the FP64 oracle.
    live = np.arange(t_max)[:, None] < cfg.steps[None, :].astype(np.int64)  # [t, sample]
    mism = total = 0
    pops = [p for p in b._pops]
    plain_rec = {0: rec[0]}
    for layer in range(1, len(cfg.sizes)):
        n = cfg.sizes[layer]
        words = (n + 31) // 32
        uid = pops[layer - 1]
        plain_rec[layer] = np.zeros((t_max, cfg.batch, words), np.uint32)
        for t in range(t_max):
            idx = b.spikes(uid, t).astype(np.int64)
            bm = plain_rec[layer][t]
            s, j = idx // n, idx % n
            np.bitwise_or.at(bm, (s, j >> 5), (np.uint32(1) << (j & 31).astype(np.uint32)))
            diff = (bm ^ rec[layer][t]) & np.where(live[t][:, None], np.uint32(0xFFFFFFFF), np.uint32(0))
            mism += int(np.unpackbits(diff.view(np.uint8)).sum())
            total += int(live[t].sum()) * n
    b.close()
    mp64, tp64 = BF.mismatch(fp64, plain_rec, cfg)
    flops = 2.0 * float(sum(int(cfg.steps.sum()) * a * c for a, c in zip(cfg.sizes[:-1], cfg.sizes[1:])))
    return {
        "workload": "batched_dense: 256 LIF samples 784-1000-1000-10, T in [50,200], inputs rate U[0,0.2], "
                    "weights N(0,1/fan_in) as BF16, FP32 accumulation, one persistent launch",
        "value": events / (ms_b / 1e3), "unit": UNIT, "ms_per_run": ms_b, "events_per_run": events,
        "plain_fp32_path": {"value": ev_p / (ms_p / 1e3), "unit": UNIT, "ms_per_run": ms_p, "events_per_run": ev_p,
                            "build_s": t_build, "mismatch_vs_fp64_oracle": mp64 / max(tp64, 1)},
        "speedup_vs_plain": (events / ms_b) / (ev_p / ms_p),
        "spike_mismatch": mism / max(total, 1), "compared": total,
        "mismatch_vs_fp64_oracle": m64 / max(t64, 1), "compared_fp64": t64,
        "fp64_oracle": "oracle/batched_fp64.py: reference LIF semantics (lif_impl.h:33-86) in FP64 over every "
                       "sample's own steps; pinned to the reference-header oracle on a smaller batch",
        "tensor": {"dense_flops_per_run": flops, "achieved_tflops": flops / (ms_b / 1e3) / 1e12},
        "dtype": "bf16 x bf16 -> fp32", "l2": "flushed (256 MB write) before each timed run",
        "launch": "one CUDA graph per batch (state memsets, input thresholds, input spike bitmaps drawn ahead, "
                  "persistent kernel of CTA-pair clusters)",
        "autotuned_ring_depth": stages, "autotuned_layer_ring_steps": ring,
        "autotune_ms": {f"depth{d}_ring{r}": v for (d, r), v in tuned.items()},
    }


def stdp_measure(device: int):
    """STDP learning config (200 samples x 100 steps: 784 rate-coded inputs -> 800 resource-STDP
    BLIFAT through all-to-all additive STDP, all-to-all lateral inhibition), input schedule resident
    on the device, all 20,000 steps timed with CUDA events. The final plastic weights are compared
    (CRC32) with the fixture the reference-header oracle wrote for the same config."""
    import zlib

    from knp_gb300 import backend as B
    from knp_gb300 import network as Nw
    from knp_gb300 import types as T

    steps = 20_000
    net, scheds = Nw.stdp_network(seed=3, samples=200, steps_per_sample=100)
    b = B.GB300Backend(device)
    b.load_network(net, record=[])
    b._init()
    fused = b.fused
    for sc in scheds:
        b.load_spike_schedule(sc)
    # The first 200 steps run phase by phase (per-phase kernels with CUDA events between the
    # phases), the rest as normal steps (the fused step kernel at this size), timed; together they
    # are the config's 20,000 steps.
    n_prof = 200
    ph = b.profile_phases(n_prof) / n_prof
    e0, _, _ = b.counters()
    ms = b.step_timed(steps - n_prof)
    events, spikes, updates = b.counters()
    w = b.read_weights(net.projections[0].uid)
    b.close()
    # The per-phase step graphs on the same config, for comparison (first 2,000 steps, timed after
    # 100 untimed ones).
    bp = B.GB300Backend(device)
    bp.load_network(net, record=[])
    bp.set_step_mode(T.STEP_PHASES)
    bp._init()
    for sc in scheds:
        bp.load_spike_schedule(sc)
    bp.step(100)
    ms_phases = bp.step_timed(1900)
    bp.close()
    crc = zlib.crc32(w.tobytes())
    # The single-threaded CPU baseline on the same config: the oracle (restated single-threaded
    # backend step, one host thread) over the first samples, about 10-20 s of CPU work.
    from oracle import oracle as orc

    o = orc.OracleNet("restated")
    o.load(net)
    t0, cpu_steps = time.perf_counter(), 0
    while cpu_steps < 2000 and (cpu_steps < 100 or time.perf_counter() - t0 < 10.0):
        for sc in scheds:
            idx = sc.at(cpu_steps)
            if idx.size:
                o.send_spikes(sc.sender, idx, cpu_steps)
        o.step()
        cpu_steps += 1
    cpu_s = time.perf_counter() - t0
    cpu_events = o.events
    o.close()
    fixture = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "stdp_full.json")
    with open(fixture) as f:
        expect = json.load(f)
    return {
        "workload": "stdp: 784 -> 800 additive STDP (tau 20) + 800 x 800 lateral inhibition, 200 samples x 100 steps",
        "value": (events - e0) / (ms / 1e3), "unit": UNIT, "timed_steps": steps - n_prof, "ms_timed": ms,
        "us_per_step": ms / (steps - n_prof) * 1e3,
        "step_kernel": "fused step kernel (one CTA cluster)" if fused else "per-phase kernels",
        "phases_us_per_step": ms_phases / 1900 * 1e3,
        "phase_us_per_step": {k: float(v) * 1e3 for k, v in zip(("population", "projection", "stdp", "step_end"), ph)},
        "events": int(events), "spikes": int(spikes),
        "cpu_baseline": {"value": cpu_events / cpu_s, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": f"the first {cpu_steps} steps of the same config on the oracle (restated "
                                   "single-threaded backend step), host-sent inputs"},
        "weights_crc32": crc, "weights_match_reference_oracle": bool(crc == expect["weights_crc"]),
        "events_match_reference_oracle": bool(int(events) == expect["events"]),
    }


def bptt_measure(device: int, iters: int = 10, warmup: int = 3):
    """Surrogate-gradient BPTT training step (LIF 784-512-512-10, batch 128, T 32, decay 0.9,
    threshold 1, fast-sigmoid slope 25, membrane checkpoint every 8 steps): forward + backward +
    SGD update of the FP32 master weights, CUDA-event timed on torch's current stream."""
    import torch

    from knp_gb300 import bptt

    dev = torch.device(f"cuda:{device}")
    torch.cuda.set_device(dev)
    x, labels = bptt.make_batch(T=32, B=128, seed=11, device=dev)
    model = bptt.SpikingMLP(sizes=(784, 512, 512, 10), checkpoint=8, seed=12, device=dev)
    opt = torch.optim.SGD(model.parameters(), lr=1e-3)

    def it():
        opt.zero_grad(set_to_none=True)
        loss = bptt.loss_fn(model(x), labels)
        loss.backward()
        opt.step()
        return loss

    def timed(step):
        for _ in range(warmup):
            step()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(iters):
            out = step()
        e1.record()
        torch.cuda.synchronize(dev)
        bptt.check_gemm_errors(dev)
        return e0.elapsed_time(e1) / iters, float(out.item())

    ms_eager, _ = timed(it)
    # The same iteration captured as one CUDA graph (the eager loop is bound by ~70 launches from Python).
    graphed = bptt.GraphedTrainStep(model, opt, x, labels)
    ms, loss = timed(graphed)
    layers = [(784, 512), (512, 512), (512, 10)]
    tb = 32 * 128
    # Algorithmic: forward GEMMs, recomputed inputs, weight and input gradients (4 per layer, no
    # input gradient for the first layer). Executed on the tensor cores: the two gradient GEMMs carry
    # dI as two BF16 terms (K doubled).
    fwd = 2.0 * tb * sum(a * c for a, c in layers)
    first = 2.0 * tb * layers[0][0] * layers[0][1]
    flops = fwd * 4 - first
    executed = fwd * 2 + 2 * (fwd * 2 - first)
    return {"workload": "bptt: LIF 784-512-512-10, batch 128, T 32, checkpoint 8", "ms_per_iter": ms,
            "execution": "one CUDA graph per iteration (forward, backward, SGD step)", "ms_per_iter_eager": ms_eager,
            "gemm_flops_per_iter": flops, "achieved_tflops": flops / (ms / 1e3) / 1e12,
            "tensor_flops_executed_per_iter": executed,
            "gemm": "tcgen05 BF16 (knp_gb300_bf16_gemm_tn: TMA-fed 128x128 tiles, 128-byte swizzle, split K "
                    "when tiles are few), FP32 accumulation; gradients as BF16 hi + lo",
            "loss": loss}


GEMM_SHAPES = [(4096, 512, 784), (784, 512, 8192), (512, 512, 8192), (4096, 784, 1024), (8192, 8192, 8192)]


def gemm_measure(device: int, shapes=None, reps: int = 20):
    """The tcgen05 BF16 GEMM (D = A B^T, FP32 accumulation) alone on the BPTT step's shapes and one
    large square, through the C ABI: `reps` calls captured in one CUDA graph (so the time is the
    kernels', not Python's), replayed 3 times untimed then once timed with CUDA events; achieved
    TFLOP/s against the measured cuBLAS BF16 burst peak."""
    import ctypes

    import torch

    from knp_gb300 import _capi

    dev = torch.device(f"cuda:{device}")
    torch.cuda.set_device(dev)
    peak, peak_source = bf16_peak()
    lib = _capi.lib()
    out = []
    for M, N, K in shapes or GEMM_SHAPES:
        g = torch.Generator(device="cpu").manual_seed(M + N + K)
        a = (torch.rand(M, K, generator=g) < 0.2).to(torch.bfloat16).to(dev)
        b = torch.randn(N, K, generator=g).to(torch.bfloat16).to(dev)
        d = torch.empty(M, N, device=dev, dtype=torch.float32)
        err = torch.zeros(1, device=dev, dtype=torch.int32)

        def call():
            _capi.check(lib.knp_gb300_bf16_gemm_tn(
                ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(d.data_ptr()), M, N, K,
                ctypes.c_void_p(err.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))

        side = torch.cuda.Stream(device=dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            call()
        torch.cuda.current_stream(dev).wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            for _ in range(reps):
                call()
        for _ in range(3):
            graph.replay()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        graph.replay()
        e1.record()
        torch.cuda.synchronize(dev)
        us = e0.elapsed_time(e1) * 1e3 / reps
        if int(err.item()) != 0:
            raise RuntimeError("a tcgen05 GEMM completion wait timed out")
        max_err = float((d - a.float() @ b.float().t()).abs().max().item())
        tf = 2.0 * M * N * K / (us * 1e-6) / 1e12
        out.append({"M": M, "N": N, "K": K, "us": us, "tflops": tf, "frac": tf / peak, "max_abs_err_vs_fp32": max_err})
        del graph
    return {"workload": "bf16 GEMM D = A B^T (A 0/1 spikes, B normal), FP32 accumulation, "
                        f"{reps} calls per CUDA graph, L2-resident operands",
            "peak_tflops": peak, "peak_source": peak_source + " cuBLAS bf16 burst", "shapes": out}


def add_rate_ceiling(device: int, n_floats: int, n_adds: int) -> float:
    """Measured ceiling of the scatter's ring adds: FP32 atomic adds at uniformly random positions of
    an `n_floats` buffer (knp_gb300_measure_add_rate, about `n_adds` adds per timed launch), adds/s."""
    import ctypes

    import torch

    from knp_gb300 import _capi

    torch.cuda.set_device(device)
    rate = ctypes.c_double(0.0)
    _capi.check(_capi.lib().knp_gb300_measure_add_rate(n_floats, n_adds, ctypes.byref(rate)))
    return rate.value


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cb = reference_mt_sample(args.warmup, args.steps, target_s=max(10.0, min(60.0, 3.0 * args.steps)))
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded)",
            "config": {"workload": f"large_sparse_plain, steps {args.warmup}..{args.warmup + args.steps - 1} "
                                   "(the GPU arm's timed window), at 1/100 scale on the host CPU (reference "
                                   "multi-threaded backend structure)",
                       "neurons": 10_000, "fan_in": FAN_IN, "p_background": P_BG},
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def algorithmic_bytes(events, neuron_updates, rows):
    """Bytes of the measurement plan: 9 B per synaptic event (int32 target + FP32 weight + u8 delay),
    32 B per neuron update, 8 B per spike row walked (a row_ptr pair)."""
    return 9.0 * events + 32.0 * neuron_updates + 8.0 * rows


def e2e_window(device, n, fan_in, pull, chan_seed, warmup, steps, sched):
    """The timed window through the C ABI with host buffers: a fresh backend runs steps 0..warmup-1
    untimed, then each timed step sends that step's background spikes from host memory (pinned
    staging, host -> device), runs the step, and reads the population's previous step back (spike
    bitmap device -> host, expanded to ascending indexes), pipelined one step deep as a caller would."""
    b, pop_uid, chan_uid = large_backend(device, n, fan_in, pull)
    b.record_spikes(pop_uid, True)
    buf = np.empty(n, np.uint32)
    for t in range(warmup):
        b.send_spikes(chan_uid, sched.at(t), t)
        b.step(1)
    b.spikes(pop_uid, warmup - 1, out=buf)
    b.discard_spikes(warmup)
    b.synchronize()
    ea, _, _ = b.counters()
    h2d = d2h = n_out = 0
    t0 = time.perf_counter()
    for k in range(steps + 1):
        if k < steps:
            idx = sched.at(warmup + k)
            b.send_spikes(chan_uid, idx, warmup + k)
            h2d += idx.nbytes
            b.step(1)
        if k > 0:
            out = b.spikes(pop_uid, warmup + k - 1, out=buf)  # ascending, as in the reference's SpikeMessage
            b.discard_spikes(warmup + k)
            d2h += (n + 31) // 32 * 4  # the step's spike bitmap crosses to the host, expanded there
            n_out += out.size
    b.synchronize()
    te = time.perf_counter() - t0
    eb, _, _ = b.counters()
    launches = b.step_kernel
    b.close()
    return {"value": (eb - ea) / te, "unit": UNIT, "h2d_bytes_per_step": h2d / steps, "d2h_bytes_per_step": d2h / steps,
            "steps": f"{warmup}..{warmup + steps - 1}", "ms_per_step": te / steps * 1e3,
            "spikes_returned_per_step": n_out / steps, "events": int(eb - ea), "step_kernel": launches}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched dense, BPTT and STDP measurements")
    ap.add_argument("--no-extra-windows", action="store_true",
                    help="skip the saturated window and the per-phase kernels on the timed window")
    ap.add_argument("--form", default="all", choices=["all", "batched", "bptt", "stdp", "gemm"],
                    help="measure one form alone: the batched dense form, the BPTT step, the STDP config or the "
                         "tcgen05 GEMM (profiling runs)")
    ap.add_argument("--gemm-shape", default=None, help="M,N,K: the GEMM form on this shape alone")
    ap.add_argument("--neurons", type=int, default=N, help="population size (profiling cases only)")
    ap.add_argument("--fan-in", type=int, default=FAN_IN, help="fan-in (profiling cases only)")
    ap.add_argument("--pull-threshold", type=float, default=0.1,
                    help="spike share above which a step is gathered instead of scattered (-1: scatter only)")
    ap.add_argument("--step-mode", default="auto", choices=["auto", "phases", "grid"])
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    if args.form != "all":
        # One form alone (profiling runs): prints that form's measurement as one JSON line.
        local = int(os.environ.get("LOCAL_RANK", "0"))
        if args.form == "gemm":
            shapes = [tuple(int(v) for v in args.gemm_shape.split(","))] if args.gemm_shape else None
            out = gemm_measure(local, shapes)
        else:
            out = {"batched": batched_dense_measure, "bptt": bptt_measure, "stdp": stdp_measure}[args.form](local)
        print(json.dumps({"form": args.form, **out}))
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")

    from knp_gb300 import network as Nw
    from knp_gb300 import types as T

    modes = {"auto": None, "phases": T.STEP_PHASES, "grid": T.STEP_GRID}
    n_neurons, W, K = args.neurons, args.warmup, args.steps
    # Ceiling of the scatter's ring adds, measured before any backend holds memory or an L2 set-aside.
    ceiling = add_rate_ceiling(local, RING_SLOTS * n_neurons, 100_000_000) if rank == 0 else None
    sat0, sat_steps = max(W + K, 40), 20  # a window of saturated steps (every neuron fires every step)
    total_steps = sat0 + sat_steps
    chan_seed = SEED + 1000 * rank
    t_build = time.perf_counter()
    b, pop_uid, chan_uid = large_backend(local, n_neurons, args.fan_in, args.pull_threshold, modes[args.step_mode])
    b.generate_bernoulli_schedule(chan_uid, n_neurons, P_BG, 0, total_steps, seed=chan_seed)
    t_build = time.perf_counter() - t_build
    step_kernel = b.step_kernel
    # The same background spikes on the host (the device generator's restatement): their count per
    # step gives the spike rows of the one-to-one projection; the e2e run sends them from host memory.
    sched = Nw.bernoulli_schedule(chan_uid, chan_seed, n_neurons, total_steps, P_BG)

    b.step(W)
    b.synchronize()
    if dist is not None:
        dist.barrier()
    ev0, sp0, _ = b.counters()
    with Clocks(local) as clk:
        ms = b.step_timed(K)
    ev1, sp1, _ = b.counters()
    t, events_all = replica_totals(ms / 1e3, ev1 - ev0, f"cuda:{local}" if dist is not None else "cpu")
    events, spikes = ev1 - ev0, sp1 - sp0
    value = events_all / t
    bg_rows = int(sched.offsets[W + K] - sched.offsets[W])
    # Roofline of the timed launch: in grid mode the K steps are one launch of the persistent step
    # kernel, timed by the CUDA events around it on the backend's stream.
    hbm, src = peaks()
    a_bytes = algorithmic_bytes(events, n_neurons * K, spikes + bg_rows)
    achieved = a_bytes / (ms / 1e3) / 1e9
    kernel_name = {T.STEP_GRID: f"grid_net_kernel (persistent step kernel, one launch of {K} steps)",
                   T.STEP_PHASES: "whole step (per-phase kernels in CUDA graphs)",
                   T.STEP_FUSED: "small_net_kernel"}[step_kernel]
    roofline = {"bound": "hbm", "kernel": kernel_name, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_source": src, "steps": f"{W}..{W + K - 1}",
                "launch_ms": ms, "algorithmic_bytes_per_launch": a_bytes,
                "bytes_model": "9 B per synaptic event + 32 B per neuron update + 8 B per spike row",
                "traffic": None}
    per_step_share = spikes / (n_neurons * K)
    if args.pull_threshold < 0:
        regime = "every step scattered (gather direction off)"
    elif per_step_share < args.pull_threshold:
        regime = "sparse (every step below the pull threshold: scattered)"
    else:
        regime = "mixed or saturated"

    extra = {}
    if rank == 0 and not args.no_extra_windows:
        # Saturated window of the same run (every neuron fires every step; steps gathered).
        b.step(sat0 - (W + K))
        s0, q0, _ = b.counters()
        ms_sat = b.step_timed(sat_steps)
        s1, q1, _ = b.counters()
        rows_sat = (q1 - q0) + int(sched.offsets[sat0 + sat_steps] - sched.offsets[sat0])
        ab = algorithmic_bytes(s1 - s0, n_neurons * sat_steps, rows_sat)
        extra["saturated_window"] = {
            "steps": f"{sat0}..{sat0 + sat_steps - 1}", "value": (s1 - s0) / (ms_sat / 1e3), "unit": UNIT,
            "ms_per_step": ms_sat / sat_steps, "firing_rate": (q1 - q0) / (n_neurons * sat_steps),
            "effective_frac": ab / (ms_sat / 1e3) / 1e9 / hbm,
            "note": "effective: the plan's 9 B per event over the step time; the gather layout moves 4 B per "
                    "synapse (dictionary weights, target and delay implied), so this can exceed 1"}
        # The persistent kernel's own phase times on the same window (global-timer stamps of CTA 0),
        # each phase against its bound: the population phase streams 32 B per neuron from HBM; the
        # scatter phase is one random FP32 add per synaptic event into the input rings (84 MB, held
        # in L2), bounded by the measured rate of such adds.
        if step_kernel == T.STEP_GRID:
            bg, _, cg = large_backend(local, n_neurons, args.fan_in, args.pull_threshold, T.STEP_GRID)
            bg.generate_bernoulli_schedule(cg, n_neurons, P_BG, 0, W + K, seed=chan_seed)
            bg.step(W)
            g0, _, _ = bg.counters()
            us = bg.profile_grid_phases(K)
            g1, _, _ = bg.counters()
            bg.close()
            pop_bytes = 32.0 * n_neurons * K
            roofline["phases"] = {
                "us_per_step": {"populations": us[0] / K, "projections": us[1] / K, "gathers": us[2] / K},
                "same_events": bool(g1 - g0 == events),
                "populations": {"bound": "hbm", "achieved": pop_bytes / (us[0] * 1e-6) / 1e9, "peak": hbm,
                                "unit": "GB/s", "frac": pop_bytes / (us[0] * 1e-6) / 1e9 / hbm,
                                "bytes_model": "32 B per neuron update"},
                "projections": {"bound": "l2-atomic", "achieved": events / (us[1] * 1e-6), "peak": ceiling,
                                "unit": "adds/s", "frac": events / (us[1] * 1e-6) / ceiling,
                                "peak_source": "measured in this run (knp_gb300_measure_add_rate): FP32 atomic "
                                               "adds at uniformly random positions of a "
                                               f"{RING_SLOTS * n_neurons * 4 // 10**6} MB buffer (the input rings' "
                                               "size), 100M adds per launch, measured before the backends were "
                                               "built (no L2 set-aside), no other traffic"},
                "whole_step_bound_us": (pop_bytes / (hbm * 1e9) + events / ceiling) * 1e6 / K,
                "whole_step_frac": (pop_bytes / (hbm * 1e9) + events / ceiling) / (ms / 1e3),
            }
        # The per-phase kernels on the same timed window (for comparison with the persistent kernel).
        if step_kernel == T.STEP_GRID:
            bp, _, cp = large_backend(local, n_neurons, args.fan_in, args.pull_threshold, T.STEP_PHASES)
            bp.generate_bernoulli_schedule(cp, n_neurons, P_BG, 0, W + K, seed=chan_seed)
            bp.step(W)
            e0p, _, _ = bp.counters()
            ms_p = bp.step_timed(K)
            e1p, _, _ = bp.counters()
            bp.close()
            extra["per_phase_kernels_same_window"] = {
                "value": (e1p - e0p) / (ms_p / 1e3), "unit": UNIT, "ms_per_step": ms_p / K,
                "same_events": bool(e1p - e0p == events)}
    b.close()

    e2e = None
    if rank == 0 and not args.no_e2e:
        e2e = e2e_window(local, n_neurons, args.fan_in, args.pull_threshold, chan_seed, W, K, sched)
        e2e["same_events_as_value"] = bool(e2e["events"] == events)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(W, K)

    batched = bp_ = stdp = None
    if rank == 0 and not args.no_forms:
        batched = batched_dense_measure(local)
        bp_ = bptt_measure(local)
        stdp = stdp_measure(local)

    if rank == 0:
        launches = (K + 65535) // 65536 if step_kernel in (T.STEP_GRID, T.STEP_FUSED) else 5 * K
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": ms / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded counter-based generator)",
            "config": {"workload": f"large_sparse_plain, steps {W}..{W + K - 1}: {regime}",
                       "neurons": n_neurons, "fan_in": args.fan_in, "synapses": n_neurons * args.fan_in,
                       "delays": "1..20", "weights": "k/256, k in [-16,48]", "p_background": P_BG,
                       "l2": "inputs larger than L2 (9 GB CSR, 4 GB gather layout), no flush",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "pull_threshold": args.pull_threshold, "step_mode": args.step_mode},
            "neuron_updates_per_s": n_neurons * world * K / t,
            "firing_rate": per_step_share,
            "events_per_step": events / K,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "build_s": t_build,
            **extra,
            "batched_dense": batched,
            "bptt": bp_,
            "stdp": stdp,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
