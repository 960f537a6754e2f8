"""Python mirror of the KNP backend plugin interface over the GB300 C ABI.

``GB300Backend`` keeps the names, argument meaning and error behaviour of ``knp::core::Backend``
(knp/core-library/include/knp/core/backend.h:55-457) as the single-threaded CPU backend implements
it (knp/backends/cpu/cpu-single-threaded-backend/include/knp/backends/cpu-single-threaded/backend.h):
``load_populations``, ``load_projections``, ``subscribe``, ``_init``, ``_step``, ``start``,
``stop``, ``get_step``, ``get_network_data``, ``start_learning`` / ``stop_learning``. Unsupported
neuron or synapse types raise, as ``knp::meta::load_from_container`` throws "Type is not supported."
(knp/meta-library/include/knp/meta/variant_helpers.h:67).

Messages that the reference exchanges through the backend's MessageBus with external endpoints are
explicit calls here: ``send_spikes`` (an input channel's SpikeMessage), ``send_impacts`` (a
SynapticImpactMessage to a population) and ``spikes`` (the SpikeMessage a subscribed output endpoint
receives). Everything between the backend's own populations and projections stays on the device.
"""
from __future__ import annotations

import copy
import ctypes

import numpy as np

from . import _capi
from . import network as N
from . import types as T

SUPPORTED_NEURONS = ["BLIFATNeuron", "SynapticResourceSTDPBLIFATNeuron", "LIFNeuron"]
SUPPORTED_SYNAPSES = ["DeltaSynapse", "AdditiveSTDPDeltaSynapse"]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class GB300Backend:
    """One GB300 backend instance on one CUDA device."""

    def __init__(self, device: int = 0):
        self._lib = _capi.lib()
        h = ctypes.c_void_p()
        _capi.check(self._lib.knp_gb300_create(device, ctypes.byref(h)))
        self._h = h
        self._pops: dict = {}
        self._projs: dict = {}
        self._recorded: set = set()
        self._initialized = False
        self._started = False
        self._stop = False

    # ------------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "_h", None):
            self._lib.knp_gb300_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _chk(self, rc):
        _capi.check(rc)

    # ------------------------------------------------------------------ interface queries (backend.h:103-127)
    def plasticity_supported(self) -> bool:
        return True

    def get_supported_neurons(self) -> list:
        return list(SUPPORTED_NEURONS)

    def get_supported_synapses(self) -> list:
        return list(SUPPORTED_SYNAPSES)

    # ------------------------------------------------------------------ loading (backend.h:137-160)
    def load_populations(self, populations):
        for pop in populations:
            if pop.kind == T.LIF:
                neurons = np.ascontiguousarray(pop.neurons, dtype=T.LIF_DTYPE)
                self._chk(self._lib.knp_gb300_load_lif_population(self._h, T.to_c_uid(pop.uid), pop.size,
                                                                  _ptr(neurons)))
                self._pops[pop.uid] = pop
                continue
            if T.is_altai(pop.kind):
                neurons = np.ascontiguousarray(pop.neurons, dtype=T.ALTAI_DTYPE)
                res = None if pop.resource is None else np.ascontiguousarray(pop.resource, dtype=T.RESOURCE_DTYPE)
                self._chk(self._lib.knp_gb300_load_altai_population(
                    self._h, T.to_c_uid(pop.uid), pop.kind, pop.size, _ptr(neurons), _ptr(res)))
                self._pops[pop.uid] = pop
                continue
            if pop.kind not in (T.BLIFAT, T.RESOURCE_STDP_BLIFAT):
                raise TypeError("Type is not supported.")
            neurons = np.ascontiguousarray(pop.neurons, dtype=T.BLIFAT_DTYPE)
            res = None if pop.resource is None else np.ascontiguousarray(pop.resource, dtype=T.RESOURCE_DTYPE)
            self._chk(self._lib.knp_gb300_load_blifat_population(
                self._h, T.to_c_uid(pop.uid), pop.kind, pop.size, _ptr(neurons), _ptr(res)))
            self._pops[pop.uid] = pop

    load_all_populations = load_populations

    def load_projections(self, projections):
        for pr in projections:
            if pr.kind not in (T.DELTA, T.ADDITIVE_STDP_DELTA, T.RESOURCE_STDP_DELTA):
                raise TypeError("Type is not supported.")
            arrs = [np.ascontiguousarray(pr.pre, np.uint32), np.ascontiguousarray(pr.post, np.uint32),
                    np.ascontiguousarray(pr.weight, np.float32), np.ascontiguousarray(pr.delay, np.uint32),
                    None if pr.out_type is None else np.ascontiguousarray(pr.out_type, np.uint8),
                    None if pr.tau_plus is None else np.ascontiguousarray(pr.tau_plus, np.float32),
                    None if pr.tau_minus is None else np.ascontiguousarray(pr.tau_minus, np.float32)]
            if pr.kind == T.RESOURCE_STDP_DELTA:
                rule = np.ascontiguousarray(pr.rule if pr.rule is not None else T.resource_synapse_defaults(pr.size),
                                            T.RESOURCE_SYNAPSE_DTYPE)
                self._chk(self._lib.knp_gb300_load_resource_stdp_projection(
                    self._h, T.to_c_uid(pr.uid), T.to_c_uid(pr.pre_uid), T.to_c_uid(pr.post_uid), pr.size,
                    *[_ptr(a) for a in arrs[:5]], _ptr(rule), int(pr.locked)))
                self._projs[pr.uid] = pr
                continue
            self._chk(self._lib.knp_gb300_load_projection(
                self._h, T.to_c_uid(pr.uid), pr.kind, T.to_c_uid(pr.pre_uid), T.to_c_uid(pr.post_uid), pr.size,
                *[_ptr(a) for a in arrs]))
            for pop_uid, ptype in pr.stdp_populations.items():
                self._chk(self._lib.knp_gb300_set_stdp_population(
                    self._h, T.to_c_uid(pr.uid), T.to_c_uid(pop_uid), ptype))
            self._projs[pr.uid] = pr

    load_all_projections = load_projections

    def generate_fixed_fan_in_projection(self, uid, pre_uid, post_uid, n_pre, n_post, fan_in, k_lo, k_hi, d_lo, d_hi,
                                         seed, stream):
        """Device-side construction of a FixedNumberPre-style delta projection (see network.fixed_fan_in_pre)."""
        self._chk(self._lib.knp_gb300_generate_fixed_fan_in_projection(
            self._h, T.to_c_uid(uid), T.to_c_uid(pre_uid), T.to_c_uid(post_uid), n_pre, n_post, fan_in, k_lo, k_hi,
            d_lo, d_hi, seed, stream))
        self._projs[uid] = None

    def generate_projection(self, uid, pre_uid, post_uid, kind, n_pre, n_post, k_lo, k_hi, d_lo, d_hi, seed, stream,
                            count=0, probability=0.0):
        """Device-side construction of a delta projection by one of the reference's synapse generators
        (kind: types.GEN_*; see network.generated_synapses for the synapses it gives)."""
        self._chk(self._lib.knp_gb300_generate_projection(
            self._h, T.to_c_uid(uid), T.to_c_uid(pre_uid), T.to_c_uid(post_uid), kind, n_pre, n_post, count,
            probability, k_lo, k_hi, d_lo, d_hi, seed, stream))
        self._projs[uid] = None

    def remove_projections(self, uids):
        """As in the single-threaded backend (backend.h:287): no effect."""

    def remove_populations(self, uids):
        """As in the single-threaded backend (backend.h:294): no effect."""

    def subscribe(self, receiver: bytes, senders):
        """Backend::subscribe (backend.h:222-226): receiver gets messages of every sender."""
        for s in ([senders] if isinstance(senders, (bytes, bytearray)) else senders):
            self._chk(self._lib.knp_gb300_subscribe(self._h, T.to_c_uid(receiver), T.to_c_uid(s)))

    def set_accumulator(self, pop_uid: bytes, mode: int):
        self._chk(self._lib.knp_gb300_set_accumulator(self._h, T.to_c_uid(pop_uid), mode))

    def set_pull_threshold(self, proj_uid: bytes, fraction: float):
        """Spike share above which a step of this projection is gathered instead of scattered
        (negative: always scatter)."""
        self._chk(self._lib.knp_gb300_set_pull_threshold(self._h, T.to_c_uid(proj_uid), float(fraction)))

    def set_step_mode(self, mode: int):
        """Step execution (before init): T.STEP_AUTO, T.STEP_PHASES (a kernel per phase),
        T.STEP_FUSED (one cluster kernel per run of steps; small networks only) or T.STEP_GRID (one
        persistent cooperative kernel of one CTA per SM per run of steps)."""
        self._chk(self._lib.knp_gb300_set_step_mode(self._h, int(mode)))

    @property
    def fused(self) -> bool:
        """True when init chose the fused step kernel."""
        v = ctypes.c_int(0)
        self._chk(self._lib.knp_gb300_step_fused(self._h, ctypes.byref(v)))
        return bool(v.value)

    @property
    def step_kernel(self) -> int:
        """The step mode init chose: T.STEP_PHASES, T.STEP_FUSED or T.STEP_GRID."""
        v = ctypes.c_int(0)
        self._chk(self._lib.knp_gb300_step_kernel(self._h, ctypes.byref(v)))
        return int(v.value)

    def record_spikes(self, pop_uid: bytes, enable: bool = True):
        self._chk(self._lib.knp_gb300_record_spikes(self._h, T.to_c_uid(pop_uid), int(enable)))
        (self._recorded.add if enable else self._recorded.discard)(pop_uid)

    def load_network(self, net: N.Network, record=None):
        """Load a network description: populations, projections, subscriptions."""
        self.load_populations(net.populations)
        self.load_projections(net.projections)
        for recv, send in net.subscriptions:
            self.subscribe(recv, [send])
        for u in ([p.uid for p in net.populations] if record is None else record):
            self.record_spikes(u, True)

    # ------------------------------------------------------------------ run (backend.h:262-321)
    def _init(self):
        self._chk(self._lib.knp_gb300_init(self._h))
        self._initialized = True

    def _step(self):
        self._chk(self._lib.knp_gb300_step(self._h, 1))

    def step(self, n: int = 1):
        self._chk(self._lib.knp_gb300_step(self._h, n))

    def step_timed(self, n: int) -> float:
        ms = ctypes.c_float(0)
        self._chk(self._lib.knp_gb300_step_timed(self._h, n, ctypes.byref(ms)))
        return float(ms.value)

    def profile_phases(self, n: int):
        """Device ms of (populations, projections, STDP, end-of-step) summed over ``n`` steps,
        kernels launched one by one with CUDA events between the phases."""
        ms = (ctypes.c_float * 4)()
        self._chk(self._lib.knp_gb300_profile_phases(self._h, n, ms))
        return np.array(list(ms), dtype=np.float64)

    def profile_grid_phases(self, n: int):
        """Device microseconds of (populations, projections, gathers) summed over ``n`` normal steps
        of the persistent grid kernel, from the kernel's own global-timer stamps."""
        us = (ctypes.c_double * 3)()
        self._chk(self._lib.knp_gb300_profile_grid_phases(self._h, n, us))
        return np.array(list(us), dtype=np.float64)

    def get_step(self) -> int:
        s = ctypes.c_uint64(0)
        self._chk(self._lib.knp_gb300_get_step(self._h, ctypes.byref(s)))
        return int(s.value)

    def start(self, pre_step=None, post_step=None):
        """Backend::start (knp/core-library/impl/backend.cpp:116-141): loop _step() while the
        predicates return true; with one argument it is the run predicate checked after a step."""
        if not self._initialized:
            self._init()
        self._started = True
        self._stop = False
        try:
            while not self._stop:
                if pre_step is not None and post_step is not None:
                    if not pre_step(self.get_step()):
                        break
                self._step()
                pred = post_step if post_step is not None else pre_step
                if pred is not None and not pred(self.get_step()):
                    break
        finally:
            self._started = False

    def stop(self):
        self._stop = True

    def running(self) -> bool:
        return self._started

    def stop_learning(self):
        self._chk(self._lib.knp_gb300_stop_learning(self._h))

    def start_learning(self):
        self._chk(self._lib.knp_gb300_start_learning(self._h))

    def synchronize(self):
        self._chk(self._lib.knp_gb300_synchronize(self._h))

    # ------------------------------------------------------------------ messages
    def send_spikes(self, sender: bytes, indexes, send_time: int | None = None):
        idx = np.ascontiguousarray(indexes, np.uint32)
        t = self.get_step() if send_time is None else send_time
        self._chk(self._lib.knp_gb300_send_spikes(self._h, T.to_c_uid(sender), t, idx.size, _ptr(idx)))

    def send_impacts(self, sender: bytes, pop: bytes, post_idx, values, out_type=None, is_forcing: bool = True):
        post_idx = np.ascontiguousarray(post_idx, np.uint32)
        values = np.ascontiguousarray(values, np.float32)
        ot = None if out_type is None else np.ascontiguousarray(out_type, np.uint8)
        self._chk(self._lib.knp_gb300_send_impacts(self._h, T.to_c_uid(sender), T.to_c_uid(pop), int(is_forcing),
                                                   post_idx.size, _ptr(post_idx), _ptr(values), _ptr(ot)))

    def load_spike_schedule(self, sched: N.SpikeSchedule, first_step: int = 0):
        offs = np.ascontiguousarray(sched.offsets, np.int64)
        idx = np.ascontiguousarray(sched.indexes, np.uint32)
        self._chk(self._lib.knp_gb300_load_spike_schedule(self._h, T.to_c_uid(sched.sender), first_step,
                                                          sched.n_steps, _ptr(offs), _ptr(idx)))

    def generate_bernoulli_schedule(self, sender, n_sources, p, first_step, n_steps, seed, stream=N.S_INPUT):
        self._chk(self._lib.knp_gb300_generate_bernoulli_schedule(self._h, T.to_c_uid(sender), n_sources, float(p),
                                                                  first_step, n_steps, seed, stream))

    def spikes(self, pop: bytes, step: int, cap: int | None = None, out: np.ndarray | None = None) -> np.ndarray:
        """Ascending spike indexes of ``pop`` at ``step`` (population must be recorded). ``out``: a
        reusable uint32 buffer to expand into (the result is a view of it when it is large enough)."""
        n = self._pops[pop].size if cap is None and pop in self._pops else (cap or 0)
        if out is None or out.dtype != np.uint32 or not out.flags.c_contiguous or out.size < max(n, 1):
            out = np.empty(max(n, 1), np.uint32)
        cnt = ctypes.c_uint32(0)
        self._chk(self._lib.knp_gb300_read_spikes(self._h, T.to_c_uid(pop), step, out.size, _ptr(out),
                                                  ctypes.byref(cnt)))
        if cnt.value > out.size:
            out = np.empty(cnt.value, np.uint32)
            self._chk(self._lib.knp_gb300_read_spikes(self._h, T.to_c_uid(pop), step, out.size, _ptr(out),
                                                      ctypes.byref(cnt)))
        return out[: cnt.value]

    def spikes_capped(self, pop: bytes, step: int, out: np.ndarray) -> int:
        """Writes at most ``out.size`` ascending spike indexes of ``pop`` at ``step`` into ``out``
        (uint32) and returns the step's full spike count."""
        cnt = ctypes.c_uint32(0)
        self._chk(self._lib.knp_gb300_read_spikes(self._h, T.to_c_uid(pop), step, out.size, _ptr(out),
                                                  ctypes.byref(cnt)))
        return int(cnt.value)

    def discard_spikes(self, before_step: int):
        self._chk(self._lib.knp_gb300_discard_spikes(self._h, before_step))

    # ------------------------------------------------------------------ readback (backend.h:420)
    def read_population(self, uid: bytes):
        """(neurons, resource-STDP extension or None) of a BLIFAT or AltAI-LIF population."""
        pop = self._pops[uid]
        if T.is_altai(pop.kind):
            out = np.empty(pop.size, T.ALTAI_DTYPE)
            ext = np.empty(pop.size, T.RESOURCE_DTYPE) if pop.kind == T.RESOURCE_STDP_ALTAI_LIF else None
            self._chk(self._lib.knp_gb300_read_altai_population(self._h, T.to_c_uid(uid), _ptr(out), _ptr(ext)))
            return out, ext
        out = np.empty(pop.size, T.BLIFAT_DTYPE)
        ext = np.empty(pop.size, T.RESOURCE_DTYPE) if pop.kind == T.RESOURCE_STDP_BLIFAT else None
        self._chk(self._lib.knp_gb300_read_blifat_population(self._h, T.to_c_uid(uid), _ptr(out), _ptr(ext)))
        return out, ext

    def read_lif(self, uid: bytes) -> np.ndarray:
        out = np.empty(self._pops[uid].size, T.LIF_DTYPE)
        self._chk(self._lib.knp_gb300_read_lif_population(self._h, T.to_c_uid(uid), _ptr(out)))
        return out

    def read_weights(self, uid: bytes) -> np.ndarray:
        n = ctypes.c_uint64(0)
        self._chk(self._lib.knp_gb300_projection_size(self._h, T.to_c_uid(uid), ctypes.byref(n)))
        out = np.empty(n.value, np.float32)
        self._chk(self._lib.knp_gb300_read_weights(self._h, T.to_c_uid(uid), _ptr(out)))
        return out

    def read_resource_synapses(self, uid: bytes) -> np.ndarray:
        """Rule state of a resource-STDP projection's synapses, in load order (RESOURCE_SYNAPSE_DTYPE)."""
        n = ctypes.c_uint64(0)
        self._chk(self._lib.knp_gb300_projection_size(self._h, T.to_c_uid(uid), ctypes.byref(n)))
        out = np.empty(n.value, T.RESOURCE_SYNAPSE_DTYPE)
        self._chk(self._lib.knp_gb300_read_resource_synapses(self._h, T.to_c_uid(uid), _ptr(out)))
        return out

    def get_network_data(self):
        """Copies of the loaded populations and projections with the device's current state and
        weights (get_network.cpp:80-93)."""
        pops, projs = [], []
        for uid, pop in self._pops.items():
            if pop.kind == T.LIF:
                pops.append(N.Population(uid, pop.kind, self.read_lif(uid)))
                continue
            neurons, ext = self.read_population(uid)
            pops.append(N.Population(uid, pop.kind, neurons, ext))
        for uid, pr in self._projs.items():
            if pr is None:
                continue
            q = copy.copy(pr)
            q.weight = self.read_weights(uid)
            if pr.kind == T.RESOURCE_STDP_DELTA:
                q.rule = self.read_resource_synapses(uid)
            projs.append(q)
        return pops, projs

    def counters(self):
        e, s, u = ctypes.c_uint64(0), ctypes.c_uint64(0), ctypes.c_uint64(0)
        self._chk(self._lib.knp_gb300_counters(self._h, ctypes.byref(e), ctypes.byref(s), ctypes.byref(u)))
        return int(e.value), int(s.value), int(u.value)


def run(net: N.Network, schedules, n_steps: int, record=None, device: int = 0, device_schedule: bool = False,
        on_step=None, accumulator=None, step_mode=None):
    """Run a network for ``n_steps`` steps through the C ABI. Input schedules are sent as host
    messages step by step (``device_schedule=False``) or uploaded once to device memory. Returns
    ({pop uid: [per-step ascending spike arrays]}, backend)."""
    b = GB300Backend(device)
    b.load_network(net, record=record)
    if accumulator is not None:
        for p in net.populations:
            b.set_accumulator(p.uid, accumulator)
    if step_mode is not None:
        b.set_step_mode(step_mode)
    b._init()
    rec = [p.uid for p in net.populations] if record is None else record
    if device_schedule:
        for s in schedules:
            b.load_spike_schedule(s)
        if on_step is None:
            b.step(n_steps)
        else:
            for t in range(n_steps):
                on_step(b, t)
                b.step(1)
    else:
        for t in range(n_steps):
            for s in schedules:
                idx = s.at(t)
                if idx.size:
                    b.send_spikes(s.sender, idx, t)
            if on_step is not None:
                on_step(b, t)
            b.step(1)
    out = {u: [b.spikes(u, t) for t in range(n_steps)] for u in rec}
    return out, b
