"""TEST INFRASTRUCTURE — ctypes driver for the CPU oracle libraries.

Only tests/, __graft_entry__.smoke() and bench.py's CPU arms import this module; the GB300 product
path never does. ``OracleNet("restated")`` loads oracle/_build/libknp_oracle.so (this repository's
restatement of the KNP single-threaded backend step); ``OracleNet("reference")`` loads
oracle/_ref/libknp_ref.so (the reference's own per-neuron / per-synapse headers, built only where
the KNP sources are present).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

from knp_gb300 import types as T

HERE = os.path.dirname(os.path.abspath(__file__))
LIBS = {
    "restated": os.path.join(HERE, "_build", "libknp_oracle.so"),
    "reference": os.path.join(HERE, "_ref", "libknp_ref.so"),
}
_lock = threading.Lock()
_loaded: dict = {}


def build(which: str = "restated", knp_ref: str | None = None) -> str:
    """Compile an oracle library with oracle/Makefile; returns its path."""
    target = "all" if which == "restated" else "ref"
    cmd = ["make", "-s", "-C", HERE, target]
    if knp_ref:
        cmd.append(f"KNP_REF={knp_ref}")
    subprocess.run(cmd, check=True)
    return LIBS[which]


def available(which: str) -> bool:
    return os.path.exists(LIBS[which])


def _load(which: str):
    with _lock:
        if which in _loaded:
            return _loaded[which]
        path = LIBS[which]
        if not os.path.exists(path):
            if which == "restated":
                build("restated")
            else:
                raise FileNotFoundError(path)
        lib = ctypes.CDLL(path)
        U = T.KnpUid
        p = ctypes.c_void_p
        u32p = ctypes.POINTER(ctypes.c_uint32)
        sig = {
            "or_last_error": ([], ctypes.c_char_p),
            "or_create": ([], p),
            "or_destroy": ([p], None),
            "or_add_blifat_population": ([p, U, ctypes.c_int, ctypes.c_uint32, p, p], ctypes.c_int),
            "or_add_lif_population": ([p, U, ctypes.c_uint32, p], ctypes.c_int),
            "or_add_projection": ([p, U, ctypes.c_int, U, U, ctypes.c_uint64, p, p, p, p, p, p, p], ctypes.c_int),
            "or_set_stdp_population": ([p, U, U, ctypes.c_int], ctypes.c_int),
            "or_subscribe": ([p, U, U], ctypes.c_int),
            "or_init": ([p], ctypes.c_int),
            "or_send_spikes": ([p, U, ctypes.c_uint64, ctypes.c_uint32, p], ctypes.c_int),
            "or_send_impacts": ([p, U, U, ctypes.c_int, ctypes.c_uint32, p, p, p], ctypes.c_int),
            "or_step": ([p], ctypes.c_int),
            "or_get_step": ([p], ctypes.c_uint64),
            "or_read_spikes": ([p, U, ctypes.c_uint32, p, u32p], ctypes.c_int),
            "or_read_blifat": ([p, U, p, p], ctypes.c_int),
            "or_read_lif": ([p, U, p], ctypes.c_int),
            "or_read_weights": ([p, U, p], ctypes.c_int),
            "or_event_count": ([p], ctypes.c_uint64),
            "or_add_resource_projection": ([p, U, U, U, ctypes.c_uint64, p, p, p, p, p, p, ctypes.c_int], ctypes.c_int),
            "or_set_learning": ([p, ctypes.c_int], ctypes.c_int),
            "or_read_resource_synapses": ([p, U, p], ctypes.c_int),
            "or_add_altai_population": ([p, U, ctypes.c_int, ctypes.c_uint32, p, p], ctypes.c_int),
            "or_read_altai": ([p, U, p, p], ctypes.c_int),
        }
        if which == "restated":
            sig["or_step_mt"] = ([p, ctypes.c_int], ctypes.c_int)
            sig["or_snapshot"] = ([p], ctypes.c_int)
            sig["or_reset"] = ([p], ctypes.c_int)
        for name, (args, res) in sig.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = res
        _loaded[which] = lib
        return lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class OracleError(RuntimeError):
    pass


class OracleNet:
    """One network instance inside an oracle library."""

    def __init__(self, which: str = "restated"):
        self.lib = _load(which)
        self.which = which
        self.h = self.lib.or_create()
        self._sizes: dict = {}
        self._keep: list = []

    def close(self):
        if self.h:
            self.lib.or_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, rc):
        if rc != 0:
            raise OracleError(self.lib.or_last_error().decode())

    def load(self, net):
        """Load a knp_gb300.network.Network and build its subscriptions."""
        for pop in net.populations:
            n = pop.size
            self._sizes[pop.uid] = (pop.kind, n)
            neurons = np.ascontiguousarray(pop.neurons)
            if pop.kind == T.LIF:
                self._chk(self.lib.or_add_lif_population(self.h, T.to_c_uid(pop.uid), n, _ptr(neurons)))
            elif T.is_altai(pop.kind):
                res = None if pop.resource is None else np.ascontiguousarray(pop.resource)
                self._chk(self.lib.or_add_altai_population(self.h, T.to_c_uid(pop.uid), pop.kind, n, _ptr(neurons),
                                                           _ptr(res)))
            else:
                res = None if pop.resource is None else np.ascontiguousarray(pop.resource)
                self._chk(self.lib.or_add_blifat_population(self.h, T.to_c_uid(pop.uid), pop.kind, n, _ptr(neurons),
                                                            _ptr(res)))
        for pr in net.projections:
            arrs = [np.ascontiguousarray(pr.pre, np.uint32), np.ascontiguousarray(pr.post, np.uint32),
                    np.ascontiguousarray(pr.weight, np.float32), np.ascontiguousarray(pr.delay, np.uint32),
                    None if pr.out_type is None else np.ascontiguousarray(pr.out_type, np.uint8),
                    None if pr.tau_plus is None else np.ascontiguousarray(pr.tau_plus, np.float32),
                    None if pr.tau_minus is None else np.ascontiguousarray(pr.tau_minus, np.float32)]
            self._sizes[pr.uid] = (pr.kind, pr.size)
            if pr.kind == T.RESOURCE_STDP_DELTA:
                rule = np.ascontiguousarray(pr.rule if pr.rule is not None else T.resource_synapse_defaults(pr.size))
                self._chk(self.lib.or_add_resource_projection(self.h, T.to_c_uid(pr.uid), T.to_c_uid(pr.pre_uid),
                                                              T.to_c_uid(pr.post_uid), pr.size,
                                                              *[_ptr(a) for a in arrs[:5]], _ptr(rule),
                                                              int(pr.locked)))
                continue
            self._chk(self.lib.or_add_projection(self.h, T.to_c_uid(pr.uid), pr.kind, T.to_c_uid(pr.pre_uid),
                                                 T.to_c_uid(pr.post_uid), pr.size, *[_ptr(a) for a in arrs]))
            for pop_uid, ptype in pr.stdp_populations.items():
                self._chk(self.lib.or_set_stdp_population(self.h, T.to_c_uid(pr.uid), T.to_c_uid(pop_uid), ptype))
        for recv, send in net.subscriptions:
            self._chk(self.lib.or_subscribe(self.h, T.to_c_uid(recv), T.to_c_uid(send)))
        self._chk(self.lib.or_init(self.h))

    def send_spikes(self, sender: bytes, indexes, send_time: int | None = None):
        idx = np.ascontiguousarray(indexes, np.uint32)
        t = self.step_count if send_time is None else send_time
        self._chk(self.lib.or_send_spikes(self.h, T.to_c_uid(sender), t, idx.size, _ptr(idx)))

    def send_impacts(self, sender: bytes, pop: bytes, post_idx, values, out_type=None, is_forcing=True):
        post_idx = np.ascontiguousarray(post_idx, np.uint32)
        values = np.ascontiguousarray(values, np.float32)
        ot = None if out_type is None else np.ascontiguousarray(out_type, np.uint8)
        self._chk(self.lib.or_send_impacts(self.h, T.to_c_uid(sender), T.to_c_uid(pop), int(is_forcing),
                                           post_idx.size, _ptr(post_idx), _ptr(values), _ptr(ot)))

    def step(self):
        self._chk(self.lib.or_step(self.h))

    def snapshot(self):
        """Keep a copy of the network as it is now (restated oracle)."""
        self._chk(self.lib.or_snapshot(self.h))

    def reset(self):
        """Return to the snapshot: step 0, no messages in flight (restated oracle)."""
        self._chk(self.lib.or_reset(self.h))

    def step_mt(self, threads: int):
        """One step with the reference multi-threaded backend's structure (timing only)."""
        self._chk(self.lib.or_step_mt(self.h, threads))

    @property
    def step_count(self) -> int:
        return int(self.lib.or_get_step(self.h))

    @property
    def events(self) -> int:
        return int(self.lib.or_event_count(self.h))

    def spikes(self, pop: bytes) -> np.ndarray:
        n = self._sizes[pop][1]
        out = np.empty(max(n, 1), np.uint32)
        cnt = ctypes.c_uint32(0)
        self._chk(self.lib.or_read_spikes(self.h, T.to_c_uid(pop), out.size, _ptr(out), ctypes.byref(cnt)))
        return out[: cnt.value].copy()

    def blifat(self, pop: bytes):
        kind, n = self._sizes[pop]
        out = np.empty(n, T.BLIFAT_DTYPE)
        ext = np.empty(n, T.RESOURCE_DTYPE) if kind == T.RESOURCE_STDP_BLIFAT else None
        self._chk(self.lib.or_read_blifat(self.h, T.to_c_uid(pop), _ptr(out), _ptr(ext)))
        return out, ext

    def altai(self, pop: bytes):
        kind, n = self._sizes[pop]
        out = np.empty(n, T.ALTAI_DTYPE)
        ext = np.empty(n, T.RESOURCE_DTYPE) if kind == T.RESOURCE_STDP_ALTAI_LIF else None
        self._chk(self.lib.or_read_altai(self.h, T.to_c_uid(pop), _ptr(out), _ptr(ext)))
        return out, ext

    def set_learning(self, on: bool):
        """Backend::start_learning / stop_learning: unlock / lock the weights of every projection."""
        self._chk(self.lib.or_set_learning(self.h, int(on)))

    def resource_synapses(self, proj: bytes) -> np.ndarray:
        out = np.empty(self._sizes[proj][1], T.RESOURCE_SYNAPSE_DTYPE)
        self._chk(self.lib.or_read_resource_synapses(self.h, T.to_c_uid(proj), _ptr(out)))
        return out

    def lif(self, pop: bytes):
        out = np.empty(self._sizes[pop][1], T.LIF_DTYPE)
        self._chk(self.lib.or_read_lif(self.h, T.to_c_uid(pop), _ptr(out)))
        return out

    def weights(self, proj: bytes) -> np.ndarray:
        out = np.empty(self._sizes[proj][1], np.float32)
        self._chk(self.lib.or_read_weights(self.h, T.to_c_uid(proj), _ptr(out)))
        return out


def run(net, schedules, n_steps: int, record=None, which: str = "restated", on_step=None):
    """Run ``n_steps`` steps; before step t every schedule sends its indexes for t (skipped when
    empty, as an input channel sends nothing then). Returns {pop uid: list of per-step spike arrays}
    and the OracleNet."""
    o = OracleNet(which)
    o.load(net)
    record = [p.uid for p in net.populations] if record is None else record
    out = {u: [] for u in record}
    for t in range(n_steps):
        for s in schedules:
            idx = s.at(t)
            if idx.size:
                o.send_spikes(s.sender, idx, t)
        if on_step is not None:
            on_step(o, t)
        o.step()
        for u in record:
            out[u].append(o.spikes(u))
    return out, o
