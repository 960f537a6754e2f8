"""ctypes binding of include/knp_gb300.h (libknp_gb300.so, built in-tree by knp_gb300/build.py).

There is no fallback: if the library is missing or fails to load, importing the binding raises.
This module is also the reference-side stub a Python KNP user would add to drive the backend.
"""
from __future__ import annotations

import ctypes
import os

from . import types as T

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libknp_gb300.so")

STATUS = {0: "OK", -1: "E_INVALID", -2: "E_STATE", -3: "E_CUDA", -4: "E_DEVICE_FLAG", -5: "E_NOMEM"}


class KnpGb300Error(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def lib():
    """The loaded library (loads it on first use; raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise FileNotFoundError(
            f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(LIB_PATH)
    U = T.KnpUid
    p = ctypes.c_void_p
    u64 = ctypes.c_uint64
    u32 = ctypes.c_uint32
    i32 = ctypes.c_int32
    c_int = ctypes.c_int
    sig = {
        "knp_gb300_last_error": ([], ctypes.c_char_p),
        "knp_gb300_version": ([], ctypes.c_char_p),
        "knp_gb300_create": ([c_int, ctypes.POINTER(p)], c_int),
        "knp_gb300_destroy": ([p], c_int),
        "knp_gb300_load_blifat_population": ([p, U, c_int, u32, p, p], c_int),
        "knp_gb300_load_lif_population": ([p, U, u32, p], c_int),
        "knp_gb300_read_lif_population": ([p, U, p], c_int),
        "knp_gb300_load_projection": ([p, U, c_int, U, U, u64, p, p, p, p, p, p, p], c_int),
        "knp_gb300_generate_fixed_fan_in_projection": ([p, U, U, U, u32, u32, u32, i32, i32, u32, u32, u64, u64], c_int),
        "knp_gb300_generate_projection": ([p, U, U, U, c_int, u32, u32, u64, ctypes.c_double, i32, i32, u32, u32, u64, u64],
                                          c_int),
        "knp_gb300_set_stdp_population": ([p, U, U, c_int], c_int),
        "knp_gb300_subscribe": ([p, U, U], c_int),
        "knp_gb300_set_accumulator": ([p, U, c_int], c_int),
        "knp_gb300_record_spikes": ([p, U, c_int], c_int),
        "knp_gb300_set_pull_threshold": ([p, U, ctypes.c_double], c_int),
        "knp_gb300_set_step_mode": ([p, c_int], c_int),
        "knp_gb300_step_fused": ([p, ctypes.POINTER(c_int)], c_int),
        "knp_gb300_step_kernel": ([p, ctypes.POINTER(c_int)], c_int),
        "knp_gb300_init": ([p], c_int),
        "knp_gb300_send_spikes": ([p, U, u64, u32, p], c_int),
        "knp_gb300_load_spike_schedule": ([p, U, u64, u64, p, p], c_int),
        "knp_gb300_generate_bernoulli_schedule": ([p, U, u32, ctypes.c_double, u64, u64, u64, u64], c_int),
        "knp_gb300_send_impacts": ([p, U, U, c_int, u32, p, p, p], c_int),
        "knp_gb300_generate_bernoulli_schedule_noalloc": ([u32, ctypes.c_double, u64, u64, u64, u64, p, p, u64,
                                                           ctypes.POINTER(u64), p], c_int),
        "knp_gb300_step": ([p, u64], c_int),
        "knp_gb300_get_step": ([p, ctypes.POINTER(u64)], c_int),
        "knp_gb300_read_spikes": ([p, U, u64, u32, p, ctypes.POINTER(u32)], c_int),
        "knp_gb300_discard_spikes": ([p, u64], c_int),
        "knp_gb300_read_blifat_population": ([p, U, p, p], c_int),
        "knp_gb300_read_weights": ([p, U, p], c_int),
        "knp_gb300_load_altai_population": ([p, U, c_int, ctypes.c_uint32, p, p], c_int),
        "knp_gb300_read_altai_population": ([p, U, p, p], c_int),
        "knp_gb300_load_resource_stdp_projection": ([p, U, U, U, u64, p, p, p, p, p, p, c_int], c_int),
        "knp_gb300_read_resource_synapses": ([p, U, p], c_int),
        "knp_gb300_projection_size": ([p, U, ctypes.POINTER(u64)], c_int),
        "knp_gb300_start_learning": ([p], c_int),
        "knp_gb300_stop_learning": ([p], c_int),
        "knp_gb300_counters": ([p, ctypes.POINTER(u64), ctypes.POINTER(u64), ctypes.POINTER(u64)], c_int),
        "knp_gb300_step_timed": ([p, u64, ctypes.POINTER(ctypes.c_float)], c_int),
        "knp_gb300_profile_phases": ([p, u64, ctypes.POINTER(ctypes.c_float)], c_int),
        "knp_gb300_profile_grid_phases": ([p, u64, ctypes.POINTER(ctypes.c_double)], c_int),
        "knp_gb300_measure_add_rate": ([u64, u64, ctypes.POINTER(ctypes.c_double)], c_int),
        "knp_gb300_bf16_operand": ([p, c_int, ctypes.c_int64, ctypes.c_int64, c_int, c_int, ctypes.c_int64, p, p], c_int),
        "knp_gb300_lif_scan_forward": ([p, p, p, c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_float, c_int, c_int,
                                        ctypes.c_float, p], c_int),
        "knp_gb300_lif_scan_backward": ([p, p, p, p, c_int, ctypes.c_int64, ctypes.c_float, ctypes.c_float, c_int,
                                         c_int, ctypes.c_float, p], c_int),
        "knp_gb300_bf16_gemm_tn": ([p, p, p, c_int, c_int, c_int, p, p], c_int),
        "knp_gb300_batched_lif_run": ([c_int, p, p, p, p, p, p, u32, p, p, u64, p, p, ctypes.POINTER(u64),
                                       ctypes.POINTER(ctypes.c_float), p], c_int),
        "knp_gb300_batched_plan_create": ([c_int, p, p, p, p, p, p, u32, p, p, p, u64, p, p, c_int, u32, p,
                                           ctypes.POINTER(p)], c_int),
        "knp_gb300_batched_plan_run": ([p, ctypes.POINTER(u64), ctypes.POINTER(ctypes.c_float)], c_int),
        "knp_gb300_batched_plan_info": ([p, ctypes.POINTER(c_int), ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_float)],
                                        c_int),
        "knp_gb300_batched_plan_destroy": ([p], None),
        "knp_gb300_synchronize": ([p], c_int),
        "knp_gb300_stream": ([p, ctypes.POINTER(p)], c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def exported_symbols() -> list:
    """Names of the C ABI entry points declared in include/knp_gb300.h."""
    hdr = os.path.join(os.path.dirname(HERE), "include", "knp_gb300.h")
    import re

    with open(hdr) as f:
        return sorted(set(re.findall(r"\b(knp_gb300_[a-z0-9_]+)\s*\(", f.read())))


def check(rc: int):
    if rc != 0:
        raise KnpGb300Error(rc, lib().knp_gb300_last_error().decode())
