"""CPU checks of the C ABI library: it builds for sm_103a, loads without a GPU, and exports every
entry point that include/knp_gb300.h declares (no compute call is made here)."""
import ctypes
import subprocess

import pytest

from knp_gb300 import _capi
from knp_gb300 import build as kb


@pytest.fixture(scope="module")
def lib_path():
    return kb.build()


def test_library_exports_every_declared_symbol(lib_path):
    declared = _capi.exported_symbols()
    assert len(declared) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    lib = ctypes.CDLL(lib_path)
    for s in declared:
        assert getattr(lib, s)


def test_binding_loads_and_reports_errors_without_gpu(lib_path):
    lib = _capi.lib()
    assert b"sm_103a" in lib.knp_gb300_version()
    # Null handles are rejected before any CUDA call.
    assert lib.knp_gb300_step(None, 1) == -1
    assert b"null" in lib.knp_gb300_last_error()
    assert lib.knp_gb300_profile_grid_phases(None, 1, None) == -1
    # Invalid sizes of the add-rate probe are refused before any CUDA call.
    import ctypes

    rate = ctypes.c_double(0.0)
    assert lib.knp_gb300_measure_add_rate(0, 10, ctypes.byref(rate)) != 0
    assert b"positive" in lib.knp_gb300_last_error()
    # GEMM operand layouts: null buffers, a bad mode and a width below the copied extent are refused
    # before any launch.
    assert lib.knp_gb300_bf16_operand(None, 0, 4, 4, 0, 0, 4, None, None) != 0
    buf = (ctypes.c_float * 16)()
    out = (ctypes.c_uint16 * 64)()
    assert lib.knp_gb300_bf16_operand(buf, 0, 4, 4, 3, 0, 4, out, None) != 0
    assert lib.knp_gb300_bf16_operand(buf, 0, 4, 4, 0, 0, 2, out, None) != 0
    assert lib.knp_gb300_bf16_operand(buf, 0, 4, 4, 1, 1, 3, out, None) != 0
    assert b"operand" in lib.knp_gb300_last_error()


def test_library_is_built_for_sm_103a_only():
    assert kb.GENCODE == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_python_constants_match_header_enums():
    """Every enumerator of the ABI headers has the same value in knp_gb300.types, and every declared
    entry point has a ctypes signature in the binding."""
    import os
    import re

    from knp_gb300 import types as T

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    prefixes = [("KNP_GB300_STEP_", "STEP_"), ("KNP_GB300_ACC_", "ACC_"), ("KNP_OUT_", ""), ("KNP_NEURON_", ""),
                ("KNP_SYNAPSE_", ""), ("KNP_STDP_", "STDP_"), ("KNP_ISI_", "ISI_")]
    seen = 0
    for hdr in ("knp_gb300.h", "knp_gb300_types.h"):
        with open(os.path.join(root, "include", hdr)) as f:
            text = f.read()
        for name, value in re.findall(r"\b(KNP_[A-Z0-9_]+)\s*=\s*(-?\d+)", text):
            for c_prefix, py_prefix in prefixes:
                if name.startswith(c_prefix):
                    py = py_prefix + name[len(c_prefix):]
                    assert getattr(T, py) == int(value), (name, py)
                    seen += 1
                    break
    assert seen >= 20
    lib = _capi.lib()
    unbound = [s for s in _capi.exported_symbols() if getattr(lib, s).argtypes is None]
    assert not unbound, unbound
