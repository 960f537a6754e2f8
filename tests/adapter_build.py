"""Builds the knp::core::Backend adapter harness (tests/adapter/harness.cpp + knp_gb300/adapter) with
g++ against the KNP core stand-ins (oracle/adapter_shim) and either the reference's own neuron and
synapse trait headers (where the KNP sources are present) or their stand-ins
(oracle/adapter_shim_traits), linked with the GB300 library. Used by the adapter tests only."""
import os
import shutil
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ADAPTER = os.path.join(ROOT, "knp_gb300", "adapter")
SHIM = os.path.join(ROOT, "oracle", "adapter_shim")
SHIM_TRAITS = os.path.join(ROOT, "oracle", "adapter_shim_traits")
OUT_DIR = os.path.join(ROOT, "oracle", "_build")


def knp_reference_dir():
    return os.environ.get("KNP_REF") or os.path.join(os.path.dirname(ROOT), "reference")


def reference_trait_includes():
    """-I flags of the reference's trait headers, or None where the KNP sources are absent."""
    ref = knp_reference_dir()
    n = os.path.join(ref, "knp", "neuron-traits-library", "include")
    s = os.path.join(ref, "knp", "synapse-traits-library", "include")
    if os.path.isdir(n) and os.path.isdir(s):
        return ["-I" + n, "-I" + s, "-include", "cstdint", "-include", "cstddef"]
    return None


def compiler():
    return os.environ.get("CXX") or shutil.which("g++") or "g++"


def flags(traits="shim"):
    inc = ["-I" + SHIM]
    if traits == "reference":
        ref = reference_trait_includes()
        if ref is None:
            raise FileNotFoundError("KNP reference sources not found")
        inc += ref
    else:
        inc += ["-I" + SHIM_TRAITS]
    return ["-std=c++17", "-O1", "-Wall", "-Werror", *inc, "-I" + os.path.join(ROOT, "include"), "-I" + ADAPTER]


def syntax_check(traits="shim"):
    cmd = [compiler(), *flags(traits), "-fsyntax-only", os.path.join(ADAPTER, "knp_gb300_backend.cpp"),
           os.path.join(ROOT, "tests", "adapter", "harness.cpp")]
    return subprocess.run(cmd, capture_output=True, text=True)


def build_harness():
    os.makedirs(OUT_DIR, exist_ok=True)
    exe = os.path.join(OUT_DIR, "adapter_harness")
    lib_dir = os.path.join(ROOT, "knp_gb300")
    cmd = [compiler(), *flags("shim"), os.path.join(ROOT, "tests", "adapter", "harness.cpp"),
           os.path.join(ADAPTER, "knp_gb300_backend.cpp"), "-L" + lib_dir, "-lknp_gb300", "-Wl,-rpath," + lib_dir,
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"adapter harness build failed:\n{r.stdout}\n{r.stderr}")
    return exe


def run_harness(exe, case, timeout=300):
    return subprocess.run([exe, case], capture_output=True, text=True, timeout=timeout)
