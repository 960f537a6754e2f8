"""The knp::core::Backend adapter (knp_gb300/adapter) on the CPU: it compiles against the KNP core
interface (stand-ins of knp/core-library/include/knp/core/*.h, whose originals need Boost) with the
reference's own neuron and synapse trait headers where the KNP sources are present, and with their
stand-ins; it lists and accepts the single-threaded backend's neuron and synapse types
(cpu-single-threaded/backend.h:58-68), AltAI-LIF populations included."""
import os

import pytest

from tests import adapter_build as AB


def test_adapter_compiles_against_trait_stand_ins():
    r = AB.syntax_check("shim")
    assert r.returncode == 0, r.stderr


@pytest.mark.skipif(AB.reference_trait_includes() is None, reason="KNP reference sources not present")
def test_adapter_compiles_against_reference_trait_headers():
    r = AB.syntax_check("reference")
    assert r.returncode == 0, r.stderr


def test_adapter_supports_the_single_threaded_backends_types():
    if not os.path.exists(os.path.join(AB.ROOT, "knp_gb300", "libknp_gb300.so")):
        pytest.skip("library not built")
    exe = AB.build_harness()
    r = AB.run_harness(exe, "types")
    assert r.returncode == 0 and r.stdout.strip() == "ok", (r.stdout, r.stderr)
