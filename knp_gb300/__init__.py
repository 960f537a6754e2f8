"""knp_gb300 — GB300 (sm_103a) backend for the Kaspersky Neuromorphic Platform hot path.

BLIFAT and synaptic-resource-STDP BLIFAT populations, delta-synapse and additive-STDP delta-synapse
projections, stepped by hand-written CUDA kernels behind the C ABI in include/knp_gb300.h
(libknp_gb300.so, built in-tree by knp_gb300/build.py). ``GB300Backend`` mirrors the reference's
``knp::core::Backend`` interface in Python; ``network`` holds the network description and the
seeded generators.
"""
from . import network, types  # noqa: F401

__all__ = ["network", "types", "GB300Backend", "run"]


def __getattr__(name):
    # The backend loads libknp_gb300.so on first use and raises if it is missing: there is no
    # CPU fallback.
    if name in ("GB300Backend", "run"):
        from . import backend

        return getattr(backend, name)
    raise AttributeError(name)
