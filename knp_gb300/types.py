"""numpy / ctypes views of the plain-data types in include/knp_gb300_types.h.

Each dtype is the byte-exact layout of the C struct, so arrays of it can be handed to the C ABI
(and to the CPU oracle) without conversion. Field names and defaults mirror the KNP reference:
``neuron_parameters<BLIFATNeuron>`` (knp/neuron-traits-library/include/knp/neuron-traits/blifat.h:47-343),
the resource-STDP neuron extension (stdp_synaptic_resource_rule.h:70-192) and
``neuron_parameters<LIFNeuron>`` (lif.h:46-118).
"""
from __future__ import annotations

import ctypes
import uuid as _uuid

import numpy as np

UINT64_MAX = np.iinfo(np.uint64).max
INT64_MAX = np.iinfo(np.int64).max
FLT_MAX = float(np.finfo(np.float32).max)

# knp_output_type (output_types.h:36-62)
EXCITATORY, INHIBITORY_CURRENT, INHIBITORY_CONDUCTANCE, DOPAMINE, BLOCKING = range(5)
# knp_neuron_kind
BLIFAT, RESOURCE_STDP_BLIFAT, LIF, ALTAI_LIF, RESOURCE_STDP_ALTAI_LIF = range(5)
# knp_synapse_kind
DELTA, ADDITIVE_STDP_DELTA, RESOURCE_STDP_DELTA = range(3)
# Device synapse generators (knp_generator_kind).
(GEN_ALL_TO_ALL, GEN_ALIGNED, GEN_EXCLUSIVE, GEN_ONE_TO_ONE, GEN_FIXED_PROBABILITY, GEN_FIXED_NUMBER_POST,
 GEN_FIXED_NUMBER_PRE) = range(7)
# knp_stdp_processing (projection.h:139-150)
STDP_ONLY, STDP_AND_SPIKE = range(2)
# knp_gb300_accumulator (input-ring accumulation of a population)
ACC_AUTO, ACC_FP32, ACC_FIXED64 = range(3)
STEP_AUTO, STEP_PHASES, STEP_FUSED, STEP_GRID = range(4)  # knp_gb300_step_mode
# knp_isi_status (stdp_synaptic_resource_rule.h:46-66)
ISI_IS_FORCED, ISI_PERIOD_STARTED, ISI_PERIOD_CONTINUED, ISI_NOT_IN_PERIOD = range(4)

BLIFAT_DTYPE = np.dtype(
    [
        ("n_time_steps_since_last_firing", "<u8"),
        ("activation_threshold", "<f8"),
        ("additional_threshold", "<f8"),
        ("dynamic_threshold", "<f8"),
        ("threshold_decay", "<f8"),
        ("threshold_increment", "<f8"),
        ("postsynaptic_trace", "<f8"),
        ("postsynaptic_trace_decay", "<f8"),
        ("postsynaptic_trace_increment", "<f8"),
        ("inhibitory_conductance", "<f8"),
        ("inhibitory_conductance_decay", "<f8"),
        ("potential", "<f8"),
        ("pre_impact_potential", "<f8"),
        ("potential_decay", "<f8"),
        ("bursting_phase", "<u4"),
        ("bursting_period", "<u4"),
        ("reflexive_weight", "<f8"),
        ("reversal_inhibitory_potential", "<f8"),
        ("absolute_refractory_period", "<u4"),
        ("pad0_", "<u4"),
        ("potential_reset_value", "<f8"),
        ("min_potential", "<f8"),
        ("total_blocking_period", "<i8"),
        ("dopamine_value", "<f8"),
        ("stochastic_stimulation", "<f8"),
        ("random_number_generator_state", "<u4"),
        ("pad1_", "<u4"),
    ]
)
assert BLIFAT_DTYPE.itemsize == 192

RESOURCE_DTYPE = np.dtype(
    [
        ("synapse_sum_threshold_coefficient", "<f4"),
        ("dopamine_plasticity_time", "<u4"),
        ("free_synaptic_resource", "<f4"),
        ("synaptic_resource_threshold", "<f4"),
        ("resource_drain_coefficient", "<u4"),
        ("stability", "<f4"),
        ("stability_change_parameter", "<f4"),
        ("stability_change_at_isi", "<f4"),
        ("isi_max", "<u4"),
        ("d_h", "<f4"),
        ("isi_status", "<i4"),
        ("is_being_forced", "<u4"),
        ("last_step", "<u8"),
        ("last_spike_step", "<u8"),
        ("first_isi_spike", "<u8"),
    ]
)
assert RESOURCE_DTYPE.itemsize == 72

# knp_resource_synapse: the rule state of one SynapticResourceSTDPDeltaSynapse
# (stdp_synaptic_resource_rule.h:45-89)
RESOURCE_SYNAPSE_DTYPE = np.dtype(
    [
        ("synaptic_resource", "<f4"),
        ("w_min", "<f4"),
        ("w_max", "<f4"),
        ("d_u", "<f4"),
        ("dopamine_plasticity_period", "<u4"),
        ("had_hebbian_update", "<u4"),
        ("last_spike_step", "<u8"),
        ("has_contributed", "<u4"),
        ("pad_", "<u4"),
    ]
)
assert RESOURCE_SYNAPSE_DTYPE.itemsize == 40

# knp_altai_neuron: neuron_parameters<AltAILIF> (altai_lif.h:164-335)
ALTAI_DTYPE = np.dtype(
    [
        ("is_diff", "u1"),
        ("is_reset", "u1"),
        ("leak_rev", "u1"),
        ("saturate", "u1"),
        ("do_not_save", "u1"),
        ("pad0_", "u1", (3,)),
        ("potential", "<f4"),
        ("pre_impact_potential", "<f4"),
        ("activation_threshold", "<u2"),
        ("negative_activation_threshold", "<u2"),
        ("potential_leak", "<i2"),
        ("potential_reset_value", "<u2"),
        ("dopamine_value", "<f8"),
        ("additional_threshold", "<f8"),
        ("activity_time", "<i8"),
    ]
)
assert ALTAI_DTYPE.itemsize == 48

LIF_DTYPE = np.dtype(
    [
        ("potential", "<f4"),
        ("potential_reset_value", "<f4"),
        ("activation_threshold", "<f4"),
        ("leak_coefficient", "<f4"),
        ("refract_counter", "<u4"),
        ("refract_period", "<u4"),
    ]
)
assert LIF_DTYPE.itemsize == 24


def blifat_defaults(n: int) -> np.ndarray:
    """``n`` BLIFAT neurons with the reference defaults (blifat.h:47-201)."""
    a = np.zeros(n, dtype=BLIFAT_DTYPE)
    a["n_time_steps_since_last_firing"] = UINT64_MAX
    a["activation_threshold"] = 1.0
    a["reversal_inhibitory_potential"] = -0.3
    a["min_potential"] = -1.0e9
    a["total_blocking_period"] = INT64_MAX
    return a


def resource_defaults(n: int) -> np.ndarray:
    """``n`` resource-STDP neuron extensions with the reference defaults (stdp_synaptic_resource_rule.h:70-192)."""
    a = np.zeros(n, dtype=RESOURCE_DTYPE)
    a["dopamine_plasticity_time"] = 1
    a["free_synaptic_resource"] = 1.0
    a["synaptic_resource_threshold"] = FLT_MAX
    a["isi_max"] = 1
    a["d_h"] = 1.0
    a["isi_status"] = ISI_NOT_IN_PERIOD
    return a


def resource_synapse_defaults(n: int) -> np.ndarray:
    """``n`` resource-STDP synapse rules with the reference defaults (stdp_synaptic_resource_rule.h:45-89)."""
    a = np.zeros(n, dtype=RESOURCE_SYNAPSE_DTYPE)
    a["w_max"] = 1.0
    return a


def altai_defaults(n: int) -> np.ndarray:
    """``n`` AltAI-LIF neurons with the reference defaults (altai_lif.h:50-157)."""
    a = np.zeros(n, dtype=ALTAI_DTYPE)
    a["is_reset"] = 1
    a["leak_rev"] = 1
    a["saturate"] = 1
    a["activation_threshold"] = 1
    a["negative_activation_threshold"] = 30000
    return a


def is_altai(kind: int) -> bool:
    return kind in (ALTAI_LIF, RESOURCE_STDP_ALTAI_LIF)


def is_resource(kind: int) -> bool:
    return kind in (RESOURCE_STDP_BLIFAT, RESOURCE_STDP_ALTAI_LIF)


def lif_defaults(n: int) -> np.ndarray:
    """``n`` LIF neurons with the reference defaults (lif.h:46-82)."""
    a = np.zeros(n, dtype=LIF_DTYPE)
    a["activation_threshold"] = 1.0
    a["leak_coefficient"] = 1.0
    return a


class KnpUid(ctypes.Structure):
    """knp_uid: 16 bytes, passed by value."""

    _fields_ = [("bytes", ctypes.c_uint8 * 16)]


NULL_UID = bytes(16)


def new_uid() -> bytes:
    """A random 16-byte identifier, as knp::core::UID() draws one."""
    return _uuid.uuid4().bytes


def uid_from_int(i: int) -> bytes:
    """A deterministic identifier (for seeded networks and tests)."""
    return int(i).to_bytes(16, "little")


def to_c_uid(u: bytes) -> KnpUid:
    if len(u) != 16:
        raise ValueError("a UID is 16 bytes")
    c = KnpUid()
    ctypes.memmove(c.bytes, u, 16)
    return c
