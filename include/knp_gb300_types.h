/*
 * Plain-data types shared by the GB300 backend C ABI (knp_gb300.h) and its CPU oracle.
 *
 * Every struct mirrors the field list and field meaning of a KNP reference type, with explicit
 * padding so that the layout is the same for C, C++, ctypes and numpy structured dtypes:
 *   knp_uid                   <- knp::core::UID (16-byte boost::uuids::uuid), knp/core-library/include/knp/core/uid.h
 *   knp_output_type           <- knp::synapse_traits::OutputType, knp/synapse-traits-library/include/knp/synapse-traits/output_types.h:36-62
 *   knp_blifat_neuron         <- neuron_parameters<BLIFATNeuron>, knp/neuron-traits-library/include/knp/neuron-traits/blifat.h:207-343
 *   knp_resource_stdp_state   <- neuron_parameters<SynapticResourceSTDPNeuron<N>> extra fields,
 *                                knp/neuron-traits-library/include/knp/neuron-traits/stdp_synaptic_resource_rule.h:70-192
 *   knp_isi_status            <- ISIPeriodType, stdp_synaptic_resource_rule.h:46-66
 *   knp_stdp_processing       <- Projection<STDP<...>>::SharedSynapseParameters::ProcessingType, knp/core-library/include/knp/core/projection.h:139-150
 */
#ifndef KNP_GB300_TYPES_H
#define KNP_GB300_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/** 16-byte entity identifier (population, projection, or external message channel). */
typedef struct knp_uid
{
    uint8_t bytes[16];
} knp_uid;

/** Synapse output type; numbering equals knp::synapse_traits::OutputType. */
typedef enum knp_output_type
{
    KNP_OUT_EXCITATORY = 0,
    KNP_OUT_INHIBITORY_CURRENT = 1,
    KNP_OUT_INHIBITORY_CONDUCTANCE = 2,
    KNP_OUT_DOPAMINE = 3,
    KNP_OUT_BLOCKING = 4
} knp_output_type;

/** Neuron model of a population. */
typedef enum knp_neuron_kind
{
    KNP_NEURON_BLIFAT = 0,
    KNP_NEURON_RESOURCE_STDP_BLIFAT = 1,
    KNP_NEURON_LIF = 2
} knp_neuron_kind;

/** Synapse model of a projection. */
typedef enum knp_synapse_kind
{
    KNP_SYNAPSE_DELTA = 0,
    KNP_SYNAPSE_ADDITIVE_STDP_DELTA = 1
} knp_synapse_kind;

/** How an STDP projection treats spikes of one of its STDP populations. */
typedef enum knp_stdp_processing
{
    KNP_STDP_ONLY = 0,
    KNP_STDP_AND_SPIKE = 1
} knp_stdp_processing;

/** Inter-spike-interval status of a resource-STDP neuron; numbering equals ISIPeriodType. */
typedef enum knp_isi_status
{
    KNP_ISI_IS_FORCED = 0,
    KNP_ISI_PERIOD_STARTED = 1,
    KNP_ISI_PERIOD_CONTINUED = 2,
    KNP_ISI_NOT_IN_PERIOD = 3
} knp_isi_status;

/**
 * BLIFAT neuron parameters and state, field for field as neuron_parameters<BLIFATNeuron>
 * (blifat.h:207-343). 192 bytes. Defaults are set by knp_blifat_neuron_defaults().
 */
typedef struct knp_blifat_neuron
{
    uint64_t n_time_steps_since_last_firing;  /* default UINT64_MAX */
    double activation_threshold;              /* default 1.0 */
    double additional_threshold;
    double dynamic_threshold;
    double threshold_decay;
    double threshold_increment;
    double postsynaptic_trace;
    double postsynaptic_trace_decay;
    double postsynaptic_trace_increment;
    double inhibitory_conductance;
    double inhibitory_conductance_decay;
    double potential;
    double pre_impact_potential;
    double potential_decay;
    uint32_t bursting_phase;
    uint32_t bursting_period;
    double reflexive_weight;
    double reversal_inhibitory_potential;  /* default -0.3 */
    uint32_t absolute_refractory_period;
    uint32_t pad0_;
    double potential_reset_value;
    double min_potential;                  /* default -1e9 */
    int64_t total_blocking_period;         /* default INT64_MAX */
    double dopamine_value;
    double stochastic_stimulation;
    uint32_t random_number_generator_state;
    uint32_t pad1_;
} knp_blifat_neuron;

/**
 * Extra state of a synaptic-resource-STDP neuron (stdp_synaptic_resource_rule.h:70-192), kept
 * beside its knp_blifat_neuron base. 72 bytes.
 */
typedef struct knp_resource_stdp_state
{
    float synapse_sum_threshold_coefficient;  /* default 0 */
    uint32_t dopamine_plasticity_time;        /* default 1 */
    float free_synaptic_resource;             /* default 1 */
    float synaptic_resource_threshold;        /* default FLT_MAX */
    uint32_t resource_drain_coefficient;      /* default 0 */
    float stability;
    float stability_change_parameter;
    float stability_change_at_isi;
    uint32_t isi_max;                         /* default 1 */
    float d_h;                                /* default 1 */
    int32_t isi_status;                       /* knp_isi_status, default KNP_ISI_NOT_IN_PERIOD */
    uint32_t is_being_forced;                 /* bool */
    uint64_t last_step;
    uint64_t last_spike_step;
    uint64_t first_isi_spike;
} knp_resource_stdp_state;

/**
 * LIF neuron parameters and state, field for field as neuron_parameters<LIFNeuron>
 * (knp/neuron-traits-library/include/knp/neuron-traits/lif.h:84-118). 24 bytes.
 */
typedef struct knp_lif_neuron
{
    float potential;
    float potential_reset_value;
    float activation_threshold;  /* default 1 */
    float leak_coefficient;      /* default 1 */
    uint32_t refract_counter;
    uint32_t refract_period;
} knp_lif_neuron;

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
static_assert(sizeof(knp_lif_neuron) == 24, "knp_lif_neuron layout");
static_assert(sizeof(knp_blifat_neuron) == 192, "knp_blifat_neuron layout");
static_assert(sizeof(knp_resource_stdp_state) == 72, "knp_resource_stdp_state layout");
#endif

#endif /* KNP_GB300_TYPES_H */
