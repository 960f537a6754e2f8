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
 *   knp_resource_synapse      <- STDPSynapticResourceRule, knp/synapse-traits-library/include/knp/synapse-traits/stdp_synaptic_resource_rule.h:45-89
 *   knp_lif_neuron            <- neuron_parameters<LIFNeuron>, knp/neuron-traits-library/include/knp/neuron-traits/lif.h:84-118
 *   knp_altai_neuron          <- neuron_parameters<AltAILIF>, knp/neuron-traits-library/include/knp/neuron-traits/altai_lif.h:164-335
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
    KNP_NEURON_LIF = 2,
    KNP_NEURON_ALTAI_LIF = 3,
    KNP_NEURON_RESOURCE_STDP_ALTAI_LIF = 4
} knp_neuron_kind;

/** Synapse model of a projection. */
typedef enum knp_synapse_kind
{
    KNP_SYNAPSE_DELTA = 0,
    KNP_SYNAPSE_ADDITIVE_STDP_DELTA = 1,
    KNP_SYNAPSE_RESOURCE_STDP_DELTA = 2
} knp_synapse_kind;

/**
 * Rule of a device-generated projection (knp_gb300_generate_projection); each is the index -> pair
 * rule of one generator of knp/base-framework/include/knp/framework/projection/synapse_generators.h.
 */
typedef enum knp_generator_kind
{
    KNP_GEN_ALL_TO_ALL = 0,          /* all_to_all (:59-69): pre = i % n_pre, post = i / n_pre */
    KNP_GEN_ALIGNED = 1,             /* aligned (:93-120) */
    KNP_GEN_EXCLUSIVE = 2,           /* exclusive (:139-154): all pairs but pre == post */
    KNP_GEN_ONE_TO_ONE = 3,          /* one_to_one (:172-178) */
    KNP_GEN_FIXED_PROBABILITY = 4,   /* FixedProbability (:259-300): all_to_all pairs kept with a probability */
    KNP_GEN_FIXED_NUMBER_POST = 5,   /* FixedNumberPost (:352-388): pre = i % n_pre, post uniform */
    KNP_GEN_FIXED_NUMBER_PRE = 6     /* FixedNumberPre (:409-445): pre uniform, post = i % n_post */
} knp_generator_kind;

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
 * Rule state of a synaptic-resource STDP delta synapse (synapse_parameters<
 * SynapticResourceSTDPDeltaSynapse>::rule_, knp/synapse-traits-library/include/knp/synapse-traits/
 * stdp_synaptic_resource_rule.h:45-89), field for field. 40 bytes.
 */
typedef struct knp_resource_synapse
{
    float synaptic_resource;              /* default 0 */
    float w_min;                          /* default 0 */
    float w_max;                          /* default 1 */
    float d_u;                            /* default 0 */
    uint32_t dopamine_plasticity_period;  /* default 0 */
    uint32_t had_hebbian_update;          /* bool */
    uint64_t last_spike_step;             /* default 0 */
    uint32_t has_contributed;             /* bool */
    uint32_t pad_;
} knp_resource_synapse;

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

/**
 * AltAI-LIF neuron parameters and state, field for field and in the same layout as
 * neuron_parameters<AltAILIF> (knp/neuron-traits-library/include/knp/neuron-traits/altai_lif.h:
 * 164-335; bools as bytes). 48 bytes. A KNP_NEURON_RESOURCE_STDP_ALTAI_LIF population keeps a
 * knp_resource_stdp_state beside each neuron, as the BLIFAT variant does.
 */
typedef struct knp_altai_neuron
{
    uint8_t is_diff;                         /* default 0 */
    uint8_t is_reset;                        /* default 1 */
    uint8_t leak_rev;                        /* default 1 */
    uint8_t saturate;                        /* default 1 */
    uint8_t do_not_save;                     /* default 0 */
    uint8_t pad0_[3];
    float potential;
    float pre_impact_potential;
    uint16_t activation_threshold;           /* default 1 */
    uint16_t negative_activation_threshold;  /* default 30000 */
    int16_t potential_leak;                  /* default 0 */
    uint16_t potential_reset_value;          /* default 0 */
    double dopamine_value;
    double additional_threshold;
    int64_t activity_time;                   /* default 0 */
} knp_altai_neuron;

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
static_assert(sizeof(knp_lif_neuron) == 24, "knp_lif_neuron layout");
static_assert(sizeof(knp_blifat_neuron) == 192, "knp_blifat_neuron layout");
static_assert(sizeof(knp_resource_stdp_state) == 72, "knp_resource_stdp_state layout");
static_assert(sizeof(knp_resource_synapse) == 40, "knp_resource_synapse layout");
static_assert(sizeof(knp_altai_neuron) == 48, "knp_altai_neuron layout");
#endif

#endif /* KNP_GB300_TYPES_H */
