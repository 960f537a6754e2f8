// TEST INFRASTRUCTURE — stand-in for the BLIFAT neuron parameters of
// knp/neuron-traits-library/include/knp/neuron-traits/blifat.h (field names, types and defaults).
#pragma once
#include <cstddef>
#include <cstdint>
#include <limits>

#include "type_traits.h"

namespace knp::neuron_traits
{
struct BLIFATNeuron;
template <>
struct neuron_parameters<BLIFATNeuron>
{
    std::size_t n_time_steps_since_last_firing_ = std::numeric_limits<std::size_t>::max();
    double activation_threshold_ = 1.0;
    double additional_threshold_ = 0.0;
    double dynamic_threshold_ = 0.0;
    double threshold_decay_ = 0.0;
    double threshold_increment_ = 0.0;
    double postsynaptic_trace_ = 0.0;
    double postsynaptic_trace_decay_ = 0.0;
    double postsynaptic_trace_increment_ = 0.0;
    double inhibitory_conductance_ = 0.0;
    double inhibitory_conductance_decay_ = 0.0;
    double potential_ = 0.0;
    double pre_impact_potential_ = 0.0;
    double potential_decay_ = 0.0;
    unsigned bursting_phase_ = 0;
    unsigned bursting_period_ = 0;
    double reflexive_weight_ = 0.0;
    double reversal_inhibitory_potential_ = -0.3;
    unsigned absolute_refractory_period_ = 0;
    double potential_reset_value_ = 0.0;
    double min_potential_ = -1.0e9;
    int64_t total_blocking_period_ = std::numeric_limits<int64_t>::max();
    double dopamine_value_ = 0.0;
    double stochastic_stimulation_ = 0.0;
    unsigned random_number_generator_state_ = 0;
};
}  // namespace knp::neuron_traits
