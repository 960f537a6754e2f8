// TEST INFRASTRUCTURE — stand-in for knp/neuron-traits-library/include/knp/neuron-traits/
// stdp_synaptic_resource_rule.h (field names, types and defaults).
#pragma once
#include <cstdint>
#include <limits>

#include "type_traits.h"

namespace knp::neuron_traits
{
template <typename NeuronType>
struct SynapticResourceSTDPNeuron;
enum class ISIPeriodType
{
    is_forced,
    period_started,
    period_continued,
    not_in_period
};
template <typename NeuronType>
struct neuron_parameters<SynapticResourceSTDPNeuron<NeuronType>> : public neuron_parameters<NeuronType>
{
    neuron_parameters() = default;
    explicit neuron_parameters(const neuron_parameters<NeuronType> &base) : neuron_parameters<NeuronType>(base) {}
    float synapse_sum_threshold_coefficient_ = 0.0F;
    uint32_t dopamine_plasticity_time_ = 1;
    float free_synaptic_resource_ = 1;
    float synaptic_resource_threshold_ = std::numeric_limits<float>::max();
    uint32_t resource_drain_coefficient_ = 0;
    float stability_ = 0;
    float stability_change_parameter_ = 0;
    float stability_change_at_isi_ = 0;
    uint32_t isi_max_ = 1;
    float d_h_ = 1.F;
    ISIPeriodType isi_status_ = ISIPeriodType::not_in_period;
    uint64_t last_step_ = 0;
    uint64_t last_spike_step_ = 0;
    uint64_t first_isi_spike_ = 0;
    bool is_being_forced_ = false;
};
}  // namespace knp::neuron_traits
