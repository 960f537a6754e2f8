// TEST INFRASTRUCTURE — stand-in for the synaptic-resource STDP rule of
// knp/synapse-traits-library/include/knp/synapse-traits/stdp_synaptic_resource_rule.h.
#pragma once
#include <cstdint>
#include <limits>

#include "stdp_common.h"

namespace knp::synapse_traits
{
template <typename SynapseType>
struct STDPSynapticResourceRule
{
    using LinkedSynapseType = SynapseType;
    float synaptic_resource_ = 0;
    float w_min_ = 0;
    float w_max_ = 1;
    float d_u_ = 0;
    uint32_t dopamine_plasticity_period_ = 0;
    uint64_t last_spike_step_ = 0;
    bool had_hebbian_update_ = false;
    bool has_contributed_ = false;
};
}  // namespace knp::synapse_traits
