// TEST INFRASTRUCTURE — stand-in for knp/synapse-traits-library/include/knp/synapse-traits/stdp_add_rule.h.
#pragma once
#include <cstdint>
#include <vector>

#include "stdp_common.h"

namespace knp::synapse_traits
{
template <typename SynapseType>
struct STDPAdditiveRule
{
    using LinkedSynapseType = SynapseType;
    float tau_plus_ = 10;
    float tau_minus_ = 10;
    std::vector<uint64_t> presynaptic_spike_times_;
    std::vector<uint64_t> postsynaptic_spike_times_;
};
}  // namespace knp::synapse_traits
