// TEST INFRASTRUCTURE — stand-in for the LIF neuron parameters of
// knp/neuron-traits-library/include/knp/neuron-traits/lif.h (field names, types and defaults).
#pragma once
#include <cstdint>

#include "type_traits.h"

namespace knp::neuron_traits
{
struct LIFNeuron;
template <>
struct neuron_parameters<LIFNeuron>
{
    float potential_ = 0;
    float potential_reset_value_ = 0;
    float activation_threshold_ = 1;
    float leak_coefficient_ = 1;
    uint32_t refract_counter_ = 0;
    uint32_t refract_period_ = 0;
};
}  // namespace knp::neuron_traits
