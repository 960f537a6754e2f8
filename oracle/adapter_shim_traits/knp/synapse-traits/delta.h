// TEST INFRASTRUCTURE — stand-in for the delta synapse parameters of
// knp/synapse-traits-library/include/knp/synapse-traits/delta.h.
#pragma once
#include <cstdint>

#include "output_types.h"
#include "type_traits.h"

namespace knp::synapse_traits
{
struct DeltaSynapse;
template <>
struct synapse_parameters<DeltaSynapse>
{
    float weight_ = 0.0F;
    uint32_t delay_ = 1;
    knp::synapse_traits::OutputType output_type_ = OutputType::EXCITATORY;
};
}  // namespace knp::synapse_traits
