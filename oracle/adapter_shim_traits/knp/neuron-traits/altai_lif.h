// TEST INFRASTRUCTURE — stand-in for the AltAI-LIF neuron parameters of
// knp/neuron-traits-library/include/knp/neuron-traits/altai_lif.h (field names, types and defaults).
#pragma once
#include <cstdint>

#include "type_traits.h"

namespace knp::neuron_traits
{
struct AltAILIF;
template <>
struct neuron_parameters<AltAILIF>
{
    bool is_diff_ = false;
    bool is_reset_ = true;
    bool leak_rev_ = true;
    bool saturate_ = true;
    bool do_not_save_ = false;
    float potential_ = 0;
    float pre_impact_potential_ = 0;
    uint16_t activation_threshold_ = 1;
    uint16_t negative_activation_threshold_ = 30000;
    int16_t potential_leak_ = 0;
    uint16_t potential_reset_value_ = 0;
    double dopamine_value_ = 0.0;
    double additional_threshold_ = 0.;
    int64_t activity_time_ = 0;
};
}  // namespace knp::neuron_traits
