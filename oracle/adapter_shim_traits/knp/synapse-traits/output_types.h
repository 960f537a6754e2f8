// TEST INFRASTRUCTURE — stand-in for knp/synapse-traits-library/include/knp/synapse-traits/output_types.h.
#pragma once
namespace knp::synapse_traits
{
enum class OutputType
{
    EXCITATORY = 0,
    INHIBITORY_CURRENT = 1,
    INHIBITORY_CONDUCTANCE = 2,
    DOPAMINE = 3,
    BLOCKING = 4
};
}  // namespace knp::synapse_traits
