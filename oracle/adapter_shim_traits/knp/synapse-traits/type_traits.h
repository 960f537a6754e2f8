// TEST INFRASTRUCTURE — stand-in for knp/synapse-traits-library/include/knp/synapse-traits/type_traits.h.
#pragma once
namespace knp::synapse_traits
{
template <class SynapseType>
struct default_values;
template <class SynapseType>
struct synapse_parameters;
template <class SynapseType>
struct shared_synapse_parameters
{
};
}  // namespace knp::synapse_traits
