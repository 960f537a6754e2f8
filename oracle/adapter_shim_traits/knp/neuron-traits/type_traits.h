// TEST INFRASTRUCTURE — stand-in for knp/neuron-traits-library/include/knp/neuron-traits/type_traits.h
// on machines without the KNP sources (names as in the reference; see oracle/adapter_shim/README.md).
#pragma once
namespace knp::neuron_traits
{
template <class NeuronType>
struct default_values;
template <class NeuronType>
struct neuron_parameters;
}  // namespace knp::neuron_traits
