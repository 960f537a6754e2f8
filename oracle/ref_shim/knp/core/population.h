// TEST INFRASTRUCTURE — minimal stand-in for knp::core::Population<Neuron>
// (knp/core-library/include/knp/core/population.h:46-285): a UID and a vector of neuron parameters.
#pragma once
#include <vector>

#include <knp/core/messaging/messaging.h>
#include <knp/neuron-traits/stdp_type_traits.h>
#include <knp/neuron-traits/lif.h>

namespace knp::core
{
template <class NeuronType>
class Population
{
public:
    using PopulationNeuronType = NeuronType;
    using NeuronParameters = neuron_traits::neuron_parameters<NeuronType>;
    Population() = default;
    Population(const UID &uid, std::vector<NeuronParameters> neurons) : uid_(uid), neurons_(std::move(neurons)) {}
    const UID &get_uid() const { return uid_; }
    size_t size() const { return neurons_.size(); }
    NeuronParameters &operator[](size_t i) { return neurons_[i]; }
    const NeuronParameters &operator[](size_t i) const { return neurons_[i]; }
    auto begin() { return neurons_.begin(); }
    auto end() { return neurons_.end(); }

private:
    UID uid_;
    std::vector<NeuronParameters> neurons_;
};
}  // namespace knp::core
