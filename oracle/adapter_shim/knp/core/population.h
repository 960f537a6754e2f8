// TEST INFRASTRUCTURE — stand-in for knp::core::Population (knp/core-library/include/knp/core/
// population.h): a UID and the neurons' parameters, built from a generator; AllPopulationsVariant over
// the neuron types the adapter handles.
#pragma once
#include <functional>
#include <optional>
#include <variant>
#include <vector>

#include <knp/core/core.h>
#include <knp/neuron-traits/altai_lif.h>
#include <knp/neuron-traits/blifat.h>
#include <knp/neuron-traits/lif.h>
#include <knp/neuron-traits/stdp_type_traits.h>

namespace knp::core
{
template <class NeuronType>
class Population final
{
public:
    using PopulationNeuronType = NeuronType;
    using PopulationType = Population<NeuronType>;
    using NeuronParameters = neuron_traits::neuron_parameters<NeuronType>;
    using NeuronGenerator = std::function<std::optional<NeuronParameters>(size_t index)>;
    using NeuronsContainer = std::vector<NeuronParameters>;

    Population(NeuronGenerator generator, size_t neurons_count) : Population(UID(), generator, neurons_count) {}
    Population(const UID &uid, NeuronGenerator generator, size_t neurons_count) : uid_(uid)
    {
        neurons_.reserve(neurons_count);
        for (size_t i = 0; i < neurons_count; ++i)
        {
            auto n = generator(i);
            if (n.has_value()) neurons_.push_back(std::move(n.value()));
        }
    }
    [[nodiscard]] const UID &get_uid() const { return uid_; }
    [[nodiscard]] const std::vector<NeuronParameters> &get_neurons_parameters() const { return neurons_; }
    [[nodiscard]] const NeuronParameters &get_neuron_parameters(size_t index) const { return neurons_[index]; }
    void set_neuron_parameters(size_t index, const NeuronParameters &parameters) { neurons_[index] = parameters; }
    void set_neurons_parameters(const std::vector<NeuronParameters> &parameters) { neurons_ = parameters; }
    [[nodiscard]] size_t size() const { return neurons_.size(); }
    const NeuronParameters &operator[](size_t index) const { return neurons_[index]; }
    NeuronParameters &operator[](size_t index) { return neurons_[index]; }
    auto begin() const { return neurons_.cbegin(); }
    auto begin() { return neurons_.begin(); }
    auto end() const { return neurons_.cend(); }
    auto end() { return neurons_.end(); }

private:
    UID uid_;
    NeuronsContainer neurons_;
};

using AllPopulationsVariant = std::variant<
    Population<neuron_traits::BLIFATNeuron>, Population<neuron_traits::SynapticResourceSTDPBLIFATNeuron>,
    Population<neuron_traits::AltAILIF>, Population<neuron_traits::SynapticResourceSTDPAltAILIFNeuron>,
    Population<neuron_traits::LIFNeuron>>;
}  // namespace knp::core
