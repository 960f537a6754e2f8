// TEST INFRASTRUCTURE — stand-in for knp::core::Projection (knp/core-library/include/knp/core/
// projection.h): synapse tuples (parameters, source, target) in index order, the STDP shared
// parameters, the weight lock; AllProjectionsVariant over the synapse types the adapter handles.
#pragma once
#include <functional>
#include <optional>
#include <tuple>
#include <unordered_map>
#include <variant>
#include <vector>

#include <knp/core/core.h>
#include <knp/synapse-traits/delta.h>
#include <knp/synapse-traits/stdp_type_traits.h>

namespace knp::core
{
enum SynapseElementAccess
{
    synapse_data = 0,
    source_neuron_id = 1,
    target_neuron_id = 2
};

template <class SynapseType>
class Projection final
{
public:
    using ProjectionSynapseType = SynapseType;
    using SynapseParameters = typename synapse_traits::synapse_parameters<SynapseType>;
    using Synapse = std::tuple<SynapseParameters, size_t, size_t>;
    using SynapseGenerator = std::function<std::optional<Synapse>(size_t)>;
    using SynapsesContainer = std::vector<Synapse>;

    template <class SynapseT>
    struct SharedSynapseParametersT
    {
    };
    template <template <typename> typename Rule, typename SynapseT>
    struct SharedSynapseParametersT<knp::synapse_traits::STDP<Rule, SynapseT>>
    {
        enum class ProcessingType
        {
            STDPOnly,
            STDPAndSpike
        };
        using ContainerType = std::unordered_map<core::UID, ProcessingType, core::uid_hash>;
        ContainerType stdp_populations_;
    };
    using SharedSynapseParameters = SharedSynapseParametersT<SynapseType>;

    Projection(UID presynaptic_uid, UID postsynaptic_uid, SynapseGenerator generator, size_t num_iterations)
        : Projection(UID(), presynaptic_uid, postsynaptic_uid, generator, num_iterations)
    {
    }
    Projection(UID uid, UID presynaptic_uid, UID postsynaptic_uid, SynapseGenerator generator, size_t num_iterations)
        : uid_(uid), presynaptic_uid_(presynaptic_uid), postsynaptic_uid_(postsynaptic_uid)
    {
        for (size_t i = 0; i < num_iterations; ++i)
        {
            auto s = generator(i);
            if (s.has_value()) parameters_.push_back(std::move(s.value()));
        }
    }
    [[nodiscard]] const UID &get_uid() const { return uid_; }
    [[nodiscard]] Synapse &operator[](size_t index) { return parameters_[index]; }
    [[nodiscard]] const Synapse &operator[](size_t index) const { return parameters_[index]; }
    [[nodiscard]] auto begin() const { return parameters_.cbegin(); }
    [[nodiscard]] auto begin() { return parameters_.begin(); }
    [[nodiscard]] auto end() const { return parameters_.cend(); }
    [[nodiscard]] auto end() { return parameters_.end(); }
    [[nodiscard]] size_t size() const { return parameters_.size(); }
    [[nodiscard]] const UID &get_presynaptic() const { return presynaptic_uid_; }
    [[nodiscard]] const UID &get_postsynaptic() const { return postsynaptic_uid_; }
    void lock_weights() { is_locked_ = true; }
    void unlock_weights() { is_locked_ = false; }
    bool is_locked() const { return is_locked_; }
    SharedSynapseParameters &get_shared_parameters() { return shared_parameters_; }
    const SharedSynapseParameters &get_shared_parameters() const { return shared_parameters_; }

private:
    UID uid_, presynaptic_uid_, postsynaptic_uid_;
    SynapsesContainer parameters_;
    SharedSynapseParameters shared_parameters_;
    bool is_locked_ = true;
};

using AllProjectionsVariant = std::variant<
    Projection<synapse_traits::DeltaSynapse>, Projection<synapse_traits::AdditiveSTDPDeltaSynapse>,
    Projection<synapse_traits::SynapticResourceSTDPDeltaSynapse>>;
}  // namespace knp::core
