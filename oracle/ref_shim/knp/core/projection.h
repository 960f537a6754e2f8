// TEST INFRASTRUCTURE — minimal stand-in for knp::core::Projection<Synapse>
// (knp/core-library/include/knp/core/projection.h:75-468): synapse tuples
// (parameters, source, target), the STDP shared parameters, and find_synapses() over a per-neuron
// index. Synapses of one neuron are returned in ascending synapse index.
#pragma once
#include <functional>
#include <tuple>
#include <unordered_map>
#include <vector>

#include <knp/core/messaging/messaging.h>
#include <knp/synapse-traits/stdp_type_traits.h>

namespace knp::core
{
enum SynapseElementAccess
{
    synapse_data = 0,
    source_neuron_id = 1,
    target_neuron_id = 2
};

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

template <class SynapseType>
class Projection
{
public:
    using ProjectionSynapseType = SynapseType;
    using SynapseParameters = synapse_traits::synapse_parameters<SynapseType>;
    using Synapse = std::tuple<SynapseParameters, size_t, size_t>;
    using SharedSynapseParameters = SharedSynapseParametersT<SynapseType>;
    enum class Search
    {
        by_postsynaptic,
        by_presynaptic
    };

    Projection() = default;
    Projection(UID uid, UID pre, UID post, std::vector<Synapse> syn)
        : uid_(uid), pre_(pre), post_(post), syn_(std::move(syn))
    {
        for (size_t i = 0; i < syn_.size(); ++i)
        {
            const size_t s = std::get<source_neuron_id>(syn_[i]);
            const size_t t = std::get<target_neuron_id>(syn_[i]);
            if (by_pre_.size() <= s) by_pre_.resize(s + 1);
            if (by_post_.size() <= t) by_post_.resize(t + 1);
            by_pre_[s].push_back(i);
            by_post_[t].push_back(i);
        }
    }
    const UID &get_uid() const { return uid_; }
    const UID &get_presynaptic() const { return pre_; }
    const UID &get_postsynaptic() const { return post_; }
    size_t size() const { return syn_.size(); }
    Synapse &operator[](size_t i) { return syn_[i]; }
    const Synapse &operator[](size_t i) const { return syn_[i]; }
    auto begin() { return syn_.begin(); }
    auto end() { return syn_.end(); }
    bool is_locked() const { return locked_; }
    void lock_weights() { locked_ = true; }
    void unlock_weights() { locked_ = false; }
    SharedSynapseParameters &get_shared_parameters() { return shared_; }
    const SharedSynapseParameters &get_shared_parameters() const { return shared_; }

    std::vector<size_t> find_synapses(size_t neuron_id, Search search) const
    {
        const auto &idx = search == Search::by_presynaptic ? by_pre_ : by_post_;
        return neuron_id < idx.size() ? idx[neuron_id] : std::vector<size_t>{};
    }

private:
    UID uid_, pre_, post_;
    std::vector<Synapse> syn_;
    std::vector<std::vector<size_t>> by_pre_, by_post_;
    SharedSynapseParameters shared_;
    bool locked_ = true;
};
}  // namespace knp::core
