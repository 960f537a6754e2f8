// GB300Backend: knp::core::Backend over the GB300 C ABI (see knp_gb300_backend.h).
#include "knp_gb300_backend.h"

#include <algorithm>
#include <array>
#include <stdexcept>
#include <type_traits>
#include <utility>

#if __has_include(<boost/dll/alias.hpp>)
#include <boost/dll/alias.hpp>
#define KNP_GB300_EXPORT_FACTORY 1
#endif

namespace knp::backends::gb300
{
namespace
{
using knp::core::UID;
namespace nt = knp::neuron_traits;
namespace st = knp::synapse_traits;

knp_uid to_c(const UID &u)
{
    knp_uid r{};
    std::copy(u.tag.begin(), u.tag.end(), r.bytes);
    return r;
}

// A UID for one of the adapter's input channels, derived from an object's UID (`salt` tells the
// spike and impact channels apart).
UID derived_uid(const UID &u, uint8_t salt)
{
    std::array<uint8_t, 16> b{};
    std::copy(u.tag.begin(), u.tag.end(), b.begin());
    b[0] ^= 0x5Au;
    b[15] ^= salt;
    return UID(b);
}

template <class Variant, class T, size_t I = 0>
constexpr size_t variant_index()
{
    if constexpr (I == std::variant_size_v<Variant>)
        return I;
    else if constexpr (std::is_same_v<std::variant_alternative_t<I, Variant>, T>)
        return I;
    else
        return variant_index<Variant, T, I + 1>();
}

template <class Variant, class... Ts>
std::vector<size_t> indexes_in()
{
    std::vector<size_t> out;
    for (size_t i : {variant_index<Variant, Ts>()...})
        if (i < std::variant_size_v<Variant>) out.push_back(i);
    return out;
}

// ------------------------------------------------------------------ neuron parameters <-> C ABI
knp_blifat_neuron to_c(const nt::neuron_parameters<nt::BLIFATNeuron> &n)
{
    knp_blifat_neuron c{};
    c.n_time_steps_since_last_firing = n.n_time_steps_since_last_firing_;
    c.activation_threshold = n.activation_threshold_;
    c.additional_threshold = n.additional_threshold_;
    c.dynamic_threshold = n.dynamic_threshold_;
    c.threshold_decay = n.threshold_decay_;
    c.threshold_increment = n.threshold_increment_;
    c.postsynaptic_trace = n.postsynaptic_trace_;
    c.postsynaptic_trace_decay = n.postsynaptic_trace_decay_;
    c.postsynaptic_trace_increment = n.postsynaptic_trace_increment_;
    c.inhibitory_conductance = n.inhibitory_conductance_;
    c.inhibitory_conductance_decay = n.inhibitory_conductance_decay_;
    c.potential = n.potential_;
    c.pre_impact_potential = n.pre_impact_potential_;
    c.potential_decay = n.potential_decay_;
    c.bursting_phase = n.bursting_phase_;
    c.bursting_period = n.bursting_period_;
    c.reflexive_weight = n.reflexive_weight_;
    c.reversal_inhibitory_potential = n.reversal_inhibitory_potential_;
    c.absolute_refractory_period = n.absolute_refractory_period_;
    c.potential_reset_value = n.potential_reset_value_;
    c.min_potential = n.min_potential_;
    c.total_blocking_period = n.total_blocking_period_;
    c.dopamine_value = n.dopamine_value_;
    c.stochastic_stimulation = n.stochastic_stimulation_;
    c.random_number_generator_state = n.random_number_generator_state_;
    return c;
}

void from_c(const knp_blifat_neuron &c, nt::neuron_parameters<nt::BLIFATNeuron> &n)
{
    n.n_time_steps_since_last_firing_ = static_cast<size_t>(c.n_time_steps_since_last_firing);
    n.activation_threshold_ = c.activation_threshold;
    n.additional_threshold_ = c.additional_threshold;
    n.dynamic_threshold_ = c.dynamic_threshold;
    n.threshold_decay_ = c.threshold_decay;
    n.threshold_increment_ = c.threshold_increment;
    n.postsynaptic_trace_ = c.postsynaptic_trace;
    n.postsynaptic_trace_decay_ = c.postsynaptic_trace_decay;
    n.postsynaptic_trace_increment_ = c.postsynaptic_trace_increment;
    n.inhibitory_conductance_ = c.inhibitory_conductance;
    n.inhibitory_conductance_decay_ = c.inhibitory_conductance_decay;
    n.potential_ = c.potential;
    n.pre_impact_potential_ = c.pre_impact_potential;
    n.potential_decay_ = c.potential_decay;
    n.bursting_phase_ = c.bursting_phase;
    n.bursting_period_ = c.bursting_period;
    n.reflexive_weight_ = c.reflexive_weight;
    n.reversal_inhibitory_potential_ = c.reversal_inhibitory_potential;
    n.absolute_refractory_period_ = c.absolute_refractory_period;
    n.potential_reset_value_ = c.potential_reset_value;
    n.min_potential_ = c.min_potential;
    n.total_blocking_period_ = c.total_blocking_period;
    n.dopamine_value_ = c.dopamine_value;
    n.stochastic_stimulation_ = c.stochastic_stimulation;
    n.random_number_generator_state_ = c.random_number_generator_state;
}

// The resource-STDP extension of a neuron of either base type (stdp_synaptic_resource_rule.h:70-192).
template <class ResourceParams>
knp_resource_stdp_state resource_to_c(const ResourceParams &n)
{
    knp_resource_stdp_state c{};
    c.synapse_sum_threshold_coefficient = n.synapse_sum_threshold_coefficient_;
    c.dopamine_plasticity_time = n.dopamine_plasticity_time_;
    c.free_synaptic_resource = n.free_synaptic_resource_;
    c.synaptic_resource_threshold = n.synaptic_resource_threshold_;
    c.resource_drain_coefficient = n.resource_drain_coefficient_;
    c.stability = n.stability_;
    c.stability_change_parameter = n.stability_change_parameter_;
    c.stability_change_at_isi = n.stability_change_at_isi_;
    c.isi_max = n.isi_max_;
    c.d_h = n.d_h_;
    c.isi_status = static_cast<int32_t>(n.isi_status_);
    c.is_being_forced = n.is_being_forced_ ? 1u : 0u;
    c.last_step = n.last_step_;
    c.last_spike_step = n.last_spike_step_;
    c.first_isi_spike = n.first_isi_spike_;
    return c;
}

template <class ResourceParams>
void resource_from_c(const knp_resource_stdp_state &c, ResourceParams &n)
{
    n.synapse_sum_threshold_coefficient_ = c.synapse_sum_threshold_coefficient;
    n.dopamine_plasticity_time_ = c.dopamine_plasticity_time;
    n.free_synaptic_resource_ = c.free_synaptic_resource;
    n.synaptic_resource_threshold_ = c.synaptic_resource_threshold;
    n.resource_drain_coefficient_ = c.resource_drain_coefficient;
    n.stability_ = c.stability;
    n.stability_change_parameter_ = c.stability_change_parameter;
    n.stability_change_at_isi_ = c.stability_change_at_isi;
    n.isi_max_ = c.isi_max;
    n.d_h_ = c.d_h;
    n.isi_status_ = static_cast<nt::ISIPeriodType>(c.isi_status);
    n.is_being_forced_ = c.is_being_forced != 0u;
    n.last_step_ = c.last_step;
    n.last_spike_step_ = c.last_spike_step;
    n.first_isi_spike_ = c.first_isi_spike;
}

// The rule state of one SynapticResourceSTDPDeltaSynapse (stdp_synaptic_resource_rule.h:45-89).
template <class Rule>
knp_resource_synapse rule_to_c(const Rule &r)
{
    knp_resource_synapse c{};
    c.synaptic_resource = r.synaptic_resource_;
    c.w_min = r.w_min_;
    c.w_max = r.w_max_;
    c.d_u = r.d_u_;
    c.dopamine_plasticity_period = r.dopamine_plasticity_period_;
    c.had_hebbian_update = r.had_hebbian_update_ ? 1u : 0u;
    c.last_spike_step = r.last_spike_step_;
    c.has_contributed = r.has_contributed_ ? 1u : 0u;
    return c;
}

template <class Rule>
void rule_from_c(const knp_resource_synapse &c, Rule &r)
{
    r.synaptic_resource_ = c.synaptic_resource;
    r.w_min_ = c.w_min;
    r.w_max_ = c.w_max;
    r.d_u_ = c.d_u;
    r.dopamine_plasticity_period_ = c.dopamine_plasticity_period;
    r.had_hebbian_update_ = c.had_hebbian_update != 0u;
    r.last_spike_step_ = c.last_spike_step;
    r.has_contributed_ = c.has_contributed != 0u;
}

knp_altai_neuron altai_to_c(const nt::neuron_parameters<nt::AltAILIF> &n)
{
    knp_altai_neuron c{};
    c.is_diff = n.is_diff_ ? 1 : 0;
    c.is_reset = n.is_reset_ ? 1 : 0;
    c.leak_rev = n.leak_rev_ ? 1 : 0;
    c.saturate = n.saturate_ ? 1 : 0;
    c.do_not_save = n.do_not_save_ ? 1 : 0;
    c.potential = n.potential_;
    c.pre_impact_potential = n.pre_impact_potential_;
    c.activation_threshold = n.activation_threshold_;
    c.negative_activation_threshold = n.negative_activation_threshold_;
    c.potential_leak = n.potential_leak_;
    c.potential_reset_value = n.potential_reset_value_;
    c.dopamine_value = n.dopamine_value_;
    c.additional_threshold = n.additional_threshold_;
    c.activity_time = n.activity_time_;
    return c;
}

void altai_from_c(const knp_altai_neuron &c, nt::neuron_parameters<nt::AltAILIF> &n)
{
    n.is_diff_ = c.is_diff != 0;
    n.is_reset_ = c.is_reset != 0;
    n.leak_rev_ = c.leak_rev != 0;
    n.saturate_ = c.saturate != 0;
    n.do_not_save_ = c.do_not_save != 0;
    n.potential_ = c.potential;
    n.pre_impact_potential_ = c.pre_impact_potential;
    n.activation_threshold_ = c.activation_threshold;
    n.negative_activation_threshold_ = c.negative_activation_threshold;
    n.potential_leak_ = c.potential_leak;
    n.potential_reset_value_ = c.potential_reset_value;
    n.dopamine_value_ = c.dopamine_value;
    n.additional_threshold_ = c.additional_threshold;
    n.activity_time_ = c.activity_time;
}

knp_lif_neuron lif_to_c(const nt::neuron_parameters<nt::LIFNeuron> &n)
{
    knp_lif_neuron c{};
    c.potential = n.potential_;
    c.potential_reset_value = n.potential_reset_value_;
    c.activation_threshold = n.activation_threshold_;
    c.leak_coefficient = n.leak_coefficient_;
    c.refract_counter = n.refract_counter_;
    c.refract_period = n.refract_period_;
    return c;
}

void lif_from_c(const knp_lif_neuron &c, nt::neuron_parameters<nt::LIFNeuron> &n)
{
    n.potential_ = c.potential;
    n.potential_reset_value_ = c.potential_reset_value;
    n.activation_threshold_ = c.activation_threshold;
    n.leak_coefficient_ = c.leak_coefficient;
    n.refract_counter_ = c.refract_counter;
    n.refract_period_ = c.refract_period;
}

// A copy of a vector of variants, walked by get_network_data's ranges.
template <class Type>
class VectorIterator final : public knp::core::Backend::BaseValueIterator<Type>
{
public:
    VectorIterator(std::shared_ptr<const std::vector<Type>> data, size_t pos) : data_(std::move(data)), pos_(pos) {}
    Type operator*() const override { return (*data_)[pos_]; }
    VectorIterator &operator++() override
    {
        ++pos_;
        return *this;
    }
    bool operator==(const knp::core::Backend::BaseValueIterator<Type> &rhs) const override
    {
        const auto *o = dynamic_cast<const VectorIterator *>(&rhs);
        return o && o->data_ == data_ && o->pos_ == pos_;
    }

private:
    std::shared_ptr<const std::vector<Type>> data_;
    size_t pos_;
};

template <class Type>
auto make_range(std::vector<Type> &&v)
{
    auto data = std::make_shared<const std::vector<Type>>(std::move(v));
    using It = knp::core::Backend::BaseValueIterator<Type>;
    return std::make_pair(std::unique_ptr<It>(new VectorIterator<Type>(data, 0)),
                          std::unique_ptr<It>(new VectorIterator<Type>(data, data->size())));
}

}  // namespace

GB300Backend::GB300Backend(int device) : device_(device) {}

knp_gb300_backend *GB300Backend::handle()
{
    if (!h_) check(knp_gb300_create(device_, &h_), "knp_gb300_create");
    return h_;
}

GB300Backend::~GB300Backend()
{
    if (h_) knp_gb300_destroy(h_);
}

std::shared_ptr<GB300Backend> GB300Backend::create() { return std::make_shared<GB300Backend>(); }

void GB300Backend::check(int rc, const char *what) const
{
    if (rc != KNP_GB300_OK) throw std::runtime_error(std::string(what) + ": " + knp_gb300_last_error());
}

std::vector<std::string> GB300Backend::get_supported_neurons() const
{
    return {"BLIFATNeuron", "SynapticResourceSTDPBLIFATNeuron", "AltAILIF", "SynapticResourceSTDPAltAILIFNeuron",
            "LIFNeuron"};
}

std::vector<std::string> GB300Backend::get_supported_synapses() const
{
    return {"DeltaSynapse", "AdditiveSTDPDeltaSynapse", "SynapticResourceSTDPDeltaSynapse"};
}

std::vector<size_t> GB300Backend::get_supported_population_indexes() const
{
    return indexes_in<knp::core::AllPopulationsVariant, BLIFATPopulation, ResourceBLIFATPopulation, AltAIPopulation,
                      ResourceAltAIPopulation, LIFPopulation>();
}

std::vector<size_t> GB300Backend::get_supported_projection_indexes() const
{
    return indexes_in<knp::core::AllProjectionsVariant, DeltaProjection, AdditiveSTDPProjection, ResourceSTDPProjection>();
}

void GB300Backend::load_all_populations(const std::vector<knp::core::AllPopulationsVariant> &populations)
{
    std::vector<PopulationVariants> supported;
    for (const auto &v : populations)
        std::visit(
            [&supported](const auto &pop)
            {
                using T = std::decay_t<decltype(pop)>;
                if constexpr (variant_index<PopulationVariants, T>() < std::variant_size_v<PopulationVariants>)
                    supported.emplace_back(pop);
                else
                    throw std::runtime_error("Type is not supported.");
            },
            v);
    load_populations(supported);
}

void GB300Backend::load_all_projections(const std::vector<knp::core::AllProjectionsVariant> &projections)
{
    std::vector<ProjectionVariants> supported;
    for (const auto &v : projections)
        std::visit(
            [&supported](const auto &proj)
            {
                using T = std::decay_t<decltype(proj)>;
                if constexpr (variant_index<ProjectionVariants, T>() < std::variant_size_v<ProjectionVariants>)
                    supported.emplace_back(proj);
                else
                    throw std::runtime_error("Type is not supported.");
            },
            v);
    load_projections(supported);
}

void GB300Backend::load_populations(const std::vector<PopulationVariants> &populations)
{
    if (initialized_) throw std::logic_error("populations cannot be loaded after initialization");
    populations_ = populations;
}

void GB300Backend::load_projections(const std::vector<ProjectionVariants> &projections)
{
    if (initialized_) throw std::logic_error("projections cannot be loaded after initialization");
    projections_ = projections;
}

std::vector<std::unique_ptr<knp::core::Device>> GB300Backend::get_devices() const { return {}; }

void GB300Backend::stop_learning()
{
    check(knp_gb300_stop_learning(handle()), "knp_gb300_stop_learning");
    learning_known_ = true;
    learning_ = false;
}

void GB300Backend::start_learning()
{
    check(knp_gb300_start_learning(handle()), "knp_gb300_start_learning");
    learning_known_ = true;
    learning_ = true;
}

void GB300Backend::_init()
{
    (void)handle();
    for (const auto &v : populations_)
        std::visit(
            [this](const auto &pop)
            {
                using T = std::decay_t<decltype(pop)>;
                const knp_uid uid = to_c(pop.get_uid());
                const auto n = static_cast<uint32_t>(pop.size());
                if constexpr (std::is_same_v<T, LIFPopulation>)
                {
                    std::vector<knp_lif_neuron> c;
                    for (const auto &x : pop) c.push_back(lif_to_c(x));
                    check(knp_gb300_load_lif_population(h_, uid, n, c.data()), "knp_gb300_load_lif_population");
                }
                else if constexpr (std::is_same_v<T, AltAIPopulation> || std::is_same_v<T, ResourceAltAIPopulation>)
                {
                    std::vector<knp_altai_neuron> c;
                    std::vector<knp_resource_stdp_state> ext;
                    for (const auto &x : pop)
                    {
                        c.push_back(altai_to_c(static_cast<const nt::neuron_parameters<nt::AltAILIF> &>(x)));
                        if constexpr (std::is_same_v<T, ResourceAltAIPopulation>) ext.push_back(resource_to_c(x));
                    }
                    constexpr int kind = std::is_same_v<T, ResourceAltAIPopulation> ? KNP_NEURON_RESOURCE_STDP_ALTAI_LIF
                                                                                    : KNP_NEURON_ALTAI_LIF;
                    check(knp_gb300_load_altai_population(h_, uid, kind, n, c.data(), ext.empty() ? nullptr : ext.data()),
                          "knp_gb300_load_altai_population");
                }
                else
                {
                    std::vector<knp_blifat_neuron> c;
                    std::vector<knp_resource_stdp_state> ext;
                    for (const auto &x : pop)
                    {
                        c.push_back(to_c(static_cast<const nt::neuron_parameters<nt::BLIFATNeuron> &>(x)));
                        if constexpr (std::is_same_v<T, ResourceBLIFATPopulation>) ext.push_back(resource_to_c(x));
                    }
                    constexpr int kind = std::is_same_v<T, ResourceBLIFATPopulation> ? KNP_NEURON_RESOURCE_STDP_BLIFAT
                                                                                     : KNP_NEURON_BLIFAT;
                    check(knp_gb300_load_blifat_population(h_, uid, kind, n, c.data(), ext.empty() ? nullptr : ext.data()),
                          "knp_gb300_load_blifat_population");
                }
                // External SynapticImpactMessages to this population enter through its impact channel;
                // its SpikeMessages leave through the step's spike recording.
                const UID chan = derived_uid(pop.get_uid(), 0xC3u);
                impact_channel_.emplace(pop.get_uid(), chan);
                check(knp_gb300_subscribe(h_, uid, to_c(chan)), "knp_gb300_subscribe");
                check(knp_gb300_record_spikes(h_, uid, 1), "knp_gb300_record_spikes");
            },
            v);
    for (const auto &v : projections_)
        std::visit(
            [this](const auto &proj)
            {
                using T = std::decay_t<decltype(proj)>;
                const size_t n = proj.size();
                std::vector<uint32_t> pre(n), post(n), delay(n);
                std::vector<float> w(n), tp, tm;
                std::vector<uint8_t> type(n);
                std::vector<knp_resource_synapse> rule;
                for (size_t i = 0; i < n; ++i)
                {
                    const auto &s = proj[i];
                    const auto &p = std::get<knp::core::synapse_data>(s);
                    pre[i] = static_cast<uint32_t>(std::get<knp::core::source_neuron_id>(s));
                    post[i] = static_cast<uint32_t>(std::get<knp::core::target_neuron_id>(s));
                    w[i] = p.weight_;
                    delay[i] = p.delay_;
                    type[i] = static_cast<uint8_t>(p.output_type_);
                    if constexpr (std::is_same_v<T, AdditiveSTDPProjection>)
                    {
                        tp.push_back(p.rule_.tau_plus_);
                        tm.push_back(p.rule_.tau_minus_);
                    }
                    if constexpr (std::is_same_v<T, ResourceSTDPProjection>) rule.push_back(rule_to_c(p.rule_));
                }
                const knp_uid uid = to_c(proj.get_uid());
                if constexpr (std::is_same_v<T, ResourceSTDPProjection>)
                {
                    check(knp_gb300_load_resource_stdp_projection(h_, uid, to_c(proj.get_presynaptic()),
                                                                  to_c(proj.get_postsynaptic()), n, pre.data(), post.data(),
                                                                  w.data(), delay.data(), type.data(), rule.data(),
                                                                  proj.is_locked() ? 1 : 0),
                          "knp_gb300_load_resource_stdp_projection");
                }
                else
                {
                constexpr int kind =
                    std::is_same_v<T, AdditiveSTDPProjection> ? KNP_SYNAPSE_ADDITIVE_STDP_DELTA : KNP_SYNAPSE_DELTA;
                check(knp_gb300_load_projection(h_, uid, kind, to_c(proj.get_presynaptic()), to_c(proj.get_postsynaptic()), n,
                                                pre.data(), post.data(), w.data(), delay.data(), type.data(),
                                                tp.empty() ? nullptr : tp.data(), tm.empty() ? nullptr : tm.data()),
                      "knp_gb300_load_projection");
                }
                if constexpr (std::is_same_v<T, AdditiveSTDPProjection>)
                {
                    using Processing = typename T::SharedSynapseParameters::ProcessingType;
                    for (const auto &[pop, how] : proj.get_shared_parameters().stdp_populations_)
                        check(knp_gb300_set_stdp_population(h_, uid, to_c(pop),
                                                            how == Processing::STDPOnly ? KNP_STDP_ONLY : KNP_STDP_AND_SPIKE),
                              "knp_gb300_set_stdp_population");
                }
                // External SpikeMessages to this projection enter through its spike channel.
                const UID chan = derived_uid(proj.get_uid(), 0x3Cu);
                spike_channel_.emplace(proj.get_uid(), chan);
                check(knp_gb300_subscribe(h_, uid, to_c(chan)), "knp_gb300_subscribe");
            },
            v);
    check(knp_gb300_init(h_), "knp_gb300_init");
    initialized_ = true;
}

void GB300Backend::_step()
{
    using knp::core::messaging::SpikeMessage;
    using knp::core::messaging::SynapticImpactMessage;
    auto &endpoint = get_message_endpoint();
    get_message_bus().route_messages();
    endpoint.receive_all_messages();
    const knp::core::Step step = get_step();
    // Messages from outside this backend: SpikeMessages to its projections (spikes of its own
    // populations already reach them on the device), SynapticImpactMessages to its populations.
    for (const auto &v : projections_)
    {
        const UID uid = std::visit([](const auto &p) { return p.get_uid(); }, v);
        for (const auto &m : endpoint.unload_messages<SpikeMessage>(uid))
        {
            if (impact_channel_.count(m.header_.sender_uid_)) continue;
            check(knp_gb300_send_spikes(h_, to_c(spike_channel_.at(uid)), step,
                                        static_cast<uint32_t>(m.neuron_indexes_.size()), m.neuron_indexes_.data()),
                  "knp_gb300_send_spikes");
        }
    }
    for (const auto &v : populations_)
    {
        const UID uid = std::visit([](const auto &p) { return p.get_uid(); }, v);
        for (const auto &m : endpoint.unload_messages<SynapticImpactMessage>(uid))
        {
            std::vector<uint32_t> post;
            std::vector<float> value;
            std::vector<uint8_t> type;
            for (const auto &imp : m.impacts_)
            {
                post.push_back(imp.postsynaptic_neuron_index_);
                value.push_back(imp.impact_value_);
                type.push_back(static_cast<uint8_t>(imp.synapse_type_));
            }
            check(knp_gb300_send_impacts(h_, to_c(impact_channel_.at(uid)), to_c(uid), m.is_forcing_ ? 1 : 0,
                                         static_cast<uint32_t>(post.size()), post.data(), value.data(), type.data()),
                  "knp_gb300_send_impacts");
        }
    }
    check(knp_gb300_step(h_, 1), "knp_gb300_step");
    // Each population that spiked sends its SpikeMessage of this step (ascending indexes).
    for (const auto &v : populations_)
    {
        const auto [uid, n] = std::visit([](const auto &p) { return std::make_pair(p.get_uid(), p.size()); }, v);
        SpikeMessage msg{{uid, step}, {}};
        msg.neuron_indexes_.resize(std::max<size_t>(n, 1));
        uint32_t count = 0;
        check(knp_gb300_read_spikes(h_, to_c(uid), step, static_cast<uint32_t>(msg.neuron_indexes_.size()),
                                    msg.neuron_indexes_.data(), &count),
              "knp_gb300_read_spikes");
        msg.neuron_indexes_.resize(count);
        if (count) endpoint.send_message(msg);
    }
    check(knp_gb300_discard_spikes(h_, step + 1), "knp_gb300_discard_spikes");
    get_message_bus().route_messages();
    endpoint.receive_all_messages();
    gad_step();
}

knp::core::Backend::DataRanges GB300Backend::get_network_data() const
{
    std::vector<knp::core::AllPopulationsVariant> pops;
    for (const auto &v : populations_)
        std::visit(
            [this, &pops](const auto &pop)
            {
                using T = std::decay_t<decltype(pop)>;
                T copy = pop;
                if (initialized_)
                {
                    const knp_uid uid = to_c(pop.get_uid());
                    if constexpr (std::is_same_v<T, LIFPopulation>)
                    {
                        std::vector<knp_lif_neuron> c(pop.size());
                        check(knp_gb300_read_lif_population(h_, uid, c.data()), "knp_gb300_read_lif_population");
                        for (size_t i = 0; i < c.size(); ++i) lif_from_c(c[i], copy[i]);
                    }
                    else if constexpr (std::is_same_v<T, AltAIPopulation> || std::is_same_v<T, ResourceAltAIPopulation>)
                    {
                        std::vector<knp_altai_neuron> c(pop.size());
                        std::vector<knp_resource_stdp_state> ext(std::is_same_v<T, ResourceAltAIPopulation> ? pop.size() : 0);
                        check(knp_gb300_read_altai_population(h_, uid, c.data(), ext.empty() ? nullptr : ext.data()),
                              "knp_gb300_read_altai_population");
                        for (size_t i = 0; i < c.size(); ++i)
                        {
                            altai_from_c(c[i], static_cast<nt::neuron_parameters<nt::AltAILIF> &>(copy[i]));
                            if constexpr (std::is_same_v<T, ResourceAltAIPopulation>) resource_from_c(ext[i], copy[i]);
                        }
                    }
                    else
                    {
                        std::vector<knp_blifat_neuron> c(pop.size());
                        std::vector<knp_resource_stdp_state> ext(std::is_same_v<T, ResourceBLIFATPopulation> ? pop.size() : 0);
                        check(knp_gb300_read_blifat_population(h_, uid, c.data(), ext.empty() ? nullptr : ext.data()),
                              "knp_gb300_read_blifat_population");
                        for (size_t i = 0; i < c.size(); ++i)
                        {
                            from_c(c[i], static_cast<nt::neuron_parameters<nt::BLIFATNeuron> &>(copy[i]));
                            if constexpr (std::is_same_v<T, ResourceBLIFATPopulation>) resource_from_c(ext[i], copy[i]);
                        }
                    }
                }
                pops.emplace_back(std::move(copy));
            },
            v);
    std::vector<knp::core::AllProjectionsVariant> projs;
    for (const auto &v : projections_)
        std::visit(
            [this, &projs](const auto &proj)
            {
                using T = std::decay_t<decltype(proj)>;
                auto copy = proj;
                if (initialized_ && proj.size())
                {
                    std::vector<float> w(proj.size());
                    check(knp_gb300_read_weights(h_, to_c(proj.get_uid()), w.data()), "knp_gb300_read_weights");
                    for (size_t i = 0; i < w.size(); ++i) std::get<knp::core::synapse_data>(copy[i]).weight_ = w[i];
                    if constexpr (std::is_same_v<T, ResourceSTDPProjection>)
                    {
                        std::vector<knp_resource_synapse> r(proj.size());
                        check(knp_gb300_read_resource_synapses(h_, to_c(proj.get_uid()), r.data()),
                              "knp_gb300_read_resource_synapses");
                        for (size_t i = 0; i < r.size(); ++i) rule_from_c(r[i], std::get<knp::core::synapse_data>(copy[i]).rule_);
                    }
                }
                // start_learning / stop_learning lock or unlock every projection.
                if (learning_known_)
                {
                    if (learning_)
                        copy.unlock_weights();
                    else
                        copy.lock_weights();
                }
                projs.emplace_back(std::move(copy));
            },
            v);
    DataRanges r;
    r.projection_range = make_range(std::move(projs));
    r.population_range = make_range(std::move(pops));
    return r;
}

}  // namespace knp::backends::gb300

#ifdef KNP_GB300_EXPORT_FACTORY
BOOST_DLL_ALIAS(knp::backends::gb300::GB300Backend::create, create_knp_backend)
#endif
