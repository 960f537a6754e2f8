// TEST INFRASTRUCTURE — the KNP reference's own hot-path arithmetic, driven by a restated step loop.
//
// Built only where the KNP sources are present (oracle/Makefile target `ref`), into
// oracle/_ref/libknp_ref.so, and used by tests to pin the restated oracle (knp_oracle.cpp) and to
// write golden fixtures. It includes, unmodified, from the reference tree:
//   cpu-library/impl/populations/blifat/blifat_impl.h (+ blifat_stdp.h, training/stdp.h)
//   cpu-library/impl/populations/lif/lif_impl.h
//   cpu-library/impl/populations/altai/altai_impl.h (+ altai_stdp.h)
//   cpu-library/impl/projections/delta/delta_impl.h (+ additive_stdp.h, synaptic_resource_stdp.h)
// with the neuron/synapse trait headers, against the small shim in oracle/ref_shim/. Message routing
// follows knp/backends/cpu/cpu-single-threaded-backend/impl/backend.cpp:89-141 exactly as in
// knp_oracle.cpp; everything that touches a neuron or a synapse is the reference's code.
#include <knp/backends/cpu-library/impl/populations/altai/altai_impl.h>
#include <knp/backends/cpu-library/impl/populations/blifat/blifat_impl.h>
#include <knp/backends/cpu-library/impl/populations/lif/lif_impl.h>
#include <knp/backends/cpu-library/impl/projections/delta/delta_impl.h>

#include <cstring>
#include <memory>
#include <string>
#include <unordered_set>
#include <variant>
#include <vector>

#include "knp_oracle.h"

namespace nt = knp::neuron_traits;
namespace st = knp::synapse_traits;
namespace kc = knp::core;
namespace msg = knp::core::messaging;

using BlifatParams = nt::neuron_parameters<nt::BLIFATNeuron>;
using ResBlifatParams = nt::neuron_parameters<nt::SynapticResourceSTDPBLIFATNeuron>;
using LifParams = nt::neuron_parameters<nt::LIFNeuron>;
using DeltaProj = kc::Projection<st::DeltaSynapse>;
using AddStdpProj = kc::Projection<st::AdditiveSTDPDeltaSynapse>;
using ResStdpProj = kc::Projection<st::SynapticResourceSTDPDeltaSynapse>;
using AltaiParams = nt::neuron_parameters<nt::AltAILIF>;
using ResAltaiParams = nt::neuron_parameters<nt::SynapticResourceSTDPAltAILIFNeuron>;

namespace
{
thread_local std::string g_error;

int fail(const std::string &m)
{
    g_error = m;
    return -1;
}

kc::UID to_uid(const knp_uid &u)
{
    kc::UID r;
    std::memcpy(r.tag.data(), u.bytes, 16);
    return r;
}

BlifatParams to_ref(const knp_blifat_neuron &a)
{
    BlifatParams b;
    b.n_time_steps_since_last_firing_ = a.n_time_steps_since_last_firing;
    b.activation_threshold_ = a.activation_threshold;
    b.additional_threshold_ = a.additional_threshold;
    b.dynamic_threshold_ = a.dynamic_threshold;
    b.threshold_decay_ = a.threshold_decay;
    b.threshold_increment_ = a.threshold_increment;
    b.postsynaptic_trace_ = a.postsynaptic_trace;
    b.postsynaptic_trace_decay_ = a.postsynaptic_trace_decay;
    b.postsynaptic_trace_increment_ = a.postsynaptic_trace_increment;
    b.inhibitory_conductance_ = a.inhibitory_conductance;
    b.inhibitory_conductance_decay_ = a.inhibitory_conductance_decay;
    b.potential_ = a.potential;
    b.pre_impact_potential_ = a.pre_impact_potential;
    b.potential_decay_ = a.potential_decay;
    b.bursting_phase_ = a.bursting_phase;
    b.bursting_period_ = a.bursting_period;
    b.reflexive_weight_ = a.reflexive_weight;
    b.reversal_inhibitory_potential_ = a.reversal_inhibitory_potential;
    b.absolute_refractory_period_ = a.absolute_refractory_period;
    b.potential_reset_value_ = a.potential_reset_value;
    b.min_potential_ = a.min_potential;
    b.total_blocking_period_ = a.total_blocking_period;
    b.dopamine_value_ = a.dopamine_value;
    b.stochastic_stimulation_ = a.stochastic_stimulation;
    b.random_number_generator_state_ = a.random_number_generator_state;
    return b;
}

knp_blifat_neuron from_ref(const BlifatParams &b)
{
    knp_blifat_neuron a{};
    a.n_time_steps_since_last_firing = b.n_time_steps_since_last_firing_;
    a.activation_threshold = b.activation_threshold_;
    a.additional_threshold = b.additional_threshold_;
    a.dynamic_threshold = b.dynamic_threshold_;
    a.threshold_decay = b.threshold_decay_;
    a.threshold_increment = b.threshold_increment_;
    a.postsynaptic_trace = b.postsynaptic_trace_;
    a.postsynaptic_trace_decay = b.postsynaptic_trace_decay_;
    a.postsynaptic_trace_increment = b.postsynaptic_trace_increment_;
    a.inhibitory_conductance = b.inhibitory_conductance_;
    a.inhibitory_conductance_decay = b.inhibitory_conductance_decay_;
    a.potential = b.potential_;
    a.pre_impact_potential = b.pre_impact_potential_;
    a.potential_decay = b.potential_decay_;
    a.bursting_phase = b.bursting_phase_;
    a.bursting_period = b.bursting_period_;
    a.reflexive_weight = b.reflexive_weight_;
    a.reversal_inhibitory_potential = b.reversal_inhibitory_potential_;
    a.absolute_refractory_period = b.absolute_refractory_period_;
    a.potential_reset_value = b.potential_reset_value_;
    a.min_potential = b.min_potential_;
    a.total_blocking_period = b.total_blocking_period_;
    a.dopamine_value = b.dopamine_value_;
    a.stochastic_stimulation = b.stochastic_stimulation_;
    a.random_number_generator_state = b.random_number_generator_state_;
    return a;
}

ResBlifatParams to_ref(const knp_blifat_neuron &a, const knp_resource_stdp_state &r)
{
    ResBlifatParams b{to_ref(a)};
    b.synapse_sum_threshold_coefficient_ = r.synapse_sum_threshold_coefficient;
    b.dopamine_plasticity_time_ = r.dopamine_plasticity_time;
    b.free_synaptic_resource_ = r.free_synaptic_resource;
    b.synaptic_resource_threshold_ = r.synaptic_resource_threshold;
    b.resource_drain_coefficient_ = r.resource_drain_coefficient;
    b.stability_ = r.stability;
    b.stability_change_parameter_ = r.stability_change_parameter;
    b.stability_change_at_isi_ = r.stability_change_at_isi;
    b.isi_max_ = r.isi_max;
    b.d_h_ = r.d_h;
    b.isi_status_ = static_cast<nt::ISIPeriodType>(r.isi_status);
    b.last_step_ = r.last_step;
    b.last_spike_step_ = r.last_spike_step;
    b.first_isi_spike_ = r.first_isi_spike;
    b.is_being_forced_ = r.is_being_forced != 0;
    return b;
}

template <class P>
knp_resource_stdp_state res_from_ref(const P &b)
{
    knp_resource_stdp_state r{};
    r.synapse_sum_threshold_coefficient = b.synapse_sum_threshold_coefficient_;
    r.dopamine_plasticity_time = b.dopamine_plasticity_time_;
    r.free_synaptic_resource = b.free_synaptic_resource_;
    r.synaptic_resource_threshold = b.synaptic_resource_threshold_;
    r.resource_drain_coefficient = b.resource_drain_coefficient_;
    r.stability = b.stability_;
    r.stability_change_parameter = b.stability_change_parameter_;
    r.stability_change_at_isi = b.stability_change_at_isi_;
    r.isi_max = b.isi_max_;
    r.d_h = b.d_h_;
    r.isi_status = static_cast<int32_t>(b.isi_status_);
    r.last_step = b.last_step_;
    r.last_spike_step = b.last_spike_step_;
    r.first_isi_spike = b.first_isi_spike_;
    r.is_being_forced = b.is_being_forced_ ? 1u : 0u;
    return r;
}

AltaiParams to_ref(const knp_altai_neuron &a)
{
    AltaiParams b;
    b.is_diff_ = a.is_diff != 0;
    b.is_reset_ = a.is_reset != 0;
    b.leak_rev_ = a.leak_rev != 0;
    b.saturate_ = a.saturate != 0;
    b.do_not_save_ = a.do_not_save != 0;
    b.potential_ = a.potential;
    b.pre_impact_potential_ = a.pre_impact_potential;
    b.activation_threshold_ = a.activation_threshold;
    b.negative_activation_threshold_ = a.negative_activation_threshold;
    b.potential_leak_ = a.potential_leak;
    b.potential_reset_value_ = a.potential_reset_value;
    b.dopamine_value_ = a.dopamine_value;
    b.additional_threshold_ = a.additional_threshold;
    b.activity_time_ = a.activity_time;
    return b;
}

knp_altai_neuron from_ref(const AltaiParams &b)
{
    knp_altai_neuron a{};
    a.is_diff = b.is_diff_ ? 1 : 0;
    a.is_reset = b.is_reset_ ? 1 : 0;
    a.leak_rev = b.leak_rev_ ? 1 : 0;
    a.saturate = b.saturate_ ? 1 : 0;
    a.do_not_save = b.do_not_save_ ? 1 : 0;
    a.potential = b.potential_;
    a.pre_impact_potential = b.pre_impact_potential_;
    a.activation_threshold = b.activation_threshold_;
    a.negative_activation_threshold = b.negative_activation_threshold_;
    a.potential_leak = b.potential_leak_;
    a.potential_reset_value = b.potential_reset_value_;
    a.dopamine_value = b.dopamine_value_;
    a.additional_threshold = b.additional_threshold_;
    a.activity_time = b.activity_time_;
    return a;
}

// The resource-STDP extension of a neuron of either base type.
template <class P>
void res_to_ref(P &b, const knp_resource_stdp_state &r)
{
    b.synapse_sum_threshold_coefficient_ = r.synapse_sum_threshold_coefficient;
    b.dopamine_plasticity_time_ = r.dopamine_plasticity_time;
    b.free_synaptic_resource_ = r.free_synaptic_resource;
    b.synaptic_resource_threshold_ = r.synaptic_resource_threshold;
    b.resource_drain_coefficient_ = r.resource_drain_coefficient;
    b.stability_ = r.stability;
    b.stability_change_parameter_ = r.stability_change_parameter;
    b.stability_change_at_isi_ = r.stability_change_at_isi;
    b.isi_max_ = r.isi_max;
    b.d_h_ = r.d_h;
    b.isi_status_ = static_cast<nt::ISIPeriodType>(r.isi_status);
    b.last_step_ = r.last_step;
    b.last_spike_step_ = r.last_spike_step;
    b.first_isi_spike_ = r.first_isi_spike;
    b.is_being_forced_ = r.is_being_forced != 0;
}

struct Pop
{
    kc::UID uid;
    int kind;
    std::variant<kc::Population<nt::BLIFATNeuron>, kc::Population<nt::SynapticResourceSTDPBLIFATNeuron>,
                 kc::Population<nt::LIFNeuron>, kc::Population<nt::AltAILIF>,
                 kc::Population<nt::SynapticResourceSTDPAltAILIFNeuron>>
        pop;
    std::unordered_set<kc::UID, kc::uid_hash> impact_senders;
    std::vector<msg::SynapticImpactMessage> inbox;
    std::vector<uint32_t> last_spikes;
};

struct Proj
{
    kc::UID uid;
    std::variant<DeltaProj, AddStdpProj, ResStdpProj> proj;
    std::unordered_set<kc::UID, kc::uid_hash> spike_senders;
    std::vector<msg::SpikeMessage> inbox;
    knp::backends::cpu::projections::MessageQueue future;
};

}  // namespace

struct or_net
{
    std::vector<std::unique_ptr<Pop>> pops;
    std::vector<std::unique_ptr<Proj>> projs;
    std::vector<std::pair<kc::UID, kc::UID>> extra_subs;
    std::vector<msg::SpikeMessage> ext_spikes;
    std::vector<msg::SynapticImpactMessage> ext_impacts;
    uint64_t step = 0;
    uint64_t events = 0;
    bool initialized = false;

    Pop *find_pop(const kc::UID &u) const
    {
        for (auto &p : pops)
            if (p->uid == u) return p.get();
        return nullptr;
    }
    Proj *find_proj(const kc::UID &u) const
    {
        for (auto &p : projs)
            if (p->uid == u) return p.get();
        return nullptr;
    }
};

namespace
{
namespace bl = knp::backends::cpu::populations::impl::blifat;
namespace li = knp::backends::cpu::populations::impl::lif;
namespace al = knp::backends::cpu::populations::impl::altai;
namespace de = knp::backends::cpu::projections::impl::delta;

template <class PopT, class Pre, class Imp, class Post>
void run_population(Pop &p, PopT &pop, Pre pre, Imp imp, Post post)
{
    auto msgs = std::move(p.inbox);
    p.inbox.clear();
    for (auto &m : msgs)
        for (auto &i : m.impacts_)
            if (i.postsynaptic_neuron_index_ >= pop.size())
                throw std::runtime_error("Impact postsynaptic index out of range.");
    // populations::calculate_{pre,post}_impact_population_state / impact_population (populations.h:53-116).
    for (size_t i = 0; i < pop.size(); ++i) pre(pop[i]);
    for (auto &m : msgs)
        for (auto &i : m.impacts_) imp(pop[i.postsynaptic_neuron_index_], i, m.is_forcing_);
    p.last_spikes.clear();
    for (size_t i = 0; i < pop.size(); ++i)
        if (post(pop[i])) p.last_spikes.push_back(static_cast<uint32_t>(i));
}

// populations_old.h:57-83, 207-209: the unlocked SynapticResourceSTDPDeltaSynapse projections into
// population `uid`, in projection order.
std::vector<std::reference_wrapper<ResStdpProj>> working_projections(or_net &net, const kc::UID &uid)
{
    std::vector<std::reference_wrapper<ResStdpProj>> working;
    for (auto &q : net.projs)
        if (auto *rp = std::get_if<ResStdpProj>(&q->proj))
            if (rp->get_postsynaptic() == uid && !rp->is_locked()) working.emplace_back(*rp);
    return working;
}

void step_population(or_net &net, Pop &p, uint64_t step)
{
    if (auto *b = std::get_if<kc::Population<nt::BLIFATNeuron>>(&p.pop))
    {
        run_population(
            p, *b, [](BlifatParams &n) { bl::calculate_pre_impact_single_neuron_state_impl(n); },
            [](BlifatParams &n, const msg::SynapticImpact &i, bool f) { bl::impact_neuron_impl(n, i, f); },
            [](BlifatParams &n) { return bl::calculate_post_impact_single_neuron_state_impl(n); });
    }
    else if (auto *r = std::get_if<kc::Population<nt::SynapticResourceSTDPBLIFATNeuron>>(&p.pop))
    {
        run_population(
            p, *r, [](ResBlifatParams &n) { bl::calculate_pre_impact_single_neuron_state_impl(n); },
            [](ResBlifatParams &n, const msg::SynapticImpact &i, bool f) { bl::impact_neuron_impl(n, i, f); },
            [](ResBlifatParams &n) { return bl::calculate_post_impact_single_neuron_state_impl(n); });
        auto working = working_projections(net, p.uid);
        msg::SpikeMessage out{{p.uid, step}, {p.last_spikes.begin(), p.last_spikes.end()}};
        bl::train_population_impl(*r, working, out, step);
    }
    else if (auto *a = std::get_if<kc::Population<nt::AltAILIF>>(&p.pop))
    {
        run_population(
            p, *a, [](AltaiParams &n) { al::calculate_pre_impact_single_neuron_state_impl(n); },
            [](AltaiParams &n, const msg::SynapticImpact &i, bool f) { al::impact_neuron_impl(n, i, f); },
            [](AltaiParams &n) { return al::calculate_post_impact_single_neuron_state_impl(n); });
    }
    else if (auto *ra = std::get_if<kc::Population<nt::SynapticResourceSTDPAltAILIFNeuron>>(&p.pop))
    {
        run_population(
            p, *ra, [](ResAltaiParams &n) { al::calculate_pre_impact_single_neuron_state_impl(n); },
            [](ResAltaiParams &n, const msg::SynapticImpact &i, bool f) { al::impact_neuron_impl(n, i, f); },
            [](ResAltaiParams &n) { return al::calculate_post_impact_single_neuron_state_impl(n); });
        auto working = working_projections(net, p.uid);
        msg::SpikeMessage out{{p.uid, step}, {p.last_spikes.begin(), p.last_spikes.end()}};
        al::train_population_impl(*ra, working, out, step);
    }
    else
    {
        auto &l = std::get<kc::Population<nt::LIFNeuron>>(p.pop);
        run_population(
            p, l, [](LifParams &n) { li::calculate_pre_impact_single_neuron_state_impl(n); },
            [](LifParams &n, const msg::SynapticImpact &i, bool f) { li::impact_neuron_impl(n, i, f); },
            [](LifParams &n) { return li::calculate_post_impact_single_neuron_state_impl(n); });
    }
}

template <class ProjT>
bool step_projection(or_net &net, Proj &p, ProjT &proj, uint64_t step, msg::SynapticImpactMessage &out)
{
    auto msgs = std::move(p.inbox);
    p.inbox.clear();
    // Events = impacts the reference appended to the future queue during this call.
    const size_t before = [&]
    {
        size_t n = 0;
        for (auto &[k, v] : p.future) n += v.impacts_.size();
        return n;
    }();
    auto it = de::calculate_projection_impl(proj, msgs, p.future, step);  // projections.h:58-84
    size_t after = 0;
    for (auto &[k, v] : p.future) after += v.impacts_.size();
    net.events += after - before;
    if (it == p.future.end()) return false;
    out = std::move(it->second);
    p.future.erase(it);
    return true;
}

template <class F>
int guarded(F &&f)
{
    try
    {
        return f();
    }
    catch (const std::exception &e)
    {
        return fail(e.what());
    }
}

}  // namespace

extern "C" {

const char *or_last_error(void) { return g_error.c_str(); }
or_net *or_create(void) { return new or_net(); }
void or_destroy(or_net *net) { delete net; }

int or_add_blifat_population(
    or_net *net, knp_uid uid, int kind, uint32_t n, const knp_blifat_neuron *neurons,
    const knp_resource_stdp_state *ext)
{
    auto p = std::make_unique<Pop>();
    p->uid = to_uid(uid);
    p->kind = kind;
    if (kind == KNP_NEURON_BLIFAT)
    {
        std::vector<BlifatParams> v;
        for (uint32_t i = 0; i < n; ++i) v.push_back(to_ref(neurons[i]));
        p->pop = kc::Population<nt::BLIFATNeuron>(p->uid, std::move(v));
    }
    else if (kind == KNP_NEURON_RESOURCE_STDP_BLIFAT && ext)
    {
        std::vector<ResBlifatParams> v;
        for (uint32_t i = 0; i < n; ++i) v.push_back(to_ref(neurons[i], ext[i]));
        p->pop = kc::Population<nt::SynapticResourceSTDPBLIFATNeuron>(p->uid, std::move(v));
    }
    else
        return fail("bad neuron kind");
    net->pops.push_back(std::move(p));
    return 0;
}

int or_add_lif_population(or_net *net, knp_uid uid, uint32_t n, const knp_lif_neuron *neurons)
{
    auto p = std::make_unique<Pop>();
    p->uid = to_uid(uid);
    p->kind = KNP_NEURON_LIF;
    std::vector<LifParams> v;
    for (uint32_t i = 0; i < n; ++i)
    {
        LifParams l;
        l.potential_ = neurons[i].potential;
        l.potential_reset_value_ = neurons[i].potential_reset_value;
        l.activation_threshold_ = neurons[i].activation_threshold;
        l.leak_coefficient_ = neurons[i].leak_coefficient;
        l.refract_counter_ = neurons[i].refract_counter;
        l.refract_period_ = neurons[i].refract_period;
        v.push_back(l);
    }
    p->pop = kc::Population<nt::LIFNeuron>(p->uid, std::move(v));
    net->pops.push_back(std::move(p));
    return 0;
}

int or_add_projection(
    or_net *net, knp_uid uid, int kind, knp_uid pre_uid, knp_uid post_uid, uint64_t n_syn,
    const uint32_t *pre_idx, const uint32_t *post_idx, const float *weight, const uint32_t *delay,
    const uint8_t *out_type, const float *tau_plus, const float *tau_minus)
{
    auto p = std::make_unique<Proj>();
    p->uid = to_uid(uid);
    if (kind == KNP_SYNAPSE_DELTA)
    {
        std::vector<DeltaProj::Synapse> v;
        for (uint64_t i = 0; i < n_syn; ++i)
        {
            st::synapse_parameters<st::DeltaSynapse> s;
            s.weight_ = weight[i];
            s.delay_ = delay[i];
            s.output_type_ = static_cast<st::OutputType>(out_type ? out_type[i] : 0);
            v.emplace_back(s, pre_idx[i], post_idx[i]);
        }
        p->proj = DeltaProj(p->uid, to_uid(pre_uid), to_uid(post_uid), std::move(v));
    }
    else if (kind == KNP_SYNAPSE_ADDITIVE_STDP_DELTA)
    {
        std::vector<AddStdpProj::Synapse> v;
        for (uint64_t i = 0; i < n_syn; ++i)
        {
            st::synapse_parameters<st::AdditiveSTDPDeltaSynapse> s;
            s.weight_ = weight[i];
            s.delay_ = delay[i];
            s.output_type_ = static_cast<st::OutputType>(out_type ? out_type[i] : 0);
            if (tau_plus) s.rule_.tau_plus_ = tau_plus[i];
            if (tau_minus) s.rule_.tau_minus_ = tau_minus[i];
            v.emplace_back(s, pre_idx[i], post_idx[i]);
        }
        p->proj = AddStdpProj(p->uid, to_uid(pre_uid), to_uid(post_uid), std::move(v));
    }
    else
        return fail("bad synapse kind");
    net->projs.push_back(std::move(p));
    return 0;
}

int or_add_resource_projection(
    or_net *net, knp_uid uid, knp_uid pre_uid, knp_uid post_uid, uint64_t n_syn, const uint32_t *pre_idx,
    const uint32_t *post_idx, const float *weight, const uint32_t *delay, const uint8_t *out_type,
    const knp_resource_synapse *rule, int locked)
{
    if (n_syn && !rule) return fail("resource-STDP synapses need their rule state");
    auto p = std::make_unique<Proj>();
    p->uid = to_uid(uid);
    std::vector<ResStdpProj::Synapse> v;
    for (uint64_t i = 0; i < n_syn; ++i)
    {
        st::synapse_parameters<st::SynapticResourceSTDPDeltaSynapse> s;
        s.weight_ = weight[i];
        s.delay_ = delay[i];
        s.output_type_ = static_cast<st::OutputType>(out_type ? out_type[i] : 0);
        s.rule_.synaptic_resource_ = rule[i].synaptic_resource;
        s.rule_.w_min_ = rule[i].w_min;
        s.rule_.w_max_ = rule[i].w_max;
        s.rule_.d_u_ = rule[i].d_u;
        s.rule_.dopamine_plasticity_period_ = rule[i].dopamine_plasticity_period;
        s.rule_.last_spike_step_ = rule[i].last_spike_step;
        s.rule_.had_hebbian_update_ = rule[i].had_hebbian_update != 0;
        s.rule_.has_contributed_ = rule[i].has_contributed != 0;
        v.emplace_back(s, pre_idx[i], post_idx[i]);
    }
    ResStdpProj proj(p->uid, to_uid(pre_uid), to_uid(post_uid), std::move(v));
    if (locked)
        proj.lock_weights();
    else
        proj.unlock_weights();
    p->proj = std::move(proj);
    net->projs.push_back(std::move(p));
    return 0;
}

int or_set_learning(or_net *net, int on)
{
    for (auto &p : net->projs)
        std::visit([on](auto &proj) { on ? proj.unlock_weights() : proj.lock_weights(); }, p->proj);
    return 0;
}

int or_read_resource_synapses(const or_net *net, knp_uid proj, knp_resource_synapse *out)
{
    const Proj *p = net->find_proj(to_uid(proj));
    const auto *r = p ? std::get_if<ResStdpProj>(&p->proj) : nullptr;
    if (!r) return fail("unknown resource-STDP projection");
    for (size_t i = 0; i < r->size(); ++i)
    {
        const auto &rule = std::get<kc::synapse_data>((*r)[i]).rule_;
        knp_resource_synapse s{};
        s.synaptic_resource = rule.synaptic_resource_;
        s.w_min = rule.w_min_;
        s.w_max = rule.w_max_;
        s.d_u = rule.d_u_;
        s.dopamine_plasticity_period = rule.dopamine_plasticity_period_;
        s.had_hebbian_update = rule.had_hebbian_update_ ? 1u : 0u;
        s.last_spike_step = rule.last_spike_step_;
        s.has_contributed = rule.has_contributed_ ? 1u : 0u;
        out[i] = s;
    }
    return 0;
}

int or_add_altai_population(
    or_net *net, knp_uid uid, int kind, uint32_t n, const knp_altai_neuron *neurons, const knp_resource_stdp_state *ext)
{
    auto p = std::make_unique<Pop>();
    p->uid = to_uid(uid);
    p->kind = kind;
    if (kind == KNP_NEURON_ALTAI_LIF)
    {
        std::vector<AltaiParams> v;
        for (uint32_t i = 0; i < n; ++i) v.push_back(to_ref(neurons[i]));
        p->pop = kc::Population<nt::AltAILIF>(p->uid, std::move(v));
    }
    else if (kind == KNP_NEURON_RESOURCE_STDP_ALTAI_LIF && ext)
    {
        std::vector<ResAltaiParams> v;
        for (uint32_t i = 0; i < n; ++i)
        {
            ResAltaiParams b{to_ref(neurons[i])};
            res_to_ref(b, ext[i]);
            v.push_back(b);
        }
        p->pop = kc::Population<nt::SynapticResourceSTDPAltAILIFNeuron>(p->uid, std::move(v));
    }
    else
        return fail("bad neuron kind");
    net->pops.push_back(std::move(p));
    return 0;
}

int or_read_altai(const or_net *net, knp_uid pop, knp_altai_neuron *out, knp_resource_stdp_state *ext)
{
    Pop *p = net->find_pop(to_uid(pop));
    if (!p) return fail("unknown population");
    if (auto *a = std::get_if<kc::Population<nt::AltAILIF>>(&p->pop))
    {
        for (size_t i = 0; i < a->size(); ++i) out[i] = from_ref((*a)[i]);
        return 0;
    }
    if (auto *ra = std::get_if<kc::Population<nt::SynapticResourceSTDPAltAILIFNeuron>>(&p->pop))
    {
        for (size_t i = 0; i < ra->size(); ++i)
        {
            out[i] = from_ref(static_cast<const AltaiParams &>((*ra)[i]));
            if (ext) ext[i] = res_from_ref((*ra)[i]);
        }
        return 0;
    }
    return fail("unknown AltAI population");
}

int or_set_stdp_population(or_net *net, knp_uid proj_uid, knp_uid pop_uid, int processing)
{
    Proj *p = net->find_proj(to_uid(proj_uid));
    if (!p) return fail("unknown projection");
    auto *a = std::get_if<AddStdpProj>(&p->proj);
    if (!a) return fail("not an STDP projection");
    a->get_shared_parameters().stdp_populations_[to_uid(pop_uid)] =
        processing == KNP_STDP_AND_SPIKE ? AddStdpProj::SharedSynapseParameters::ProcessingType::STDPAndSpike
                                         : AddStdpProj::SharedSynapseParameters::ProcessingType::STDPOnly;
    return 0;
}

int or_subscribe(or_net *net, knp_uid receiver, knp_uid sender)
{
    net->extra_subs.emplace_back(to_uid(receiver), to_uid(sender));
    if (net->initialized)
    {
        if (Proj *p = net->find_proj(to_uid(receiver))) p->spike_senders.insert(to_uid(sender));
        if (Pop *q = net->find_pop(to_uid(receiver))) q->impact_senders.insert(to_uid(sender));
    }
    return 0;
}

int or_init(or_net *net)
{
    for (auto &p : net->projs)
    {
        std::visit(
            [&](auto &proj)
            {
                using T = std::decay_t<decltype(proj)>;
                if constexpr (std::is_same_v<T, AddStdpProj>)
                    for (auto &[u, _] : proj.get_shared_parameters().stdp_populations_)
                        if (u) p->spike_senders.insert(u);
                if (proj.get_presynaptic()) p->spike_senders.insert(proj.get_presynaptic());
                if (proj.get_postsynaptic())
                    if (Pop *q = net->find_pop(proj.get_postsynaptic())) q->impact_senders.insert(p->uid);
            },
            p->proj);
    }
    for (auto &[recv, send] : net->extra_subs)
    {
        if (Proj *p = net->find_proj(recv)) p->spike_senders.insert(send);
        if (Pop *q = net->find_pop(recv)) q->impact_senders.insert(send);
    }
    net->initialized = true;
    return 0;
}

int or_send_spikes(or_net *net, knp_uid sender, uint64_t send_time, uint32_t n, const uint32_t *idx)
{
    net->ext_spikes.push_back(msg::SpikeMessage{{to_uid(sender), send_time}, {idx, idx + n}});
    return 0;
}

int or_send_impacts(
    or_net *net, knp_uid sender, knp_uid receiver_pop, int is_forcing, uint32_t n, const uint32_t *post_idx,
    const float *value, const uint8_t *out_type)
{
    msg::SynapticImpactMessage m{{to_uid(sender), net->step}, kc::UID{}, to_uid(receiver_pop), is_forcing != 0, {}};
    for (uint32_t i = 0; i < n; ++i)
        m.impacts_.push_back(
            msg::SynapticImpact{0, value[i], static_cast<st::OutputType>(out_type ? out_type[i] : 0), 0, post_idx[i]});
    net->ext_impacts.push_back(std::move(m));
    return 0;
}

int or_step(or_net *net)
{
    return guarded(
        [&]
        {
            if (!net->initialized) throw std::runtime_error("or_init was not called");
            const uint64_t step = net->step;
            for (auto &m : net->ext_spikes)
                for (auto &p : net->projs)
                    if (p->spike_senders.count(m.header_.sender_uid_)) p->inbox.push_back(m);
            for (auto &m : net->ext_impacts)
                for (auto &q : net->pops)
                    if (q->impact_senders.count(m.header_.sender_uid_)) q->inbox.push_back(m);
            net->ext_spikes.clear();
            net->ext_impacts.clear();
            std::vector<msg::SpikeMessage> sent;
            for (auto &q : net->pops)
            {
                step_population(*net, *q, step);
                if (!q->last_spikes.empty())
                    sent.push_back(msg::SpikeMessage{{q->uid, step}, {q->last_spikes.begin(), q->last_spikes.end()}});
            }
            for (auto &m : sent)
                for (auto &p : net->projs)
                    if (p->spike_senders.count(m.header_.sender_uid_)) p->inbox.push_back(m);
            std::vector<msg::SynapticImpactMessage> out;
            for (auto &p : net->projs)
            {
                msg::SynapticImpactMessage m;
                const bool due = std::visit([&](auto &proj) { return step_projection(*net, *p, proj, step, m); }, p->proj);
                if (due) out.push_back(std::move(m));
            }
            for (auto &m : out)
                for (auto &q : net->pops)
                    if (q->impact_senders.count(m.header_.sender_uid_)) q->inbox.push_back(m);
            ++net->step;
            return 0;
        });
}

uint64_t or_get_step(const or_net *net) { return net->step; }

int or_read_spikes(const or_net *net, knp_uid pop, uint32_t cap, uint32_t *out, uint32_t *n)
{
    const Pop *q = net->find_pop(to_uid(pop));
    if (!q) return fail("unknown population");
    *n = static_cast<uint32_t>(q->last_spikes.size());
    if (q->last_spikes.size() > cap) return fail("spike buffer too small");
    std::copy(q->last_spikes.begin(), q->last_spikes.end(), out);
    return 0;
}

int or_read_blifat(const or_net *net, knp_uid pop, knp_blifat_neuron *out, knp_resource_stdp_state *ext)
{
    Pop *q = net->find_pop(to_uid(pop));
    if (!q) return fail("unknown population");
    if (auto *b = std::get_if<kc::Population<nt::BLIFATNeuron>>(&q->pop))
    {
        for (size_t i = 0; i < b->size(); ++i) out[i] = from_ref((*b)[i]);
        return 0;
    }
    if (auto *r = std::get_if<kc::Population<nt::SynapticResourceSTDPBLIFATNeuron>>(&q->pop))
    {
        for (size_t i = 0; i < r->size(); ++i)
        {
            out[i] = from_ref((*r)[i]);
            if (ext) ext[i] = res_from_ref((*r)[i]);
        }
        return 0;
    }
    return fail("not a BLIFAT population");
}

int or_read_lif(const or_net *net, knp_uid pop, knp_lif_neuron *out)
{
    Pop *q = net->find_pop(to_uid(pop));
    if (!q) return fail("unknown population");
    auto *l = std::get_if<kc::Population<nt::LIFNeuron>>(&q->pop);
    if (!l) return fail("not a LIF population");
    for (size_t i = 0; i < l->size(); ++i)
    {
        const auto &n = (*l)[i];
        out[i] = knp_lif_neuron{n.potential_, n.potential_reset_value_, n.activation_threshold_, n.leak_coefficient_,
                                n.refract_counter_, n.refract_period_};
    }
    return 0;
}

int or_read_weights(const or_net *net, knp_uid proj, float *out)
{
    Proj *p = net->find_proj(to_uid(proj));
    if (!p) return fail("unknown projection");
    std::visit(
        [&](auto &pr)
        {
            for (size_t i = 0; i < pr.size(); ++i) out[i] = std::get<kc::synapse_data>(pr[i]).weight_;
        },
        p->proj);
    return 0;
}

uint64_t or_event_count(const or_net *net) { return net->events; }

}  // extern "C"
