// TEST INFRASTRUCTURE — CPU restatement of the KNP single-threaded backend step (the oracle).
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU arms load this library; the GB300 product
// path never calls it. It restates, with FP64 neuron state and the reference's own container
// structure (unordered_map future-impact queue, per-spike synapse lookup, impact vectors copied
// through a FIFO bus), the following reference code (paths inside the KNP project):
//
//   step loop       knp/backends/cpu/cpu-single-threaded-backend/impl/backend.cpp:89-141
//   subscriptions   knp/backends/cpu/cpu-library/include/knp/backends/cpu-library/init.h:46-110
//   bus order       knp/core-library/impl/message_bus_cpu_impl/message_bus_cpu_impl.cpp:41-88 (route = pop_back)
//                   + message_endpoint_cpu_impl.h:62-76 (receive = pop_back): the two LIFOs give FIFO
//   population      cpu-library/populations_old.h:104-121 (any), :195-217 (resource STDP)
//   BLIFAT          cpu-library/impl/populations/blifat/blifat_impl.h:31-168
//   resource STDP   cpu-library/impl/populations/blifat/blifat_stdp.h:35-172, impl/populations/training/stdp.h:88-186
//   LIF             cpu-library/impl/populations/lif/lif_impl.h:33-86
//   projection      cpu-library/projections.h:58-84, impl/projections/delta/delta_impl.h:54-114
//   additive STDP   cpu-library/impl/projections/training/stdp/additive_stdp.h:42-196
//
// Synapses of one presynaptic (or postsynaptic) neuron are visited in ascending synapse index. The
// reference visits them in Boost.MultiIndex hashed-index order (knp/core-library/impl/projection.cpp:168-188);
// that order only changes FP64 rounding of impact sums, never the set of impacts.
#include "knp_oracle.h"

#include <algorithm>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace
{

thread_local std::string g_error;

struct Uid
{
    knp_uid v;
    bool operator==(const Uid &o) const { return std::memcmp(v.bytes, o.v.bytes, 16) == 0; }
    bool is_null() const
    {
        for (auto b : v.bytes)
            if (b) return false;
        return true;
    }
};

struct UidHash
{
    size_t operator()(const Uid &u) const
    {
        uint64_t a, b;
        std::memcpy(&a, u.v.bytes, 8);
        std::memcpy(&b, u.v.bytes + 8, 8);
        return static_cast<size_t>(a * 0x9E3779B97F4A7C15ull ^ b);
    }
};

struct SpikeMessage
{
    Uid sender;
    uint64_t send_time;
    std::vector<uint32_t> idx;
};

struct Impact
{
    uint64_t connection_index;
    float value;
    uint8_t type;
    uint32_t pre;
    uint32_t post;
};

struct ImpactMessage
{
    Uid sender;
    uint64_t send_time;
    Uid pre_uid;
    Uid post_uid;
    bool is_forcing;
    std::vector<Impact> impacts;
};

struct Population
{
    Uid uid;
    int kind;
    std::vector<knp_blifat_neuron> blifat;
    std::vector<knp_resource_stdp_state> res;
    std::vector<knp_lif_neuron> lif;
    std::vector<knp_altai_neuron> altai;
    std::vector<uint32_t> last_spikes;
    std::unordered_set<Uid, UidHash> impact_senders;  // impact-message subscription
    std::vector<ImpactMessage> inbox;
    size_t size() const
    {
        return kind == KNP_NEURON_LIF ? lif.size() : is_altai() ? altai.size() : blifat.size();
    }
    bool is_altai() const { return kind == KNP_NEURON_ALTAI_LIF || kind == KNP_NEURON_RESOURCE_STDP_ALTAI_LIF; }
    bool is_resource() const
    {
        return kind == KNP_NEURON_RESOURCE_STDP_BLIFAT || kind == KNP_NEURON_RESOURCE_STDP_ALTAI_LIF;
    }
};

struct Synapse
{
    float weight;
    uint32_t delay;
    uint8_t type;
    float tau_plus;
    float tau_minus;
    std::vector<uint64_t> pre_times;
    std::vector<uint64_t> post_times;
    uint32_t pre;
    uint32_t post;
    knp_resource_synapse rule{};  // synaptic-resource STDP rule state
};

struct Projection
{
    Uid uid;
    int kind;
    Uid pre_uid;
    Uid post_uid;
    std::vector<Synapse> syn;
    std::vector<std::vector<size_t>> by_pre;
    std::vector<std::vector<size_t>> by_post;
    bool locked = true;  // is_locked() (projection.h:384-396); only resource-STDP training reads it
    std::unordered_map<Uid, int, UidHash> stdp_pops;
    std::unordered_set<Uid, UidHash> spike_senders;  // spike-message subscription
    std::vector<SpikeMessage> inbox;
    std::unordered_map<uint64_t, ImpactMessage> future;  // MessageQueue (message_queue.h:34)

    const std::vector<size_t> &find_by_pre(uint32_t i) const
    {
        static const std::vector<size_t> none;
        return i < by_pre.size() ? by_pre[i] : none;
    }
    const std::vector<size_t> &find_by_post(uint32_t i) const
    {
        static const std::vector<size_t> none;
        return i < by_post.size() ? by_post[i] : none;
    }
};

// Fixed-size worker pool with post/join, standing in for the reference's Boost.Asio thread pool
// (knp/backends/cpu/thread_pool/include/knp/backends/thread_pool/thread_pool.h:36-77).
class ThreadPool
{
public:
    explicit ThreadPool(int n)
    {
        for (int i = 0; i < n; ++i) workers_.emplace_back([this] { loop(); });
    }
    ~ThreadPool()
    {
        {
            std::lock_guard<std::mutex> l(m_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto &w : workers_) w.join();
    }
    void post(std::function<void()> f)
    {
        {
            std::lock_guard<std::mutex> l(m_);
            q_.push_back(std::move(f));
            ++pending_;
        }
        cv_.notify_one();
    }
    void join()
    {
        std::unique_lock<std::mutex> l(m_);
        done_.wait(l, [this] { return pending_ == 0; });
    }
    int size() const { return static_cast<int>(workers_.size()); }

private:
    void loop()
    {
        for (;;)
        {
            std::function<void()> f;
            {
                std::unique_lock<std::mutex> l(m_);
                cv_.wait(l, [this] { return stop_ || !q_.empty(); });
                if (stop_ && q_.empty()) return;
                f = std::move(q_.front());
                q_.pop_front();
            }
            f();
            {
                std::lock_guard<std::mutex> l(m_);
                if (--pending_ == 0) done_.notify_all();
            }
        }
    }
    std::vector<std::thread> workers_;
    std::deque<std::function<void()>> q_;
    std::mutex m_;
    std::condition_variable cv_, done_;
    size_t pending_ = 0;
    bool stop_ = false;
};

}  // namespace

struct or_net
{
    std::unique_ptr<ThreadPool> pool;
    std::vector<std::unique_ptr<Population>> pops;
    std::vector<std::unique_ptr<Projection>> projs;
    std::vector<std::pair<Uid, Uid>> extra_subs;  // receiver, sender
    std::vector<SpikeMessage> ext_spikes;
    std::vector<ImpactMessage> ext_impacts;
    uint64_t step = 0;
    uint64_t events = 0;
    bool initialized = false;
    // The network as built by or_init, for or_reset (repeated timing windows of the CPU baseline).
    std::vector<Population> pops0;
    std::vector<Projection> projs0;

    Population *find_pop(const Uid &u) const
    {
        for (auto &p : pops)
            if (p->uid == u) return p.get();
        return nullptr;
    }
    Projection *find_proj(const Uid &u) const
    {
        for (auto &p : projs)
            if (p->uid == u) return p.get();
        return nullptr;
    }
};

namespace
{

int fail(const std::string &msg)
{
    g_error = msg;
    return -1;
}

// ---------------------------------------------------------------- BLIFAT (blifat_impl.h:31-168)

void blifat_pre_impact(knp_blifat_neuron &n)
{
    ++n.n_time_steps_since_last_firing;
    n.dynamic_threshold *= n.threshold_decay;
    n.postsynaptic_trace *= n.postsynaptic_trace_decay;
    n.inhibitory_conductance *= n.inhibitory_conductance_decay;
    n.potential *= n.potential_decay;
    if (1 == n.bursting_phase)
    {
        --n.bursting_phase;
        n.potential += n.reflexive_weight;
    }
    n.pre_impact_potential = n.potential;
}

// Resource-STDP variant (blifat_impl.h:50-65): resets dopamine and forcing, and does not decrement
// the bursting phase.
void resource_blifat_pre_impact(knp_blifat_neuron &n, knp_resource_stdp_state &r)
{
    ++n.n_time_steps_since_last_firing;
    n.dynamic_threshold *= n.threshold_decay;
    n.postsynaptic_trace *= n.postsynaptic_trace_decay;
    n.inhibitory_conductance *= n.inhibitory_conductance_decay;
    n.dopamine_value = 0.0;
    r.is_being_forced = 0;
    n.potential *= n.potential_decay;
    if (1 == n.bursting_phase) n.potential += n.reflexive_weight;
    n.pre_impact_potential = n.potential;
}

void blifat_impact(knp_blifat_neuron &n, const Impact &imp)
{
    switch (imp.type)
    {
        case KNP_OUT_EXCITATORY:
            n.potential += imp.value;
            break;
        case KNP_OUT_INHIBITORY_CURRENT:
            n.potential -= imp.value;
            break;
        case KNP_OUT_INHIBITORY_CONDUCTANCE:
            n.inhibitory_conductance += imp.value;
            break;
        case KNP_OUT_DOPAMINE:
            n.dopamine_value += imp.value;
            break;
        case KNP_OUT_BLOCKING:
            n.total_blocking_period = static_cast<int64_t>(imp.value);
            break;
        default:
            throw std::runtime_error("Unhandled synapse type.");
    }
}

bool blifat_post_impact(knp_blifat_neuron &n)
{
    if (n.total_blocking_period <= 0) n.potential = n.pre_impact_potential;
    if (n.total_blocking_period < 0)
    {
        ++n.total_blocking_period;
        if (n.total_blocking_period == 0) n.total_blocking_period = std::numeric_limits<int64_t>::max();
    }
    else if (n.total_blocking_period > 0)
    {
        n.total_blocking_period -= 1;
    }
    if (n.inhibitory_conductance < 1.0)
        n.potential -= (n.potential - n.reversal_inhibitory_potential) * n.inhibitory_conductance;
    else
        n.potential = n.reversal_inhibitory_potential;

    const bool spike = (n.n_time_steps_since_last_firing > n.absolute_refractory_period) &&
                       (n.potential >= n.activation_threshold + n.dynamic_threshold + n.additional_threshold);
    if (spike)
    {
        n.dynamic_threshold += n.threshold_increment;
        n.postsynaptic_trace += n.postsynaptic_trace_increment;
        n.potential = n.potential_reset_value;
        n.bursting_phase = n.bursting_period;
        n.n_time_steps_since_last_firing = 0;
    }
    if (n.potential < n.min_potential) n.potential = n.min_potential;
    return spike;
}

// ------------------------------------------- resource-STDP neuron training (blifat_stdp.h:35-172)
// The population's training over the unlocked SynapticResourceSTDPDeltaSynapse projections into it:
// ISI status, stability, additional threshold, Hebbian and dopamine changes of the synaptic
// resource, free-resource renormalisation and the weights that follow from the resource.

template <class Neuron>
int update_isi(knp_resource_stdp_state &r, const Neuron &n, uint64_t step)  // training/stdp.h:88-126
{
    if (r.is_being_forced)
    {
        r.isi_status = KNP_ISI_IS_FORCED;
        return r.isi_status;
    }
    switch (r.isi_status)
    {
        case KNP_ISI_NOT_IN_PERIOD:
        case KNP_ISI_IS_FORCED:
            r.isi_status = KNP_ISI_PERIOD_STARTED;
            r.first_isi_spike = step;
            break;
        case KNP_ISI_PERIOD_STARTED:
            // Unsigned difference, as in the reference.
            if (r.last_step - step < r.isi_max) r.isi_status = KNP_ISI_PERIOD_CONTINUED;
            break;
        case KNP_ISI_PERIOD_CONTINUED:
            if (r.last_step - step >= r.isi_max || n.dopamine_value != 0)
            {
                r.isi_status = KNP_ISI_PERIOD_STARTED;
                r.first_isi_spike = step;
            }
            break;
        default:
            throw std::runtime_error("Not supported ISI status.");
    }
    r.last_step = step;
    return r.isi_status;
}

// recalculate_synapse_weights (training/stdp.h:40-52).
void recalc_weight(Synapse &s)
{
    const float syn_w = std::max(s.rule.synaptic_resource, 0.F);
    const float weight_diff = s.rule.w_max - s.rule.w_min;
    s.weight = s.rule.w_min + weight_diff * syn_w / (weight_diff + syn_w);
}

// min(2^-stability, 1) as the reference evaluates it: std::pow(2, -stability) in double, then float.
float resource_factor(float stability) { return std::min(static_cast<float>(std::pow(2, -stability)), 1.F); }

// The SynapticResourceSTDPDeltaSynapse projections into a population that are not locked, in the
// backend's projection order (populations_old.h:57-83, 207-209).
std::vector<Projection *> working_projections(or_net &net, const Population &pop)
{
    std::vector<Projection *> out;
    for (auto &p : net.projs)
        if (p->kind == KNP_SYNAPSE_RESOURCE_STDP_DELTA && p->post_uid == pop.uid && !p->locked) out.push_back(p.get());
    return out;
}

// get_all_connected_synapses (training/stdp.h:55-72): synapses into neuron i, projection by projection.
std::vector<Synapse *> connected(const std::vector<Projection *> &working, uint32_t i)
{
    std::vector<Synapse *> out;
    for (Projection *p : working)
        for (size_t si : p->find_by_post(i)) out.push_back(&p->syn[si]);
    return out;
}

bool is_point_in_interval(uint64_t a, uint64_t b, uint64_t point)  // training/stdp.h:129-133
{
    if (a > b) std::swap(a, b);
    return a <= point && point <= b;
}

// train_population_impl (blifat_stdp.h:158-172): process_spiking_neurons_impl (:35-103),
// do_dopamine_plasticity_impl (:106-155), renormalize_resource (training/stdp.h:152-186). The
// AltAI-LIF variant (altai/altai_stdp.h) is the same computation on the AltAI neuron's dopamine value
// and additional threshold.
template <class Neuron>
void train_resource_population(or_net &net, Population &pop, std::vector<Neuron> &neurons,
                               const std::vector<uint32_t> &spikes, uint64_t step)
{
    const std::vector<Projection *> working = working_projections(net, pop);
    for (uint32_t i : spikes)
    {
        auto &n = neurons[i];
        auto &r = pop.res[i];
        const std::vector<Synapse *> syns = connected(working, i);
        r.last_spike_step = step;
        update_isi(r, n, step);
        if (KNP_ISI_PERIOD_STARTED == r.isi_status) r.stability -= r.stability_change_at_isi;
        n.additional_threshold = 0.0;
        for (Synapse *s : syns)
        {
            n.additional_threshold += s->weight * (s->weight > 0);
            const bool had_spike =
                is_point_in_interval(step - s->rule.dopamine_plasticity_period, step, s->rule.last_spike_step + s->delay - 1);
            if (KNP_ISI_PERIOD_CONTINUED != r.isi_status || had_spike) s->rule.has_contributed = had_spike;
        }
        n.additional_threshold *= r.synapse_sum_threshold_coefficient;
        if (r.isi_status != KNP_ISI_PERIOD_CONTINUED)
            for (Synapse *s : syns) s->rule.had_hebbian_update = 0;
        if (r.isi_status != KNP_ISI_IS_FORCED)
        {
            for (Synapse *s : syns)
            {
                s->rule.synaptic_resource -= s->rule.d_u;
                r.free_synaptic_resource += s->rule.d_u;
                if (s->rule.has_contributed && !s->rule.had_hebbian_update)
                {
                    const float d_h = r.d_h * resource_factor(r.stability);
                    s->rule.synaptic_resource += d_h;
                    r.free_synaptic_resource -= d_h;
                    s->rule.had_hebbian_update = 1;
                }
            }
        }
        for (Synapse *s : syns) recalc_weight(*s);
    }
    for (uint32_t i = 0; i < neurons.size(); ++i)
    {
        auto &n = neurons[i];
        auto &r = pop.res[i];
        if (n.dopamine_value > 0.0 || (n.dopamine_value < 0.0 && r.isi_status != KNP_ISI_IS_FORCED))
        {
            const std::vector<Synapse *> syns = connected(working, i);
            for (Synapse *s : syns)
            {
                if (step - r.last_spike_step <= r.dopamine_plasticity_time && s->rule.has_contributed)
                {
                    const float resource_change = n.dopamine_value * resource_factor(r.stability);
                    s->rule.synaptic_resource += resource_change;
                    r.free_synaptic_resource -= resource_change;
                }
            }
            if (r.is_being_forced || n.dopamine_value < 0)
            {
                r.stability -= n.dopamine_value * r.stability_change_parameter;
                r.stability = std::max(r.stability, 0.0F);
            }
            else
            {
                const double dopamine_constant = 2.0;
                const double difference = std::fabs(step - r.first_isi_spike - r.isi_max);
                r.stability += r.stability_change_parameter * n.dopamine_value *
                               std::max(dopamine_constant - difference / r.isi_max, -1.0);
            }
            for (Synapse *s : syns) recalc_weight(*s);
        }
    }
    for (uint32_t i = 0; i < neurons.size(); ++i)
    {
        auto &r = pop.res[i];
        if (step - r.last_step <= r.isi_max && r.isi_status != KNP_ISI_IS_FORCED) continue;
        if (std::fabs(r.free_synaptic_resource) < r.synaptic_resource_threshold) continue;
        const std::vector<Synapse *> syns = connected(working, i);
        const float add_resource_value = r.free_synaptic_resource / (syns.size() + r.resource_drain_coefficient);
        for (Synapse *s : syns) s->rule.synaptic_resource += add_resource_value;
        r.free_synaptic_resource = 0.0F;
        for (Synapse *s : syns) recalc_weight(*s);
    }
}

// ----------------------------------------------------------------------- LIF (lif_impl.h:33-86)

void lif_pre_impact(knp_lif_neuron &n)
{
    if (0 == n.refract_counter) n.potential *= n.leak_coefficient;
}

void lif_impact(knp_lif_neuron &n, const Impact &imp)
{
    switch (imp.type)
    {
        case KNP_OUT_EXCITATORY:
            if (0 == n.refract_counter) n.potential += imp.value;
            break;
        case KNP_OUT_INHIBITORY_CURRENT:
            if (0 == n.refract_counter) n.potential -= imp.value;
            break;
        default:
            throw std::runtime_error("Unhandled synapse type.");
    }
}

bool lif_post_impact(knp_lif_neuron &n)
{
    if (0 == n.refract_counter)
    {
        if (n.potential > n.activation_threshold)
        {
            n.potential = n.potential_reset_value;
            n.refract_counter = n.refract_period;
            return true;
        }
    }
    else
    {
        --n.refract_counter;
    }
    return false;
}

// ---------------------------------------------------------- AltAI-LIF (altai/altai_impl.h:33-168)

void altai_pre_impact(knp_altai_neuron &n, knp_resource_stdp_state *r)
{
    n.potential = n.do_not_save ? static_cast<float>(n.potential_reset_value) : std::round(n.potential);
    if (r)
    {
        n.dopamine_value = 0.0;
        r->is_being_forced = 0;
    }
    n.pre_impact_potential = n.potential;
}

void altai_impact(knp_altai_neuron &n, const Impact &imp)
{
    switch (imp.type)
    {
        case KNP_OUT_EXCITATORY:
            n.potential += imp.value;
            break;
        case KNP_OUT_INHIBITORY_CURRENT:
            n.potential -= imp.value;
            break;
        case KNP_OUT_DOPAMINE:
            n.dopamine_value += imp.value;
            break;
        case KNP_OUT_BLOCKING:
            // A blocking impact replaces the activity time unless it has the same sign and a smaller
            // magnitude (signs of the values as doubles).
            if (std::signbit(static_cast<double>(n.activity_time)) != std::signbit(static_cast<double>(imp.value)) ||
                std::abs(n.activity_time) <= std::abs(imp.value))
                n.activity_time = static_cast<int64_t>(imp.value);
            break;
        default:
            throw std::runtime_error("Unhandled synapse type.");
    }
}

bool altai_post_impact(knp_altai_neuron &n)
{
    const int sign = (n.leak_rev && n.potential < 0) ? -1 : 1;
    n.potential += n.potential_leak * sign;
    bool spiked = false;
    if (n.activity_time > 0)
        --n.activity_time;
    else if (n.activity_time < 0)
        ++n.activity_time;
    if (n.activity_time == 0) n.activity_time = std::numeric_limits<int64_t>::max();
    bool was_reset = false;
    if (n.potential >= n.activation_threshold + n.additional_threshold)
    {
        if (n.activity_time > 0) spiked = true;
        if (n.is_diff) n.potential -= n.activation_threshold + n.additional_threshold;
        if (n.is_reset)
        {
            n.potential = n.potential_reset_value;
            was_reset = true;
        }
    }
    if (n.potential <= -static_cast<float>(n.negative_activation_threshold) && !was_reset)
    {
        if (n.saturate)
            n.potential = -static_cast<float>(n.negative_activation_threshold);
        else if (n.is_reset)
            n.potential = -n.potential_reset_value;
        else if (n.is_diff)
            n.potential += n.negative_activation_threshold;
    }
    return spiked;
}

// ------------------------------------------------------------------ one population step

void check_impacts(const Population &pop, const std::vector<ImpactMessage> &msgs)
{
    for (auto &m : msgs)
        for (auto &imp : m.impacts)
            if (imp.post >= pop.size()) throw std::runtime_error("Impact postsynaptic index out of range.");
}

// Per-neuron phases of any population kind.
void pre_impact(Population &q, size_t i)
{
    switch (q.kind)
    {
        case KNP_NEURON_LIF:
            lif_pre_impact(q.lif[i]);
            break;
        case KNP_NEURON_RESOURCE_STDP_BLIFAT:
            resource_blifat_pre_impact(q.blifat[i], q.res[i]);
            break;
        case KNP_NEURON_ALTAI_LIF:
            altai_pre_impact(q.altai[i], nullptr);
            break;
        case KNP_NEURON_RESOURCE_STDP_ALTAI_LIF:
            altai_pre_impact(q.altai[i], &q.res[i]);
            break;
        default:
            blifat_pre_impact(q.blifat[i]);
    }
}

void impact(Population &q, const Impact &imp, bool is_forcing)
{
    if (q.kind == KNP_NEURON_LIF)
    {
        lif_impact(q.lif[imp.post], imp);
        return;
    }
    if (q.is_altai())
        altai_impact(q.altai[imp.post], imp);
    else
        blifat_impact(q.blifat[imp.post], imp);
    if (q.is_resource() && imp.type == KNP_OUT_EXCITATORY) q.res[imp.post].is_being_forced |= is_forcing ? 1u : 0u;
}

bool post_impact(Population &q, size_t i)
{
    if (q.kind == KNP_NEURON_LIF) return lif_post_impact(q.lif[i]);
    if (q.is_altai()) return altai_post_impact(q.altai[i]);
    return blifat_post_impact(q.blifat[i]);
}

void train(or_net &net, Population &q, uint64_t step)
{
    if (q.kind == KNP_NEURON_RESOURCE_STDP_BLIFAT) train_resource_population(net, q, q.blifat, q.last_spikes, step);
    if (q.kind == KNP_NEURON_RESOURCE_STDP_ALTAI_LIF) train_resource_population(net, q, q.altai, q.last_spikes, step);
}

// calculate_any_population / calculate_resource_stdp_population (populations_old.h:104-121, 195-217).
void calculate_population(or_net &net, Population &pop, uint64_t step)
{
    std::vector<ImpactMessage> msgs = std::move(pop.inbox);
    pop.inbox.clear();
    check_impacts(pop, msgs);
    pop.last_spikes.clear();
    const size_t n = pop.size();
    for (size_t i = 0; i < n; ++i) pre_impact(pop, i);
    for (auto &m : msgs)
        for (auto &imp : m.impacts) impact(pop, imp, m.is_forcing);
    for (uint32_t i = 0; i < n; ++i)
        if (post_impact(pop, i)) pop.last_spikes.push_back(i);
    train(net, pop, step);
}

// --------------------------------------------------------- additive STDP (additive_stdp.h:42-196)

// STDPFormula::stdp_w with a_plus = a_minus = 1 (additive_stdp.h:50-55, :187). The argument is the
// unsigned step difference converted to float, as in stdp_delta_w (:72): a negative difference wraps
// to a huge positive value, whose term is exp(-huge) = 0.
float stdp_w(float tau_plus, float tau_minus, float weight_diff)
{
    return weight_diff > 0 ? 1.0F * std::exp(-weight_diff / tau_plus) : 1.0F * std::exp(weight_diff / tau_minus);
}

float stdp_delta_w(const Synapse &s)
{
    float w_j = 0;
    for (uint64_t t_f : s.pre_times)
        for (uint64_t t_n : s.post_times) w_j += stdp_w(s.tau_plus, s.tau_minus, static_cast<float>(t_n - t_f));
    return w_j;
}

// init_projection (additive_stdp.h:117-170): fill spike-time lists from messages of STDP populations.
void stdp_init_projection(Projection &proj, std::vector<SpikeMessage> &msgs)
{
    for (auto &msg : msgs)
    {
        auto it = proj.stdp_pops.find(msg.sender);
        if (it == proj.stdp_pops.end()) continue;
        const int type = it->second;
        auto append = [&](bool post_list)
        {
            for (uint32_t j : msg.idx)
                for (size_t si : proj.find_by_post(j))
                {
                    Synapse &s = proj.syn[si];
                    auto &q = post_list ? s.post_times : s.pre_times;
                    if (q.size() < s.tau_minus + s.tau_plus) q.push_back(msg.send_time);
                }
        };
        append(true);
        if (type == KNP_STDP_AND_SPIKE) append(false);
        if (type == KNP_STDP_ONLY) msg.idx.clear();
    }
}

// modify_weights (additive_stdp.h:173-196).
void stdp_modify_weights(Projection &proj)
{
    for (auto &s : proj.syn)
    {
        const float period = s.tau_plus + s.tau_minus;
        if (s.pre_times.size() >= period && s.post_times.size() >= period)
        {
            s.weight += stdp_delta_w(s);
            s.pre_times.clear();
            s.post_times.clear();
        }
    }
}

// ----------------------------------------------------------------- one projection step

// projections::calculate_projection + delta::calculate_projection_impl (projections.h:58-84,
// delta_impl.h:54-114). Returns true and fills `out` if an impact message is due this step.
bool calculate_projection(or_net &net, Projection &proj, uint64_t step, ImpactMessage &out)
{
    std::vector<SpikeMessage> msgs = std::move(proj.inbox);
    proj.inbox.clear();
    const bool stdp = proj.kind == KNP_SYNAPSE_ADDITIVE_STDP_DELTA;
    const bool resource = proj.kind == KNP_SYNAPSE_RESOURCE_STDP_DELTA;
    if (stdp) stdp_init_projection(proj, msgs);
    for (auto &msg : msgs)
        for (uint32_t spiked : msg.idx)
            for (size_t si : proj.find_by_pre(spiked))
            {
                Synapse &s = proj.syn[si];
                // init_synapse (synaptic_resource_stdp.h:36-41): the step of the presynaptic spike.
                if (resource) s.rule.last_spike_step = step;
                // The message is sent on step N - 1 and received on step N.
                const uint64_t future_step = s.delay + step - 1;
                Impact imp{si, s.weight, s.type, s.pre, s.post};
                ++net.events;
                auto it = proj.future.find(future_step);
                if (it != proj.future.end())
                {
                    it->second.impacts.push_back(imp);
                }
                else
                {
                    // is_forced(): true for plain delta projections, false for additive and resource
                    // STDP (stdp_dispatcher.h:54-58, additive_stdp.h:199-203, synaptic_resource_stdp.h:58-62).
                    ImpactMessage m{proj.uid, step, proj.pre_uid, proj.post_uid, proj.kind == KNP_SYNAPSE_DELTA, {imp}};
                    proj.future.emplace(future_step, std::move(m));
                }
            }
    if (stdp) stdp_modify_weights(proj);
    auto it = proj.future.find(step);
    if (it == proj.future.end()) return false;
    out = std::move(it->second);
    proj.future.erase(it);
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
    if (kind != KNP_NEURON_BLIFAT && kind != KNP_NEURON_RESOURCE_STDP_BLIFAT) return fail("bad neuron kind");
    if (kind == KNP_NEURON_RESOURCE_STDP_BLIFAT && !ext) return fail("resource-STDP population needs ext state");
    auto p = std::make_unique<Population>();
    p->uid = Uid{uid};
    p->kind = kind;
    p->blifat.assign(neurons, neurons + n);
    if (ext) p->res.assign(ext, ext + n);
    net->pops.push_back(std::move(p));
    return 0;
}

int or_add_altai_population(
    or_net *net, knp_uid uid, int kind, uint32_t n, const knp_altai_neuron *neurons, const knp_resource_stdp_state *ext)
{
    if (kind != KNP_NEURON_ALTAI_LIF && kind != KNP_NEURON_RESOURCE_STDP_ALTAI_LIF) return fail("bad neuron kind");
    if (kind == KNP_NEURON_RESOURCE_STDP_ALTAI_LIF && !ext) return fail("resource-STDP population needs ext state");
    auto p = std::make_unique<Population>();
    p->uid = Uid{uid};
    p->kind = kind;
    p->altai.assign(neurons, neurons + n);
    if (kind == KNP_NEURON_RESOURCE_STDP_ALTAI_LIF) p->res.assign(ext, ext + n);
    net->pops.push_back(std::move(p));
    return 0;
}

int or_read_altai(const or_net *net, knp_uid pop, knp_altai_neuron *out, knp_resource_stdp_state *ext)
{
    const Population *q = net->find_pop(Uid{pop});
    if (!q || !q->is_altai()) return fail("unknown AltAI population");
    std::copy(q->altai.begin(), q->altai.end(), out);
    if (ext && !q->res.empty()) std::copy(q->res.begin(), q->res.end(), ext);
    return 0;
}

int or_add_lif_population(or_net *net, knp_uid uid, uint32_t n, const knp_lif_neuron *neurons)
{
    auto p = std::make_unique<Population>();
    p->uid = Uid{uid};
    p->kind = KNP_NEURON_LIF;
    p->lif.assign(neurons, neurons + n);
    net->pops.push_back(std::move(p));
    return 0;
}

int or_add_projection(
    or_net *net, knp_uid uid, int kind, knp_uid pre_uid, knp_uid post_uid, uint64_t n_syn,
    const uint32_t *pre_idx, const uint32_t *post_idx, const float *weight, const uint32_t *delay,
    const uint8_t *out_type, const float *tau_plus, const float *tau_minus)
{
    if (kind != KNP_SYNAPSE_DELTA && kind != KNP_SYNAPSE_ADDITIVE_STDP_DELTA && kind != KNP_SYNAPSE_RESOURCE_STDP_DELTA)
        return fail("bad synapse kind");
    auto p = std::make_unique<Projection>();
    p->uid = Uid{uid};
    p->kind = kind;
    p->pre_uid = Uid{pre_uid};
    p->post_uid = Uid{post_uid};
    p->syn.resize(n_syn);
    uint32_t max_pre = 0, max_post = 0;
    for (uint64_t i = 0; i < n_syn; ++i)
    {
        Synapse &s = p->syn[i];
        s.weight = weight[i];
        s.delay = delay[i];
        s.type = out_type ? out_type[i] : KNP_OUT_EXCITATORY;
        s.tau_plus = tau_plus ? tau_plus[i] : 10.0F;
        s.tau_minus = tau_minus ? tau_minus[i] : 10.0F;
        s.pre = pre_idx[i];
        s.post = post_idx[i];
        max_pre = std::max(max_pre, s.pre + 1);
        max_post = std::max(max_post, s.post + 1);
    }
    p->by_pre.resize(max_pre);
    p->by_post.resize(max_post);
    for (uint64_t i = 0; i < n_syn; ++i)
    {
        p->by_pre[p->syn[i].pre].push_back(i);
        p->by_post[p->syn[i].post].push_back(i);
    }
    net->projs.push_back(std::move(p));
    return 0;
}

int or_add_resource_projection(
    or_net *net, knp_uid uid, knp_uid pre_uid, knp_uid post_uid, uint64_t n_syn, const uint32_t *pre_idx,
    const uint32_t *post_idx, const float *weight, const uint32_t *delay, const uint8_t *out_type,
    const knp_resource_synapse *rule, int locked)
{
    if (n_syn && !rule) return fail("resource-STDP synapses need their rule state");
    const int rc = or_add_projection(net, uid, KNP_SYNAPSE_RESOURCE_STDP_DELTA, pre_uid, post_uid, n_syn, pre_idx,
                                     post_idx, weight, delay, out_type, nullptr, nullptr);
    if (rc) return rc;
    Projection &p = *net->projs.back();
    for (uint64_t i = 0; i < n_syn; ++i) p.syn[i].rule = rule[i];
    p.locked = locked != 0;
    return 0;
}

int or_set_learning(or_net *net, int on)
{
    // start_learning / stop_learning unlock / lock every projection (cpu-single-threaded/backend.h:315-332).
    for (auto &p : net->projs) p->locked = on == 0;
    return 0;
}

int or_read_resource_synapses(const or_net *net, knp_uid proj, knp_resource_synapse *out)
{
    const Projection *p = net->find_proj(Uid{proj});
    if (!p || p->kind != KNP_SYNAPSE_RESOURCE_STDP_DELTA) return fail("unknown resource-STDP projection");
    for (size_t i = 0; i < p->syn.size(); ++i) out[i] = p->syn[i].rule;
    return 0;
}

int or_set_stdp_population(or_net *net, knp_uid proj_uid, knp_uid pop_uid, int processing)
{
    Projection *p = net->find_proj(Uid{proj_uid});
    if (!p) return fail("unknown projection");
    if (p->kind != KNP_SYNAPSE_ADDITIVE_STDP_DELTA) return fail("not an STDP projection");
    p->stdp_pops[Uid{pop_uid}] = processing;
    return 0;
}

int or_subscribe(or_net *net, knp_uid receiver, knp_uid sender)
{
    net->extra_subs.emplace_back(Uid{receiver}, Uid{sender});
    if (net->initialized)
    {
        if (Projection *p = net->find_proj(Uid{receiver})) p->spike_senders.insert(Uid{sender});
        if (Population *q = net->find_pop(Uid{receiver})) q->impact_senders.insert(Uid{sender});
    }
    return 0;
}

int or_init(or_net *net)
{
    // cpu::init (init.h:93-110) + subscribe_stdp_projection (init.h:46-82).
    for (auto &p : net->projs)
    {
        for (auto &[pop_uid, _] : p->stdp_pops)
            if (!pop_uid.is_null()) p->spike_senders.insert(pop_uid);
        if (!p->pre_uid.is_null()) p->spike_senders.insert(p->pre_uid);
        if (!p->post_uid.is_null())
            if (Population *q = net->find_pop(p->post_uid)) q->impact_senders.insert(p->uid);
    }
    for (auto &[recv, send] : net->extra_subs)
    {
        if (Projection *p = net->find_proj(recv)) p->spike_senders.insert(send);
        if (Population *q = net->find_pop(recv)) q->impact_senders.insert(send);
    }
    net->initialized = true;
    net->pops0.clear();
    net->projs0.clear();
    return 0;
}

int or_snapshot(or_net *net)
{
    net->pops0.clear();
    net->projs0.clear();
    for (auto &p : net->pops) net->pops0.push_back(*p);
    for (auto &p : net->projs) net->projs0.push_back(*p);
    return 0;
}

int or_reset(or_net *net)
{
    if (net->pops0.size() != net->pops.size()) return fail("no snapshot to reset to");
    for (size_t i = 0; i < net->pops.size(); ++i) *net->pops[i] = net->pops0[i];
    for (size_t i = 0; i < net->projs.size(); ++i) *net->projs[i] = net->projs0[i];
    net->ext_spikes.clear();
    net->ext_impacts.clear();
    net->step = 0;
    net->events = 0;
    return 0;
}

int or_send_spikes(or_net *net, knp_uid sender, uint64_t send_time, uint32_t n, const uint32_t *idx)
{
    net->ext_spikes.push_back(SpikeMessage{Uid{sender}, send_time, std::vector<uint32_t>(idx, idx + n)});
    return 0;
}

int or_send_impacts(
    or_net *net, knp_uid sender, knp_uid receiver_pop, int is_forcing, uint32_t n, const uint32_t *post_idx,
    const float *value, const uint8_t *out_type)
{
    ImpactMessage m{Uid{sender}, net->step, Uid{knp_uid{}}, Uid{receiver_pop}, is_forcing != 0, {}};
    for (uint32_t i = 0; i < n; ++i)
        m.impacts.push_back(Impact{0, value[i], out_type ? out_type[i] : uint8_t(KNP_OUT_EXCITATORY), 0, post_idx[i]});
    net->ext_impacts.push_back(std::move(m));
    return 0;
}

// SingleThreadedCPUBackend::_step (backend.cpp:89-141): route, populations, route, projections, route.
int or_step(or_net *net)
{
    return guarded(
        [&]
        {
            if (!net->initialized) throw std::runtime_error("or_init was not called");
            const uint64_t step = net->step;
            // Route #1: external messages sent before this step.
            for (auto &m : net->ext_spikes)
                for (auto &p : net->projs)
                    if (p->spike_senders.count(m.sender)) p->inbox.push_back(m);
            for (auto &m : net->ext_impacts)
                for (auto &q : net->pops)
                    if (q->impact_senders.count(m.sender)) q->inbox.push_back(m);
            net->ext_spikes.clear();
            net->ext_impacts.clear();
            // Populations, in load order; their spike messages are routed after all of them ran.
            std::vector<SpikeMessage> sent;
            for (auto &q : net->pops)
            {
                calculate_population(*net, *q, step);
                if (!q->last_spikes.empty()) sent.push_back(SpikeMessage{q->uid, step, q->last_spikes});
            }
            for (auto &m : sent)  // Route #2.
                for (auto &p : net->projs)
                    if (p->spike_senders.count(m.sender)) p->inbox.push_back(m);
            // Projections, in load order.
            std::vector<ImpactMessage> out;
            for (auto &p : net->projs)
            {
                ImpactMessage m;
                if (calculate_projection(*net, *p, step, m)) out.push_back(std::move(m));
            }
            for (auto &m : out)  // Route #3: delivered to populations for the next step.
                for (auto &q : net->pops)
                    if (q->impact_senders.count(m.sender)) q->inbox.push_back(m);
            ++net->step;
            return 0;
        });
}

// MultiThreadedCPUBackend::_step (knp/backends/cpu/cpu-multi-threaded-backend/impl/backend.cpp:310-323),
// restated for timing the reference's multi-threaded CPU path: populations in parts of 1000 neurons
// (:77-200), one impact task per population (:101-118); every delta projection scans all of its
// synapses in parts of 1000 against the neuron->count map of its FIRST spike message only (:250-295,
// delta_impl.h:117-175) and merges impacts (weight x count) under one mutex. The MT backend has no
// additive STDP, and its spike order within a step is not deterministic.
int or_step_mt(or_net *net, int threads)
{
    return guarded(
        [&]
        {
            if (!net->initialized) throw std::runtime_error("or_init was not called");
            if (threads < 1) threads = 1;
            if (!net->pool || net->pool->size() != threads) net->pool = std::make_unique<ThreadPool>(threads);
            ThreadPool &pool = *net->pool;
            const uint64_t step = net->step;
            const size_t part = 1000;
            std::mutex merge;
            for (auto &m : net->ext_spikes)
                for (auto &p : net->projs)
                    if (p->spike_senders.count(m.sender)) p->inbox.push_back(m);
            for (auto &m : net->ext_impacts)
                for (auto &q : net->pops)
                    if (q->impact_senders.count(m.sender)) q->inbox.push_back(m);
            net->ext_spikes.clear();
            net->ext_impacts.clear();
            std::vector<std::vector<ImpactMessage>> msgs(net->pops.size());
            for (size_t k = 0; k < net->pops.size(); ++k)
            {
                Population &q = *net->pops[k];
                msgs[k] = std::move(q.inbox);
                q.inbox.clear();
                q.last_spikes.clear();
                check_impacts(q, msgs[k]);
                const size_t n = q.size();
                for (size_t a = 0; a < n; a += part)
                    pool.post(
                        [&q, a, n, part]
                        {
                            const size_t b = std::min(a + part, n);
                            for (size_t i = a; i < b; ++i) pre_impact(q, i);
                        });
            }
            pool.join();
            for (size_t k = 0; k < net->pops.size(); ++k)
                pool.post(
                    [&, k]
                    {
                        Population &q = *net->pops[k];
                        for (auto &m : msgs[k])
                            for (auto &imp : m.impacts) impact(q, imp, m.is_forcing);
                    });
            pool.join();
            for (auto &qp : net->pops)
            {
                Population &q = *qp;
                const size_t n = q.size();
                for (size_t a = 0; a < n; a += part)
                    pool.post(
                        [&q, a, n, part, &merge]
                        {
                            std::vector<uint32_t> local;
                            const size_t b = std::min(a + part, n);
                            for (size_t i = a; i < b; ++i)
                            {
                                if (post_impact(q, i)) local.push_back(static_cast<uint32_t>(i));
                            }
                            std::lock_guard<std::mutex> l(merge);
                            q.last_spikes.insert(q.last_spikes.end(), local.begin(), local.end());
                        });
            }
            pool.join();
            std::vector<SpikeMessage> sent;
            for (auto &q : net->pops)
            {
                train(*net, *q, step);
                if (!q->last_spikes.empty()) sent.push_back(SpikeMessage{q->uid, step, q->last_spikes});
            }
            for (auto &m : sent)
                for (auto &p : net->projs)
                    if (p->spike_senders.count(m.sender)) p->inbox.push_back(m);
            std::vector<std::unordered_map<uint64_t, size_t>> converted;
            converted.reserve(net->projs.size());
            std::vector<uint64_t> events(net->projs.size(), 0);
            for (size_t k = 0; k < net->projs.size(); ++k)
            {
                Projection &p = *net->projs[k];
                std::vector<SpikeMessage> in = std::move(p.inbox);
                p.inbox.clear();
                if (in.empty()) continue;
                converted.emplace_back();
                auto &counts = converted.back();
                for (uint32_t i : in[0].idx) ++counts[i];
                const size_t S = p.syn.size();
                for (size_t a = 0; a < S; a += part)
                    pool.post(
                        [&p, &counts, &merge, &events, k, a, S, part, step]
                        {
                            std::vector<std::pair<uint64_t, Impact>> container;
                            const size_t b = std::min(a + part, S);
                            for (size_t si = a; si < b; ++si)
                            {
                                const Synapse &s = p.syn[si];
                                auto it = counts.find(s.pre);
                                if (it == counts.end()) continue;
                                container.emplace_back(s.delay + step - 1,
                                                       Impact{si, s.weight * static_cast<float>(it->second), s.type,
                                                              s.pre, s.post});
                            }
                            std::lock_guard<std::mutex> l(merge);
                            events[k] += container.size();
                            for (auto &[key, imp] : container)
                            {
                                auto f = p.future.find(key);
                                if (f != p.future.end())
                                    f->second.impacts.push_back(imp);
                                else
                                    p.future.emplace(key, ImpactMessage{p.uid, step, p.post_uid, p.pre_uid, true, {imp}});
                            }
                        });
            }
            pool.join();
            std::vector<ImpactMessage> out;
            for (size_t k = 0; k < net->projs.size(); ++k)
            {
                Projection &p = *net->projs[k];
                net->events += events[k];
                auto it = p.future.find(step);
                if (it != p.future.end())
                {
                    out.push_back(std::move(it->second));
                    p.future.erase(it);
                }
            }
            for (auto &m : out)
                for (auto &q : net->pops)
                    if (q->impact_senders.count(m.sender)) q->inbox.push_back(m);
            ++net->step;
            return 0;
        });
}

uint64_t or_get_step(const or_net *net) { return net->step; }

int or_read_spikes(const or_net *net, knp_uid pop, uint32_t cap, uint32_t *out, uint32_t *n)
{
    const Population *q = net->find_pop(Uid{pop});
    if (!q) return fail("unknown population");
    *n = static_cast<uint32_t>(q->last_spikes.size());
    if (q->last_spikes.size() > cap) return fail("spike buffer too small");
    std::copy(q->last_spikes.begin(), q->last_spikes.end(), out);
    return 0;
}

int or_read_blifat(const or_net *net, knp_uid pop, knp_blifat_neuron *out, knp_resource_stdp_state *ext)
{
    const Population *q = net->find_pop(Uid{pop});
    if (!q || q->kind == KNP_NEURON_LIF || q->is_altai()) return fail("unknown BLIFAT population");
    std::copy(q->blifat.begin(), q->blifat.end(), out);
    if (ext && !q->res.empty()) std::copy(q->res.begin(), q->res.end(), ext);
    return 0;
}

int or_read_lif(const or_net *net, knp_uid pop, knp_lif_neuron *out)
{
    const Population *q = net->find_pop(Uid{pop});
    if (!q || q->kind != KNP_NEURON_LIF) return fail("unknown LIF population");
    std::copy(q->lif.begin(), q->lif.end(), out);
    return 0;
}

int or_read_weights(const or_net *net, knp_uid proj, float *out)
{
    const Projection *p = net->find_proj(Uid{proj});
    if (!p) return fail("unknown projection");
    for (size_t i = 0; i < p->syn.size(); ++i) out[i] = p->syn[i].weight;
    return 0;
}

uint64_t or_event_count(const or_net *net) { return net->events; }

}  // extern "C"
