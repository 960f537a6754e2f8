// Drives knp::backends::gb300::GB300Backend (knp_gb300/adapter) through the knp::core::Backend
// interface and its message bus, as the reference's backend tests drive a backend
// (knp/tests/backend/single_thread_cpu_test.cpp:54-176, tests_messaging_common.h:34-56): the
// one-neuron network input -> input projection (w 1.0, delay 1) -> population <-> loop projection
// (delta: w 1.1, delay 6; additive STDP: w 1.0, delay 6, tau {1, 1}, input tau {2, 2}, the population
// registered STDPAndSpike), input SpikeMessages on steps 0, 5, 10, 15 from an external endpoint, the
// population's SpikeMessages received on that endpoint. Also checks the interface queries, a type the
// backend does not take, external SynapticImpactMessages (lif_test.cpp:60-100 style) and
// get_network_data. Prints "steps: ..." (steps with output), "weights: ..." (loop and input weights
// after 20 steps, from get_network_data) and "ok".
//
// The resource_stdp case is single_thread_cpu_test.cpp:179-264: SynapticResourceSTDPDeltaSynapse input
// (rule {0, 1, 2, 0.1}) and loop (rule {0, 1, 2}, delay 6) projections onto one resource-STDP BLIFAT
// neuron (synaptic resource threshold 1, free resource 2, isi_max 0), start_learning after _init;
// it also prints the loop synapse's rule state from get_network_data ("rule: ...").
//
// Usage: harness delta|stdp|resource|resource_stdp|impacts|types
#include <cstdio>
#include <cstring>
#include <optional>
#include <string>
#include <vector>

#include "knp_gb300_backend.h"

using knp::backends::gb300::GB300Backend;
using knp::core::UID;
using knp::core::messaging::SpikeMessage;
namespace nt = knp::neuron_traits;
namespace st = knp::synapse_traits;

// Inside lambdas (which cannot return the harness's status): record the failure.
static bool failed = false;
#define EXPECT_VOID(c)                                                            \
    do                                                                            \
    {                                                                             \
        if (!(c))                                                                 \
        {                                                                         \
            std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
            failed = true;                                                        \
        }                                                                         \
    } while (0)

#define EXPECT(c)                                                  \
    do                                                             \
    {                                                              \
        if (!(c))                                                  \
        {                                                          \
            std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
            return 1;                                              \
        }                                                          \
    } while (0)

template <class Proj>
Proj one_synapse(const UID &pre, const UID &post, float w, uint32_t d, float tau)
{
    return Proj(pre, post,
                [w, d, tau](size_t) -> std::optional<typename Proj::Synapse>
                {
                    typename Proj::SynapseParameters p{};
                    p.weight_ = w;
                    p.delay_ = d;
                    p.output_type_ = st::OutputType::EXCITATORY;
                    if constexpr (!std::is_same_v<Proj, GB300Backend::DeltaProjection>)
                    {
                        p.rule_.tau_plus_ = tau;
                        p.rule_.tau_minus_ = tau;
                    }
                    return typename Proj::Synapse{p, 0, 0};
                },
                1);
}

int run_golden(const std::string &kind)
{
    GB300Backend backend;
    EXPECT(backend.plasticity_supported());
    EXPECT(backend.get_supported_neurons().size() == 5);
    EXPECT(backend.get_supported_population_indexes().size() == 5);
    EXPECT(backend.get_supported_projection_indexes().size() == 3);
    EXPECT(backend.get_supported_synapses().size() == 3);

    std::vector<knp::core::AllPopulationsVariant> pops;
    UID pop_uid;
    if (kind == "resource_stdp")
    {
        GB300Backend::ResourceBLIFATPopulation pop(
            [](size_t)
            {
                nt::neuron_parameters<nt::SynapticResourceSTDPBLIFATNeuron> n{};
                n.synaptic_resource_threshold_ = 1;
                n.free_synaptic_resource_ = 2;
                n.isi_max_ = 0;
                return std::make_optional(n);
            },
            1);
        pop_uid = pop.get_uid();
        pops.emplace_back(pop);
    }
    else if (kind == "resource")
    {
        GB300Backend::ResourceBLIFATPopulation pop(
            [](size_t) { return std::make_optional(nt::neuron_parameters<nt::SynapticResourceSTDPBLIFATNeuron>{}); }, 1);
        pop_uid = pop.get_uid();
        pops.emplace_back(pop);
    }
    else
    {
        GB300Backend::BLIFATPopulation pop([](size_t) { return std::make_optional(nt::neuron_parameters<nt::BLIFATNeuron>{}); },
                                           1);
        pop_uid = pop.get_uid();
        pops.emplace_back(pop);
    }
    std::vector<knp::core::AllProjectionsVariant> projs;
    UID input_uid, loop_uid;
    if (kind == "delta")
    {
        auto input = one_synapse<GB300Backend::DeltaProjection>(UID{false}, pop_uid, 1.0f, 1, 0);
        auto loop = one_synapse<GB300Backend::DeltaProjection>(pop_uid, pop_uid, 1.1f, 6, 0);
        input_uid = input.get_uid();
        loop_uid = loop.get_uid();
        projs.emplace_back(input);
        projs.emplace_back(loop);
    }
    else if (kind == "resource_stdp")
    {
        using RP = GB300Backend::ResourceSTDPProjection;
        auto make = [](const UID &pre, const UID &post, uint32_t d, float d_u)
        {
            return RP(pre, post,
                      [d, d_u](size_t) -> std::optional<RP::Synapse>
                      {
                          RP::SynapseParameters p{};
                          p.weight_ = 1.0f;
                          p.delay_ = d;
                          p.output_type_ = st::OutputType::EXCITATORY;
                          p.rule_.synaptic_resource_ = 0;
                          p.rule_.w_min_ = 1;
                          p.rule_.w_max_ = 2;
                          p.rule_.d_u_ = d_u;
                          return RP::Synapse{p, 0, 0};
                      },
                      1);
        };
        auto input = make(UID{false}, pop_uid, 1, 0.1f);
        auto loop = make(pop_uid, pop_uid, 6, 0.0f);
        input_uid = input.get_uid();
        loop_uid = loop.get_uid();
        projs.emplace_back(input);
        projs.emplace_back(loop);
    }
    else
    {
        auto input = one_synapse<GB300Backend::AdditiveSTDPProjection>(UID{false}, pop_uid, 1.0f, 1, 2);
        auto loop = one_synapse<GB300Backend::AdditiveSTDPProjection>(pop_uid, pop_uid, 1.0f, 6, 1);
        using Processing = GB300Backend::AdditiveSTDPProjection::SharedSynapseParameters::ProcessingType;
        loop.get_shared_parameters().stdp_populations_[pop_uid] = Processing::STDPAndSpike;
        input_uid = input.get_uid();
        loop_uid = loop.get_uid();
        projs.emplace_back(input);
        projs.emplace_back(loop);
    }
    backend.load_all_populations(pops);
    backend.load_all_projections(projs);
    backend._init();
    if (kind == "resource_stdp") backend.start_learning();
    auto endpoint = backend.get_message_bus().create_endpoint();
    const UID in_channel_uid, out_channel_uid;
    backend.subscribe<SpikeMessage>(input_uid, {in_channel_uid});
    endpoint.subscribe<SpikeMessage>(out_channel_uid, {pop_uid});

    std::printf("steps:");
    for (knp::core::Step step = 0; step < 20; ++step)
    {
        if (step % 5 == 0) endpoint.send_message(SpikeMessage{{in_channel_uid, 0}, {0}});
        backend._step();
        endpoint.receive_all_messages();
        auto out = endpoint.unload_messages<SpikeMessage>(out_channel_uid);
        if (!out.empty())
        {
            EXPECT(out.size() == 1 && out[0].header_.sender_uid_ == pop_uid && out[0].header_.send_time_ == step);
            EXPECT(out[0].neuron_indexes_ == std::vector<uint32_t>{0});
            std::printf(" %llu", static_cast<unsigned long long>(step));
        }
    }
    std::printf("\n");
    EXPECT(backend.get_step() == 20);

    // Network data: two projections (weights after the run), one population.
    auto data = backend.get_network_data();
    std::vector<float> weights;
    size_t n_proj = 0, n_pop = 0;
    for (auto &it = *data.projection_range.first; it != *data.projection_range.second; ++it)
    {
        ++n_proj;
        std::visit(
            [&](const auto &p)
            {
                using T = std::decay_t<decltype(p)>;
                weights.push_back(std::get<knp::core::synapse_data>(p[0]).weight_);
                if constexpr (std::is_same_v<T, GB300Backend::ResourceSTDPProjection>)
                {
                    EXPECT_VOID(!p.is_locked());
                    if (p.get_uid() == loop_uid)
                    {
                        const auto &r = std::get<knp::core::synapse_data>(p[0]).rule_;
                        std::printf("rule: %.9g %llu %d %d\n", r.synaptic_resource_,
                                    static_cast<unsigned long long>(r.last_spike_step_), r.had_hebbian_update_ ? 1 : 0,
                                    r.has_contributed_ ? 1 : 0);
                    }
                }
            },
            *it);
    }
    EXPECT(!failed);
    for (auto &it = *data.population_range.first; it != *data.population_range.second; ++it)
    {
        ++n_pop;
        const UID u = std::visit([](const auto &p) { return p.get_uid(); }, *it);
        EXPECT(u == pop_uid);
    }
    EXPECT(n_proj == 2 && n_pop == 1);
    std::printf("weights: %.9g %.9g\n", weights[1], weights[0]);
    return 0;
}

// External SynapticImpactMessages to a LIF population (lif_test.cpp:60-100): one impact per step.
int run_impacts()
{
    GB300Backend backend;
    GB300Backend::LIFPopulation pop([](size_t) { return std::make_optional(nt::neuron_parameters<nt::LIFNeuron>{}); }, 1);
    const UID pop_uid = pop.get_uid();
    backend.load_all_populations({pop});
    backend.load_all_projections({});
    backend._init();
    auto endpoint = backend.get_message_bus().create_endpoint();
    const UID in_uid, out_uid;
    backend.subscribe<knp::core::messaging::SynapticImpactMessage>(pop_uid, {in_uid});
    endpoint.subscribe<SpikeMessage>(out_uid, {pop_uid});
    const float impacts[] = {0.5f, 0.6f, 0.2f, 0.9f, 0.1f, 1.5f};
    std::printf("steps:");
    for (knp::core::Step step = 0; step < 6; ++step)
    {
        knp::core::messaging::SynapticImpactMessage m{{in_uid, step}, UID{false}, pop_uid, false, {}};
        m.impacts_.push_back({0, impacts[step], st::OutputType::EXCITATORY, 0, 0});
        endpoint.send_message(m);
        backend._step();
        endpoint.receive_all_messages();
        if (!endpoint.unload_messages<SpikeMessage>(out_uid).empty())
            std::printf(" %llu", static_cast<unsigned long long>(step));
    }
    std::printf("\n");
    return 0;
}

int main(int argc, char **argv)
{
    const std::string kind = argc > 1 ? argv[1] : "delta";
    try
    {
        if (kind == "types")
        {
            // The single-threaded backend's neuron and synapse lists (cpu-single-threaded/backend.h:58-68),
            // every population and projection type of the core variants accepted, without a GPU.
            GB300Backend backend;
            EXPECT(backend.get_supported_neurons() ==
                   (std::vector<std::string>{"BLIFATNeuron", "SynapticResourceSTDPBLIFATNeuron", "AltAILIF",
                                             "SynapticResourceSTDPAltAILIFNeuron", "LIFNeuron"}));
            EXPECT(backend.get_supported_synapses() ==
                   (std::vector<std::string>{"DeltaSynapse", "AdditiveSTDPDeltaSynapse", "SynapticResourceSTDPDeltaSynapse"}));
            EXPECT(backend.get_supported_population_indexes().size() ==
                   std::variant_size_v<knp::core::AllPopulationsVariant>);
            EXPECT(backend.get_supported_projection_indexes().size() ==
                   std::variant_size_v<knp::core::AllProjectionsVariant>);
            knp::core::Population<nt::AltAILIF> p(
                [](size_t) { return std::make_optional(nt::neuron_parameters<nt::AltAILIF>{}); }, 1);
            backend.load_all_populations({p});
            std::printf("ok\n");
            return 0;
        }
        const int rc = kind == "impacts" ? run_impacts() : run_golden(kind);
        if (rc == 0) std::printf("ok\n");
        return rc;
    }
    catch (const std::exception &e)
    {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 2;
    }
}
