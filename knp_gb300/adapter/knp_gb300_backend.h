/*
 * GB300Backend: the KNP backend plugin (knp::core::Backend, knp/core-library/include/knp/core/
 * backend.h:55-457) over the GB300 backend's C ABI (include/knp_gb300.h).
 *
 * A KNP maintainer builds this file inside the KNP tree as the shared library of a backend
 * (libknp-gb300-backend.so, linked with knp_gb300/libknp_gb300.so) and exports the factory as the
 * other backends do:
 *     BOOST_DLL_ALIAS(knp::backends::gb300::GB300Backend::create, create_knp_backend)
 * (the single-threaded backend: knp/backends/cpu/cpu-single-threaded-backend/impl/backend.cpp:340),
 * which BackendLoader::load resolves (knp/base-framework/impl/backend_loader.cpp:34-77). The
 * export line is the only Boost-dependent line and is compiled only where Boost is available.
 *
 * It keeps the single-threaded backend's behaviour: the same supported neuron and synapse types
 * (BLIFAT, AltAI-LIF and their synaptic-resource-STDP variants, LIF; delta, additive-STDP delta and
 * synaptic-resource-STDP delta), the same message
 * semantics on the backend's bus (SpikeMessages sent to a projection's UID reach that projection
 * at the next step; SynapticImpactMessages sent to a population's UID are applied at the next
 * step; each population that spiked sends its SpikeMessage {population UID, step, ascending
 * indexes}), and the same step order (_step: route, receive, populations, projections, route).
 * Everything between the backend's own populations and projections stays on the GPU.
 */
#pragma once

#include <knp/core/backend.h>
#include <knp/core/population.h>
#include <knp/core/projection.h>
#include <knp/neuron-traits/altai_lif.h>
#include <knp/neuron-traits/blifat.h>
#include <knp/neuron-traits/lif.h>
#include <knp/neuron-traits/stdp_type_traits.h>
#include <knp/synapse-traits/delta.h>
#include <knp/synapse-traits/stdp_type_traits.h>

#include <memory>
#include <string>
#include <unordered_map>
#include <variant>
#include <vector>

#include "knp_gb300.h"

namespace knp::backends::gb300
{

class GB300Backend : public knp::core::Backend
{
public:
    using BLIFATPopulation = knp::core::Population<knp::neuron_traits::BLIFATNeuron>;
    using ResourceBLIFATPopulation = knp::core::Population<knp::neuron_traits::SynapticResourceSTDPBLIFATNeuron>;
    using LIFPopulation = knp::core::Population<knp::neuron_traits::LIFNeuron>;
    using AltAIPopulation = knp::core::Population<knp::neuron_traits::AltAILIF>;
    using ResourceAltAIPopulation = knp::core::Population<knp::neuron_traits::SynapticResourceSTDPAltAILIFNeuron>;
    using DeltaProjection = knp::core::Projection<knp::synapse_traits::DeltaSynapse>;
    using AdditiveSTDPProjection = knp::core::Projection<knp::synapse_traits::AdditiveSTDPDeltaSynapse>;
    using ResourceSTDPProjection = knp::core::Projection<knp::synapse_traits::SynapticResourceSTDPDeltaSynapse>;
    /** The population and projection types this backend runs (the single-threaded backend's set). */
    using PopulationVariants = std::variant<BLIFATPopulation, ResourceBLIFATPopulation, AltAIPopulation,
                                            ResourceAltAIPopulation, LIFPopulation>;
    using ProjectionVariants = std::variant<DeltaProjection, AdditiveSTDPProjection, ResourceSTDPProjection>;

    /** A backend on CUDA device `device`; the device backend (knp_gb300_create) is created at first
     * use (init, or a learning switch), so constructing and loading need no GPU. */
    explicit GB300Backend(int device = 0);
    ~GB300Backend() override;
    /** The factory exported as create_knp_backend. */
    static std::shared_ptr<GB300Backend> create();

    [[nodiscard]] bool plasticity_supported() const override { return true; }
    [[nodiscard]] std::vector<std::string> get_supported_neurons() const override;
    [[nodiscard]] std::vector<std::string> get_supported_synapses() const override;
    [[nodiscard]] std::vector<size_t> get_supported_population_indexes() const override;
    [[nodiscard]] std::vector<size_t> get_supported_projection_indexes() const override;

    /** Copies supported projections; any other type throws "Type is not supported." as
     * knp::meta::load_from_container does (knp/meta-library/include/knp/meta/variant_helpers.h:67). */
    void load_all_projections(const std::vector<knp::core::AllProjectionsVariant> &projections) override;
    void load_all_populations(const std::vector<knp::core::AllPopulationsVariant> &populations) override;
    void load_populations(const std::vector<PopulationVariants> &populations);
    void load_projections(const std::vector<ProjectionVariants> &projections);
    /** No-ops, as in the single-threaded backend. */
    void remove_projections(const std::vector<knp::core::UID> &) override {}
    void remove_populations(const std::vector<knp::core::UID> &) override {}
    [[nodiscard]] std::vector<std::unique_ptr<knp::core::Device>> get_devices() const override;

    void stop_learning() override;
    void start_learning() override;

    /** Copies of the loaded populations and projections with their current state read back from the
     * GPU (neuron state; projection weights in the loaded synapse order; the rule state of
     * synaptic-resource-STDP synapses; the lock flag of every projection). The additive-STDP spike
     * time lists of a synapse keep their loaded contents: the GPU keeps one history per
     * postsynaptic neuron, not per synapse. */
    [[nodiscard]] DataRanges get_network_data() const override;

    /** Uploads the network (knp_gb300_load_* for every population and projection, the STDP
     * population maps), enables spike recording for every population and builds the device network
     * (knp_gb300_init). */
    void _init() override;
    /** One step: route and receive the bus's messages; hand this step's external SpikeMessages to
     * their projections and SynapticImpactMessages to their populations; run the step on the GPU;
     * send each population's SpikeMessage; route again; advance the step number. */
    void _step() override;

    /** The C-ABI handle (for callers that mix this interface with the C ABI); created on first use. */
    [[nodiscard]] knp_gb300_backend *handle();

private:
    void check(int rc, const char *what) const;
    int device_ = 0;
    knp_gb300_backend *h_ = nullptr;
    std::vector<PopulationVariants> populations_;
    std::vector<ProjectionVariants> projections_;
    bool initialized_ = false;
    // The last start_learning / stop_learning: every projection's lock flag follows it.
    bool learning_known_ = false, learning_ = false;
    // External messages reach the C ABI through one input channel per projection (spikes) and one
    // per population (impacts), subscribed at _init.
    std::unordered_map<knp::core::UID, knp::core::UID, knp::core::uid_hash> spike_channel_, impact_channel_;
};

}  // namespace knp::backends::gb300
