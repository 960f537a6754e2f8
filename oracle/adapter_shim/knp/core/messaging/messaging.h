// TEST INFRASTRUCTURE — stand-ins for the KNP message types with the reference's field names and order
// (knp/core-library/include/knp/core/messaging/{message_header,spike_message,synaptic_impact_message,
// messaging}.h).
#pragma once
#include <cstdint>
#include <variant>
#include <vector>

#include <knp/core/core.h>
#include <knp/synapse-traits/output_types.h>

namespace knp::core::messaging
{
struct MessageHeader
{
    knp::core::UID sender_uid_;
    knp::core::Step send_time_;
};

using SpikeIndex = uint32_t;
using SpikeData = std::vector<SpikeIndex>;

struct SpikeMessage
{
    MessageHeader header_;
    SpikeData neuron_indexes_;
};

struct SynapticImpact
{
    uint64_t connection_index_;
    float impact_value_;
    knp::synapse_traits::OutputType synapse_type_;
    uint32_t presynaptic_neuron_index_;
    uint32_t postsynaptic_neuron_index_;
};

struct SynapticImpactMessage
{
    MessageHeader header_;
    knp::core::UID presynaptic_population_uid_;
    knp::core::UID postsynaptic_population_uid_;
    bool is_forcing_ = false;
    std::vector<SynapticImpact> impacts_;
};

using MessageVariant = std::variant<SpikeMessage, SynapticImpactMessage>;
}  // namespace knp::core::messaging
