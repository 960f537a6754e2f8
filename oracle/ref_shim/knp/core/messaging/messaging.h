// TEST INFRASTRUCTURE — minimal stand-ins for the KNP message types, with the reference's field names
// and order (knp/core-library/include/knp/core/messaging/{message_header,spike_message,
// synaptic_impact_message}.h) and a 16-byte UID (knp/core-library/include/knp/core/uid.h).
#pragma once
#include <array>
#include <cstdint>
#include <cstring>
#include <vector>

#include <knp/synapse-traits/output_types.h>

namespace knp::core
{
using Step = uint64_t;

struct UID
{
    std::array<uint8_t, 16> tag{};
    UID() = default;
    explicit UID(bool) {}
    explicit operator bool() const
    {
        for (auto b : tag)
            if (b) return true;
        return false;
    }
    bool operator==(const UID &o) const { return tag == o.tag; }
    bool operator!=(const UID &o) const { return !(*this == o); }
};

struct uid_hash
{
    size_t operator()(const UID &u) const
    {
        uint64_t a, b;
        std::memcpy(&a, u.tag.data(), 8);
        std::memcpy(&b, u.tag.data() + 8, 8);
        return static_cast<size_t>(a * 0x9E3779B97F4A7C15ull ^ b);
    }
};
}  // namespace knp::core

namespace knp::core::messaging
{
struct MessageHeader
{
    knp::core::UID sender_uid_;
    Step send_time_;
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
    UID presynaptic_population_uid_;
    UID postsynaptic_population_uid_;
    bool is_forcing_ = false;
    std::vector<SynapticImpact> impacts_;
};
}  // namespace knp::core::messaging
