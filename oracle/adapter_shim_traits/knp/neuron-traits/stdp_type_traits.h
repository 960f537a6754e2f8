// TEST INFRASTRUCTURE — stand-in for knp/neuron-traits-library/include/knp/neuron-traits/stdp_type_traits.h.
#pragma once
#include "altai_lif.h"
#include "blifat.h"
#include "stdp_synaptic_resource_rule.h"

namespace knp::neuron_traits
{
using SynapticResourceSTDPBLIFATNeuron = SynapticResourceSTDPNeuron<BLIFATNeuron>;
using SynapticResourceSTDPAltAILIFNeuron = SynapticResourceSTDPNeuron<AltAILIF>;
}  // namespace knp::neuron_traits
