// TEST INFRASTRUCTURE — stand-in for knp/synapse-traits-library/include/knp/synapse-traits/stdp_type_traits.h.
#pragma once
#include "delta.h"
#include "stdp_add_rule.h"
#include "stdp_synaptic_resource_rule.h"

namespace knp::synapse_traits
{
using AdditiveSTDPDeltaSynapse = STDP<STDPAdditiveRule, DeltaSynapse>;
using SynapticResourceSTDPDeltaSynapse = STDP<STDPSynapticResourceRule, DeltaSynapse>;
}  // namespace knp::synapse_traits
