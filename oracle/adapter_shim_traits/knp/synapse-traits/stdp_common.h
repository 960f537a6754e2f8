// TEST INFRASTRUCTURE — stand-in for knp/synapse-traits-library/include/knp/synapse-traits/stdp_common.h.
#pragma once
#include "type_traits.h"

namespace knp::synapse_traits
{
template <template <typename> typename Rule, typename Synapse>
struct STDP;
template <template <typename> typename Rule, typename Synapse>
struct synapse_parameters<STDP<Rule, Synapse>> : public synapse_parameters<Synapse>
{
    using RuleType = Rule<Synapse>;
    using SynapseType = Synapse;
    RuleType rule_;
};
}  // namespace knp::synapse_traits
