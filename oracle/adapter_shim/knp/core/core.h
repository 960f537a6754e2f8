// TEST INFRASTRUCTURE — stand-in for knp/core-library/include/knp/core/core.h: the step type.
#pragma once
#include <cstdint>

#include <knp/core/uid.h>

namespace knp::core
{
using Step = uint64_t;
}  // namespace knp::core
