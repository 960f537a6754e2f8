// TEST INFRASTRUCTURE — stand-in for knp::core::Device (knp/core-library/include/knp/core/device.h).
#pragma once
#include <string>

#include <knp/core/uid.h>

namespace knp::core
{
class Device
{
public:
    virtual ~Device() = default;
    [[nodiscard]] virtual const std::string &get_name() const = 0;
};
}  // namespace knp::core
