// TEST INFRASTRUCTURE — empty stand-in for knp::core::MessageEndpoint (the oracle driver routes messages itself).
#pragma once
#include <knp/core/messaging/messaging.h>
namespace knp::core
{
class MessageEndpoint
{
};
}  // namespace knp::core
