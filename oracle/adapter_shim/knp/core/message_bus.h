// TEST INFRASTRUCTURE — the stand-in MessageBus is declared beside the endpoint.
#pragma once
#include <knp/core/message_endpoint.h>
