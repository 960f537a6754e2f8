// TEST INFRASTRUCTURE — stand-in for knp::core::UID (knp/core-library/include/knp/core/uid.h):
// 16 bytes, nil or pseudo-random, ordered, hashable.
#pragma once
#include <array>
#include <cstdint>
#include <cstring>
#include <functional>
#include <random>

namespace knp::core
{
struct UID
{
    explicit UID(bool random)
    {
        if (!random) return;
        static std::mt19937_64 gen(0x5EED5EEDull);
        const uint64_t a = gen(), b = gen();
        std::memcpy(tag.data(), &a, 8);
        std::memcpy(tag.data() + 8, &b, 8);
    }
    UID() : UID(true) {}
    explicit UID(const std::array<uint8_t, 16> &value) : tag(value) {}
    explicit operator bool() const
    {
        for (auto b : tag)
            if (b) return true;
        return false;
    }
    bool operator<(const UID &uid) const { return uid.tag < tag; }
    bool operator==(const UID &uid) const { return uid.tag == tag; }
    bool operator!=(const UID &uid) const { return uid.tag != tag; }
    std::array<uint8_t, 16> tag{};
};

struct uid_hash
{
    size_t operator()(const UID &uid) const
    {
        uint64_t a, b;
        std::memcpy(&a, uid.tag.data(), 8);
        std::memcpy(&b, uid.tag.data() + 8, 8);
        return static_cast<size_t>(a * 0x9E3779B97F4A7C15ull ^ b);
    }
};
}  // namespace knp::core
