// TEST INFRASTRUCTURE — stand-ins for knp::core::MessageEndpoint and knp::core::MessageBus
// (knp/core-library/include/knp/core/{message_endpoint,message_bus}.h) with the reference's
// delivery order: every message sent through any endpoint of a bus reaches every endpoint of the bus
// in send order (route_messages), and each endpoint files it under the subscriptions of its type
// that list its sender (receive_all_messages); unload_messages hands a receiver its messages.
#pragma once
#include <deque>
#include <map>
#include <memory>
#include <utility>
#include <variant>
#include <vector>

#include <knp/core/messaging/messaging.h>
#include <knp/core/subscription.h>

namespace knp::core
{
class MessageBus;

namespace detail
{
struct BusState
{
    std::vector<messaging::MessageVariant> outbox;  // sent, not yet routed
    std::vector<std::deque<messaging::MessageVariant> *> inboxes;
};
}  // namespace detail

class MessageEndpoint
{
public:
    using SubscriptionVariant =
        std::variant<Subscription<messaging::SpikeMessage>, Subscription<messaging::SynapticImpactMessage>>;
    using SubscriptionContainer = std::map<std::pair<size_t, UID>, SubscriptionVariant>;

    template <typename Variant, typename Type>
    static constexpr size_t type_index()
    {
        if constexpr (std::is_same_v<std::variant_alternative_t<0, Variant>, Type>)
            return 0;
        else
            return 1;
    }

    MessageEndpoint(MessageEndpoint &&) noexcept = default;
    MessageEndpoint &operator=(const MessageEndpoint &) = delete;
    virtual ~MessageEndpoint()
    {
        if (!bus_) return;
        for (auto &p : bus_->inboxes)
            if (p == inbox_.get()) p = nullptr;
    }

    template <typename MessageType>
    Subscription<MessageType> &subscribe(const UID &receiver, const std::vector<UID> &senders)
    {
        constexpr size_t index = type_index<messaging::MessageVariant, MessageType>();
        auto key = std::make_pair(index, receiver);
        auto it = subscriptions_.find(key);
        if (it == subscriptions_.end())
            it = subscriptions_.emplace(key, Subscription<MessageType>(receiver, senders)).first;
        else
            std::get<Subscription<MessageType>>(it->second).add_senders(senders);
        return std::get<Subscription<MessageType>>(it->second);
    }

    void send_message(const messaging::MessageVariant &message) { bus_->outbox.push_back(message); }

    size_t receive_all_messages()
    {
        size_t n = 0;
        while (!inbox_->empty())
        {
            const messaging::MessageVariant m = std::move(inbox_->front());
            inbox_->pop_front();
            ++n;
            std::visit(
                [this](const auto &msg)
                {
                    using M = std::decay_t<decltype(msg)>;
                    constexpr size_t index = type_index<messaging::MessageVariant, M>();
                    for (auto &[key, sub] : subscriptions_)
                    {
                        if (key.first != index) continue;
                        auto &s = std::get<Subscription<M>>(sub);
                        if (s.has_sender(msg.header_.sender_uid_)) s.add_message(msg);
                    }
                },
                m);
        }
        return n;
    }

    template <class MessageType>
    std::vector<MessageType> unload_messages(const UID &receiver_uid)
    {
        constexpr size_t index = type_index<messaging::MessageVariant, MessageType>();
        auto it = subscriptions_.find(std::make_pair(index, receiver_uid));
        if (it == subscriptions_.end()) return {};
        auto &msgs = std::get<Subscription<MessageType>>(it->second).get_messages();
        std::vector<MessageType> out = std::move(msgs);
        msgs.clear();
        return out;
    }

    const SubscriptionContainer &get_endpoint_subscriptions() const { return subscriptions_; }

private:
    friend class MessageBus;
    explicit MessageEndpoint(std::shared_ptr<detail::BusState> bus)
        : bus_(std::move(bus)), inbox_(std::make_unique<std::deque<messaging::MessageVariant>>())
    {
        bus_->inboxes.push_back(inbox_.get());
    }
    std::shared_ptr<detail::BusState> bus_;
    std::unique_ptr<std::deque<messaging::MessageVariant>> inbox_;
    SubscriptionContainer subscriptions_;
};

class MessageBus
{
public:
    static std::shared_ptr<MessageBus> construct_bus() { return std::shared_ptr<MessageBus>(new MessageBus()); }
    [[nodiscard]] MessageEndpoint create_endpoint() { return MessageEndpoint(state_); }
    size_t route_messages()
    {
        std::vector<messaging::MessageVariant> out = std::move(state_->outbox);
        state_->outbox.clear();
        for (auto &m : out)
            for (auto *box : state_->inboxes)
                if (box) box->push_back(m);
        return out.size();
    }

private:
    MessageBus() : state_(std::make_shared<detail::BusState>()) {}
    std::shared_ptr<detail::BusState> state_;
};
}  // namespace knp::core
