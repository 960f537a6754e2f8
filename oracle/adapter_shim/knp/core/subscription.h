// TEST INFRASTRUCTURE — stand-in for knp::core::Subscription (knp/core-library/include/knp/core/
// subscription.h): a receiver, its senders and the messages received from them.
#pragma once
#include <iterator>
#include <unordered_set>
#include <vector>

#include <knp/core/uid.h>

namespace knp::core
{
template <class MessageT>
class Subscription final
{
public:
    using MessageType = MessageT;
    using MessageContainerType = std::vector<MessageType>;
    using UidSet = std::unordered_set<knp::core::UID, knp::core::uid_hash>;
    Subscription(const UID &receiver, const std::vector<UID> &senders) : receiver_(receiver) { add_senders(senders); }
    [[nodiscard]] const UidSet &get_senders() const { return senders_; }
    [[nodiscard]] UID get_receiver_uid() const { return receiver_; }
    size_t add_sender(const UID &uid) { return senders_.insert(uid).second; }
    size_t add_senders(const std::vector<UID> &senders)
    {
        const size_t before = senders_.size();
        std::copy(senders.begin(), senders.end(), std::inserter(senders_, senders_.end()));
        return senders_.size() - before;
    }
    [[nodiscard]] bool has_sender(const UID &uid) const { return senders_.count(uid) != 0; }
    void add_message(const MessageType &message) { messages_.push_back(message); }
    MessageContainerType &get_messages() { return messages_; }
    const MessageContainerType &get_messages() const { return messages_; }

private:
    UID receiver_;
    UidSet senders_;
    MessageContainerType messages_;
};
}  // namespace knp::core
