// TEST INFRASTRUCTURE — stand-in for knp::core::Backend (knp/core-library/include/knp/core/backend.h:
// 55-457): the same pure virtual interface (the operations a backend plugin implements) and the base
// services a backend's _step uses (its message bus and endpoint, the step counter, start/stop).
#pragma once
#include <atomic>
#include <functional>
#include <memory>
#include <set>
#include <string>
#include <utility>
#include <vector>

#include <knp/core/core.h>
#include <knp/core/device.h>
#include <knp/core/message_bus.h>
#include <knp/core/population.h>
#include <knp/core/projection.h>

namespace knp::core
{
class Backend
{
public:
    using RunPredicate = std::function<bool(knp::core::Step)>;
    virtual ~Backend() = default;

    [[nodiscard]] virtual bool plasticity_supported() const = 0;
    [[nodiscard]] virtual std::vector<std::string> get_supported_neurons() const = 0;
    [[nodiscard]] virtual std::vector<std::string> get_supported_synapses() const = 0;
    [[nodiscard]] virtual std::vector<size_t> get_supported_population_indexes() const = 0;
    [[nodiscard]] virtual std::vector<size_t> get_supported_projection_indexes() const = 0;
    virtual void load_all_projections(const std::vector<AllProjectionsVariant> &projections) = 0;
    virtual void load_all_populations(const std::vector<AllPopulationsVariant> &populations) = 0;
    virtual void remove_projections(const std::vector<UID> &uids) = 0;
    virtual void remove_populations(const std::vector<UID> &uids) = 0;
    [[nodiscard]] virtual std::vector<std::unique_ptr<Device>> get_devices() const = 0;

    template <typename MessageType>
    Subscription<MessageType> &subscribe(const UID &receiver, const std::vector<UID> &senders)
    {
        return message_endpoint_.subscribe<MessageType>(receiver, senders);
    }
    [[nodiscard]] MessageBus &get_message_bus() { return *message_bus_; }
    [[nodiscard]] const MessageBus &get_message_bus() const { return *message_bus_; }
    [[nodiscard]] virtual const core::MessageEndpoint &get_message_endpoint() const { return message_endpoint_; }
    [[nodiscard]] virtual core::MessageEndpoint &get_message_endpoint() { return message_endpoint_; }

    void start()
    {
        pre_start();
        while (started_) _step();
    }
    void start(const RunPredicate &pre_step, const RunPredicate &post_step)
    {
        pre_start();
        while (started_)
        {
            if (pre_step && !pre_step(get_step())) break;
            _step();
            if (post_step && !post_step(get_step())) break;
        }
        started_ = false;
    }
    void start(const RunPredicate &run_predicate) { start(run_predicate, RunPredicate{}); }
    void stop() { started_ = false; }
    [[nodiscard]] core::Step get_step() const { return step_; }
    virtual void stop_learning() = 0;
    virtual void start_learning() = 0;
    [[nodiscard]] bool running() const { return started_; }

    virtual void _init() = 0;
    virtual void _step() = 0;
    virtual void _uninit() {}

    template <class Type>
    class BaseValueIterator
    {
    public:
        BaseValueIterator() = default;
        using iterator_category = std::input_iterator_tag;
        using value_type = Type;
        virtual Type operator*() const = 0;
        virtual BaseValueIterator &operator++() = 0;
        virtual bool operator==(const BaseValueIterator &rhs) const = 0;
        virtual bool operator!=(const BaseValueIterator &rhs) const { return !(*this == rhs); }
        virtual ~BaseValueIterator() = default;
    };

    struct DataRanges
    {
        std::pair<std::unique_ptr<BaseValueIterator<AllProjectionsVariant>>,
                  std::unique_ptr<BaseValueIterator<AllProjectionsVariant>>>
            projection_range;
        std::pair<std::unique_ptr<BaseValueIterator<AllPopulationsVariant>>,
                  std::unique_ptr<BaseValueIterator<AllPopulationsVariant>>>
            population_range;
    };
    [[nodiscard]] virtual DataRanges get_network_data() const = 0;

protected:
    Backend() : message_bus_(MessageBus::construct_bus()), message_endpoint_(message_bus_->create_endpoint()) {}
    core::Step gad_step() { return step_++; }

private:
    void pre_start()
    {
        if (!initialized_)
        {
            _init();
            initialized_ = true;
        }
        started_ = true;
    }
    bool initialized_ = false;
    std::atomic<bool> started_ = false;
    std::shared_ptr<MessageBus> message_bus_;
    MessageEndpoint message_endpoint_;
    core::Step step_ = 0;
};
}  // namespace knp::core
