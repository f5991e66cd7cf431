// bbfft::plan and bbfft::plan_unmanaged_event; mirror the reference's
// include/bbfft/plan.hpp:24-184 (same members and semantics; copies share the plan).
#ifndef BBFFT_GB300_PLAN_HPP
#define BBFFT_GB300_PLAN_HPP

#include "bbfft/detail/plan_impl.hpp"

#include <cstdint>
#include <memory>
#include <utility>
#include <vector>

namespace bbfft {

template <class Impl> class base_plan {
  public:
    base_plan() : impl_(nullptr) {}
    base_plan(std::shared_ptr<Impl> impl) : impl_(std::move(impl)) {}
    inline explicit operator bool() const noexcept { return bool(impl_); }

  protected:
    std::shared_ptr<Impl> impl_;
};

template <typename EventT> class plan : public base_plan<detail::plan_impl<EventT>> {
  public:
    using base_plan<detail::plan_impl<EventT>>::base_plan;
    using event_t = EventT;

    auto execute(void const *in, void *out) -> event_t { return this->impl_->execute(in, out); }
    auto execute(void const *in, void *out, event_t dep_event) -> event_t {
        return this->impl_->execute(in, out, std::move(dep_event));
    }
    auto execute(void const *in, void *out, std::vector<event_t> const &dep_events) -> event_t {
        return this->impl_->execute(in, out, dep_events);
    }
    auto execute(void *inout) -> event_t { return this->impl_->execute(inout, inout); }
    auto execute(void *inout, event_t dep_event) -> event_t {
        return this->impl_->execute(inout, inout, dep_event);
    }
    auto execute(void *inout, std::vector<event_t> const &dep_events) -> event_t {
        return this->impl_->execute(inout, inout, dep_events);
    }
};

template <typename EventT>
class plan_unmanaged_event : public base_plan<detail::plan_unmanaged_event_impl<EventT>> {
  public:
    using base_plan<detail::plan_unmanaged_event_impl<EventT>>::base_plan;
    using event_t = EventT;

    void execute(void const *in, void *out, event_t signal_event = nullptr,
                 std::uint32_t num_wait_events = 0, event_t *wait_events = nullptr) {
        this->impl_->execute(in, out, signal_event, num_wait_events, wait_events);
    }
    void execute(void *inout, event_t signal_event = nullptr, std::uint32_t num_wait_events = 0,
                 event_t *wait_events = nullptr) {
        this->impl_->execute(inout, inout, signal_event, num_wait_events, wait_events);
    }
};

} // namespace bbfft

#endif
