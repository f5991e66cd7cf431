// Plan implementation interfaces; mirror the reference's include/bbfft/detail/plan_impl.hpp:21-63.
#ifndef BBFFT_GB300_PLAN_IMPL_HPP
#define BBFFT_GB300_PLAN_IMPL_HPP

#include <cstdint>
#include <utility>
#include <vector>

namespace bbfft::detail {

template <typename EventT> class plan_impl {
  public:
    using event_t = EventT;
    virtual ~plan_impl() {}
    virtual auto execute(void const *in, void *out) -> event_t {
        return execute(in, out, std::vector<event_t>{});
    }
    virtual auto execute(void const *in, void *out, event_t dep_event) -> event_t {
        return execute(in, out, std::vector<event_t>{std::move(dep_event)});
    }
    virtual auto execute(void const *in, void *out, std::vector<event_t> const &dep_events)
        -> event_t = 0;
};

template <typename EventT> class plan_unmanaged_event_impl {
  public:
    using event_t = EventT;
    virtual ~plan_unmanaged_event_impl() {}
    virtual void execute(void const *in, void *out, event_t signal_event,
                         std::uint32_t num_wait_events, event_t *wait_events) = 0;
};

} // namespace bbfft::detail

#endif
