// bbfft::make_plan for CUDA streams on GB300.
// Replaces the reference's backend overloads (include/bbfft/sycl/make_plan.hpp:27,40,
// cl/make_plan.hpp:27,40, ze/make_plan.hpp:29) with one taking a cudaStream_t:
//   plan<cudaEvent_t> p = make_plan(cfg, stream[, cache]);
//   cudaEvent_t done = p.execute(in, out[, deps]);   // caller destroys `done`
// and the unmanaged-event form of the Level Zero backend:
//   plan_unmanaged_event<cudaEvent_t> q = make_plan_unmanaged(cfg, stream[, cache]);
//   q.execute(in, out, signal, n_wait, wait);        // caller owns all events
#ifndef BBFFT_GB300_CUDA_MAKE_PLAN_HPP
#define BBFFT_GB300_CUDA_MAKE_PLAN_HPP

#include "bbfft/configuration.hpp"
#include "bbfft/jit_cache.hpp"
#include "bbfft/plan.hpp"
#include "bbfft_gb300.h"

#include <cuda_runtime_api.h>

#include <memory>
#include <stdexcept>
#include <vector>

namespace bbfft {

namespace detail {
class cuda_plan_handle {
  public:
    cuda_plan_handle(configuration const &cfg, cudaStream_t stream, jit_cache *cache, bool adjoint)
        : stream_(stream) {
        bbfft_configuration c = cfg.to_c();
        bbfft_cache_t ch = cache ? cache->native_handle() : nullptr;
        check(adjoint ? bbfft_plan_create_adjoint(&c, stream, ch, &plan_)
                      : bbfft_plan_create(&c, stream, ch, &plan_));
    }
    ~cuda_plan_handle() { bbfft_plan_destroy(plan_); }
    cuda_plan_handle(cuda_plan_handle const &) = delete;
    cuda_plan_handle &operator=(cuda_plan_handle const &) = delete;
    bbfft_plan_t get() const { return plan_; }
    cudaStream_t stream() const { return stream_; }

  private:
    bbfft_plan_t plan_ = nullptr;
    cudaStream_t stream_;
};

class cuda_plan_impl : public plan_impl<cudaEvent_t> {
  public:
    cuda_plan_impl(configuration const &cfg, cudaStream_t stream, jit_cache *cache, bool adjoint)
        : h_(cfg, stream, cache, adjoint) {}
    using plan_impl<cudaEvent_t>::execute;
    auto execute(void const *in, void *out, std::vector<cudaEvent_t> const &dep_events)
        -> cudaEvent_t override {
        cudaEvent_t done = nullptr;
        if (cudaEventCreateWithFlags(&done, cudaEventDisableTiming) != cudaSuccess) {
            throw std::runtime_error("cudaEventCreateWithFlags failed");
        }
        int status = bbfft_plan_execute(h_.get(), in, out,
                                        static_cast<uint32_t>(dep_events.size()),
                                        dep_events.empty() ? nullptr : dep_events.data(), done);
        if (status != BBFFT_SUCCESS) {
            cudaEventDestroy(done);
            check(status);
        }
        return done;
    }

  private:
    cuda_plan_handle h_;
};

class cuda_plan_unmanaged_impl : public plan_unmanaged_event_impl<cudaEvent_t> {
  public:
    cuda_plan_unmanaged_impl(configuration const &cfg, cudaStream_t stream, jit_cache *cache)
        : h_(cfg, stream, cache, false) {}
    void execute(void const *in, void *out, cudaEvent_t signal_event,
                 std::uint32_t num_wait_events, cudaEvent_t *wait_events) override {
        check(bbfft_plan_execute(h_.get(), in, out, num_wait_events, wait_events, signal_event));
    }

  private:
    cuda_plan_handle h_;
};
} // namespace detail

using cuda_plan = plan<cudaEvent_t>;
using cuda_plan_unmanaged = plan_unmanaged_event<cudaEvent_t>;

inline auto make_plan(configuration const &cfg, cudaStream_t stream, jit_cache *cache = nullptr)
    -> cuda_plan {
    return cuda_plan(std::make_shared<detail::cuda_plan_impl>(cfg, stream, cache, false));
}

inline auto make_plan_unmanaged(configuration const &cfg, cudaStream_t stream,
                                jit_cache *cache = nullptr) -> cuda_plan_unmanaged {
    return cuda_plan_unmanaged(std::make_shared<detail::cuda_plan_unmanaged_impl>(cfg, stream, cache));
}

// Adjoint of the transform (no counterpart in the reference): maps tensors laid out like
// cfg's output to tensors laid out like cfg's input (see bbfft_plan_create_adjoint).
inline auto make_adjoint_plan(configuration const &cfg, cudaStream_t stream,
                              jit_cache *cache = nullptr) -> cuda_plan {
    return cuda_plan(std::make_shared<detail::cuda_plan_impl>(cfg, stream, cache, true));
}

// AOT generation of callback kernels (reference tools/aot/main.cpp:22-60).
inline aot_module generate_aot_module(std::vector<configuration> const &cfgs, int device_id = 0) {
    std::vector<bbfft_configuration> cs;
    for (auto const &c : cfgs) {
        cs.push_back(c.to_c());
    }
    std::size_t img = 0, nn = 0;
    detail::check(bbfft_aot_generate(cs.data(), cs.size(), nullptr, 0, &img, nullptr, 0, &nn));
    aot_module m;
    m.image.resize(img);
    std::string names(nn, '\0');
    detail::check(bbfft_aot_generate(cs.data(), cs.size(), m.image.data(), img, nullptr, &names[0], nn,
                                     nullptr));
    std::size_t pos = 0;
    while (pos < names.size()) {
        std::size_t nl = names.find('\n', pos);
        if (nl == std::string::npos) {
            break;
        }
        m.kernel_names.push_back(names.substr(pos, nl - pos));
        pos = nl + 1;
    }
    m.device_id = device_id;
    return m;
}

} // namespace bbfft

#endif
