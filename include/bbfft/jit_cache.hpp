// Plan caches.  Mirror the reference's include/bbfft/jit_cache.hpp:23-69,
// jit_cache_all.hpp:20-37 and aot_cache.hpp:21-48.  On GB300 only plans with user callbacks
// compile code (NVRTC); the cache objects hold those modules keyed by kernel name and
// device.  jit_cache_all and aot_cache wrap the library's cache objects; make_plan uses a
// cache through native_handle() (a cache class that does not provide one is ignored).
#ifndef BBFFT_GB300_JIT_CACHE_HPP
#define BBFFT_GB300_JIT_CACHE_HPP

#include "bbfft/bad_configuration.hpp"
#include "bbfft_gb300.h"

#include <cstdint>
#include <limits>
#include <string>
#include <vector>

namespace bbfft {

using device_handle_t = std::uintptr_t;
using module_handle_t = std::uintptr_t;

struct jit_cache_key {
    std::string kernel_name = {};
    std::uint64_t device_id = std::numeric_limits<std::uint64_t>::max();
    bool operator==(jit_cache_key const &other) const {
        return kernel_name == other.kernel_name && device_id == other.device_id;
    }
};

class jit_cache {
  public:
    virtual ~jit_cache() {}
    virtual bbfft_cache_t native_handle() const { return nullptr; }
};

namespace detail {
class native_cache : public jit_cache {
  public:
    native_cache(bool aot) {
        check(aot ? bbfft_aot_cache_create(&h_) : bbfft_jit_cache_create(&h_));
    }
    ~native_cache() override { bbfft_cache_destroy(h_); }
    native_cache(native_cache const &) = delete;
    native_cache &operator=(native_cache const &) = delete;
    bbfft_cache_t native_handle() const override { return h_; }
    auto kernel_names() const -> std::vector<std::string> {
        std::size_t needed = 0;
        check(bbfft_cache_kernel_names(h_, nullptr, 0, &needed));
        std::string all(needed, '\0');
        check(bbfft_cache_kernel_names(h_, &all[0], needed, nullptr));
        std::vector<std::string> names;
        std::size_t pos = 0;
        while (pos < all.size()) {
            std::size_t nl = all.find('\n', pos);
            if (nl == std::string::npos) {
                break;
            }
            names.push_back(all.substr(pos, nl - pos));
            pos = nl + 1;
        }
        return names;
    }

  private:
    bbfft_cache_t h_ = nullptr;
};
} // namespace detail

class jit_cache_all : public detail::native_cache {
  public:
    jit_cache_all() : native_cache(false) {}
};

struct aot_module {
    std::vector<char> image;                ///< cubin / fatbin for sm_103a
    std::vector<std::string> kernel_names;  ///< kernels in the image
    int device_id = 0;                      ///< CUDA device ordinal
};

class aot_cache : public detail::native_cache {
  public:
    aot_cache() : native_cache(true) {}
    void register_module(aot_module const &m) {
        std::vector<char const *> names;
        for (auto const &n : m.kernel_names) {
            names.push_back(n.c_str());
        }
        detail::check(bbfft_aot_cache_register_module(native_handle(), m.image.data(),
                                                      m.image.size(), names.data(), names.size(),
                                                      m.device_id));
    }
};

} // namespace bbfft

#endif
