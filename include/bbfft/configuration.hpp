// bbfft::configuration for the GB300 library (header-only, over include/bbfft_gb300.h).
// Mirrors the reference's include/bbfft/configuration.hpp:151-192 and the stride rules of
// src/base/configuration.cpp:24-160: same names, values and meaning.
#ifndef BBFFT_GB300_CONFIGURATION_HPP
#define BBFFT_GB300_CONFIGURATION_HPP

#include "bbfft/bad_configuration.hpp"
#include "bbfft/user_module.hpp"
#include "bbfft_gb300.h"

#include <array>
#include <cstddef>
#include <ostream>
#include <string>

namespace bbfft {

enum class precision : int { f32 = 4, f64 = 8 };
template <typename T> struct to_precision;
template <> struct to_precision<float> {
    static constexpr precision value = precision::f32;
};
template <> struct to_precision<double> {
    static constexpr precision value = precision::f64;
};
template <typename T> inline constexpr precision to_precision_v = to_precision<T>::value;

enum class direction : int { forward = -1, backward = 1 };
enum class transform_type : int { c2c, r2c, c2r };

inline char const *to_string(transform_type type) {
    switch (type) {
    case transform_type::c2c:
        return "c2c";
    case transform_type::r2c:
        return "r2c";
    case transform_type::c2r:
        return "c2r";
    }
    return "unknown";
}

constexpr unsigned max_fft_dim = BBFFT_MAX_FFT_DIM;
constexpr unsigned max_tensor_dim = BBFFT_MAX_TENSOR_DIM;

inline auto default_istride(unsigned dim, std::array<std::size_t, max_tensor_dim> const &shape,
                            transform_type type, bool inplace)
    -> std::array<std::size_t, max_tensor_dim> {
    std::array<std::size_t, max_tensor_dim> s = {};
    detail::check(bbfft_default_istride(dim, shape.data(), static_cast<int32_t>(type), inplace,
                                        s.data()));
    return s;
}

inline auto default_ostride(unsigned dim, std::array<std::size_t, max_tensor_dim> const &shape,
                            transform_type type, bool inplace)
    -> std::array<std::size_t, max_tensor_dim> {
    std::array<std::size_t, max_tensor_dim> s = {};
    detail::check(bbfft_default_ostride(dim, shape.data(), static_cast<int32_t>(type), inplace,
                                        s.data()));
    return s;
}

struct configuration {
    unsigned dim;
    std::array<std::size_t, max_tensor_dim> shape;
    precision fp;
    direction dir = direction::forward;
    transform_type type = transform_type::c2c;
    std::array<std::size_t, max_tensor_dim> istride = default_istride(dim, shape, type, true);
    std::array<std::size_t, max_tensor_dim> ostride = default_ostride(dim, shape, type, true);
    user_module callbacks = {};

    void set_strides_default(bool inplace) {
        istride = default_istride(dim, shape, type, inplace);
        ostride = default_ostride(dim, shape, type, inplace);
    }

    // C ABI view of this configuration (pointers refer to this object's callbacks)
    bbfft_configuration to_c(int32_t compute = BBFFT_COMPUTE_NATIVE) const {
        bbfft_configuration c = {};
        c.dim = dim;
        c.precision = static_cast<int32_t>(fp);
        c.direction = static_cast<int32_t>(dir);
        c.type = static_cast<int32_t>(type);
        for (unsigned i = 0; i < max_tensor_dim; ++i) {
            c.shape[i] = shape[i];
            c.istride[i] = istride[i];
            c.ostride[i] = ostride[i];
        }
        c.callback_source = callbacks.data;
        c.callback_length = callbacks.length;
        c.load_function = callbacks.load_function;
        c.store_function = callbacks.store_function;
        c.compute = compute;
        return c;
    }

    std::string to_string() const {
        bbfft_configuration c = to_c();
        std::size_t needed = 0;
        detail::check(bbfft_configuration_to_string(&c, nullptr, 0, &needed));
        std::string s(needed, '\0');
        detail::check(bbfft_configuration_to_string(&c, &s[0], needed, nullptr));
        s.resize(needed - 1);
        return s;
    }
};

inline std::ostream &operator<<(std::ostream &os, configuration const &cfg) {
    return os << cfg.to_string();
}

} // namespace bbfft

#endif
