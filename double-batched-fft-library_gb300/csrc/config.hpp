// Internal host-side helpers shared by the library translation units.
#pragma once

#include "bbfft_gb300.h"

#include <array>
#include <cstddef>
#include <stdexcept>
#include <string>

namespace gbfft {

constexpr unsigned max_fft_dim = BBFFT_MAX_FFT_DIM;
constexpr unsigned max_tensor_dim = BBFFT_MAX_TENSOR_DIM;
using stride_t = std::array<std::size_t, max_tensor_dim>;

// Exception carrying a C-ABI status; converted to a return code at the boundary.
class status_error : public std::runtime_error {
  public:
    status_error(int status, std::string const &what) : std::runtime_error(what), status_(status) {}
    int status() const noexcept { return status_; }

  private:
    int status_;
};

inline stride_t to_array(std::size_t const *a) {
    stride_t r;
    for (unsigned i = 0; i < max_tensor_dim; ++i) {
        r[i] = a[i];
    }
    return r;
}
inline void from_array(stride_t const &r, std::size_t *a) {
    for (unsigned i = 0; i < max_tensor_dim; ++i) {
        a[i] = r[i];
    }
}

stride_t default_istride(unsigned dim, stride_t const &shape, int type, bool inplace);
stride_t default_ostride(unsigned dim, stride_t const &shape, int type, bool inplace);
std::string to_descriptor(bbfft_configuration const &cfg);
bbfft_configuration parse_descriptor(std::string const &desc);

} // namespace gbfft
