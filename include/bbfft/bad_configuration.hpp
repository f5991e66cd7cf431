// bbfft::bad_configuration on top of the GB300 C ABI.
// Mirrors the reference's include/bbfft/bad_configuration.hpp:17-40: thrown for
// unsupported configurations (status BBFFT_BAD_CONFIGURATION of the C ABI).
#ifndef BBFFT_GB300_BAD_CONFIGURATION_HPP
#define BBFFT_GB300_BAD_CONFIGURATION_HPP

#include "bbfft_gb300.h"

#include <exception>
#include <stdexcept>
#include <string>

namespace bbfft {

class bad_configuration : public std::exception {
  public:
    bad_configuration(std::string what) : what_(std::move(what)) {}
    bad_configuration(char const *what) : what_(what) {}
    char const *what() const noexcept override { return what_.c_str(); }

  private:
    std::string what_;
};

namespace detail {
// Converts a C ABI status into the exception the reference throws for it.
inline void check(int status) {
    if (status == BBFFT_SUCCESS) {
        return;
    }
    std::string msg = bbfft_last_error();
    if (status == BBFFT_BAD_CONFIGURATION) {
        throw bad_configuration(msg);
    }
    throw std::runtime_error(msg);
}
} // namespace detail

} // namespace bbfft

#endif
