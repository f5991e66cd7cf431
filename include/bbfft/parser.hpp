// bbfft::parse_fft_descriptor for the GB300 library.
// Mirrors the reference's include/bbfft/parser.hpp:24 (src/base/parser.cpp:59-211): throws
// std::runtime_error with a caret under the offending character on malformed input.
#ifndef BBFFT_GB300_PARSER_HPP
#define BBFFT_GB300_PARSER_HPP

#include "bbfft/configuration.hpp"

#include <stdexcept>
#include <string>
#include <string_view>

namespace bbfft {

inline configuration parse_fft_descriptor(std::string_view desc) {
    bbfft_configuration c = {};
    std::string d(desc);
    int status = bbfft_parse_fft_descriptor(d.c_str(), &c);
    if (status != BBFFT_SUCCESS) {
        throw std::runtime_error(bbfft_last_error());
    }
    std::array<std::size_t, max_tensor_dim> shape = {}, is = {}, os = {};
    for (unsigned i = 0; i < max_tensor_dim; ++i) {
        shape[i] = c.shape[i];
        is[i] = c.istride[i];
        os[i] = c.ostride[i];
    }
    return configuration{c.dim, shape, static_cast<precision>(c.precision),
                         static_cast<direction>(c.direction), static_cast<transform_type>(c.type),
                         is, os};
}

} // namespace bbfft

#endif
