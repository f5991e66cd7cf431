// Configuration semantics: default strides, descriptor printing and parsing.
//
// Behaviour follows the reference:
//   default_istride / default_ostride   src/base/configuration.cpp:24-56
//   operator<< (descriptor string)      src/base/configuration.cpp:69-160
//   parse_fft_descriptor                src/base/parser.cpp:59-211
#include "config.hpp"

#include <cctype>
#include <sstream>
#include <stdexcept>
#include <string>

namespace gbfft {

stride_t default_istride(unsigned dim, stride_t const &shape, int type, bool inplace) {
    std::size_t n1 = shape[1];
    if (type == BBFFT_R2C) {
        n1 = inplace ? 2 * (shape[1] / 2 + 1) : shape[1];
    } else if (type == BBFFT_C2R) {
        n1 = shape[1] / 2 + 1;
    }
    stride_t s = {1, shape[0], n1 * shape[0], 0, 0};
    for (unsigned d = 1; d < dim && d + 2 < max_tensor_dim; ++d) {
        s[d + 2] = shape[d + 1] * s[d + 1];
    }
    return s;
}

stride_t default_ostride(unsigned dim, stride_t const &shape, int type, bool inplace) {
    int swapped = type == BBFFT_R2C ? BBFFT_C2R : type == BBFFT_C2R ? BBFFT_R2C : BBFFT_C2C;
    return default_istride(dim, shape, swapped, inplace);
}

static bool strides_equal(stride_t const &a, stride_t const &b, unsigned dim) {
    for (unsigned d = 0; d < dim + 2 && d < max_tensor_dim; ++d) {
        if (a[d] != b[d]) {
            return false;
        }
    }
    return true;
}

std::string to_descriptor(bbfft_configuration const &cfg) {
    std::ostringstream os;
    if (cfg.precision == BBFFT_PRECISION_F32) {
        os << 's';
    } else if (cfg.precision == BBFFT_PRECISION_F64) {
        os << 'd';
    } else {
        throw status_error(BBFFT_INVALID_ARGUMENT, "Unsupported precision");
    }
    if (cfg.type == BBFFT_C2C) {
        os << 'c';
    } else if (cfg.type == BBFFT_R2C || cfg.type == BBFFT_C2R) {
        os << 'r';
    } else {
        throw status_error(BBFFT_INVALID_ARGUMENT, "Unsupported transform type");
    }
    if (cfg.direction == BBFFT_FORWARD) {
        os << 'f';
    } else if (cfg.direction == BBFFT_BACKWARD) {
        os << 'b';
    } else {
        throw status_error(BBFFT_INVALID_ARGUMENT, "Unsupported direction");
    }
    if ((cfg.type == BBFFT_R2C && cfg.direction == BBFFT_BACKWARD) ||
        (cfg.type == BBFFT_C2R && cfg.direction == BBFFT_FORWARD)) {
        throw status_error(BBFFT_INVALID_ARGUMENT,
                           "r2c direction must be forward and c2r direction must be backward");
    }
    if (cfg.dim < 1 || cfg.dim > max_fft_dim) {
        throw status_error(BBFFT_INVALID_ARGUMENT, "Unsupported FFT dimension");
    }
    // placement: compare strides measured in real numbers on the complex side
    stride_t is = to_array(cfg.istride), ost = to_array(cfg.ostride);
    if (cfg.type == BBFFT_R2C) {
        for (unsigned d = 2; d < max_tensor_dim; ++d) {
            ost[d] *= 2;
        }
    } else if (cfg.type == BBFFT_C2R) {
        for (unsigned d = 2; d < max_tensor_dim; ++d) {
            is[d] *= 2;
        }
    }
    bool inplace = strides_equal(is, ost, cfg.dim);
    os << (inplace ? 'i' : 'o');
    if (cfg.shape[0] != 1u) {
        os << cfg.shape[0] << '.';
    }
    os << cfg.shape[1];
    for (unsigned d = 1; d < cfg.dim; ++d) {
        os << 'x' << cfg.shape[1 + d];
    }
    if (cfg.shape[cfg.dim + 1] != 1u) {
        os << '*' << cfg.shape[cfg.dim + 1];
    }
    stride_t shape = to_array(cfg.shape);
    if (to_array(cfg.istride) != default_istride(cfg.dim, shape, cfg.type, inplace)) {
        os << 'i' << cfg.istride[0];
        for (unsigned d = 1; d < cfg.dim + 2; ++d) {
            os << ',' << cfg.istride[d];
        }
    }
    if (to_array(cfg.ostride) != default_ostride(cfg.dim, shape, cfg.type, inplace)) {
        os << 'o' << cfg.ostride[0];
        for (unsigned d = 1; d < cfg.dim + 2; ++d) {
            os << ',' << cfg.ostride[d];
        }
    }
    return os.str();
}

namespace {
class parser {
  public:
    explicit parser(std::string const &d) : desc_(d) {}

    [[noreturn]] void fail(std::string const &msg, bool caret = true) {
        std::ostringstream oss;
        oss << "==> " << desc_ << " is malformed: " << msg;
        if (caret) {
            oss << '\n' << std::string(4 + pos_, ' ') << '^';
        }
        throw status_error(BBFFT_PARSE_ERROR, oss.str());
    }
    bool at_end() const { return pos_ >= desc_.size(); }
    char peek() const { return at_end() ? '\0' : desc_[pos_]; }
    char next() { return at_end() ? '\0' : desc_[pos_++]; }
    std::size_t number() {
        std::size_t begin = pos_;
        while (!at_end() && std::isdigit(static_cast<unsigned char>(desc_[pos_]))) {
            ++pos_;
        }
        if (begin == pos_) {
            fail("expected number");
        }
        return std::stoull(desc_.substr(begin, pos_ - begin));
    }
    std::size_t pos_ = 0;
    std::string desc_;
};
} // namespace

bbfft_configuration parse_descriptor(std::string const &desc) {
    bbfft_configuration cfg = {};
    parser p(desc);
    bool inplace = false;
    auto expect = [&](char c, char const *what) {
        if (c == '\0') {
            p.fail(std::string("expected ") + what);
        }
        --p.pos_;
        p.fail(std::string("expected ") + what);
    };
    char c = p.next();
    if (c == 's') {
        cfg.precision = BBFFT_PRECISION_F32;
    } else if (c == 'd') {
        cfg.precision = BBFFT_PRECISION_F64;
    } else {
        expect(c, "'s' (single) or 'd' (double)");
    }
    c = p.next();
    if (c == 'c') {
        cfg.type = BBFFT_C2C;
    } else if (c == 'r') {
        cfg.type = BBFFT_R2C;
    } else {
        expect(c, "'c' (complex) or 'r' (real)");
    }
    c = p.next();
    if (c == 'f') {
        cfg.direction = BBFFT_FORWARD;
    } else if (c == 'b') {
        cfg.direction = BBFFT_BACKWARD;
        if (cfg.type == BBFFT_R2C) {
            cfg.type = BBFFT_C2R;
        }
    } else {
        expect(c, "'f' (forward) or 'b' (backward)");
    }
    c = p.next();
    if (c == 'i') {
        inplace = true;
    } else if (c == 'o') {
        inplace = false;
    } else {
        expect(c, "'i' (in-place) or 'o' (out-of-place)");
    }

    std::array<char, max_tensor_dim> ops = {};
    std::array<std::size_t, max_tensor_dim + 1> nums = {};
    int n = 0;
    nums[n++] = p.number();
    while (!p.at_end()) {
        char op = p.peek();
        if (op != '.' && op != 'x' && op != '*') {
            break;
        }
        if (n >= static_cast<int>(max_tensor_dim)) {
            p.fail("tensor dimension must not be larger than " + std::to_string(max_tensor_dim),
                   false);
        }
        p.next();
        ops[n - 1] = op;
        nums[n++] = p.number();
    }
    bool has_M = n >= 2 && ops[0] == '.';
    bool has_K = n >= 2 && ops[n - 2] == '*';
    unsigned num_x = 0;
    for (int i = has_M ? 1 : 0; i < n - 1 - (has_K ? 1 : 0); ++i) {
        if (ops[i] == 'x') {
            ++num_x;
        } else {
            p.fail("'.' or '*' must only appear at the beginning or end of the tensor shape, "
                   "respectively",
                   false);
        }
    }
    cfg.dim = 1 + num_x;
    if (cfg.dim > max_fft_dim) {
        p.fail("only " + std::to_string(max_fft_dim - 1) + " 'x' are supported", false);
    }
    int s = 0;
    cfg.shape[s++] = has_M ? nums[0] : 1;
    for (int i = has_M ? 1 : 0; i < n; ++i) {
        cfg.shape[s++] = nums[i];
    }
    if (!has_K) {
        cfg.shape[s++] = 1;
    }
    bool custom_i = false, custom_o = false;
    auto parse_stride = [&](std::size_t *st) {
        for (unsigned d = 0; d < cfg.dim + 2; ++d) {
            st[d] = p.number();
            if (d + 1 < cfg.dim + 2) {
                char cc = p.next();
                if (cc != ',') {
                    expect(cc, "','");
                }
            }
        }
    };
    while (!p.at_end()) {
        char cc = p.next();
        if (cc == 'i') {
            parse_stride(cfg.istride);
            custom_i = true;
        } else if (cc == 'o') {
            parse_stride(cfg.ostride);
            custom_o = true;
        } else {
            expect(cc, "'i' (istride) or 'o' (ostride)");
        }
    }
    stride_t shape = to_array(cfg.shape);
    if (!custom_i) {
        from_array(default_istride(cfg.dim, shape, cfg.type, inplace), cfg.istride);
    }
    if (!custom_o) {
        from_array(default_ostride(cfg.dim, shape, cfg.type, inplace), cfg.ostride);
    }
    return cfg;
}

} // namespace gbfft
