// bbfft::tensor_indexer: offsets of multi-dimensional tensors with shapes and strides.
// Same interface as the reference's include/bbfft/tensor_indexer.hpp:24-357 (layout,
// fit_array, tensor_indexer with fuse / reshape, vector_indexer, matrix_indexer), written
// for this library.  Internally shape and stride are kept fastest-varying mode first.
#ifndef BBFFT_GB300_TENSOR_INDEXER_HPP
#define BBFFT_GB300_TENSOR_INDEXER_HPP

#include <algorithm>
#include <array>
#include <cstddef>

namespace bbfft {

enum class layout {
    row_major, ///< last index varies fastest
    col_major  ///< first index varies fastest
};

// Copies min(Din, Dout) entries of `in` into an array of length Dout padded with fill_value.
template <std::size_t Dout, typename IdxT, std::size_t Din>
constexpr auto fit_array(std::array<IdxT, Din> const &in, IdxT fill_value = IdxT(0)) {
    std::array<IdxT, Dout> out = {};
    for (std::size_t i = 0; i < Dout; ++i) {
        out[i] = i < Din ? in[i] : fill_value;
    }
    return out;
}

template <typename IdxT, unsigned int D, layout L = layout::row_major> class tensor_indexer {
  public:
    using multi_idx_t = std::array<IdxT, D>;

    tensor_indexer() : shape_{}, stride_{} {}
    tensor_indexer(multi_idx_t shape) : shape_(to_internal(shape)) {
        stride_[0] = IdxT(1);
        for (unsigned d = 1; d < D; ++d) {
            stride_[d] = stride_[d - 1] * shape_[d - 1];
        }
    }
    tensor_indexer(multi_idx_t shape, multi_idx_t stride)
        : shape_(to_internal(shape)), stride_(to_internal(stride)) {}

    template <typename... Indices, typename = std::enable_if_t<sizeof...(Indices) == D, int>>
    IdxT operator()(Indices &&...is) const {
        multi_idx_t idx = {static_cast<IdxT>(is)...};
        return (*this)(idx);
    }
    IdxT operator()(multi_idx_t const &idx) const {
        multi_idx_t in = to_internal(idx);
        IdxT off = IdxT(0);
        for (unsigned d = 0; d < D; ++d) {
            off += in[d] * stride_[d];
        }
        return off;
    }

    auto shape() const { return to_internal(shape_); }
    auto shape(unsigned int d) const { return shape_[internal(d)]; }
    auto stride() const { return to_internal(stride_); }
    auto stride(unsigned int d) const { return stride_[internal(d)]; }
    IdxT size() const { return stride_[D - 1] * shape_[D - 1]; }
    constexpr auto dim() const { return D; }

    // Modes Dfrom..Dto (user numbering) may be fused if they are packed in memory.
    template <unsigned int Dfrom = 0, unsigned int Dto = D - 1> bool may_fuse() const {
        static_assert(Dfrom <= Dto && Dto <= D - 1);
        unsigned lo = std::min(internal(Dfrom), internal(Dto));
        unsigned hi = std::max(internal(Dfrom), internal(Dto));
        for (unsigned d = lo; d < hi; ++d) {
            if (stride_[d] * shape_[d] != stride_[d + 1]) {
                return false;
            }
        }
        return true;
    }

    template <unsigned int Dfrom = 0, unsigned int Dto = D - 1> auto fused() const {
        static_assert(Dfrom <= Dto && Dto <= D - 1);
        constexpr unsigned E = D - (Dto - Dfrom);
        std::array<IdxT, E> shp = {}, str = {};
        auto ushape = shape();
        auto ustride = stride();
        unsigned o = 0;
        for (unsigned d = 0; d < D; ++d) {
            if (d > Dfrom && d <= Dto) {
                shp[o - 1] *= ushape[d];
                if constexpr (L == layout::row_major) {
                    str[o - 1] = ustride[d];
                }
                continue;
            }
            shp[o] = ushape[d];
            str[o] = ustride[d];
            ++o;
        }
        return tensor_indexer<IdxT, E, L>(shp, str);
    }

    template <std::size_t E>
    bool may_reshape_mode(int mode, std::array<IdxT, E> const &mode_shape) const {
        IdxT n = IdxT(1);
        for (auto m : mode_shape) {
            n *= m;
        }
        return n == shape(static_cast<unsigned>(mode));
    }

    // Splits user mode `mode` into E modes of shape mode_shape (given in the layout's order).
    template <std::size_t E> auto reshaped_mode(int mode, std::array<IdxT, E> mode_shape) const {
        static_assert(E > 0u);
        constexpr unsigned F = D + E - 1;
        std::array<IdxT, F> shp = {}, str = {};
        auto ushape = shape();
        auto ustride = stride();
        unsigned o = 0;
        for (unsigned d = 0; d < D; ++d) {
            if (static_cast<int>(d) != mode) {
                shp[o] = ushape[d];
                str[o] = ustride[d];
                ++o;
                continue;
            }
            // stride of each new mode, fastest-varying first in memory
            std::array<IdxT, E> s = {};
            if constexpr (L == layout::col_major) {
                s[0] = ustride[d];
                for (std::size_t e = 1; e < E; ++e) {
                    s[e] = s[e - 1] * mode_shape[e - 1];
                }
            } else {
                s[E - 1] = ustride[d];
                for (std::size_t e = E - 1; e-- > 0;) {
                    s[e] = s[e + 1] * mode_shape[e + 1];
                }
            }
            for (std::size_t e = 0; e < E; ++e) {
                shp[o] = mode_shape[e];
                str[o] = s[e];
                ++o;
            }
        }
        return tensor_indexer<IdxT, F, L>(shp, str);
    }

  private:
    static constexpr unsigned internal(unsigned d) {
        return L == layout::col_major ? d : D - 1 - d;
    }
    static multi_idx_t to_internal(multi_idx_t const &a) {
        if constexpr (L == layout::col_major) {
            return a;
        } else {
            multi_idx_t r = {};
            for (unsigned d = 0; d < D; ++d) {
                r[d] = a[D - 1 - d];
            }
            return r;
        }
    }

    multi_idx_t shape_;
    multi_idx_t stride_;
};

template <typename IdxT, layout L = layout::row_major>
using vector_indexer = tensor_indexer<IdxT, 1u, L>;
template <typename IdxT, layout L = layout::row_major>
using matrix_indexer = tensor_indexer<IdxT, 2u, L>;

} // namespace bbfft

#endif
