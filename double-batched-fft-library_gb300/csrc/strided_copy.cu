// Strided tensor copy for nd plans with non-default layouts: the input is gathered into
// the default (packed) layout before the chain of 1d passes and the result is scattered
// into the caller's output layout after it.  Element (c_0, .., c_{r-1}) of the packed side
// (c_0 fastest) maps to offset sum_d c_d * stride_d of the strided side.  The reference
// rejects these layouts (src/common/algorithm/nd_fft.hpp:47-49).
#include "kernels.hpp"

#include <cuda_runtime.h>

namespace gbfft {

template <class T>
__global__ void __launch_bounds__(256) strided_copy_kernel(const copy_params p) {
    const T *src = static_cast<const T *>(p.src);
    T *dst = static_cast<T *>(p.dst);
    for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < p.total;
         i += static_cast<long long>(gridDim.x) * blockDim.x) {
        long long rem = i, off = 0;
#pragma unroll
        for (int d = 0; d < copy_max_rank; ++d) {
            if (d < p.rank) {
                const long long c = rem % p.shape[d];
                rem /= p.shape[d];
                off += c * p.stride[d];
            }
        }
        if (p.gather) {
            dst[i] = src[off];
        } else {
            dst[off] = src[i];
        }
    }
}

const void *strided_copy_kernel_ptr(int elem_bytes) {
    switch (elem_bytes) {
    case 4:
        return reinterpret_cast<const void *>(&strided_copy_kernel<float>);
    case 8:
        return reinterpret_cast<const void *>(&strided_copy_kernel<float2>);
    case 16:
        return reinterpret_cast<const void *>(&strided_copy_kernel<double2>);
    default:
        return nullptr;
    }
}

} // namespace gbfft
