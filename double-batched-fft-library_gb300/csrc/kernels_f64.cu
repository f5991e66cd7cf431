// AOT instantiation of the double-batched FFT kernels, double precision.
// The kernel body is the stage engine of engine.cuh; one kernel per transform kind.
#include "engine.cuh"
#include "kernels.hpp"

namespace gbfft {

template <class R, int Kind>
__global__ void __launch_bounds__(512) fft_kernel(const __grid_constant__ fft_params p) {
    fft_tile<R, Kind, default_io>(p);
}

const void *kernel_f64(int kind) {
    switch (kind) {
    case kind_c2c:
        return reinterpret_cast<const void *>(&fft_kernel<double, kind_c2c>);
    case kind_r2c_half:
        return reinterpret_cast<const void *>(&fft_kernel<double, kind_r2c_half>);
    case kind_r2c_full:
        return reinterpret_cast<const void *>(&fft_kernel<double, kind_r2c_full>);
    case kind_c2r_half:
        return reinterpret_cast<const void *>(&fft_kernel<double, kind_c2r_half>);
    case kind_c2r_full:
        return reinterpret_cast<const void *>(&fft_kernel<double, kind_c2r_full>);
    }
    return nullptr;
}

} // namespace gbfft
