// Persistent kernel for ragged batches: many independent 1d transforms of different
// lengths, kinds and batch sizes in ONE launch.
//
// The host splits every transform into CTA tiles ("units"), orders the units largest
// first and stores them in a table.  Each persistent CTA repeatedly takes the next unit
// index from a device counter (one atomicAdd by one thread -- no thread ever waits on
// another CTA), stages the unit's parameters in shared memory and runs the runtime-size
// engine on it.  The counter is reset before every launch (a memset node in the graph).
// The reference launches one kernel per plan (src/common/algorithm/small_batch_fft.hpp:111);
// it has no ragged form.
#include "engine.cuh"
#include "engine_ct.cuh"
#include "kernels.hpp"

namespace gbfft {

// ragged_ct_call(vid, p, tile): the compile-time-size tile functions (generated units,
// linked as relocatable device code)
#include "ragged_ct_dispatch.inc"

template <class R>
__global__ void __launch_bounds__(256, 2) ragged_kernel(const ragged_item_dev *__restrict__ items,
                                                     const int2 *__restrict__ units, int n_units,
                                                     unsigned *counter) {
    __shared__ int s_unit;
    __shared__ __align__(16) fft_params s_p;
    __shared__ int s_kind;
    __shared__ int s_vid;
    for (;;) {
        if (threadIdx.x == 0) {
            s_unit = static_cast<int>(atomicAdd(counter, 1u));
        }
        __syncthreads();
        const int u = s_unit;
        if (u >= n_units) {
            return;
        }
        const int2 un = units[u];
        const int *src = reinterpret_cast<const int *>(&items[un.x].p);
        int *dst = reinterpret_cast<int *>(&s_p);
        for (int i = threadIdx.x; i < static_cast<int>(sizeof(fft_params) / sizeof(int)); i += blockDim.x) {
            dst[i] = src[i];
        }
        if (threadIdx.x == 0) {
            s_kind = items[un.x].kind;
            s_vid = items[un.x].vid;
        }
        __syncthreads();
        if (s_vid >= 0) {
            if constexpr (sizeof(R) == 4) {
                ragged_ct_call(s_vid, s_p, un.y);
            }
        } else {
            switch (s_kind) {
            case kind_c2c:
                fft_tile_at<R, kind_c2c, default_io>(s_p, un.y);
                break;
            case kind_r2c_half:
                fft_tile_at<R, kind_r2c_half, default_io>(s_p, un.y);
                break;
            case kind_r2c_full:
                fft_tile_at<R, kind_r2c_full, default_io>(s_p, un.y);
                break;
            case kind_c2r_half:
                fft_tile_at<R, kind_c2r_half, default_io>(s_p, un.y);
                break;
            case kind_c2r_full:
                fft_tile_at<R, kind_c2r_full, default_io>(s_p, un.y);
                break;
            }
        }
        __syncthreads(); // shared memory and s_p are reused by the next unit
    }
}

const void *ragged_kernel_ptr(int prec) {
    return prec == 4 ? reinterpret_cast<const void *>(&ragged_kernel<float>)
                     : reinterpret_cast<const void *>(&ragged_kernel<double>);
}

} // namespace gbfft
