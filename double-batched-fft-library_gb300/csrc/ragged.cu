// Persistent kernel for ragged batches: many independent 1d transforms of different
// lengths, kinds and batch sizes in ONE launch.
//
// The host splits every transform into CTA tiles ("units"), orders the units largest
// first and stores them in a table.  A unit runs on its compile-time-size tile function
// when one exists, else on the runtime-size engine.  Two launch forms share the table:
// persistent CTAs taking units from a counter, or one CTA per unit.
// The reference launches one kernel per plan (src/common/algorithm/small_batch_fft.hpp:111);
// it has no ragged form.
#include "engine.cuh"
#include "engine_ct.cuh"
#include "kernels.hpp"

namespace gbfft {

// ragged_ct_call(vid, p, tile): the compile-time-size tile functions (generated units,
// linked as relocatable device code)
#include "ragged_ct_dispatch.inc"

// One unit: its parameters staged in shared memory, then its tile.
template <class R>
__device__ __forceinline__ void ragged_unit(const ragged_item_dev *__restrict__ items, int2 un,
                                            fft_params &s_p, int &s_kind, int &s_vid) {
    constexpr int NW = static_cast<int>(sizeof(fft_params) / sizeof(int));
    const int tid = threadIdx.x;
    if (tid < NW) {
        reinterpret_cast<int *>(&s_p)[tid] = __ldg(reinterpret_cast<const int *>(&items[un.x].p) + tid);
    }
    if (tid == 0) {
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
}

// Persistent form: G CTAs; each takes the next unit from a device counter (one atomicAdd
// by one thread; no thread waits on another CTA) until the table is exhausted.  The
// counter is reset before every launch.
template <class R>
__global__ void __launch_bounds__(256, 2) ragged_kernel(const ragged_item_dev *__restrict__ items,
                                                     const int2 *__restrict__ units, int n_units,
                                                     unsigned *counter) {
    static_assert(sizeof(fft_params) / sizeof(int) <= 256, "parameter block larger than the block");
    __shared__ int s_unit;
    __shared__ __align__(16) fft_params s_p;
    __shared__ int s_kind, s_vid;
    for (;;) {
        if (threadIdx.x == 0) {
            s_unit = static_cast<int>(atomicAdd(counter, 1u));
        }
        __syncthreads();
        const int u = s_unit;
        if (u >= n_units) {
            return;
        }
        ragged_unit<R>(items, units[u], s_p, s_kind, s_vid);
        __syncthreads(); // shared memory and s_p are reused by the next unit
    }
}

// Grid form: one CTA per unit, scheduled by the hardware (same unit table and tiles).
template <class R>
__global__ void __launch_bounds__(256, 2) ragged_grid_kernel(const ragged_item_dev *__restrict__ items,
                                                          const int2 *__restrict__ units, int n_units,
                                                          unsigned *counter) {
    (void)counter;
    __shared__ __align__(16) fft_params s_p;
    __shared__ int s_kind, s_vid;
    if (static_cast<int>(blockIdx.x) < n_units) {
        ragged_unit<R>(items, units[blockIdx.x], s_p, s_kind, s_vid);
    }
}

// Class form: one kernel per class of units; this one runs the classes without a
// compile-time-size tile function.
template <class R, int Kind>
__global__ void __launch_bounds__(256, 2) ragged_class_rt(const ragged_item_dev *__restrict__ items,
                                                       const int2 *__restrict__ units) {
    __shared__ __align__(16) fft_params s_p;
    const int2 un = stage_unit_params(items, units, s_p);
    fft_tile_at<R, Kind, default_io>(s_p, un.y);
}

const void *ragged_class_runtime_kernel(int prec, int kind) {
#define GBFFT_RT_CASE(K)                                                                         \
    case K:                                                                                      \
        return prec == 4 ? reinterpret_cast<const void *>(&ragged_class_rt<float, K>)            \
                         : reinterpret_cast<const void *>(&ragged_class_rt<double, K>);
    switch (kind) {
        GBFFT_RT_CASE(kind_c2c)
        GBFFT_RT_CASE(kind_r2c_half)
        GBFFT_RT_CASE(kind_r2c_full)
        GBFFT_RT_CASE(kind_c2r_half)
        GBFFT_RT_CASE(kind_c2r_full)
    default:
        return nullptr;
    }
#undef GBFFT_RT_CASE
}

const void *ragged_kernel_ptr(int prec, bool persistent) {
    if (persistent) {
        return prec == 4 ? reinterpret_cast<const void *>(&ragged_kernel<float>)
                         : reinterpret_cast<const void *>(&ragged_kernel<double>);
    }
    return prec == 4 ? reinterpret_cast<const void *>(&ragged_grid_kernel<float>)
                     : reinterpret_cast<const void *>(&ragged_grid_kernel<double>);
}

} // namespace gbfft
