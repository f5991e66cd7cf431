// Persistent kernel for ragged batches: many independent 1d transforms of different
// lengths, kinds and batch sizes in ONE launch.
//
// The host splits every transform into CTA tiles ("units"), orders the units largest
// first and stores them in a table.  Persistent CTA b runs units b, b + G, b + 2G, ...
// (G CTAs; no CTA ever waits on another), with the parameters of the next unit fetched
// while the current one runs, and each unit on its compile-time-size tile function when
// one exists, else on the runtime-size engine.
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
    (void)counter;
    constexpr int NW = static_cast<int>(sizeof(fft_params) / sizeof(int));
    static_assert(NW <= 256, "parameter block larger than the block");
    __shared__ __align__(16) fft_params s_p[2];
    __shared__ int s_kind[2], s_vid[2];
    __shared__ long long s_tile[2];
    const int tid = threadIdx.x;
    const int G = gridDim.x;
    int u = blockIdx.x;
    if (u >= n_units) {
        return;
    }
    {
        const int2 un = units[u];
        if (tid < NW) {
            reinterpret_cast<int *>(&s_p[0])[tid] = reinterpret_cast<const int *>(&items[un.x].p)[tid];
        }
        if (tid == 0) {
            s_kind[0] = items[un.x].kind;
            s_vid[0] = items[un.x].vid;
            s_tile[0] = un.y;
        }
    }
    __syncthreads();
    for (int slot = 0;; slot ^= 1) {
        // the units of a block are u, u + G, u + 2G, ... (LPT order, round robin): the
        // parameters of the next one are loaded into registers before this tile runs and
        // stored into the other slot after it, so no tile waits for them
        const int un_i = u + G;
        const bool more = un_i < n_units;
        int pw = 0, nk = 0, nv = 0;
        long long nt = 0;
        if (more) {
            const int2 un = units[un_i];
            if (tid < NW) {
                pw = __ldg(reinterpret_cast<const int *>(&items[un.x].p) + tid);
            }
            if (tid == 0) {
                nk = __ldg(&items[un.x].kind);
                nv = __ldg(&items[un.x].vid);
                nt = un.y;
            }
        }
        const fft_params &p = s_p[slot];
        if (s_vid[slot] >= 0) {
            if constexpr (sizeof(R) == 4) {
                ragged_ct_call(s_vid[slot], p, s_tile[slot]);
            }
        } else {
            switch (s_kind[slot]) {
            case kind_c2c:
                fft_tile_at<R, kind_c2c, default_io>(p, s_tile[slot]);
                break;
            case kind_r2c_half:
                fft_tile_at<R, kind_r2c_half, default_io>(p, s_tile[slot]);
                break;
            case kind_r2c_full:
                fft_tile_at<R, kind_r2c_full, default_io>(p, s_tile[slot]);
                break;
            case kind_c2r_half:
                fft_tile_at<R, kind_c2r_half, default_io>(p, s_tile[slot]);
                break;
            case kind_c2r_full:
                fft_tile_at<R, kind_c2r_full, default_io>(p, s_tile[slot]);
                break;
            }
        }
        if (!more) {
            return;
        }
        if (tid < NW) {
            reinterpret_cast<int *>(&s_p[slot ^ 1])[tid] = pw;
        }
        if (tid == 0) {
            s_kind[slot ^ 1] = nk;
            s_vid[slot ^ 1] = nv;
            s_tile[slot ^ 1] = nt;
        }
        __syncthreads(); // the next tile's parameters are visible; shared data is free
        u = un_i;
    }
}

const void *ragged_kernel_ptr(int prec) {
    return prec == 4 ? reinterpret_cast<const void *>(&ragged_kernel<float>)
                     : reinterpret_cast<const void *>(&ragged_kernel<double>);
}

} // namespace gbfft
