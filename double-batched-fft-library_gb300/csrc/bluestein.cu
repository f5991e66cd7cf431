// Bluestein's algorithm for float transforms whose complex length Nc has a prime factor
// above 61, fused into one kernel per tile.
//
// Those lengths have no efficient radix stage: the generic odd-radix stage costs O(P) per
// output.  With c_n = exp(-i pi n^2 / Nc) and nk = (n^2 + k^2 - (k-n)^2) / 2,
//   X_k = c_k sum_n (x_n c_n) conj(c_{k-n}),
// a cyclic convolution of a_n = x_n c_n with b_m = conj(c_m) (m mod L) of any length
// L >= 2 Nc - 1 (a power of two here, 128..1024): X = c . IFFT_L(FFT_L(a) . FFT_L(b)).
// FFT_L(b) / L is a table of the plan (host, long double, rounded once).  Every transform
// of the tile is loaded once (the kind's own load: c2c, the real even / odd forms and the
// reference's c2r pre-process, engine.cuh gload), multiplied by the chirp and zero-padded
// to L in shared memory; the two length-L transforms run there as radix-4 (and one radix-2)
// Stockham stages on 64 threads per transform (the inverse as conj(FFT(conj(.)))); the
// result is multiplied by the chirp and stored by the kind's own store (with the r2c
// post-process from shared memory for even real N).  One read and one write of the tensor.
#include "engine.cuh"
#include "kernels.hpp"

namespace gbfft {
namespace blu {

constexpr int kTT = 64; // threads per transform

// One radix-R stage of the length-L Stockham transform, in place in shared memory: every
// thread holds its butterflies in registers across the barrier.
template <int R, int L, class Ctx>
__device__ __forceinline__ void stage(const Ctx &c, int j, int Ns, const float2 *__restrict__ wL) {
    constexpr int nb = L / R;
    constexpr int IT = (nb + kTT - 1) / kTT;
    float2 v[IT][R];
    const int twstride = L / (Ns * R);
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const int b = j + it * kTT;
        if (b < nb) { // threads beyond the tile hold j = 1 << 20
            const int kk = b % Ns;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                float2 x = c.sm[c.sidx(0, b + r * nb)];
                if (r > 0 && Ns > 1) {
                    x = cmul(x, __ldg(wL + r * kk * twstride));
                }
                v[it][r] = x;
            }
            dft<R, float>::run(v[it]);
        }
    }
    __syncthreads();
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const int b = j + it * kTT;
        if (b < nb) {
            const int o = b + (b / Ns) * Ns * (R - 1);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                c.sm[c.sidx(0, o + r * Ns)] = v[it][r];
            }
        }
    }
    __syncthreads();
}

__host__ __device__ constexpr int log2i(int n) { return n > 1 ? 1 + log2i(n / 2) : 0; }

// forward length-L transform: radix-4 stages, then one radix-2 stage when log2 L is odd
template <int L, class Ctx>
__device__ __forceinline__ void fft_l(const Ctx &c, int j, const float2 *wL) {
    constexpr int S4 = log2i(L) / 2;
    int Ns = 1;
#pragma unroll
    for (int s = 0; s < S4; ++s) {
        stage<4, L>(c, j, Ns, wL);
        Ns *= 4;
    }
    if constexpr (log2i(L) % 2 == 1) {
        stage<2, L>(c, j, Ns, wL);
    }
}

template <int Kind, int L> __device__ __forceinline__ void tile(const fft_params &p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int j;
    auto c = make_ctx<float, Kind, default_io>(p, smem_raw, kTT, L, j, blockIdx.x);
    const bool work = j < kTT; // threads beyond the tile hold j = 1 << 20
    const int Nc = p.Nc;
    const float2 *chirp = static_cast<const float2 *>(p.bs);
    const float2 *bhat = chirp + Nc;
    const float2 *wL = bhat + L;
    if (work) {
        for (int n = j; n < L; n += kTT) {
            float2 v = make_float2(0.f, 0.f);
            if (n < Nc) {
                if (c.active) {
                    v = cmul(c.template gload<0>(n), __ldg(chirp + n));
                }
            }
            c.sm[c.sidx(0, n)] = v;
        }
    }
    __syncthreads();
    fft_l<L>(c, work ? j : 1 << 20, wL);
    // A . FFT(b) / L, conjugated for the inverse transform
    if (work) {
        for (int l = j; l < L; l += kTT) {
            const float2 v = cmul(c.sm[c.sidx(0, l)], __ldg(bhat + l));
            c.sm[c.sidx(0, l)] = make_float2(v.x, -v.y);
        }
    }
    __syncthreads();
    fft_l<L>(c, work ? j : 1 << 20, wL);
    if constexpr (Kind == kind_r2c_half) {
        // Z_k = c_k conj(y_k) into shared memory, then the r2c post-process
        if (work) {
            for (int k = j; k < Nc; k += kTT) {
                const float2 y = c.sm[c.sidx(0, k)];
                c.sm[c.sidx(0, k)] = cmul(make_float2(y.x, -y.y), __ldg(chirp + k));
            }
        }
        __syncthreads();
        r2c_post<0, 0>(c, work ? j : 1 << 20, 0);
    } else {
        if (work && c.active) {
            for (int k = j; k < Nc; k += kTT) {
                const float2 y = c.sm[c.sidx(0, k)];
                c.template gstore<0>(k, cmul(make_float2(y.x, -y.y), __ldg(chirp + k)));
            }
        }
    }
}

template <int Kind>
__global__ void __launch_bounds__(256) bluestein_kernel(const __grid_constant__ fft_params p) {
    switch (p.bL) {
    case 128:
        tile<Kind, 128>(p);
        break;
    case 256:
        tile<Kind, 256>(p);
        break;
    case 512:
        tile<Kind, 512>(p);
        break;
    case 1024:
        tile<Kind, 1024>(p);
        break;
    }
}

} // namespace blu

const void *bluestein_kernel(int kind) {
    switch (kind) {
    case kind_c2c:
        return reinterpret_cast<const void *>(&blu::bluestein_kernel<kind_c2c>);
    case kind_r2c_half:
        return reinterpret_cast<const void *>(&blu::bluestein_kernel<kind_r2c_half>);
    case kind_r2c_full:
        return reinterpret_cast<const void *>(&blu::bluestein_kernel<kind_r2c_full>);
    case kind_c2r_half:
        return reinterpret_cast<const void *>(&blu::bluestein_kernel<kind_c2r_half>);
    case kind_c2r_full:
        return reinterpret_cast<const void *>(&blu::bluestein_kernel<kind_c2r_full>);
    }
    return nullptr;
}

} // namespace gbfft
