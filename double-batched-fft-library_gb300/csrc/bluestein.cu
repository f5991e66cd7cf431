// Bluestein's algorithm for float transforms whose complex length Nc has a prime factor
// above 61, fused into one kernel per tile.
//
// Those lengths have no efficient radix stage: the generic odd-radix stage costs O(P) per
// output.  With c_n = exp(-i pi n^2 / Nc) and nk = (n^2 + k^2 - (k-n)^2) / 2,
//   X_k = c_k sum_n (x_n c_n) conj(c_{k-n}),
// a cyclic convolution of a_n = x_n c_n with b_m = conj(c_m) (m mod L) of any length
// L >= 2 Nc - 1 (a power of two: 256, 512 or 1024, since Nc >= 67 here):
// X = c . IFFT_L(FFT_L(a) . FFT_L(b)).  FFT_L(b) / L is a table of the plan (host, long
// double, rounded once); the inverse runs as conj(FFT(conj(.))).
//
// The two length-L transforms are Stockham stages of radix 16 / 8 / 4 (256 = 16 x 16 on 16
// threads per transform, 512 = 8 x 8 x 8 and 1024 = 16 x 16 x 4 on 64) exchanging through
// shared memory; each thread holds its butterflies in registers across the barrier of an
// in-place stage.  The steps around them are fused into the first and last stages:
// - the first stage of the forward transform loads its butterfly's inputs from global
//   memory (the kind's own load: c2c, the real even / odd forms, the reference's c2r
//   pre-process; engine.cuh gload) and multiplies them by the chirp; inputs at n >= L / 2
//   are zero padding (L / 2 >= Nc) and are not loaded;
// - the last stage of the forward transform multiplies by FFT_L(b) / L and conjugates;
// - the last stage of the inverse conjugates, multiplies by the chirp and stores outputs
//   k < Nc (all below L / 2) to global memory with the kind's own store (for even real N
//   into shared memory, then the r2c post-process).
// One read and one write of the tensor.
#include "engine.cuh"
#include "kernels.hpp"

namespace gbfft {
namespace blu {

// threads per transform and radices of the length-L transform
__host__ __device__ constexpr int threads_of(int L) { return L == 256 ? 16 : 64; }
__host__ __device__ constexpr int radix_of(int L, int s) {
    return L == 256 ? (s < 2 ? 16 : 1) : L == 512 ? (s < 3 ? 8 : 1) : (s < 2 ? 16 : s == 2 ? 4 : 1);
}
__host__ __device__ constexpr int stages_of(int L) { return L == 256 ? 2 : 3; }
__host__ __device__ constexpr int span_of(int L, int s) { // product of the radices before s
    return s == 0 ? 1 : span_of(L, s - 1) * radix_of(L, s - 1);
}

// One radix-R Stockham stage of the length-L transform on T threads per transform, the
// earlier stages spanning Ns: butterfly b reads elements b + r L / R (times the twiddles
// w_L^{-r (b mod Ns) L / (Ns R)}) and writes (b / Ns) Ns R + (b mod Ns) + r Ns.
// `load(n)` / `store(n, v)` move element n; `HALF_IN`: inputs at r >= R / 2 are zero;
// `HALF_OUT`: outputs at r >= R / 2 are not needed; `MID`: barrier between the loads and
// the stores (in-place shared-memory stage).  Threads beyond the tile hold j = 1 << 20.
template <int L, int T, int R, int Ns, bool HALF_IN, bool HALF_OUT, bool MID, class Load, class Store>
__device__ __forceinline__ void stage(int j, const float2 *__restrict__ wL, Load load, Store store) {
    constexpr int nb = L / R;
    constexpr int IT = (nb + T - 1) / T;
    constexpr int tws = L / (Ns * R);
    float2 v[IT][R];
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const int b = j + it * T;
        if (b < nb) {
            const int kk = b % Ns;
#pragma unroll
            for (int r = 0; r < R; ++r) {
                float2 x = make_float2(0.f, 0.f);
                if (!HALF_IN || r < R / 2) {
                    x = load(b + r * nb);
                    if (Ns > 1 && r > 0) {
                        x = cmul(x, __ldg(wL + r * kk * tws));
                    }
                }
                v[it][r] = x;
            }
            dft<R, float>::run(v[it]);
        }
    }
    if constexpr (MID) {
        __syncthreads();
    }
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const int b = j + it * T;
        if (b < nb) {
            const int o = (b / Ns) * Ns * R + b % Ns;
#pragma unroll
            for (int r = 0; r < (HALF_OUT ? R / 2 : R); ++r) {
                store(o + r * Ns, v[it][r]);
            }
        }
    }
}

// Middle stages s = 1 .. S - 2 of a transform, shared memory to shared memory.
template <int L, int s, class SmLoad, class SmStore>
__device__ __forceinline__ void middle(int j, const float2 *wL, SmLoad ld, SmStore st) {
    if constexpr (s < stages_of(L) - 1) {
        stage<L, threads_of(L), radix_of(L, s), span_of(L, s), false, false, true>(j, wL, ld, st);
        __syncthreads();
        middle<L, s + 1>(j, wL, ld, st);
    }
}

template <int Kind, int L> __device__ __forceinline__ void tile(const fft_params &p) {
    constexpr int T = threads_of(L);
    constexpr int S = stages_of(L);
    constexpr int R0 = radix_of(L, 0);
    constexpr int RL = radix_of(L, S - 1);
    constexpr int NL = span_of(L, S - 1);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int j;
    auto c = make_ctx<float, Kind, default_io>(p, smem_raw, T, L, j, blockIdx.x);
    const int Nc = p.Nc;
    const float2 *chirp = static_cast<const float2 *>(p.bs);
    const float2 *bhat = chirp + Nc;
    const float2 *wL = bhat + L;
    auto sm_load = [&](int n) { return c.sm[c.sidx(0, n)]; };
    auto sm_store = [&](int n, float2 v) { c.sm[c.sidx(0, n)] = v; };
    // forward transform of a = x . chirp: first stage from global memory
    auto g_load = [&](int n) {
        float2 v = make_float2(0.f, 0.f);
        if (n < Nc && c.active) {
            v = cmul(c.template gload<0>(n), __ldg(chirp + n));
        }
        return v;
    };
    stage<L, T, R0, 1, true, false, false>(j, wL, g_load, sm_store);
    __syncthreads();
    middle<L, 1>(j, wL, sm_load, sm_store);
    // last forward stage: times FFT(b) / L, conjugated for the inverse transform
    auto mul_store = [&](int n, float2 v) {
        v = cmul(v, __ldg(bhat + n));
        c.sm[c.sidx(0, n)] = make_float2(v.x, -v.y);
    };
    stage<L, T, RL, NL, false, false, true>(j, wL, sm_load, mul_store);
    __syncthreads();
    // inverse transform (of the conjugate)
    stage<L, T, R0, 1, false, false, true>(j, wL, sm_load, sm_store);
    __syncthreads();
    middle<L, 1>(j, wL, sm_load, sm_store);
    if constexpr (Kind == kind_r2c_half) {
        // Z_k = c_k conj(y_k) into shared memory, then the r2c post-process
        auto z_store = [&](int k, float2 y) {
            if (k < Nc) {
                c.sm[c.sidx(0, k)] = cmul(make_float2(y.x, -y.y), __ldg(chirp + k));
            }
        };
        stage<L, T, RL, NL, false, true, true>(j, wL, sm_load, z_store);
        __syncthreads();
        r2c_post<0, T>(c, j, 0);
    } else {
        auto g_store = [&](int k, float2 y) {
            if (k < Nc && c.active) {
                c.template gstore<0>(k, cmul(make_float2(y.x, -y.y), __ldg(chirp + k)));
            }
        };
        stage<L, T, RL, NL, false, true, false>(j, wL, sm_load, g_store);
    }
}

template <int Kind>
__global__ void __launch_bounds__(256, 4) bluestein_kernel(const __grid_constant__ fft_params p) {
    switch (p.bL) {
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

int bluestein_threads(int L) { return blu::threads_of(L); }

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
