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
// in-place stage.  The twiddles of the stages after the first are a table of the plan laid
// out per stage as [r - 1][b mod Ns] (consecutive butterflies read consecutive entries:
// no bank conflicts), which each CTA copies into shared memory (at most 1008 entries; the
// scattered twiddle reads from global memory cost a sector each).  A tile loop over
// persistent CTAs was not kept: it held the per-thread addresses of every stage across the
// loop and spilled.  The steps around the transforms are fused into the first
// and last stages:
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
// offset of stage s's twiddles ((R - 1) Ns entries from stage 1 on) and the table size
__host__ __device__ constexpr int tw_offset(int L, int s) {
    return s <= 1 ? 0 : tw_offset(L, s - 1) + (radix_of(L, s - 1) - 1) * span_of(L, s - 1);
}
__host__ __device__ constexpr int tw_entries(int L) { return tw_offset(L, stages_of(L)); }
// spare shared elements after every 16 (chosen with a model of the 32 banks, 8-byte
// elements in half-warp phases, over every shared access of the tile)
__host__ __device__ constexpr int pad_of(int L, int MB) { return L == 512 && MB % 2 == 0 ? 2 : 1; }

// Shared index of element i of the tile buffer (MB transforms along M interleaved): PAD
// spare elements after every 16.
template <int PAD> __device__ __forceinline__ int padded(int i) { return i + (i >> 4) * PAD; }

// Shared indices of the elements n0 + r * STEP (r = 0, 1, ...) of a transform whose
// element 0 sits at `base`: when STEP * MB is a multiple of 16 the padding is linear in r
// and the index is a compile-time offset from the first one.
template <int MB, int PAD, int STEP> struct sm_run {
    int a0, i0;
    __device__ __forceinline__ sm_run(int base, int n0) : i0(base + n0 * MB) { a0 = padded<PAD>(i0); }
    __device__ __forceinline__ int at(int r) const {
        if constexpr ((STEP * MB) % 16 == 0) {
            return a0 + r * (STEP * MB / 16) * (16 + PAD);
        } else {
            return padded<PAD>(i0 + r * STEP * MB);
        }
    }
};

// One radix-R Stockham stage of the length-L transform on T threads per transform, the
// earlier stages spanning Ns: butterfly b reads elements b + r L / R (times the twiddles
// w_L^{-r (b mod Ns) L / (Ns R)} = tw[(r - 1) Ns + b mod Ns]) and writes
// (b / Ns) Ns R + (b mod Ns) + r Ns.  `load(n, a)` / `store(n, a, v)` move element n, a its
// shared index (SRC_SM / DST_SM: the stage reads / writes the tile buffer sm itself);
// `HALF_IN`: inputs at r >= R / 2 are zero; `HALF_OUT`: outputs at r >= R / 2 are not
// needed; `MID`: barrier between the loads and the stores (in-place shared-memory stage).
// Threads beyond the tile hold j = 1 << 20.
template <int L, int T, int MB, int PAD, int R, int Ns, bool HALF_IN, bool HALF_OUT, bool MID,
          class Load, class Store>
__device__ __forceinline__ void stage(int j, int base, const float2 *tw, Load load, Store store) {
    constexpr int nb = L / R;
    constexpr int IT = (nb + T - 1) / T;
    float2 v[IT][R];
#pragma unroll
    for (int it = 0; it < IT; ++it) {
        const int b = j + it * T;
        if (b < nb) {
            const int kk = b % Ns;
            const sm_run<MB, PAD, nb> in(base, b);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                float2 x = make_float2(0.f, 0.f);
                if (!HALF_IN || r < R / 2) {
                    x = load(b + r * nb, in.at(r));
                    if (Ns > 1 && r > 0) {
                        x = cmul(x, tw[(r - 1) * Ns + kk]);
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
            const sm_run<MB, PAD, Ns> out(base, o);
#pragma unroll
            for (int r = 0; r < (HALF_OUT ? R / 2 : R); ++r) {
                store(o + r * Ns, out.at(r), v[it][r]);
            }
        }
    }
}

// Middle stages s = 1 .. S - 2 of a transform, shared memory to shared memory.
template <int L, int MB, int PAD, int s, class SmLoad, class SmStore>
__device__ __forceinline__ void middle(int j, int base, const float2 *tw, SmLoad ld, SmStore st) {
    if constexpr (s < stages_of(L) - 1) {
        stage<L, threads_of(L), MB, PAD, radix_of(L, s), span_of(L, s), false, false, true>(
            j, base, tw + tw_offset(L, s), ld, st);
        __syncthreads();
        middle<L, MB, PAD, s + 1>(j, base, tw, ld, st);
    }
}

// PAIR (odd real N, no adjoint weights): one complex transform serves the real transforms
// k0 = 2k and k0 + 1 of the tile's pair index k.  r2c: z = x_k0 + i x_k0+1, and with
// Z = FFT(z), X_k0[k] = (Z_k + conj Z_{N-k}) / 2, X_k0+1[k] = -i (Z_k - conj Z_{N-k}) / 2.
// c2r: the engine's load gives A = conj X_k0 and B = conj X_k0+1 (Hermitian extensions),
// the forward transform of A - i B is x_k0 - i x_k0+1.  MB: transforms along M per tile
// (1, 2 or 4, compile-time so that the shared indices of a butterfly are constant
// offsets of one another).
template <int Kind, int L, bool PAIR, int MB>
__device__ __forceinline__ void tile(const fft_params &p, long long t, const float2 *tw) {
    constexpr int T = threads_of(L);
    constexpr int S = stages_of(L);
    constexpr int R0 = radix_of(L, 0);
    constexpr int RL = radix_of(L, S - 1);
    constexpr int NL = span_of(L, S - 1);
    constexpr int PAD = pad_of(L, MB);
    const float2 *twl = tw + tw_offset(L, S - 1); // last stage's twiddles
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int j;
    auto c = make_ctx<float, Kind, default_io>(p, smem_raw, T, L, j, t);
    auto c2 = c; // the second transform of a pair
    if constexpr (PAIR) {
        const int m_l = threadIdx.x % MB;
        const int k_l = threadIdx.x / (MB * T);
        const long long m = (t % p.m_tiles) * MB + m_l;
        const long long k0 = 2 * ((t / p.m_tiles) * p.Kb + k_l);
        c.ib = m + k0 * p.is2;
        c.ob = m + k0 * p.os2;
        c.active = m < p.M && k0 < p.K && k_l < p.Kb;
        c2.ib = c.ib + p.is2;
        c2.ob = c.ob + p.os2;
        c2.active = c.active && k0 + 1 < p.K;
    }
    const int Nc = p.Nc;
    const int base = c.sbase;
    float2 *sm = c.sm;
    const float2 *chirp = static_cast<const float2 *>(p.bs);
    const float2 *bhat = chirp + Nc;
    auto sm_load = [&](int, int a) { return sm[a]; };
    auto sm_store = [&](int, int a, float2 v) { sm[a] = v; };
    // forward transform of a = x . chirp: first stage from global memory
    auto g_load = [&](int n, int) {
        float2 v = make_float2(0.f, 0.f);
        if (n < Nc && c.active) {
            v = c.template gload<0>(n);
            if constexpr (PAIR) {
                const float2 b = c2.active ? c2.template gload<0>(n) : make_float2(0.f, 0.f);
                v = Kind == kind_r2c_full ? make_float2(v.x, b.x) : make_float2(v.x + b.y, v.y - b.x);
            }
            v = cmul(v, __ldg(chirp + n));
        }
        return v;
    };
    stage<L, T, MB, PAD, R0, 1, true, false, false>(j, base, tw, g_load, sm_store);
    __syncthreads();
    middle<L, MB, PAD, 1>(j, base, tw, sm_load, sm_store);
    // last forward stage: times FFT(b) / L, conjugated for the inverse transform
    auto mul_store = [&](int n, int a, float2 v) {
        v = cmul(v, __ldg(bhat + n));
        sm[a] = make_float2(v.x, -v.y);
    };
    stage<L, T, MB, PAD, RL, NL, false, false, true>(j, base, twl, sm_load, mul_store);
    __syncthreads();
    // inverse transform (of the conjugate)
    stage<L, T, MB, PAD, R0, 1, false, false, true>(j, base, tw, sm_load, sm_store);
    __syncthreads();
    middle<L, MB, PAD, 1>(j, base, tw, sm_load, sm_store);
    if constexpr (Kind == kind_r2c_half || (PAIR && Kind == kind_r2c_full)) {
        // Z_k = c_k conj(y_k) into shared memory, then the r2c post-process
        auto z_store = [&](int k, int a, float2 y) {
            if (k < Nc) {
                sm[a] = cmul(make_float2(y.x, -y.y), __ldg(chirp + k));
            }
        };
        stage<L, T, MB, PAD, RL, NL, false, true, true>(j, base, twl, sm_load, z_store);
        __syncthreads();
        if constexpr (Kind == kind_r2c_half) {
            r2c_post<0, T>(c, j, 0);
        } else if (c.active) {
            // split the spectra of the two real transforms
            for (int k = j; 2 * k <= Nc; k += T) {
                const float2 zk = sm[padded<PAD>(base + k * MB)];
                const float2 zn = sm[padded<PAD>(base + (k == 0 ? 0 : Nc - k) * MB)];
                c.template gstore<0>(k, make_float2(0.5f * (zk.x + zn.x), 0.5f * (zk.y - zn.y)));
                if (c2.active) {
                    c2.template gstore<0>(k, make_float2(0.5f * (zk.y + zn.y), 0.5f * (zn.x - zk.x)));
                }
            }
        }
    } else {
        auto g_store = [&](int k, int, float2 y) {
            if (k < Nc && c.active) {
                const float2 v = cmul(make_float2(y.x, -y.y), __ldg(chirp + k));
                c.template gstore<0>(k, v);
                if constexpr (PAIR) {
                    if (c2.active) {
                        c2.template gstore<0>(k, make_float2(-v.y, 0.f));
                    }
                }
            }
        };
        stage<L, T, MB, PAD, RL, NL, false, true, false>(j, base, twl, sm_load, g_store);
    }
}

// One tile per CTA; the stage twiddles are copied into shared memory after the tile buffer
template <int Kind, int L, bool PAIR, int MB> __device__ __forceinline__ void tiles(const fft_params &p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *tw = reinterpret_cast<float2 *>(smem_raw) + p.buf_elems;
    const float2 *gtw = static_cast<const float2 *>(p.bs) + p.Nc + L;
    for (int i = threadIdx.x; i < tw_entries(L); i += blockDim.x) {
        tw[i] = __ldg(gtw + i);
    }
    __syncthreads();
    tile<Kind, L, PAIR, MB>(p, blockIdx.x, tw);
}

template <int Kind, bool PAIR, int MB>
__global__ void __launch_bounds__(256, 5) bluestein_kernel(const __grid_constant__ fft_params p) {
    switch (p.bL) {
    case 256:
        tiles<Kind, 256, PAIR, MB>(p);
        break;
    case 512:
        tiles<Kind, 512, PAIR, MB>(p);
        break;
    case 1024:
        tiles<Kind, 1024, PAIR, MB>(p);
        break;
    }
}

template <int Kind, bool PAIR> const void *kernel_mb(int mb) {
    switch (mb) {
    case 1:
        return reinterpret_cast<const void *>(&bluestein_kernel<Kind, PAIR, 1>);
    case 2:
        return reinterpret_cast<const void *>(&bluestein_kernel<Kind, PAIR, 2>);
    case 4:
        return reinterpret_cast<const void *>(&bluestein_kernel<Kind, PAIR, 4>);
    }
    return nullptr;
}

} // namespace blu

int bluestein_threads(int L) { return blu::threads_of(L); }
int bluestein_stages(int L) { return blu::stages_of(L); }
int bluestein_radix(int L, int s) { return blu::radix_of(L, s); }

int bluestein_pad(int L, int mb) { return blu::pad_of(L, mb); }

const void *bluestein_kernel(int kind, bool pair, int mb) {
    switch (kind) {
    case kind_c2c:
        return blu::kernel_mb<kind_c2c, false>(mb);
    case kind_r2c_half:
        return blu::kernel_mb<kind_r2c_half, false>(mb);
    case kind_r2c_full:
        return pair ? blu::kernel_mb<kind_r2c_full, true>(mb) : blu::kernel_mb<kind_r2c_full, false>(mb);
    case kind_c2r_half:
        return blu::kernel_mb<kind_c2r_half, false>(mb);
    case kind_c2r_full:
        return pair ? blu::kernel_mb<kind_c2r_full, true>(mb) : blu::kernel_mb<kind_c2r_full, false>(mb);
    }
    return nullptr;
}

} // namespace gbfft
