// Double-batched FFT engine for sm_103a.
//
// One CTA transforms a tile of Mb x Kb independent 1d FFTs of an M x N x K tensor
// (column-major; element (m, n, k) at m*s0 + n*s1 + k*s2 with s0 = 1, the layout of
// include/bbfft/configuration.hpp:151-192 in the reference).  The M-mode and the
// K-mode are both batch modes ("double batching", reference README.md:25-29).
//
// Algorithm: Stockham autosort over a list of radices (stage s has radix p_s,
// Ns = p_0 ... p_{s-1}).  Stage s, butterfly b (0 <= b < Nc/p):
//   v[r]  = src[b + r Nc/p] * w_{Ns p}^{-r (b mod Ns)}                (r = 0..p-1)
//   v     = DFT_p(v)
//   dst[(b / Ns) Ns p + (b mod Ns) + r Ns] = v[r]
// The first stage reads global memory directly and the last stage writes global
// memory directly (both accesses are unit-stride across neighbouring butterflies,
// hence coalesced); stages in between exchange through padded shared memory.
// Twiddles for the stages come from a table w_Nt^{-i}, computed on the host in
// extended precision and rounded once (the reference does the same for its
// factor2-SLM kernels, src/common/algorithm/factor2_slm_fft.hpp:49-90).
//
// The same stage code runs with runtime sizes (one kernel per kind for any N) or with
// compile-time sizes (specialised kernels for the frequent N), see fft_tile / fft_tile_ct.
//
// Real transforms follow the reference's generator:
//  * even N: an N/2-point complex FFT of z[n] = x[2n] + i x[2n+1] with a twiddled
//    post-process (r2c, src/base/generator/sbfft_gen.cpp:162-200) or pre-process
//    (c2r, sbfft_gen.cpp:202-247; imag(X[0]) is ignored, imag(X[N/2]) is used as the
//    reference's formula uses it).  The c2r pre-process is fused into the loads of
//    the first stage: Z[n] needs X[n] and X[N/2-n] only.
//  * odd N: an N-point complex FFT of the real data (r2c) or of the Hermitian
//    extension (c2r, imag(X[0]) ignored).  The reference packs two K-slices into one
//    complex FFT for this case (sbfft_gen.cpp:249-351); the result is the same DFT.
//
// Backward transforms run the forward engine on conjugated data:
//   DFT^+(x) = conj(DFT^-(conj(x))).
#pragma once

#include "params.h"
#include "radix.cuh"
#ifndef GBFFT_NVRTC
#include "prime_tc.cuh"
#endif

namespace gbfft {

// Default memory access policy: plain loads and stores at tensor + base + off.  The
// JIT path generates a policy with the same interface that calls user callbacks with
// the element offset base + off (reference callback_accessor,
// src/base/generator/tensor_accessor.cpp:34-55).
struct default_io {
    static constexpr bool direct = true;
    template <class T>
    static __device__ __forceinline__ T load(const T *t, long long base, int off) {
        return (t + base)[off];
    }
    template <class T>
    static __device__ __forceinline__ void store(T *t, long long base, int off, T v) {
        (t + base)[off] = v;
    }
};

template <class R, int Kind, class IO> struct transform_ctx {
    using C = cplx<R>;
    static constexpr int kind_v = Kind;
    const fft_params &p;
    C *sm;        // shared memory
    long long ib; // input base offset (elements)
    long long ob; // output base offset (elements)
    int sbase;    // shared index of element 0 of this transform
    int sstep;    // shared stride between elements (= Mb)
    int bufe;     // elements per shared buffer
    int pshift, padd;
    bool active;

    __device__ __forceinline__ int sidx(int buf, int n) const {
        int i = sbase + n * sstep;
        return buf * bufe + i + (i >> pshift) * padd;
    }

    // Adjoint of r2c: interior bins halved, imaginary parts of DC and Nyquist dropped.
    __device__ __forceinline__ C adj_r2c_weight(C v, int k) const {
        if (k == 0 || 2 * k == p.N) {
            v.y = R(0);
        } else {
            v.x *= R(0.5);
            v.y *= R(0.5);
        }
        return v;
    }
    // Adjoint of c2r (the reference's c2r, including its use of imag(X[N/2]) for even N):
    // interior bins doubled, DC imaginary part zero, Nyquist imaginary part = -sum(g)
    // (the derivative of every output sample w.r.t. imag(X[N/2]) is -1).
    __device__ __forceinline__ C adj_c2r_weight(C v, int k, R g0) const {
        if (k == 0) {
            v.y = R(0);
        } else if (2 * k == p.N) {
            v.y = -g0;
        } else {
            v.x *= R(2);
            v.y *= R(2);
        }
        return v;
    }

    // ---------------- global load of element n of the complex FFT input -----------------
    template <int NC> __device__ __forceinline__ C gload(int n) const {
        if constexpr (Kind == kind_c2c) {
            C v = IO::load(static_cast<const C *>(p.in), ib, n * p.is1);
            if (p.flags & flag_conj_in) {
                v.y = -v.y;
            }
            return v;
        } else if constexpr (Kind == kind_r2c_half) {
            const R *x = static_cast<const R *>(p.in);
            if constexpr (IO::direct) {
                if (p.flags & flag_vec_in) {
                    return reinterpret_cast<const C *>(x + ib)[n];
                }
            }
            R a = IO::load(x, ib, (2 * n) * p.is1);
            R b = IO::load(x, ib, (2 * n + 1) * p.is1);
            return mk<R>(a, b);
        } else if constexpr (Kind == kind_r2c_full) {
            const R *x = static_cast<const R *>(p.in);
            return mk<R>(IO::load(x, ib, n * p.is1), R(0));
        } else if constexpr (Kind == kind_c2r_full) {
            // Hermitian extension of X[0..N/2], conjugated for the forward engine
            const C *X = static_cast<const C *>(p.in);
            const int N = NC ? NC : p.N;
            if (2 * n <= N) {
                C v = IO::load(X, ib, n * p.is1);
                if (n == 0) {
                    v.y = R(0);
                }
                if (p.flags & flag_adj_r2c) {
                    v = adj_r2c_weight(v, n);
                }
                v.y = -v.y;
                return v;
            } else {
                C v = IO::load(X, ib, (N - n) * p.is1);
                if (p.flags & flag_adj_r2c) {
                    v = adj_r2c_weight(v, N - n);
                }
                return v;
            }
        } else {
            // c2r_half: Z[n] = (x1 + x2) + (x1 - x2) i w_N^{+n}, x1 = X[n], x2 = conj X[Nc-n]
            // (sbfft_gen.cpp:209-246), returned conjugated for the forward engine
            const C *X = static_cast<const C *>(p.in);
            const int Nc = NC ? NC : p.Nc;
            C x1 = IO::load(X, ib, n * p.is1);
            C x2 = IO::load(X, ib, (Nc - n) * p.is1);
            if (n == 0) {
                x1.y = R(0);
            }
            if (p.flags & flag_adj_r2c) {
                x1 = adj_r2c_weight(x1, n);
                x2 = adj_r2c_weight(x2, Nc - n);
            }
            x2.y = -x2.y;
            C a = cadd(x1, x2);
            C b = csub(x1, x2);
            C w = __ldg(static_cast<const C *>(p.tw) + n); // w_N^{-n}
            b = cmul(b, mk<R>(w.y, w.x));                  // * i conj(w)
            C z = cadd(a, b);
            z.y = -z.y;
            return z;
        }
    }

    // ---------------- global store of element n of the complex FFT output ---------------
    template <int NC> __device__ __forceinline__ void gstore(int n, C v) const {
        if constexpr (Kind == kind_c2c) {
            if (p.flags & flag_conj_out) {
                v.y = -v.y;
            }
            if (p.flags & flag_scale_out) {
                v.x *= R(p.scale);
                v.y *= R(p.scale);
            }
            IO::store(static_cast<C *>(p.out), ob, n * p.os1, v);
        } else if constexpr (Kind == kind_r2c_full) {
            const int N = NC ? NC : p.N;
            if (2 * n <= N) {
                if (p.flags & flag_adj_c2r) {
                    v = adj_c2r_weight(v, n, R(0));
                }
                IO::store(static_cast<C *>(p.out), ob, n * p.os1, v);
            }
        } else if constexpr (Kind == kind_c2r_full) {
            IO::store(static_cast<R *>(p.out), ob, n * p.os1, v.x);
        } else if constexpr (Kind == kind_c2r_half) {
            R *x = static_cast<R *>(p.out);
            if constexpr (IO::direct) {
                if (p.flags & flag_vec_out) {
                    reinterpret_cast<C *>(x + ob)[n] = mk<R>(v.x, -v.y);
                    return;
                }
            }
            IO::store(x, ob, (2 * n) * p.os1, v.x);
            IO::store(x, ob, (2 * n + 1) * p.os1, R(-v.y));
        }
    }
};

// One Stockham stage for all butterflies of this thread.  NC / TT are the complex FFT
// length and the threads per transform when known at compile time (0 = runtime).
template <int P, int NC, int TT, class R, int Kind, class IO>
__device__ __forceinline__ void run_stage(const transform_ctx<R, Kind, IO> &c, int j, int Ns,
                                          bool src_g, int src_buf, bool dst_g, int dst_buf) {
    using C = cplx<R>;
    constexpr bool half = Kind == kind_r2c_half || Kind == kind_c2r_half;
    const int Nc = NC ? NC : c.p.Nc;
    const int T = TT ? TT : c.p.T;
    const int Nt = NC ? (half ? 2 * NC : NC) : c.p.Nt;
    const int nb = Nc / P;
    const C *tw = static_cast<const C *>(c.p.tw);
    const int twstride = Nt / (Ns * P);
    const int iters = (nb + T - 1) / T;
#pragma unroll
    for (int it = 0; it < iters; ++it) {
        const int b = j + it * T;
        if ((NC == 0 || nb % T != 0) && b >= nb) {
            break;
        }
        C v[P];
        if (src_g) {
            if (c.active) {
                sfor<0, P>([&](auto I) { v[I.value] = c.template gload<NC>(b + I.value * nb); });
            } else {
                sfor<0, P>([&](auto I) { v[I.value] = mk<R>(R(0), R(0)); });
            }
        } else {
            sfor<0, P>([&](auto I) { v[I.value] = c.sm[c.sidx(src_buf, b + I.value * nb)]; });
        }
        const int kk = b % Ns;
        if (P > 1 && Ns > 1) {
            const int base = kk * twstride;
            sfor<1, P>([&](auto I) { v[I.value] = cmul(v[I.value], __ldg(tw + I.value * base)); });
        }
        dft<P, R>::run(v);
        const int o = b + (b / Ns) * Ns * (P - 1);
        if (dst_g) {
            if (c.active) {
                sfor<0, P>([&](auto I) { c.template gstore<NC>(o + I.value * Ns, v[I.value]); });
            }
        } else {
            sfor<0, P>([&](auto I) { c.sm[c.sidx(dst_buf, o + I.value * Ns)] = v[I.value]; });
        }
    }
}

// Odd radix P without an unrolled butterfly (primes above 13).  The stage twiddles are
// first applied in place to the shared source; then every output pair (k, P-k) comes
// from the pair sums s_j = x_j + x_{P-j}, d_j = x_j - x_{P-j} (the reference's pair
// optimisation, src/base/mixed_radix_fft.cpp:55-126):
//   X_k = x_0 + sum_j cos(2 pi jk/P) s_j - i sum_j sin(2 pi jk/P) d_j,  X_{P-k} likewise.
// O(P) work per output.
//
// P <= gen_table_max_p: a task computes G output pairs of one butterfly in one sweep over
// the input pairs, with the coefficients from a k-major table w_P^{-(jk mod P)} in shared
// memory (rows padded to a multiple of G with zeros); lanes working on the same group of
// outputs read the same coefficient (one broadcast load per four FMAs).
// Larger P: tasks of G output pairs over the threads, coefficients from the w_P table.
__device__ __forceinline__ int gen_table_rows(int P) {
    return ((P - 1) / 2 + gen_group - 1) / gen_group * gen_group;
}

#ifndef GBFFT_NVRTC
// Float prime radix 17..61 on the tensor cores (prime_tc.cuh): the block's butterflies
// (Mb * Kb transforms x Nc / P) in groups of 8 per full warp, shared source buffer to
// shared destination buffer, stage twiddles applied as the inputs are loaded.  The host
// launches such kernels with a multiple of 32 threads.
template <int P, class R, int Kind, class IO>
__device__ __forceinline__ void run_stage_prime_tc(const transform_ctx<R, Kind, IO> &c, int Ns,
                                                   int src_buf, int dst_buf) {
    const fft_params &p = c.p;
    const int nb = p.Nc / P;
    const int mb = p.Mb;
    const int nbf = mb * p.Kb * nb;
    const int ngrp = (nbf + 7) / 8;
    const int lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const int twstride = p.Nt / (Ns * P);
    const float2 *tw = static_cast<const float2 *>(p.tw);
    float2 *sm = c.sm;
    const int pshift = c.pshift, padd = c.padd, bufe = c.bufe;
    // butterflies in groups of 8: the same butterfly of 8 neighbouring transforms when
    // Mb >= 8 (adjacent in shared memory), else 8 butterflies of one transform
    const int ntr = mb * p.Kb;
    const bool mfast = mb >= 8;
    for (int grp = threadIdx.x >> 5; grp < ngrp; grp += nwarps) {
        const int q = grp * 8 + (lane >> 2);
        const bool valid = q < nbf;
        const int tr = !valid ? 0 : mfast ? q % ntr : q / nb;
        const int b = !valid ? 0 : mfast ? q / ntr : q - tr * nb;
        const int base = (tr / mb) * p.Nc * mb + (tr % mb);
        const int kk = b % Ns;
        const int o = b + (b / Ns) * Ns * (P - 1);
        auto in = [&](int r) {
            const int i = base + (b + r * nb) * mb;
            return sm + src_buf * bufe + i + (i >> pshift) * padd;
        };
        auto out = [&](int k) {
            const int i = base + (o + k * Ns) * mb;
            return sm + dst_buf * bufe + i + (i >> pshift) * padd;
        };
        ptc::butterflies8<P>(lane, valid, tw, kk * twstride, in, out);
    }
}

#endif

template <class R, int Kind, class IO>
__device__ __forceinline__ void run_stage_generic(const transform_ctx<R, Kind, IO> &c, int j,
                                                  int P, int Ns, int src_buf, bool dst_g,
                                                  int dst_buf) {
    using C = cplx<R>;
    const fft_params &p = c.p;
#ifndef GBFFT_NVRTC
    if constexpr (sizeof(R) == 4) {
        if (!dst_g) {
            switch (P) {
#define GBFFT_PTC_CASE(Q)                                                                        \
    case Q:                                                                                      \
        run_stage_prime_tc<Q>(c, Ns, src_buf, dst_buf);                                          \
        return;
                GBFFT_PTC_CASE(17)
                GBFFT_PTC_CASE(19)
                GBFFT_PTC_CASE(23)
                GBFFT_PTC_CASE(29)
                GBFFT_PTC_CASE(31)
                GBFFT_PTC_CASE(37)
                GBFFT_PTC_CASE(41)
                GBFFT_PTC_CASE(43)
                GBFFT_PTC_CASE(47)
                GBFFT_PTC_CASE(53)
                GBFFT_PTC_CASE(59)
                GBFFT_PTC_CASE(61)
#undef GBFFT_PTC_CASE
            default:
                break;
            }
        }
    }
#endif
    const int Nc = p.Nc;
    const int T = p.T;
    const int nb = Nc / P;
    const C *tw = static_cast<const C *>(p.tw);
    C *wtab = c.sm + p.nbuf * p.buf_elems;
    const int wstride = p.Nt / P;
    const int H = (P - 1) / 2;
    const bool table = P <= gen_table_max_p;
    if (table) {
        // wtab[(k - 1) * H + (jj - 1)] = w_P^{-(jj k mod P)}, k = 1 .. rows
        const int rows = gen_table_rows(P);
        for (int e = threadIdx.x; e < rows * H; e += blockDim.x) {
            const int k = e / H + 1;
            const int jj = e % H + 1;
            wtab[e] = k <= H ? __ldg(tw + ((jj * k) % P) * wstride) : mk<R>(R(0), R(0));
        }
    } else {
        for (int q = threadIdx.x; q < P; q += blockDim.x) {
            wtab[q] = __ldg(tw + q * wstride);
        }
    }
    if (Ns > 1) {
        const int twstride = p.Nt / (Ns * P);
        for (int e = j; e < Nc; e += T) {
            const int b = e % nb;
            const int r = e / nb;
            if (r > 0) {
                C &v = c.sm[c.sidx(src_buf, e)];
                v = cmul(v, __ldg(tw + r * (b % Ns) * twstride));
            }
        }
    }
    __syncthreads();
    auto put = [&](int o, int kf, C v) {
        if (dst_g) {
            if (c.active) {
                c.template gstore<0>(o + kf * Ns, v);
            }
        } else {
            c.sm[c.sidx(dst_buf, o + kf * Ns)] = v;
        }
    };
    constexpr int G = gen_group;
    if (table) {
        // task = (group of G output pairs, butterfly), group-major so that the lanes of a
        // warp mostly share a group and read the same coefficients
        const int tpb = gen_table_rows(P) / G;
        for (int task = j; task < nb * tpb; task += T) {
            const int b = task % nb;
            const int k0 = 1 + (task / nb) * G;
            const int o = b + (b / Ns) * Ns * (P - 1);
            const C x0 = c.sm[c.sidx(src_buf, b)];
            const C *w = wtab + (k0 - 1) * H;
            C acc[G], dd[G];
#pragma unroll
            for (int g = 0; g < G; ++g) {
                acc[g] = x0;
                dd[g] = mk<R>(R(0), R(0));
            }
            C sum = x0;
#pragma unroll 2
            for (int jj = 1; jj <= H; ++jj) {
                const C xa = c.sm[c.sidx(src_buf, b + jj * nb)];
                const C xb = c.sm[c.sidx(src_buf, b + (P - jj) * nb)];
                const C sj = cadd(xa, xb);
                const C dj = csub(xa, xb);
                sum = cadd(sum, sj);
#pragma unroll
                for (int g = 0; g < G; ++g) {
                    const C cw = w[g * H + jj - 1]; // (cos, -sin)(2 pi jj k / P)
                    acc[g].x += cw.x * sj.x;
                    acc[g].y += cw.x * sj.y;
                    dd[g].x += cw.y * dj.x;
                    dd[g].y += cw.y * dj.y;
                }
            }
            if (k0 == 1) {
                put(o, 0, sum);
            }
#pragma unroll
            for (int g = 0; g < G; ++g) {
                const int k = k0 + g;
                if (k <= H) {
                    put(o, k, mk<R>(acc[g].x - dd[g].y, acc[g].y + dd[g].x));
                    put(o, P - k, mk<R>(acc[g].x + dd[g].y, acc[g].y - dd[g].x));
                }
            }
        }
        return;
    }
    // a task computes G output pairs (k, P-k) of one butterfly, so every input pair it
    // loads serves G outputs; the first task of a butterfly also forms X_0 = x_0 + sum s_j
    const int tpb = (H + G - 1) / G; // tasks per butterfly
    for (int task = j; task < nb * tpb; task += T) {
        const int b = task % nb;
        const int k0 = 1 + (task / nb) * G;
        const int o = b + (b / Ns) * Ns * (P - 1);
        const C x0 = c.sm[c.sidx(src_buf, b)];
        C acc[G], bb[G];
        int q[G];
        for (int g = 0; g < G; ++g) {
            acc[g] = x0;
            bb[g] = mk<R>(R(0), R(0));
            q[g] = k0 + g;
        }
        C sum = x0;
        for (int jj = 1; jj <= H; ++jj) {
            const C xa = c.sm[c.sidx(src_buf, b + jj * nb)];
            const C xb = c.sm[c.sidx(src_buf, b + (P - jj) * nb)];
            const C sj = cadd(xa, xb);
            const C dj = csub(xa, xb);
            sum = cadd(sum, sj);
#pragma unroll
            for (int g = 0; g < G; ++g) {
                const C w = wtab[q[g] < P ? q[g] : 0]; // (cos, -sin)(2 pi q / P)
                acc[g].x += w.x * sj.x;
                acc[g].y += w.x * sj.y;
                bb[g].x += w.y * dj.x;
                bb[g].y += w.y * dj.y;
                q[g] += k0 + g;
                if (q[g] >= P) {
                    q[g] -= P;
                }
            }
        }
        if (k0 == 1) {
            put(o, 0, sum);
        }
#pragma unroll
        for (int g = 0; g < G; ++g) {
            const int k = k0 + g;
            if (k <= H) {
                put(o, k, mk<R>(acc[g].x - bb[g].y, acc[g].y + bb[g].x));
                put(o, P - k, mk<R>(acc[g].x + bb[g].y, acc[g].y - bb[g].x));
            }
        }
    }
}

template <class R, int Kind, class IO>
__device__ __forceinline__ void dispatch_stage(const transform_ctx<R, Kind, IO> &c, int j, int P,
                                               int Ns, bool src_g, int src_buf, bool dst_g,
                                               int dst_buf) {
    switch (P) {
    case 1:
        run_stage<1, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 2:
        run_stage<2, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 3:
        run_stage<3, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 4:
        run_stage<4, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 5:
        run_stage<5, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 6:
        run_stage<6, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 7:
        run_stage<7, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 8:
        run_stage<8, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 9:
        run_stage<9, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 10:
        run_stage<10, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 11:
        run_stage<11, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 12:
        run_stage<12, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 13:
        run_stage<13, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 16:
        run_stage<16, 0, 0>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    default:
        run_stage_generic(c, j, P, Ns, src_buf, dst_g, dst_buf);
        break;
    }
}

// r2c (even N) post-process: Z (N/2-point FFT in shared buffer `buf`) -> X[0..N/2].
template <int NC, int TT, class R, int Kind, class IO>
__device__ __forceinline__ void r2c_post(const transform_ctx<R, Kind, IO> &c, int j, int buf) {
    using C = cplx<R>;
    const fft_params &p = c.p;
    const int Nc = NC ? NC : p.Nc;
    const int T = TT ? TT : p.T;
    const C *tw = static_cast<const C *>(p.tw); // w_N^{-i}
    C *X = static_cast<C *>(p.out);
    R g0 = R(0);
    if (p.flags & flag_adj_c2r) {
        // sum of the real input = Re X[0] = Re Z[0] + Im Z[0]
        C z0 = c.sm[c.sidx(buf, 0)];
        g0 = z0.x + z0.y;
    }
    const int cnt = Nc / 2 + 1;
    const int iters = (cnt + T - 1) / T;
#pragma unroll
    for (int it = 0; it < iters; ++it) {
        const int i = j + it * T;
        if ((NC == 0 || cnt % T != 0) && i >= cnt) {
            break;
        }
        const int io = Nc - i;
        C y1 = c.sm[c.sidx(buf, i)];
        C y2 = c.sm[c.sidx(buf, io == Nc ? 0 : io)];
        y2.y = -y2.y;
        C a = mk<R>((y2.x + y1.x) * R(0.5), (y2.y + y1.y) * R(0.5));
        C bb = mk<R>((y2.x - y1.x) * R(0.5), (y2.y - y1.y) * R(0.5));
        C w = __ldg(tw + i);
        bb = cmul(bb, mk<R>(-w.y, w.x)); // * i w_N^{-i}
        C xi = cadd(a, bb);
        C xo = mk<R>(a.x - bb.x, bb.y - a.y);
        if (p.flags & flag_adj_c2r) {
            xi = c.adj_c2r_weight(xi, i, g0);
            xo = c.adj_c2r_weight(xo, io, g0);
        }
        if (c.active) {
            IO::store(X, c.ob, i * p.os1, xi);
            if (i != io) {
                IO::store(X, c.ob, io * p.os1, xo);
            }
        }
    }
}

template <class R, int Kind, class IO>
__device__ __forceinline__ transform_ctx<R, Kind, IO> make_ctx(const fft_params &p, void *smem,
                                                                int T, int Nc, int &j,
                                                                long long tile) {
    const int tid = threadIdx.x;
    const int m_l = tid % p.Mb;
    j = (tid / p.Mb) % T;
    int k_l = tid / (p.Mb * T);
    const long long mt = tile % p.m_tiles;
    const long long kt = tile / p.m_tiles;
    const long long m = mt * p.Mb + m_l;
    const long long k = kt * p.Kb + k_l;
    transform_ctx<R, Kind, IO> c{p, reinterpret_cast<cplx<R> *>(smem), 0, 0, 0, 0, 0, 0, 0, false};
    c.active = (m < p.M) && (k < p.K) && (k_l < p.Kb);
    if (k_l >= p.Kb) {
        // thread beyond the tile (persistent CTAs larger than the tile): no butterflies
        j = 1 << 20;
        k_l = 0;
    }
    c.ib = m + k * p.is2;
    c.ob = m + k * p.os2;
    c.sbase = k_l * Nc * p.Mb + m_l;
    c.sstep = p.Mb;
    c.bufe = p.buf_elems;
    c.pshift = p.pad_shift;
    c.padd = p.pad_add;
    return c;
}

// ---------------------------------------------------------------- runtime-size kernel body
template <class R, int Kind, class IO>
__device__ __forceinline__ void fft_tile_at(const fft_params &p, long long tile) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int j;
    auto c = make_ctx<R, Kind, IO>(p, smem_raw, p.T, p.Nc, j, tile);
    constexpr bool post = Kind == kind_r2c_half;
    int cur = 0;
    int Ns = 1;
    for (int s = 0; s < p.L; ++s) {
        const int P = p.radix[s];
        const bool src_g = s == 0;
        const bool dst_g = (s == p.L - 1) && !post;
        const int dst = (p.nbuf > 1 && !src_g) ? 1 - cur : 0;
        dispatch_stage(c, j, P, Ns, src_g, cur, dst_g, dst);
        cur = dst;
        Ns *= P;
        if (!dst_g) {
            __syncthreads();
        }
    }
    if constexpr (post) {
        r2c_post<0, 0>(c, j, cur);
    }
}

template <class R, int Kind, class IO> __device__ __forceinline__ void fft_tile(const fft_params &p) {
    fft_tile_at<R, Kind, IO>(p, blockIdx.x);
}

} // namespace gbfft
