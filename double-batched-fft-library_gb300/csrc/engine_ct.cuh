// Compile-time-size FFT kernels, vectorised over the left batch mode M.
//
// Same algorithm and data semantics as the runtime engine (engine.cuh), specialised for
// a fixed complex length NC, radix list and threads per transform TT:
//  * every index, trip count and twiddle stride is a compile-time constant;
//  * each thread owns V consecutive m of the M-mode (M is the fastest-varying mode of the
//    column-major tensor, so the V transforms sit next to each other in memory): global
//    and shared accesses move V elements at once (16-byte vectors), and every twiddle load
//    and index computation is shared by V transforms;
//  * stages run in place in ONE shared buffer: a thread keeps all butterflies of a stage
//    in registers, so after a barrier it can overwrite the values it read.
#pragma once

#include "engine.cuh"
#include "prime_tc.cuh"

namespace gbfft {

// ---- vector access of V consecutive elements (aligned to V * sizeof(element)) ----------
template <int V> __device__ __forceinline__ void ldv(const float2 *p, float2 *o) {
    if constexpr (V == 1) {
        o[0] = p[0];
    } else {
        sfor<0, V / 2>([&](auto I) {
            float4 q = reinterpret_cast<const float4 *>(p)[I.value];
            o[2 * I.value] = mk<float>(q.x, q.y);
            o[2 * I.value + 1] = mk<float>(q.z, q.w);
        });
    }
}
template <int V> __device__ __forceinline__ void stv(float2 *p, const float2 *o) {
    if constexpr (V == 1) {
        p[0] = o[0];
    } else {
        sfor<0, V / 2>([&](auto I) {
            float4 q;
            q.x = o[2 * I.value].x;
            q.y = o[2 * I.value].y;
            q.z = o[2 * I.value + 1].x;
            q.w = o[2 * I.value + 1].y;
            reinterpret_cast<float4 *>(p)[I.value] = q;
        });
    }
}
template <int V> __device__ __forceinline__ void ldv(const double2 *p, double2 *o) {
    sfor<0, V>([&](auto I) { o[I.value] = p[I.value]; });
}
template <int V> __device__ __forceinline__ void stv(double2 *p, const double2 *o) {
    sfor<0, V>([&](auto I) { p[I.value] = o[I.value]; });
}
template <int V> __device__ __forceinline__ void ldv(const float *p, float *o) {
    if constexpr (V == 1) {
        o[0] = p[0];
    } else if constexpr (V == 2) {
        float2 q = *reinterpret_cast<const float2 *>(p);
        o[0] = q.x;
        o[1] = q.y;
    } else {
        sfor<0, V / 4>([&](auto I) {
            float4 q = reinterpret_cast<const float4 *>(p)[I.value];
            o[4 * I.value] = q.x;
            o[4 * I.value + 1] = q.y;
            o[4 * I.value + 2] = q.z;
            o[4 * I.value + 3] = q.w;
        });
    }
}
template <int V> __device__ __forceinline__ void stv(float *p, const float *o) {
    if constexpr (V == 1) {
        p[0] = o[0];
    } else if constexpr (V == 2) {
        *reinterpret_cast<float2 *>(p) = mk<float>(o[0], o[1]);
    } else {
        sfor<0, V / 4>([&](auto I) {
            float4 q;
            q.x = o[4 * I.value];
            q.y = o[4 * I.value + 1];
            q.z = o[4 * I.value + 2];
            q.w = o[4 * I.value + 3];
            reinterpret_cast<float4 *>(p)[I.value] = q;
        });
    }
}
template <int V> __device__ __forceinline__ void ldv(const double *p, double *o) {
    if constexpr (V == 1) {
        o[0] = p[0];
    } else {
        sfor<0, V / 2>([&](auto I) {
            double2 q = reinterpret_cast<const double2 *>(p)[I.value];
            o[2 * I.value] = q.x;
            o[2 * I.value + 1] = q.y;
        });
    }
}
template <int V> __device__ __forceinline__ void stv(double *p, const double *o) {
    if constexpr (V == 1) {
        p[0] = o[0];
    } else {
        sfor<0, V / 2>([&](auto I) {
            reinterpret_cast<double2 *>(p)[I.value] = mk<double>(o[2 * I.value], o[2 * I.value + 1]);
        });
    }
}

template <class R, int Kind, int NC, int TT, int V, bool MI = false, bool PAIR = false,
          bool TWO = false, bool REGP = false>
struct ct_ctx {
    using C = cplx<R>;
    static constexpr int kind_v = Kind;
    // may_idle: the block has more threads than the tile (persistent ragged kernel); the
    // threads beyond the tile (live == false) only take part in the barriers
    static constexpr bool may_idle = MI;
    // c2r (even N): form Z[n] and Z[NC-n] together in a pre-pass into shared memory
    static constexpr bool paired_c2r = PAIR;
    // odd real N (r2c_full / c2r_full): with flag_pair, the real transforms k0 and k0 + 1
    // (input / output offsets ib, ob and + is2, + os2) share one complex FFT:
    //   r2c: z = x_k0 + i x_k0+1; X_k0[k] = (Z_k + conj Z_{N-k}) / 2,
    //        X_k0+1[k] = -i (Z_k - conj Z_{N-k}) / 2 (post-process from shared memory);
    //   c2r: the forward FFT of A - i B (A, B: the conjugated Hermitian extensions the
    //        load forms) is x_k0 - i x_k0+1.
    // Without the flag a TWO tile runs single transforms (r2c still through the
    // post-process, which then returns Z_k).
    static constexpr bool two = TWO && (Kind == kind_r2c_full || Kind == kind_c2r_full);
    // the prime radix 17..47 of a short length runs in registers, one butterfly per thread
    // (the generic stage with dft<P>), instead of the tensor-core / shared-memory form
    static constexpr bool reg_prime = REGP;
    static constexpr bool half = Kind == kind_r2c_half || Kind == kind_c2r_half;
    static constexpr int NN = half ? 2 * NC : NC; // logical length (odd kinds: N = NC)
    // lane vectors of 16 bytes or more are stored as 16-byte chunks in NQ planes with an
    // XOR swizzle; 8-byte elements (float, V = 1) use the padded linear layout
    static constexpr bool LIN = sizeof(C) * V < 16;
    static constexpr int NQ = LIN ? 1 : int(sizeof(C)) * V / 16;
    static constexpr int PER = LIN ? 1 : 16 / int(sizeof(C)); // complex per chunk
    const fft_params &p;
    C *sm;
    long long ib, ob;
    int sbase; // LIN: shared index of element 0; else chunk index of element 0
    int pshift, padd;
    bool active;
    bool live = true;
    bool active2 = false; // the second transform of a pair (two)

    __device__ __forceinline__ int sidx(int n) const { // LIN layout
        int i = sbase + n * p.Mb;
        return i + (i >> pshift) * padd;
    }
    __device__ __forceinline__ int chunk(int n) const { // plane layout
        int c = sbase + n * (p.Mb / V);
        return c ^ (((c >> p.sw_a) & p.sw_mask) << p.sw_b);
    }
    __device__ __forceinline__ void sload(int n, C *o) const {
        if constexpr (LIN) {
            ldv<V>(sm + sidx(n), o);
        } else {
            const int c = chunk(n);
            sfor<0, NQ>([&](auto Q) { ldv<PER>(sm + (Q.value * p.plane_chunks + c) * PER, o + Q.value * PER); });
        }
    }
    __device__ __forceinline__ void sstore(int n, const C *o) const {
        if constexpr (LIN) {
            stv<V>(sm + sidx(n), o);
        } else {
            const int c = chunk(n);
            sfor<0, NQ>([&](auto Q) { stv<PER>(sm + (Q.value * p.plane_chunks + c) * PER, o + Q.value * PER); });
        }
    }

    __device__ __forceinline__ C adj_r2c_weight(C v, int k) const {
        if (k == 0 || 2 * k == NN) {
            v.y = R(0);
        } else {
            v.x *= R(0.5);
            v.y *= R(0.5);
        }
        return v;
    }
    __device__ __forceinline__ C adj_c2r_weight(C v, int k, R g0) const {
        if (k == 0) {
            v.y = R(0);
        } else if (2 * k == NN) {
            v.y = -g0;
        } else {
            v.x *= R(2);
            v.y *= R(2);
        }
        return v;
    }

    __device__ __forceinline__ void gload(int n, C *o) const {
        if constexpr (Kind == kind_c2c) {
            ldv<V>(static_cast<const C *>(p.in) + ib + n * p.is1, o);
            if (p.flags & flag_conj_in) {
                sfor<0, V>([&](auto U) { o[U.value].y = -o[U.value].y; });
            }
        } else if constexpr (Kind == kind_r2c_half) {
            const R *x = static_cast<const R *>(p.in) + ib;
            if (V == 1 && (p.flags & flag_vec_in)) {
                o[0] = reinterpret_cast<const C *>(x)[n];
                return;
            }
            R a[V], b[V];
            ldv<V>(x + (2 * n) * p.is1, a);
            ldv<V>(x + (2 * n + 1) * p.is1, b);
            sfor<0, V>([&](auto U) { o[U.value] = mk<R>(a[U.value], b[U.value]); });
        } else if constexpr (Kind == kind_r2c_full) {
            R a[V], b[V];
            ldv<V>(static_cast<const R *>(p.in) + ib + n * p.is1, a);
            sfor<0, V>([&](auto U) { b[U.value] = R(0); });
            if constexpr (two) {
                if (active2) {
                    ldv<V>(static_cast<const R *>(p.in) + ib + p.is2 + n * p.is1, b);
                }
            }
            sfor<0, V>([&](auto U) { o[U.value] = mk<R>(a[U.value], b[U.value]); });
        } else if constexpr (Kind == kind_c2r_full) {
            c2r_full_load(static_cast<const C *>(p.in) + ib, n, o);
            if constexpr (two) {
                if (active2) {
                    C b[V];
                    c2r_full_load(static_cast<const C *>(p.in) + ib + p.is2, n, b);
                    sfor<0, V>([&](auto U) {
                        o[U.value] = mk<R>(o[U.value].x + b[U.value].y, o[U.value].y - b[U.value].x);
                    });
                }
            }
        } else {
            c2r_half_load(n, o);
        }
    }

    // c2r_full: the Hermitian extension of X[0..N/2] at n, conjugated for the forward engine
    __device__ __forceinline__ void c2r_full_load(const C *X, int n, C *o) const {
        if constexpr (Kind == kind_c2r_full) {
            if (2 * n <= NN) {
                ldv<V>(X + n * p.is1, o);
                sfor<0, V>([&](auto U) {
                    C v = o[U.value];
                    if (n == 0) {
                        v.y = R(0);
                    }
                    if (p.flags & flag_adj_r2c) {
                        v = adj_r2c_weight(v, n);
                    }
                    v.y = -v.y;
                    o[U.value] = v;
                });
            } else {
                ldv<V>(X + (NN - n) * p.is1, o);
                if (p.flags & flag_adj_r2c) {
                    sfor<0, V>([&](auto U) { o[U.value] = adj_r2c_weight(o[U.value], NN - n); });
                }
            }
        }
    }

    __device__ __forceinline__ void c2r_half_load(int n, C *o) const {
        if constexpr (Kind == kind_c2r_half) {
            // c2r_half: Z[n] = (x1 + x2) + (x1 - x2) i w_N^{+n}, x1 = X[n], x2 = conj X[NC-n]
            const C *X = static_cast<const C *>(p.in) + ib;
            C x1[V], x2[V];
            ldv<V>(X + n * p.is1, x1);
            ldv<V>(X + (NC - n) * p.is1, x2);
            C w = __ldg(static_cast<const C *>(p.tw) + n);
            C iw = mk<R>(w.y, w.x);
            sfor<0, V>([&](auto U) {
                C a1 = x1[U.value], a2 = x2[U.value];
                if (n == 0) {
                    a1.y = R(0);
                }
                if (p.flags & flag_adj_r2c) {
                    a1 = adj_r2c_weight(a1, n);
                    a2 = adj_r2c_weight(a2, NC - n);
                }
                a2.y = -a2.y;
                C a = cadd(a1, a2);
                C b = cmul(csub(a1, a2), iw);
                C z = cadd(a, b);
                z.y = -z.y;
                o[U.value] = z;
            });
        }
    }

    __device__ __forceinline__ void gstore(int n, C *v) const {
        if constexpr (Kind == kind_c2c) {
            if (p.flags & flag_conj_out) {
                sfor<0, V>([&](auto U) { v[U.value].y = -v[U.value].y; });
            }
            if (p.flags & flag_scale_out) {
                sfor<0, V>([&](auto U) {
                    v[U.value].x *= R(p.scale);
                    v[U.value].y *= R(p.scale);
                });
            }
            stv<V>(static_cast<C *>(p.out) + ob + n * p.os1, v);
        } else if constexpr (Kind == kind_r2c_full) {
            if (2 * n <= NN) {
                if (p.flags & flag_adj_c2r) {
                    sfor<0, V>([&](auto U) { v[U.value] = adj_c2r_weight(v[U.value], n, R(0)); });
                }
                stv<V>(static_cast<C *>(p.out) + ob + n * p.os1, v);
            }
        } else if constexpr (Kind == kind_c2r_full) {
            R a[V];
            sfor<0, V>([&](auto U) { a[U.value] = v[U.value].x; });
            stv<V>(static_cast<R *>(p.out) + ob + n * p.os1, a);
            if constexpr (two) {
                if (active2) {
                    sfor<0, V>([&](auto U) { a[U.value] = -v[U.value].y; });
                    stv<V>(static_cast<R *>(p.out) + ob + p.os2 + n * p.os1, a);
                }
            }
        } else if constexpr (Kind == kind_c2r_half) {
            R *x = static_cast<R *>(p.out) + ob;
            if (V == 1 && (p.flags & flag_vec_out)) {
                reinterpret_cast<C *>(x)[n] = mk<R>(v[0].x, -v[0].y);
                return;
            }
            R a[V], b[V];
            sfor<0, V>([&](auto U) {
                a[U.value] = v[U.value].x;
                b[U.value] = -v[U.value].y;
            });
            stv<V>(x + (2 * n) * p.os1, a);
            stv<V>(x + (2 * n + 1) * p.os1, b);
        }
    }
};

// Odd prime radix 17..61 with compile-time roots of unity (shared memory in and out, one
// transform per thread along M).  A task is one group of G output pairs (k, P-k) of one
// butterfly; consecutive threads take consecutive butterflies of the same group, so the
// lanes of a warp mostly run the same group and every coefficient is a literal operand
// of its FMA.  With s_j = x_j + x_{P-j}, d_j = x_j - x_{P-j} (the reference's pair
// optimisation, src/base/mixed_radix_fft.cpp:55-126):
//   X_k = x_0 + sum_j cos(2 pi jk/P) s_j - i sum_j sin(2 pi jk/P) d_j,  X_{P-k} likewise.
// The stage twiddles are applied in place first; the results stay in registers until
// every task has read its inputs (the stage runs in place).
__host__ __device__ constexpr bool ct_big_prime(int P) { return P > 16 && P <= 61 && P % 2 == 1; }

template <int P, int GRP, int G, class Ctx, class R>
__device__ __forceinline__ void ct_prime_group(const Ctx &c, int b, int nb, cplx<R> *out) {
    using C = cplx<R>;
    constexpr int H = (P - 1) / 2;
    C x0[1];
    c.sload(b, x0);
    C acc[G], dd[G];
    sfor<0, G>([&](auto Q) {
        acc[Q.value] = x0[0];
        dd[Q.value] = mk<R>(R(0), R(0));
    });
    C sum = x0[0];
    sfor<1, H + 1>([&](auto J) {
        constexpr int jj = decltype(J)::value;
        C xa[1], xb[1];
        c.sload(b + jj * nb, xa);
        c.sload(b + (P - jj) * nb, xb);
        const C sj = cadd(xa[0], xb[0]);
        const C dj = csub(xa[0], xb[0]);
        if constexpr (GRP == 0) {
            sum = cadd(sum, sj);
        }
        sfor<0, G>([&](auto Q) {
            constexpr int k = GRP * G + decltype(Q)::value + 1;
            if constexpr (k <= H) {
                constexpr R cr = W<R, P, jj * k>::re; //  cos(2 pi jj k / P)
                constexpr R ci = W<R, P, jj * k>::im; // -sin(2 pi jj k / P)
                acc[Q.value].x += cr * sj.x;
                acc[Q.value].y += cr * sj.y;
                dd[Q.value].x += ci * dj.x;
                dd[Q.value].y += ci * dj.y;
            }
        });
    });
    out[0] = sum;
    sfor<0, G>([&](auto Q) {
        out[1 + 2 * Q.value] = mk<R>(acc[Q.value].x - dd[Q.value].y, acc[Q.value].y + dd[Q.value].x);
        out[2 + 2 * Q.value] = mk<R>(acc[Q.value].x + dd[Q.value].y, acc[Q.value].y - dd[Q.value].x);
    });
}

// Float prime radix as the last stage: the tile's butterflies in groups of 8 per warp on
// the tensor cores (prime_tc.cuh), in place (a butterfly's outputs overwrite its own
// inputs when NS * P == NC).  Every full warp of the block takes part; the host launches
// these tiles with a multiple of 32 threads.
template <int P, int NS, class Ctx, int NC>
__device__ __forceinline__ void ct_stage_prime_tc(const Ctx &c) {
    static_assert(NS * P == NC && Ctx::LIN, "tensor-core prime stage: last stage, scalar layout");
    constexpr int nb = NC / P;
    constexpr int twstride = (Ctx::half ? 2 * NC : NC) / NC;
    const fft_params &p = c.p;
    const int mb = p.Mb;
    const int nbf = mb * p.Kb * nb; // butterflies of the tile
    const int ngrp = (nbf + 7) / 8;
    const int lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    const float2 *tw = static_cast<const float2 *>(p.tw);
    float2 *sm = c.sm;
    const int pshift = c.pshift, padd = c.padd;
    // butterflies in groups of 8: with 8 or more transforms along M the group's butterflies
    // are the same butterfly of 8 neighbouring transforms (adjacent in shared memory), else
    // 8 butterflies of one transform (adjacent when Mb = 1)
    const int ntr = mb * p.Kb;
    const bool mfast = mb >= 8;
    for (int grp = threadIdx.x >> 5; grp < ngrp; grp += nwarps) {
        const int q = grp * 8 + (lane >> 2);
        const bool valid = q < nbf;
        const int tr = !valid ? 0 : mfast ? q % ntr : q / nb;
        const int b = !valid ? 0 : mfast ? q / ntr : q - tr * nb;
        const int base = (tr / mb) * NC * mb + (tr % mb) + b * mb;
        auto at = [&](int n) {
            const int i = base + n * (nb * mb);
            return sm + i + (i >> pshift) * padd;
        };
        ptc::butterflies8<P>(lane, valid, tw, b * twstride, at, at);
    }
}

template <int P, int NS, class Ctx, class R, int NC, int TT>
__device__ __forceinline__ void ct_stage_prime(const Ctx &c, int j) {
    using C = cplx<R>;
    if constexpr (sizeof(R) == 4 && NS * P == NC && ptc::supported(P)) {
        (void)j;
        ct_stage_prime_tc<P, NS, Ctx, NC>(c);
    } else {
    constexpr int nb = NC / P;
    constexpr int H = (P - 1) / 2;
    constexpr int G = sizeof(R) == 4 ? 8 : 4;
    constexpr int NG = (H + G - 1) / G;
    constexpr int NT = nb * NG;
    constexpr int ITERS = (NT + TT - 1) / TT;
    constexpr int twstride = (Ctx::half ? 2 * NC : NC) / (NS * P);
    const bool live = !Ctx::may_idle || c.live;
    if constexpr (NS > 1) {
        const C *tw = static_cast<const C *>(c.p.tw);
        constexpr int IE = (NC + TT - 1) / TT;
#pragma unroll
        for (int it = 0; it < IE; ++it) {
            const int e = j + it * TT;
            if (live && (NC % TT == 0 || e < NC)) {
                const int b = e % nb;
                const int r = e / nb;
                if (r > 0) {
                    C v[1];
                    c.sload(e, v);
                    v[0] = cmul(v[0], __ldg(tw + r * (b % NS) * twstride));
                    c.sstore(e, v);
                }
            }
        }
        __syncthreads();
    }
    C out[ITERS][2 * G + 1];
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = j + it * TT;
        if (live && (NT % TT == 0 || t < NT)) {
            const int grp = t / nb;
            const int b = t % nb;
            sfor<0, NG>([&](auto Gi) {
                if (grp == Gi.value) {
                    ct_prime_group<P, Gi.value, G, Ctx, R>(c, b, nb, out[it]);
                }
            });
        }
    }
    __syncthreads(); // every input is read before the outputs overwrite the buffer
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int t = j + it * TT;
        if (live && (NT % TT == 0 || t < NT)) {
            const int grp = t / nb;
            const int b = t % nb;
            const int o = b + (b / NS) * NS * (P - 1);
            if (grp == 0) {
                c.sstore(o, &out[it][0]);
            }
            sfor<0, G>([&](auto Q) {
                const int k = grp * G + Q.value + 1;
                if (k <= H) {
                    c.sstore(o + k * NS, &out[it][1 + 2 * Q.value]);
                    c.sstore(o + (P - k) * NS, &out[it][2 + 2 * Q.value]);
                }
            });
        }
    }
    }
}

// One in-place Stockham stage with compile-time sizes (see engine.cuh for the formulas).
// A prime radix 17..61 takes the shared-memory / tensor-core form (ct_stage_prime) unless
// the tile runs it in registers (Ctx::reg_prime): then it is an ordinary stage whose
// butterfly is dft<P> (radix.cuh, pair sums with literal coefficients), one per thread.
template <int P, int NS, bool SRC_G, bool DST_G, class Ctx, class R, int NC, int TT, int V>
__device__ __forceinline__ void ct_stage(const Ctx &c, int j) {
    if constexpr (ct_big_prime(P) && !Ctx::reg_prime) {
        static_assert(!SRC_G && !DST_G && V == 1, "prime stages run shared to shared, V = 1");
        ct_stage_prime<P, NS, Ctx, R, NC, TT>(c, j);
        return;
    } else {
    using C = cplx<R>;
    constexpr int nb = NC / P;
    constexpr int ITERS = (nb + TT - 1) / TT;
    constexpr int twstride = (Ctx::half ? 2 * NC : NC) / (NS * P);
    const C *tw = static_cast<const C *>(c.p.tw);
    C v[ITERS][V][P];
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int b = j + it * TT;
        if ((nb % TT == 0 || b < nb) && (!Ctx::may_idle || c.live)) {
            if constexpr (SRC_G) {
                if (c.active) {
                    sfor<0, P>([&](auto I) {
                        C t[V];
                        c.gload(b + I.value * nb, t);
                        sfor<0, V>([&](auto U) { v[it][U.value][I.value] = t[U.value]; });
                    });
                } else {
                    sfor<0, P>([&](auto I) {
                        sfor<0, V>([&](auto U) { v[it][U.value][I.value] = mk<R>(R(0), R(0)); });
                    });
                }
            } else {
                sfor<0, P>([&](auto I) {
                    C t[V];
                    c.sload(b + I.value * nb, t);
                    sfor<0, V>([&](auto U) { v[it][U.value][I.value] = t[U.value]; });
                });
            }
            if constexpr (P > 1 && NS > 1) {
                const int kk = b % NS;
                sfor<1, P>([&](auto I) {
                    C w = __ldg(tw + I.value * kk * twstride);
                    sfor<0, V>([&](auto U) { v[it][U.value][I.value] = cmul(v[it][U.value][I.value], w); });
                });
            }
            sfor<0, V>([&](auto U) { dft<P, R>::run(v[it][U.value]); });
        }
    }
    if constexpr (!SRC_G && !DST_G) {
        __syncthreads(); // every value of the buffer is read before it is overwritten
    }
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int b = j + it * TT;
        if ((nb % TT == 0 || b < nb) && (!Ctx::may_idle || c.live)) {
            const int o = b + (b / NS) * NS * (P - 1);
            sfor<0, P>([&](auto I) {
                C t[V];
                sfor<0, V>([&](auto U) { t[U.value] = v[it][U.value][I.value]; });
                if constexpr (DST_G) {
                    if (c.active) {
                        c.gstore(o + I.value * NS, t);
                    }
                } else {
                    c.sstore(o + I.value * NS, t);
                }
            });
        }
    }
    }
}

// r2c (even N) post-process from the shared buffer, V transforms per thread.
template <class Ctx, class R, int NC, int TT, int V>
__device__ __forceinline__ void ct_r2c_post(const Ctx &c, int j) {
    using C = cplx<R>;
    const C *tw = static_cast<const C *>(c.p.tw);
    constexpr int cnt = NC / 2 + 1;
    constexpr int ITERS = (cnt + TT - 1) / TT;
    if constexpr (Ctx::may_idle) {
        if (!c.live) {
            return;
        }
    }
    R g0[V];
    if (c.p.flags & flag_adj_c2r) {
        C z0[V];
        c.sload(0, z0);
        sfor<0, V>([&](auto U) { g0[U.value] = z0[U.value].x + z0[U.value].y; });
    }
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int i = j + it * TT;
        if (cnt % TT == 0 || i < cnt) {
            const int io = NC - i;
            C y1[V], y2[V], xi[V], xo[V];
            c.sload(i, y1);
            c.sload(io == NC ? 0 : io, y2);
            C w = __ldg(tw + i);
            C iw = mk<R>(-w.y, w.x);
            sfor<0, V>([&](auto U) {
                C a2 = y2[U.value], a1 = y1[U.value];
                a2.y = -a2.y;
                C a = mk<R>((a2.x + a1.x) * R(0.5), (a2.y + a1.y) * R(0.5));
                C b = mk<R>((a2.x - a1.x) * R(0.5), (a2.y - a1.y) * R(0.5));
                b = cmul(b, iw);
                C p1 = cadd(a, b);
                C p2 = mk<R>(a.x - b.x, b.y - a.y);
                if (c.p.flags & flag_adj_c2r) {
                    p1 = c.adj_c2r_weight(p1, i, g0[U.value]);
                    p2 = c.adj_c2r_weight(p2, io, g0[U.value]);
                }
                xi[U.value] = p1;
                xo[U.value] = p2;
            });
            if (c.active) {
                C *X = static_cast<C *>(c.p.out) + c.ob;
                stv<V>(X + i * c.p.os1, xi);
                if (i != io) {
                    stv<V>(X + io * c.p.os1, xo);
                }
            }
        }
    }
}

// c2r (even N) pre-process into the shared buffer, V transforms per thread.  Z[n] and
// Z[NC-n] need the same two inputs X[n], X[NC-n] and twiddles w_N^{-n}, w_N^{-(NC-n)} =
// -conj(w_N^{-n}), so one thread forms both (reference formula: sbfft_gen.cpp:209-246):
//   Z[n] = (x1 + x2) + (x1 - x2) i conj(w_N^{-n}),  x1 = X[n], x2 = conj X[NC-n]
// (imag X[0] ignored), stored conjugated for the forward engine.
template <class Ctx, class R, int NC, int TT, int V>
__device__ __forceinline__ void ct_c2r_pre(const Ctx &c, int j) {
    using C = cplx<R>;
    constexpr int cnt = NC / 2 + 1;
    constexpr int ITERS = (cnt + TT - 1) / TT;
    const C *X = static_cast<const C *>(c.p.in) + c.ib;
    const C *tw = static_cast<const C *>(c.p.tw);
    const bool adj = c.p.flags & flag_adj_r2c;
    auto z_of = [&](C a1, C a2, C iw, int k1, int k2, bool zero_im) {
        if (zero_im) {
            a1.y = R(0);
        }
        if (adj) {
            a1 = c.adj_r2c_weight(a1, k1);
            a2 = c.adj_r2c_weight(a2, k2);
        }
        a2.y = -a2.y;
        C z = cadd(cadd(a1, a2), cmul(csub(a1, a2), iw));
        z.y = -z.y;
        return z;
    };
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int n = j + it * TT;
        if ((cnt % TT == 0 || n < cnt) && (!Ctx::may_idle || c.live)) {
            const int m = NC - n;
            C x1[V], x2[V], zn[V], zm[V];
            if (c.active) {
                ldv<V>(X + n * c.p.is1, x1);
                ldv<V>(X + m * c.p.is1, x2);
            } else {
                sfor<0, V>([&](auto U) {
                    x1[U.value] = mk<R>(R(0), R(0));
                    x2[U.value] = mk<R>(R(0), R(0));
                });
            }
            const C w = __ldg(tw + n);
            const C iw = mk<R>(w.y, w.x);  // i conj(w_N^{-n})
            const C iwm = mk<R>(w.y, -w.x); // i conj(w_N^{-(NC-n)}), w_N^{-(NC-n)} = -conj(w)
            sfor<0, V>([&](auto U) {
                zn[U.value] = z_of(x1[U.value], x2[U.value], iw, n, m, n == 0);
                zm[U.value] = z_of(x2[U.value], x1[U.value], iwm, m, n, false);
            });
            c.sstore(n, zn);
            if (n != 0 && m != n) {
                c.sstore(m, zm);
            }
        }
    }
}

// r2c (odd N) of a TWO tile: split Z (shared buffer) into the spectra of the pair's two
// real transforms, X_k0[k] = (Z_k + conj Z_{N-k}) / 2, X_k0+1[k] = -i (Z_k - conj Z_{N-k}) / 2,
// k = 0..(N-1)/2.
template <class Ctx, class R, int NC, int TT, int V>
__device__ __forceinline__ void ct_r2c_two_post(const Ctx &c, int j) {
    using C = cplx<R>;
    constexpr int cnt = NC / 2 + 1;
    constexpr int ITERS = (cnt + TT - 1) / TT;
    if constexpr (Ctx::may_idle) {
        if (!c.live) {
            return;
        }
    }
#pragma unroll
    for (int it = 0; it < ITERS; ++it) {
        const int k = j + it * TT;
        if ((cnt % TT == 0 || k < cnt) && c.active) {
            C zk[V], zn[V], x0[V], x1[V];
            c.sload(k, zk);
            c.sload(k == 0 ? 0 : NC - k, zn);
            sfor<0, V>([&](auto U) {
                const C a = zk[U.value], b = zn[U.value];
                C v = mk<R>((a.x + b.x) * R(0.5), (a.y - b.y) * R(0.5));
                if (c.p.flags & flag_adj_c2r) {
                    v = c.adj_c2r_weight(v, k, R(0));
                }
                x0[U.value] = v;
                x1[U.value] = mk<R>((a.y + b.y) * R(0.5), (b.x - a.x) * R(0.5));
            });
            C *X = static_cast<C *>(c.p.out) + c.ob + k * c.p.os1;
            stv<V>(X, x0);
            if (c.active2) {
                stv<V>(X + c.p.os2, x1);
            }
        }
    }
}

template <class Ctx, class R, int NC, int TT, int V, int S, int L, int NS, int P, int... Rest>
__device__ __forceinline__ void ct_run(const Ctx &c, int j) {
    constexpr bool two_post = Ctx::two && Ctx::kind_v == kind_r2c_full;
    constexpr bool post = Ctx::kind_v == kind_r2c_half || two_post;
    // c2r (even N), paired variant: the pre-process fills the shared buffer and the first
    // stage reads it; otherwise the first stage forms Z[n] in its own loads
    constexpr bool pre = S == 0 && Ctx::kind_v == kind_c2r_half && Ctx::paired_c2r;
    constexpr bool src_g = S == 0 && !pre;
    constexpr bool dst_g = (S == L - 1) && !post;
    if constexpr (pre) {
        ct_c2r_pre<Ctx, R, NC, TT, V>(c, j);
        __syncthreads();
    }
    ct_stage<P, NS, src_g, dst_g, Ctx, R, NC, TT, V>(c, j);
    if constexpr (!dst_g) {
        __syncthreads();
    }
    if constexpr (sizeof...(Rest) > 0) {
        ct_run<Ctx, R, NC, TT, V, S + 1, L, NS * P, Rest...>(c, j);
    } else if constexpr (two_post) {
        ct_r2c_two_post<Ctx, R, NC, TT, V>(c, j);
    } else if constexpr (post) {
        ct_r2c_post<Ctx, R, NC, TT, V>(c, j);
    }
}

template <class R, int Kind, int NC, int TT, int V, bool PAIR, int... Ps>
__device__ __forceinline__ void fft_tile_ct(const fft_params &p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using Ctx = ct_ctx<R, Kind, NC, TT, V, false, PAIR>;
    const int tid = threadIdx.x;
    const int mvb = p.Mb / V;
    const int mv = tid % mvb;
    const int j = (tid / mvb) % TT;
    const int k_l = tid / (mvb * TT);
    const long long mt = blockIdx.x % p.m_tiles;
    const long long kt = blockIdx.x / p.m_tiles;
    const int m_l = mv * V;
    const long long m = mt * p.Mb + m_l;
    const long long k = kt * p.Kb + k_l;
    const int sbase = Ctx::LIN ? k_l * NC * p.Mb + m_l : k_l * NC * mvb + mv;
    Ctx c{p, reinterpret_cast<cplx<R> *>(smem_raw), m + k * p.is2, m + k * p.os2, sbase,
          p.pad_shift, p.pad_add, (m < p.M) && (k < p.K)};
    ct_run<Ctx, R, NC, TT, V, 0, sizeof...(Ps), 1, Ps...>(c, j);
}

// The same tile for the persistent ragged kernel: tile index given, block possibly larger
// than the tile's (Mb / V) * TT * Kb threads.  TWO: odd real N, the tile's k index counts
// pairs of transforms when the plan sets flag_pair (ct_ctx::two); REGP: the prime stage
// runs in registers (ct_ctx::reg_prime).
template <class R, int Kind, int NC, int TT, int V, bool TWO, bool REGP, int... Ps>
__device__ __forceinline__ void fft_tile_ct_ragged_t(const fft_params &p, long long tile) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using Ctx = ct_ctx<R, Kind, NC, TT, V, true, false, TWO, REGP>;
    const int tid = threadIdx.x;
    const int mvb = p.Mb / V;
    const bool live = tid < mvb * TT * p.Kb;
    const int mv = tid % mvb;
    const int j = (tid / mvb) % TT;
    const int k_l = live ? tid / (mvb * TT) : 0;
    const long long mt = tile % p.m_tiles;
    const long long kt = tile / p.m_tiles;
    const int m_l = mv * V;
    const long long m = mt * p.Mb + m_l;
    long long k = kt * p.Kb + k_l;
    bool pair = false;
    if constexpr (Ctx::two) {
        pair = (p.flags & flag_pair) != 0;
        if (pair) {
            k *= 2;
        }
    }
    const int sbase = Ctx::LIN ? k_l * NC * p.Mb + m_l : k_l * NC * mvb + mv;
    Ctx c{p, reinterpret_cast<cplx<R> *>(smem_raw), m + k * p.is2, m + k * p.os2, sbase,
          p.pad_shift, p.pad_add, live && (m < p.M) && (k < p.K), live};
    c.active2 = pair && c.active && k + 1 < p.K;
    ct_run<Ctx, R, NC, TT, V, 0, sizeof...(Ps), 1, Ps...>(c, j);
}

template <class R, int Kind, int NC, int TT, int V, int... Ps>
__device__ __forceinline__ void fft_tile_ct_ragged(const fft_params &p, long long tile) {
    fft_tile_ct_ragged_t<R, Kind, NC, TT, V, false, false, Ps...>(p, tile);
}

// Ragged batches, one CTA per unit: stage the unit's parameters (item un.x, tile un.y)
// in shared memory.
__device__ __forceinline__ int2 stage_unit_params(const ragged_item_dev *__restrict__ items,
                                                  const int2 *__restrict__ units,
                                                  fft_params &s_p) {
    constexpr int NW = static_cast<int>(sizeof(fft_params) / sizeof(int));
    const int2 un = units[blockIdx.x];
    // the block may have fewer threads than the parameter block has words
    for (int i = threadIdx.x; i < NW; i += blockDim.x) {
        reinterpret_cast<int *>(&s_p)[i] = __ldg(reinterpret_cast<const int *>(&items[un.x].p) + i);
    }
    __syncthreads();
    return un;
}

} // namespace gbfft
