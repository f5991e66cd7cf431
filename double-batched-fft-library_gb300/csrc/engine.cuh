// Double-batched FFT engine for sm_103a.
//
// One CTA transforms a tile of Mb x Kb independent 1d FFTs of an M x N x K tensor
// (column-major; element (m, n, k) at m*s0 + n*s1 + k*s2 with s0 = 1, the layout of
// include/bbfft/configuration.hpp:151-192 in the reference).  The M-mode and the
// K-mode are both batch modes ("double batching", reference README.md:25-29).
//
// Algorithm: Stockham autosort over a runtime list of radices (stage s has radix
// p_s, Ns = p_0 ... p_{s-1}).  Stage s, butterfly b (0 <= b < Nc/p):
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
// Real transforms follow the reference's generator:
//  * even N: an N/2-point complex FFT of z[n] = x[2n] + i x[2n+1] with a twiddled
//    post-process (r2c, src/base/generator/sbfft_gen.cpp:162-200) or pre-process
//    (c2r, sbfft_gen.cpp:202-247; imag(X[0]) is ignored, imag(X[N/2]) is used as the
//    reference's formula uses it);
//  * odd N: an N-point complex FFT of the real data (r2c) or of the Hermitian
//    extension (c2r, imag(X[0]) ignored).  The reference packs two K-slices into one
//    complex FFT for this case (sbfft_gen.cpp:249-351); the arithmetic result is the
//    same DFT.
//
// Backward transforms run the forward engine on conjugated data:
//   DFT^+(x) = conj(DFT^-(conj(x))).
#pragma once

#include "params.h"
#include "radix.cuh"

namespace gbfft {




// ---------------------------------------------------------------------------------------------
// Shared-memory padding: one element every (128 bytes / element size) so that strided
// Stockham writes and the column reads of the next stage avoid bank conflicts.
template <class R> __device__ __forceinline__ int spad(int i) {
    if constexpr (sizeof(R) == 4) {
        return i + (i >> 4);
    } else {
        return i + (i >> 3);
    }
}
template <class R> constexpr int spad_host(int i) { return sizeof(R) == 4 ? i + (i >> 4) : i + (i >> 3); }

// Default memory access policy: plain loads and stores.  A user-callback policy with
// the same interface is generated by the JIT path.
struct default_io {
    template <class T> static __device__ __forceinline__ T load(const T *p, unsigned long long off) {
        return p[off];
    }
    template <class T>
    static __device__ __forceinline__ void store(T *p, unsigned long long off, T v) {
        p[off] = v;
    }
};

template <class R, int Kind, class IO> struct transform_ctx {
    using C = cplx<R>;
    const fft_params &p;
    C *sm;        // shared memory
    long long ib; // input base offset (elements)
    long long ob; // output base offset (elements)
    int sbase;    // shared index of element 0 of this transform
    int sstep;    // shared stride between elements (= Mb)
    bool active;

    __device__ __forceinline__ int sidx(int buf, int n) const {
        return buf * p.buf_elems + spad<R>(sbase + n * sstep);
    }

    // ---------------- global load of element n of the complex FFT input -----------------
    __device__ __forceinline__ C gload(int n) const {
        if constexpr (Kind == kind_c2c) {
            C v = IO::load(static_cast<const C *>(p.in), (unsigned long long)(ib + n * p.is1));
            if (p.flags & flag_conj_in) {
                v.y = -v.y;
            }
            return v;
        } else if constexpr (Kind == kind_r2c_half) {
            const R *x = static_cast<const R *>(p.in);
            R a = IO::load(x, (unsigned long long)(ib + (2 * n) * p.is1));
            R b = IO::load(x, (unsigned long long)(ib + (2 * n + 1) * p.is1));
            return mk<R>(a, b);
        } else if constexpr (Kind == kind_r2c_full) {
            const R *x = static_cast<const R *>(p.in);
            return mk<R>(IO::load(x, (unsigned long long)(ib + n * p.is1)), R(0));
        } else if constexpr (Kind == kind_c2r_full) {
            // Hermitian extension of X[0..N/2], conjugated for the forward engine
            const C *X = static_cast<const C *>(p.in);
            int h = p.N / 2;
            if (n <= h) {
                C v = IO::load(X, (unsigned long long)(ib + n * p.is1));
                if (n == 0) {
                    v.y = R(0);
                }
                if (p.flags & flag_adj_r2c) {
                    v = adj_r2c_weight(v, n);
                }
                v.y = -v.y;
                return v;
            } else {
                C v = IO::load(X, (unsigned long long)(ib + (p.N - n) * p.is1));
                if (p.flags & flag_adj_r2c) {
                    v = adj_r2c_weight(v, p.N - n);
                }
                return v;
            }
        } else {
            return mk<R>(R(0), R(0)); // c2r_half is loaded by its pre-process
        }
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

    // ---------------- global store of element n of the complex FFT output ---------------
    __device__ __forceinline__ void gstore(int n, C v) const {
        if constexpr (Kind == kind_c2c) {
            if (p.flags & flag_conj_out) {
                v.y = -v.y;
            }
            if (p.flags & flag_scale_out) {
                v.x *= R(p.scale);
                v.y *= R(p.scale);
            }
            IO::store(static_cast<C *>(p.out), (unsigned long long)(ob + n * p.os1), v);
        } else if constexpr (Kind == kind_r2c_full) {
            if (2 * n <= p.N) {
                if (p.flags & flag_adj_c2r) {
                    v = adj_c2r_weight(v, n, 0);
                }
                IO::store(static_cast<C *>(p.out), (unsigned long long)(ob + n * p.os1), v);
            }
        } else if constexpr (Kind == kind_c2r_full) {
            IO::store(static_cast<R *>(p.out), (unsigned long long)(ob + n * p.os1), v.x);
        } else if constexpr (Kind == kind_c2r_half) {
            R *x = static_cast<R *>(p.out);
            IO::store(x, (unsigned long long)(ob + (2 * n) * p.os1), v.x);
            IO::store(x, (unsigned long long)(ob + (2 * n + 1) * p.os1), R(-v.y));
        }
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
};

// One stage for all butterflies of this thread. Src/Dst: 0 = global, 1 = shared
template <int P, class R, int Kind, class IO>
__device__ __forceinline__ void run_stage(const transform_ctx<R, Kind, IO> &c, int j, int Ns,
                                          bool src_g, int src_buf, bool dst_g, int dst_buf) {
    using C = cplx<R>;
    const fft_params &p = c.p;
    const int Nc = p.Nc;
    const int nb = Nc / P;
    const C *tw = static_cast<const C *>(p.tw);
    const int twstride = p.Nt / (Ns * P);
    for (int b = j; b < nb; b += p.T) {
        C v[P];
        if (src_g) {
            if (c.active) {
                sfor<0, P>([&](auto I) { v[I.value] = c.gload(b + I.value * nb); });
            } else {
                sfor<0, P>([&](auto I) { v[I.value] = mk<R>(R(0), R(0)); });
            }
        } else {
            sfor<0, P>([&](auto I) { v[I.value] = c.sm[c.sidx(src_buf, b + I.value * nb)]; });
        }
        const int kk = b % Ns;
        if (Ns > 1) {
            const int base = kk * twstride;
            sfor<1, P>([&](auto I) { v[I.value] = cmul(v[I.value], __ldg(tw + I.value * base)); });
        }
        dft<P, R>::run(v);
        const int o = b + (b / Ns) * Ns * (P - 1);
        if (dst_g) {
            if (c.active) {
                sfor<0, P>([&](auto I) { c.gstore(o + I.value * Ns, v[I.value]); });
            }
        } else {
            sfor<0, P>([&](auto I) { c.sm[c.sidx(dst_buf, o + I.value * Ns)] = v[I.value]; });
        }
    }
}

// Radix without an unrolled butterfly: every output is a length-P sum read from shared
// memory (src must be shared).  O(P) work per output.
template <class R, int Kind, class IO>
__device__ __forceinline__ void run_stage_generic(const transform_ctx<R, Kind, IO> &c, int j,
                                                  int P, int Ns, int src_buf, bool dst_g,
                                                  int dst_buf) {
    using C = cplx<R>;
    const fft_params &p = c.p;
    const int Nc = p.Nc;
    const int nb = Nc / P;
    const C *tw = static_cast<const C *>(p.tw);
    const int twstride = p.Nt / (Ns * P); // stage twiddle: w_{Ns P}
    const int wstride = p.Nt / P;         // DFT kernel: w_P
    for (int idx = j; idx < Nc; idx += p.T) {
        const int b = idx % nb;
        const int kf = idx / nb;
        const int kk = b % Ns;
        C acc = mk<R>(R(0), R(0));
        int q = 0; // (jf * kf) mod P
        for (int jf = 0; jf < P; ++jf) {
            C x = c.sm[c.sidx(src_buf, b + jf * nb)];
            if (Ns > 1 && jf > 0) {
                x = cmul(x, __ldg(tw + jf * kk * twstride));
            }
            C w = __ldg(tw + q * wstride);
            acc.x += x.x * w.x - x.y * w.y;
            acc.y += x.x * w.y + x.y * w.x;
            q += kf;
            if (q >= P) {
                q -= P;
            }
        }
        const int o = b + (b / Ns) * Ns * (P - 1) + kf * Ns;
        if (dst_g) {
            if (c.active) {
                c.gstore(o, acc);
            }
        } else {
            c.sm[c.sidx(dst_buf, o)] = acc;
        }
    }
}

template <class R, int Kind, class IO>
__device__ __forceinline__ void run_copy(const transform_ctx<R, Kind, IO> &c, int j, bool src_g,
                                         int src_buf, bool dst_g, int dst_buf) {
    using C = cplx<R>;
    for (int n = j; n < c.p.Nc; n += c.p.T) {
        C v;
        if (src_g) {
            v = c.active ? c.gload(n) : mk<R>(R(0), R(0));
        } else {
            v = c.sm[c.sidx(src_buf, n)];
        }
        if (dst_g) {
            if (c.active) {
                c.gstore(n, v);
            }
        } else {
            c.sm[c.sidx(dst_buf, n)] = v;
        }
    }
}

template <class R, int Kind, class IO>
__device__ __forceinline__ void dispatch_stage(const transform_ctx<R, Kind, IO> &c, int j, int P,
                                               int Ns, bool src_g, int src_buf, bool dst_g,
                                               int dst_buf) {
    switch (P) {
    case 1:
        run_copy(c, j, src_g, src_buf, dst_g, dst_buf);
        break;
    case 2:
        run_stage<2>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 3:
        run_stage<3>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 4:
        run_stage<4>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 5:
        run_stage<5>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 6:
        run_stage<6>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 7:
        run_stage<7>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 8:
        run_stage<8>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 9:
        run_stage<9>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 10:
        run_stage<10>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 11:
        run_stage<11>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 12:
        run_stage<12>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 13:
        run_stage<13>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    case 16:
        run_stage<16>(c, j, Ns, src_g, src_buf, dst_g, dst_buf);
        break;
    default:
        run_stage_generic(c, j, P, Ns, src_buf, dst_g, dst_buf);
        break;
    }
}

// True if radix P has an unrolled butterfly (must match dispatch_stage).
__host__ __device__ constexpr bool radix_unrolled(int P) {
    return P == 1 || (P >= 2 && P <= 13) || P == 16;
}

// r2c (even N) post-process: Z (N/2-point FFT in shared buffer `buf`) -> X[0..N/2].
template <class R, int Kind, class IO>
__device__ __forceinline__ void r2c_post(const transform_ctx<R, Kind, IO> &c, int j, int buf) {
    using C = cplx<R>;
    const fft_params &p = c.p;
    const int Nc = p.Nc;
    const C *tw = static_cast<const C *>(p.tw); // w_N^{-i}
    C *X = static_cast<C *>(p.out);
    R g0 = R(0);
    if (p.flags & flag_adj_c2r) {
        // sum of the real input = Re X[0] = Re Z[0] + Im Z[0]
        C z0 = c.sm[c.sidx(buf, 0)];
        g0 = z0.x + z0.y;
    }
    for (int i = j; 2 * i <= Nc; i += p.T) {
        const int io = Nc - i;
        C y1 = c.sm[c.sidx(buf, i)];
        C y2 = c.sm[c.sidx(buf, io == Nc ? 0 : io)];
        y2.y = -y2.y;
        C a = mk<R>((y2.x + y1.x) * R(0.5), (y2.y + y1.y) * R(0.5));
        C bb = mk<R>((y2.x - y1.x) * R(0.5), (y2.y - y1.y) * R(0.5));
        // b *= i * w_N^{-i}
        C w = __ldg(tw + i);
        C iw = mk<R>(-w.y, w.x);
        bb = cmul(bb, iw);
        C xi = cadd(a, bb);
        C xo = mk<R>(a.x - bb.x, bb.y - a.y);
        if (p.flags & flag_adj_c2r) {
            xi = c.adj_c2r_weight(xi, i, g0);
            xo = c.adj_c2r_weight(xo, io, g0);
        }
        if (c.active) {
            IO::store(X, (unsigned long long)(c.ob + i * p.os1), xi);
            if (i != io) {
                IO::store(X, (unsigned long long)(c.ob + io * p.os1), xo);
            }
        }
    }
}

// c2r (even N) pre-process: X[0..N/2] (global) -> conj(Z) in shared buffer `buf`.
template <class R, int Kind, class IO>
__device__ __forceinline__ void c2r_pre(const transform_ctx<R, Kind, IO> &c, int j, int buf) {
    using C = cplx<R>;
    const fft_params &p = c.p;
    const int Nc = p.Nc;
    const C *tw = static_cast<const C *>(p.tw); // w_N^{-i}
    const C *X = static_cast<const C *>(p.in);
    for (int i = j; 2 * i <= Nc; i += p.T) {
        const int io = Nc - i;
        C x1 = mk<R>(R(0), R(0)), x2 = mk<R>(R(0), R(0));
        if (c.active) {
            x1 = IO::load(X, (unsigned long long)(c.ib + i * p.is1));
            x2 = IO::load(X, (unsigned long long)(c.ib + io * p.is1));
        }
        if (i == 0) {
            x1.y = R(0);
        }
        if (p.flags & flag_adj_r2c) {
            x1 = c.adj_r2c_weight(x1, i);
            x2 = c.adj_r2c_weight(x2, io);
        }
        x2.y = -x2.y;
        C a = cadd(x1, x2);
        C bb = csub(x1, x2);
        // b *= i * w_N^{+i} = i * conj(w_N^{-i})
        C w = __ldg(tw + i);
        C iw = mk<R>(w.y, w.x);
        bb = cmul(bb, iw);
        C z = cadd(a, bb);
        C zo = mk<R>(a.x - bb.x, bb.y - a.y);
        // store conj for the forward engine
        c.sm[c.sidx(buf, i)] = cconj(z);
        if (i != 0 && i != io) {
            c.sm[c.sidx(buf, io)] = cconj(zo);
        }
    }
}

template <class R, int Kind, class IO> __device__ __forceinline__ void fft_tile(const fft_params &p) {
    using C = cplx<R>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C *sm = reinterpret_cast<C *>(smem_raw);

    const int tid = threadIdx.x;
    const int m_l = tid % p.Mb;
    const int j = (tid / p.Mb) % p.T;
    const int k_l = tid / (p.Mb * p.T);
    const long long mt = blockIdx.x % p.m_tiles;
    const long long kt = blockIdx.x / p.m_tiles;
    const long long m = mt * p.Mb + m_l;
    const long long k = kt * p.Kb + k_l;

    transform_ctx<R, Kind, IO> c{p, sm, 0, 0, 0, 0, false};
    c.active = (m < p.M) && (k < p.K) && (k_l < p.Kb);
    c.ib = m + k * p.is2;
    c.ob = m + k * p.os2;
    c.sbase = k_l * p.Nc * p.Mb + m_l;
    c.sstep = p.Mb;

    constexpr bool pre = Kind == kind_c2r_half;
    constexpr bool post = Kind == kind_r2c_half;

    int cur = 0; // shared buffer holding the current data
    if constexpr (pre) {
        c2r_pre(c, j, 0);
        __syncthreads();
    }
    int Ns = 1;
    for (int s = 0; s < p.L; ++s) {
        const int P = p.radix[s];
        const bool src_g = (s == 0) && !pre;
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
        r2c_post(c, j, cur);
    }
}

} // namespace gbfft
