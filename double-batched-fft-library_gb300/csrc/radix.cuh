// In-register radix-P DFT butterflies with compile-time roots of unity.
//
// Semantics follow the reference's mixed-radix core: an unnormalised DFT
//   X[k] = sum_j x[j] * w_P^{-j k},  w_P = exp(2 pi i / P)        (forward, sign -1)
// (src/base/mixed_radix_fft.cpp:46-53 basic_esum, 215-254 inplace<ESum>).
// Odd primes use the reference's "pair optimisation": the products with w and
// conj(w) share one real and one imaginary multiply
// (src/base/mixed_radix_fft.cpp:55-126).  Composite P are split in registers by a
// Cooley-Tukey step with compile-time twiddles.  Only the forward sign is
// implemented; the backward transform is obtained by conjugating input and
// output at the load/store boundary.
//
// Everything here compiles both under nvcc and under NVRTC (no standard headers).
#pragma once

#include "root_of_unity_table.cuh"

namespace gbfft {

template <class R> struct cplx_of;
template <> struct cplx_of<float> {
    using type = float2;
};
template <> struct cplx_of<double> {
    using type = double2;
};
template <class R> using cplx = typename cplx_of<R>::type;

template <class R> __device__ __forceinline__ cplx<R> mk(R x, R y) {
    cplx<R> c;
    c.x = x;
    c.y = y;
    return c;
}
template <class C> __device__ __forceinline__ C cadd(C a, C b) {
    a.x += b.x;
    a.y += b.y;
    return a;
}
template <class C> __device__ __forceinline__ C csub(C a, C b) {
    a.x -= b.x;
    a.y -= b.y;
    return a;
}
template <class C> __device__ __forceinline__ C cmul(C a, C b) {
    C c;
    c.x = a.x * b.x - a.y * b.y;
    c.y = a.x * b.y + a.y * b.x;
    return c;
}
// a * (-i)
template <class C> __device__ __forceinline__ C cmul_mi(C a) {
    C c;
    c.x = a.y;
    c.y = -a.x;
    return c;
}
template <class C> __device__ __forceinline__ C cconj(C a) {
    a.y = -a.y;
    return a;
}

// ---- compile-time integer helpers -------------------------------------------------
template <int I> struct ic {
    static constexpr int value = I;
};
template <int B, int E, class F> __device__ __forceinline__ void sfor(F &&f) {
    if constexpr (B < E) {
        f(ic<B>{});
        sfor<B + 1, E>(f);
    }
}
__host__ __device__ constexpr int smallest_factor(int n) {
    for (int f = 2; f * f <= n; ++f) {
        if (n % f == 0) {
            return f;
        }
    }
    return n;
}
__host__ __device__ constexpr bool is_prime_ct(int n) { return n >= 2 && smallest_factor(n) == n; }

// ---- compile-time roots of unity ------------------------------------------------------
// W<R,P,K>::re/im = cos/sin(-2 pi K / P): the forward twiddle w_P^{-K}.
template <class R, int P, int K> struct W;
template <int P, int K> struct W<double, P, K> {
    static_assert(P >= 1 && P <= rou::kMaxP, "root of unity order out of table range");
    static constexpr int k = ((K % P) + P) % P;
    static constexpr double re = rou::kCosD[rou::kOffset[P] + k];
    static constexpr double im = -rou::kSinD[rou::kOffset[P] + k];
};
template <int P, int K> struct W<float, P, K> {
    static_assert(P >= 1 && P <= rou::kMaxP, "root of unity order out of table range");
    static constexpr int k = ((K % P) + P) % P;
    static constexpr float re = rou::kCosF[rou::kOffset[P] + k];
    static constexpr float im = -rou::kSinF[rou::kOffset[P] + k];
};

// multiply by the compile-time constant w_P^{-K}, with the trivial cases folded
template <class R, int P, int K> __device__ __forceinline__ cplx<R> twc(cplx<R> a) {
    constexpr int k = ((K % P) + P) % P;
    if constexpr (k == 0) {
        return a;
    } else if constexpr (4 * k == P) { // -i
        return cmul_mi(a);
    } else if constexpr (2 * k == P) { // -1
        return mk<R>(-a.x, -a.y);
    } else if constexpr (4 * k == 3 * P) { // +i
        return mk<R>(-a.y, a.x);
    } else {
        constexpr R c = W<R, P, k>::re;
        constexpr R s = W<R, P, k>::im;
        return mk<R>(a.x * c - a.y * s, a.x * s + a.y * c);
    }
}

// ---- butterflies --------------------------------------------------------------------------
template <int P, class R> struct dft;

template <class R> struct dft<1, R> {
    static __device__ __forceinline__ void run(cplx<R> *) {}
};

template <class R> struct dft<2, R> {
    static __device__ __forceinline__ void run(cplx<R> *v) {
        cplx<R> a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};

template <class R> struct dft<4, R> {
    static __device__ __forceinline__ void run(cplx<R> *v) {
        cplx<R> a0 = cadd(v[0], v[2]);
        cplx<R> a1 = csub(v[0], v[2]);
        cplx<R> a2 = cadd(v[1], v[3]);
        cplx<R> a3 = cmul_mi(csub(v[1], v[3]));
        v[0] = cadd(a0, a2);
        v[2] = csub(a0, a2);
        v[1] = cadd(a1, a3);
        v[3] = csub(a1, a3);
    }
};

template <class R> struct dft<8, R> {
    static __device__ __forceinline__ void run(cplx<R> *v) {
        cplx<R> e[4] = {v[0], v[2], v[4], v[6]};
        cplx<R> o[4] = {v[1], v[3], v[5], v[7]};
        dft<4, R>::run(e);
        dft<4, R>::run(o);
        constexpr R h = W<R, 8, 1>::re; // sqrt(1/2)
        cplx<R> o1 = mk<R>((o[1].x + o[1].y) * h, (o[1].y - o[1].x) * h);   // * w8^-1
        cplx<R> o2 = cmul_mi(o[2]);                                            // * w8^-2
        cplx<R> o3 = mk<R>((o[3].y - o[3].x) * h, -(o[3].x + o[3].y) * h);  // * w8^-3
        v[0] = cadd(e[0], o[0]);
        v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], o1);
        v[5] = csub(e[1], o1);
        v[2] = cadd(e[2], o2);
        v[6] = csub(e[2], o2);
        v[3] = cadd(e[3], o3);
        v[7] = csub(e[3], o3);
    }
};

// Odd prime P: pair optimisation (w and conj(w) share the multiply).
template <int P, class R> struct dft_prime {
    static __device__ __forceinline__ void run(cplx<R> *v) {
        constexpr int H = (P - 1) / 2;
        cplx<R> s[H + 1], d[H + 1];
        cplx<R> x0 = v[0];
        cplx<R> sum = x0;
        sfor<1, H + 1>([&](auto J) {
            constexpr int j = decltype(J)::value;
            s[j] = cadd(v[j], v[P - j]);
            d[j] = csub(v[j], v[P - j]);
            sum = cadd(sum, s[j]);
        });
        sfor<1, H + 1>([&](auto Kc) {
            constexpr int k = decltype(Kc)::value;
            cplx<R> a = x0;
            cplx<R> b = mk<R>(R(0), R(0));
            sfor<1, H + 1>([&](auto J) {
                constexpr int j = decltype(J)::value;
                constexpr R c = W<R, P, j * k>::re;
                constexpr R sn = -W<R, P, j * k>::im; // sin(2 pi jk / P)
                a.x += c * s[j].x;
                a.y += c * s[j].y;
                b.x += sn * d[j].x;
                b.y += sn * d[j].y;
            });
            // X_k = a - i b, X_{P-k} = a + i b
            v[k] = mk<R>(a.x + b.y, a.y - b.x);
            v[P - k] = mk<R>(a.x - b.y, a.y + b.x);
        });
        v[0] = sum;
    }
};

// Composite P = A * B, decimation in time:
//   n = B n1 + n2, k = k1 + A k2
//   X[k1 + A k2] = sum_n2 w_B^{-n2 k2} w_P^{-n2 k1} sum_n1 x[B n1 + n2] w_A^{-n1 k1}
template <int P, int A, class R> struct dft_ct {
    static constexpr int B = P / A;
    static __device__ __forceinline__ void run(cplx<R> *v) {
        cplx<R> y[P];
        sfor<0, B>([&](auto N2) {
            constexpr int n2 = decltype(N2)::value;
            cplx<R> u[A];
            sfor<0, A>([&](auto N1) { u[N1.value] = v[B * N1.value + n2]; });
            dft<A, R>::run(u);
            sfor<0, A>([&](auto K1) {
                constexpr int k1 = decltype(K1)::value;
                y[k1 * B + n2] = twc<R, P, n2 * k1>(u[k1]);
            });
        });
        sfor<0, A>([&](auto K1) {
            constexpr int k1 = decltype(K1)::value;
            cplx<R> t[B];
            sfor<0, B>([&](auto N2) { t[N2.value] = y[k1 * B + N2.value]; });
            dft<B, R>::run(t);
            sfor<0, B>([&](auto K2) { v[k1 + A * K2.value] = t[K2.value]; });
        });
    }
};

template <int P> __host__ __device__ constexpr int ct_split() {
    // preferred first factor for in-register Cooley-Tukey
    if constexpr (P % 4 == 0 && P != 8) {
        return 4;
    } else {
        return smallest_factor(P);
    }
}

template <int P, class R> struct dft {
    static __device__ __forceinline__ void run(cplx<R> *v) {
        if constexpr (is_prime_ct(P)) {
            dft_prime<P, R>::run(v);
        } else {
            dft_ct<P, ct_split<P>(), R>::run(v);
        }
    }
};

} // namespace gbfft
