// Radix stages on the tensor cores (float transforms): the odd primes 17..61 and 16, 32.
//
// A radix-P butterfly is a P x P complex DFT: O(P) work per output on the CUDA cores,
// which made the lengths with a prime factor 17..61 the slowest of the engine.  With the
// reference's pair optimisation (src/base/mixed_radix_fft.cpp:55-126), s_j = x_j + x_{P-j},
// d_j = x_j - x_{P-j} for j = 1..H (H = (P-1)/2 for odd P; P/2 - 1 for even P, where
// x_h = x_{P/2} has no partner and enters with the sign (-1)^k):
//   X_0 = x_0 + x_h + sum_j s_j,  X_{P/2} = x_0 + x_h + sum_j (-1)^j s_j  (even P, P/2 even),
//   X_k = x_0 + (-1)^k x_h + U_k + i W_k,  X_{P-k} = x_0 + (-1)^k x_h + U_k - i W_k  (k = 1..H),
//   U_k = sum_j cos(2 pi jk/P) s_j,  W_k = sum_j -sin(2 pi jk/P) d_j
// (x_h = 0 for odd P).
// U and W are real matrix products with K = j and N = k (padded to multiples of 8).  One
// warp runs them for 8 butterflies at a time as mma.sync.m16n8k8 TF32 with FP32
// accumulation: the 16 rows of A are the real and imaginary parts of the 8 butterflies'
// s (or d) values, B holds the coefficients.  Precision: every operand is split into two
// TF32 pieces (hi + lo, about 22 bits) and three products are accumulated,
// A_lo B_hi + A_hi B_lo + A_hi B_hi (the lo * lo term is below 2^-22 relative), which keeps
// the stage at FP32 accuracy.  The coefficient fragments are precomputed per lane
// (gen_prime_frags.py, evaluated in double and split once).
//
// Lane l = 4 g + t of the warp works on butterfly g of the group of 8: it loads that
// butterfly's inputs j = 8 ks + t + 1 and 8 ks + t + 5 of every k-step ks (the A fragment
// entries (row g, col t), (row g + 8, col t), (row g, col t + 4), (row g + 8, col t + 4)),
// and receives the outputs k = 8 nt + 2 t + 1 and + 2 of every n-tile nt (the accumulator
// entries (row g, cols 2t, 2t + 1) and (row g + 8, same cols)).  A lane therefore reads
// and writes only its own butterfly's elements, and the four lanes of a butterfly finish
// their reads before any of them writes (the MMAs consume every loaded value): a
// butterfly whose outputs overwrite its own inputs (the last stage of a transform) runs
// in place without a block barrier.
#pragma once

#include "prime_frag_table.cuh"

namespace gbfft {
namespace ptc {

__host__ __device__ constexpr bool supported(int P) {
    return P == 17 || P == 19 || P == 23 || P == 29 || P == 31 || P == 37 || P == 41 || P == 43 ||
           P == 47 || P == 53 || P == 59 || P == 61;
}
__host__ __device__ constexpr int pairs(int P) { return P % 2 ? (P - 1) / 2 : P / 2 - 1; }

__device__ __forceinline__ unsigned to_tf32(float x) {
    unsigned r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

// x = hi + lo with both pieces TF32
__device__ __forceinline__ void split_tf32(float x, unsigned &hi, unsigned &lo) {
    hi = to_tf32(x);
    lo = to_tf32(x - __uint_as_float(hi));
}

__device__ __forceinline__ void mma_tf32(float *d, const unsigned *a, unsigned b0, unsigned b1) {
    asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, "
                 "{%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One group of 8 butterflies of radix P on the calling warp (all 32 lanes must call it
// together).  `valid`: this lane's butterfly exists; in(r) / out(k): pointers to element r
// of its input and element k of its output; tw: the twiddle table w^{-i}, twb: the
// butterfly's twiddle exponent step (element r is multiplied by tw[r * twb]; twb = 0 for
// none).
template <int P, class In, class Out>
__device__ __forceinline__ void butterflies8(int lane, bool valid, const float2 *__restrict__ tw,
                                             int twb, In in, Out out) {
    static_assert(P % 2 == 1 || (P / 2) % 2 == 0, "even radices with an even half (16, 32)");
    constexpr bool EVEN = P % 2 == 0;
    constexpr int H = pairs(P);
    constexpr int KS = (H + 7) / 8; // k-steps (input pairs) = n-tiles (output pairs)
    const uint4 *__restrict__ frag = frag_table<P>();
    const int t = lane & 3;
    float2 x0 = make_float2(0.f, 0.f), xh = make_float2(0.f, 0.f);
    if (valid) {
        x0 = *in(0);
        if constexpr (EVEN) {
            xh = *in(P / 2);
            if (twb) {
                const float2 w = __ldg(tw + (P / 2) * twb);
                xh = make_float2(xh.x * w.x - xh.y * w.y, xh.x * w.y + xh.y * w.x);
            }
        }
    }
    float sre = 0.f, sim = 0.f; // sum of the lane's s_j
    float are = 0.f, aim = 0.f; // sum of (-1)^j s_j (even P)
    float u[KS][4], w[KS][4];
#pragma unroll
    for (int n = 0; n < KS; ++n) {
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            u[n][e] = 0.f;
            w[n][e] = 0.f;
        }
    }
#pragma unroll
    for (int ks = 0; ks < KS; ++ks) {
        float sv[4], dv[4]; // (re, im) of j0 and j1
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int j = 8 * ks + t + 1 + 4 * h;
            float2 a = make_float2(0.f, 0.f), b = make_float2(0.f, 0.f);
            if (valid && j <= H) {
                a = *in(j);
                b = *in(P - j);
                if (twb) {
                    const float2 wa = __ldg(tw + j * twb);
                    const float2 wb = __ldg(tw + (P - j) * twb);
                    a = make_float2(a.x * wa.x - a.y * wa.y, a.x * wa.y + a.y * wa.x);
                    b = make_float2(b.x * wb.x - b.y * wb.y, b.x * wb.y + b.y * wb.x);
                }
            }
            sv[2 * h] = a.x + b.x;
            sv[2 * h + 1] = a.y + b.y;
            dv[2 * h] = a.x - b.x;
            dv[2 * h + 1] = a.y - b.y;
            sre += sv[2 * h];
            sim += sv[2 * h + 1];
            if constexpr (EVEN) {
                are += (j & 1) ? -sv[2 * h] : sv[2 * h];
                aim += (j & 1) ? -sv[2 * h + 1] : sv[2 * h + 1];
            }
        }
        // A fragments: a0 = re(j0), a1 = im(j0), a2 = re(j1), a3 = im(j1)
        unsigned sh[4], sl[4], dh[4], dl[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            split_tf32(sv[e], sh[e], sl[e]);
            split_tf32(dv[e], dh[e], dl[e]);
        }
#pragma unroll
        for (int nt = 0; nt < KS; ++nt) {
            const uint4 fc = __ldg(frag + ((ks * KS + nt) * 32 + lane) * 2);
            const uint4 fs = __ldg(frag + ((ks * KS + nt) * 32 + lane) * 2 + 1);
            mma_tf32(u[nt], sl, fc.x, fc.y);
            mma_tf32(u[nt], sh, fc.z, fc.w);
            mma_tf32(u[nt], sh, fc.x, fc.y);
            mma_tf32(w[nt], dl, fs.x, fs.y);
            mma_tf32(w[nt], dh, fs.z, fs.w);
            mma_tf32(w[nt], dh, fs.x, fs.y);
        }
    }
    // X_0 (and X_{P/2}) = constant part + sum of all s_j of the butterfly: the four lanes
    // of a butterfly hold disjoint parts of the sums
    sre += __shfl_xor_sync(0xffffffffu, sre, 1);
    sim += __shfl_xor_sync(0xffffffffu, sim, 1);
    sre += __shfl_xor_sync(0xffffffffu, sre, 2);
    sim += __shfl_xor_sync(0xffffffffu, sim, 2);
    if constexpr (EVEN) {
        are += __shfl_xor_sync(0xffffffffu, are, 1);
        aim += __shfl_xor_sync(0xffffffffu, aim, 1);
        are += __shfl_xor_sync(0xffffffffu, are, 2);
        aim += __shfl_xor_sync(0xffffffffu, aim, 2);
    }
    __syncwarp();
    if (!valid) {
        return;
    }
    // x_0 + x_h and x_0 - x_h: the constant part of the outputs of even and odd k
    const float2 ev = make_float2(x0.x + xh.x, x0.y + xh.y);
    const float2 od = make_float2(x0.x - xh.x, x0.y - xh.y);
    if (t == 0) {
        *out(0) = make_float2(ev.x + sre, ev.y + sim);
    }
    if constexpr (EVEN) {
        if (t == 1) {
            *out(P / 2) = make_float2(ev.x + are, ev.y + aim);
        }
    }
#pragma unroll
    for (int nt = 0; nt < KS; ++nt) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int k = 8 * nt + 2 * t + 1 + e;
            if (k <= H) {
                const float2 b = (k & 1) ? od : ev;
                const float ur = u[nt][e], ui = u[nt][2 + e];
                const float wr = w[nt][e], wi = w[nt][2 + e];
                *out(k) = make_float2(b.x + ur - wi, b.y + ui + wr);
                *out(P - k) = make_float2(b.x + ur + wi, b.y + ui - wr);
            }
        }
    }
}

} // namespace ptc
} // namespace gbfft
