// Tensor-core DFT stages for c2c float transforms (complex length 64, 256, 512).
//
// A radix-16 Stockham stage is a product of 16-point input vectors with the DFT-16 matrix.
// Written over the reals, [yr | yi] = [xr | xi] * [[C, -S], [S, C]] with C = cos(2 pi nk/16)
// and S = sin(2 pi nk/16): a 32 x 32 real matrix.  Sixteen butterflies (rows) of a stage
// form one 16 x 32 operand A; the product runs on the tensor cores as 2 (K) x 4 (N) warp-level
// m16n8k16 BF16 MMAs with FP32 accumulation.
//
// Precision: every FP32 operand is split into PIECES bfloat16 numbers, x = x0 + x1 (+ x2),
// likewise the matrix, and all products x_i W_j with i + j < PIECES are accumulated:
//   PIECES = 1: plain BF16 (1 term, ~3 significant digits);
//   PIECES = 2: 3 terms (x0W0 + x0W1 + x1W0), ~2^-16 relative per stage;
//   PIECES = 3: 6 terms, ~2^-24: the FP32 result within FP32 rounding.
// Stage twiddles, the radix-2/4 stages and all data movement stay in FP32 on CUDA cores.
// The reference has no tensor-core path.
#include "engine.cuh"
#include "kernels.hpp"
#include "prime_tc.cuh"

#include <cuda_bf16.h>

namespace gbfft {

namespace tc {

constexpr int kThreads = 256;
constexpr int kElems = 2048; // complex elements per CTA tile

// padded shared index: three spare elements per 16 (per 8 for length 256), which keeps a
// warp's 8-byte accesses of every stage at about 2.5 wavefronts (2 is the minimum)
template <int NC> __host__ __device__ constexpr int pad(int i) {
    return NC == 256 ? i + (i >> 3) * 3 : i + (i >> 4) * 3;
}
constexpr int kBufElems = kElems + (kElems >> 3) * 3 + 8; // covers every length's padding

__device__ __forceinline__ unsigned pack(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return static_cast<unsigned>(__bfloat16_as_ushort(lo)) |
           (static_cast<unsigned>(__bfloat16_as_ushort(hi)) << 16);
}

// splits (x0, x1) into PIECES packed bfloat16 pairs whose sums approximate x0 and x1 (one
// paired conversion per piece; the low half holds x0)
template <int PIECES> __device__ __forceinline__ void split2(float x0, float x1, unsigned *out) {
    float r0 = x0, r1 = x1;
#pragma unroll
    for (int i = 0; i < PIECES; ++i) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(r0, r1);
        const unsigned u = *reinterpret_cast<const unsigned *>(&h);
        out[i] = u;
        if (i + 1 < PIECES) {
            r0 -= __uint_as_float(u << 16);
            r1 -= __uint_as_float(u & 0xffff0000u);
        }
    }
}

// splits x into PIECES bfloat16 numbers whose sum approximates x
template <int PIECES> __device__ __forceinline__ void split(float x, __nv_bfloat16 *out) {
    float r = x;
#pragma unroll
    for (int i = 0; i < PIECES; ++i) {
        out[i] = __float2bfloat16_rn(r);
        r = r - __bfloat162float(out[i]);
    }
}

__device__ __forceinline__ void mma_bf16(float *d, unsigned a0, unsigned a1, unsigned a2,
                                         unsigned a3, unsigned b0, unsigned b1) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, "
                 "{%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// B fragment of the real DFT-16 matrix for this lane: b[piece][s][j][e], where k-step s
// selects the real (0) or imaginary (1) input half, n-tile j the 8 output columns and e the
// two registers (input rows 2q + 8e + {0, 1}, output column 8j + g).
template <int PIECES> struct dft16_b {
    unsigned b[PIECES][2][4][2];
    __device__ __forceinline__ void init(int lane) {
        float c16[16], s16[16];
        sfor<0, 16>([&](auto M) {
            c16[M.value] = W<float, 16, M.value>::re;
            s16[M.value] = -W<float, 16, M.value>::im; // sin(2 pi m / 16)
        });
        const int g = lane >> 2, q = lane & 3;
#pragma unroll
        for (int s = 0; s < 2; ++s) {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    __nv_bfloat16 p0[PIECES], p1[PIECES];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int n = 2 * q + 8 * e + h; // input index within the half
                        const int col = 8 * j + g;
                        const int k = col & 15;
                        const bool out_im = col >= 16;
                        const int m = (n * k) & 15;
                        float v;
                        if (s == 0) {
                            v = out_im ? -s16[m] : c16[m]; // xr -> yr: C, xr -> yi: -S
                        } else {
                            v = out_im ? c16[m] : s16[m]; // xi -> yr: S, xi -> yi: C
                        }
                        split<PIECES>(v, h == 0 ? p0 : p1);
                    }
#pragma unroll
                    for (int pc = 0; pc < PIECES; ++pc) {
                        b[pc][s][j][e] = pack(p0[pc], p1[pc]);
                    }
                }
            }
        }
    }
};

// One radix-16 stage on the tensor cores: src -> dst (shared), all transforms of the tile.
template <int PIECES, int NC>
__device__ __forceinline__ void stage16(const float2 *src, float2 *dst, int Ns, const float2 *tw,
                                        const dft16_b<PIECES> &B, int tiles) {
    constexpr int nb = NC / 16;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, q = lane & 3;
    const int rows = tiles * nb;
    const int twstride = NC / (Ns * 16);
    for (int base = warp * 16; base < rows; base += (kThreads / 32) * 16) {
        // rows (butterflies) handled by this lane: base + g and base + g + 8
        float xr[2][4], xi[2][4];
        int tt[2], bb[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int row = base + g + 8 * h;
            tt[h] = row / nb;
            bb[h] = row % nb;
            const int kk = bb[h] % Ns;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int r = 2 * q + (u & 1) + 8 * (u >> 1); // 2q, 2q+1, 2q+8, 2q+9
                float2 v = src[pad<NC>(tt[h] * NC + bb[h] + r * nb)];
                if (Ns > 1 && r > 0) {
                    v = cmul(v, __ldg(tw + r * kk * twstride));
                }
                xr[h][u] = v.x;
                xi[h][u] = v.y;
            }
        }
        // A fragments per piece: k-step 0 = real parts, k-step 1 = imaginary parts
        unsigned a[PIECES][2][4];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const float(*x)[4] = s == 0 ? xr : xi;
            unsigned t[4][PIECES];
            split2<PIECES>(x[0][0], x[0][1], t[0]); // row g, cols 2q, 2q+1
            split2<PIECES>(x[1][0], x[1][1], t[1]); // row g+8
            split2<PIECES>(x[0][2], x[0][3], t[2]); // row g, cols 2q+8, 2q+9
            split2<PIECES>(x[1][2], x[1][3], t[3]); // row g+8
#pragma unroll
            for (int pc = 0; pc < PIECES; ++pc) {
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    a[pc][s][r] = t[r][pc];
                }
            }
        }
        float d[4][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            d[j][0] = d[j][1] = d[j][2] = d[j][3] = 0.f;
            // small terms first: pieces pa + pb < PIECES, in decreasing pa + pb
#pragma unroll
            for (int lvl = PIECES - 1; lvl >= 0; --lvl) {
#pragma unroll
                for (int pa = 0; pa <= lvl; ++pa) {
                    const int pb = lvl - pa;
#pragma unroll
                    for (int s = 0; s < 2; ++s) {
                        mma_bf16(d[j], a[pa][s][0], a[pa][s][1], a[pa][s][2], a[pa][s][3],
                                 B.b[pb][s][j][0], B.b[pb][s][j][1]);
                    }
                }
            }
        }
        // outputs k in {2q, 2q+1} (n-tiles 0 and 2) and {2q+8, 2q+9} (n-tiles 1 and 3)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int o = bb[h] + (bb[h] / Ns) * Ns * 15;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int k = 2 * q + (u & 1) + 8 * (u >> 1);
                const int jr = (u >> 1);    // n-tile of the real part
                const int ji = 2 + (u >> 1); // n-tile of the imaginary part
                const int e = (u & 1) + 2 * h;
                dst[pad<NC>(tt[h] * NC + o + k * Ns)] = mk<float>(d[jr][e], d[ji][e]);
            }
        }
    }
}

// Radix-P stage on CUDA cores from shared memory to global memory (last stage).
template <int P, int NC>
__device__ __forceinline__ void stage_last(const float2 *src, float2 *out, int Ns,
                                           const float2 *tw, int tiles, long long t0, long long K,
                                           bool conj_out) {
    constexpr int nb = NC / P;
    const int twstride = NC / (Ns * P);
    for (int idx = threadIdx.x; idx < tiles * nb; idx += kThreads) {
        const int t = idx / nb, b = idx % nb;
        float2 v[P];
        const int kk = b % Ns;
        sfor<0, P>([&](auto I) {
            v[I.value] = src[pad<NC>(t * NC + b + I.value * nb)];
            if (I.value > 0) {
                v[I.value] = cmul(v[I.value], __ldg(tw + I.value * kk * twstride));
            }
        });
        dft<P, float>::run(v);
        if (t0 + t < K) {
            float2 *y = out + (t0 + t) * NC;
            sfor<0, P>([&](auto I) {
                float2 r = v[I.value];
                if (conj_out) {
                    r.y = -r.y;
                }
                y[b + I.value * Ns] = r; // last stage: o = b
            });
        }
    }
}

// One radix-P stage (P = 16 or 32) on the tensor cores with split TF32 operands
// (prime_tc.cuh: the pair sums and differences of each butterfly against the cosine and
// sine matrices, two TF32 pieces per operand, three products): src -> dst, all transforms
// of the tile, eight butterflies per warp at a time.
template <int P, int NC>
__device__ __forceinline__ void stage_tf32(const float2 *src, float2 *dst, int Ns, const float2 *tw,
                                           int tiles) {
    constexpr int nb = NC / P;
    const int lane = threadIdx.x & 31;
    const int ngrp = tiles * nb / 8; // tiles * nb = kElems / P, a multiple of 8
    const int twstride = NC / (Ns * P);
    for (int grp = threadIdx.x >> 5; grp < ngrp; grp += kThreads / 32) {
        const int q = grp * 8 + (lane >> 2);
        const int t = q / nb, b = q % nb;
        const int kk = b % Ns;
        const int o = b + (b / Ns) * Ns * (P - 1);
        auto in = [&](int r) { return src + pad<NC>(t * NC + b + r * nb); };
        auto out = [&](int k) { return dst + pad<NC>(t * NC + o + k * Ns); };
        ptc::butterflies8<P>(lane, true, tw, kk * twstride, in, out);
    }
}

// contiguous tile in shared memory -> global (16-byte stores), conjugated for backward
template <int NC>
__device__ __forceinline__ void store_tile(const float2 *buf, float2 *yt, long long nt, bool conj_out) {
    for (int i = threadIdx.x; i < kElems / 2; i += kThreads) {
        if (2 * i < nt * NC) {
            float2 a = buf[pad<NC>(2 * i)], b = buf[pad<NC>(2 * i + 1)];
            if (conj_out) {
                a.y = -a.y;
                b.y = -b.y;
            }
            reinterpret_cast<float4 *>(yt)[i] = make_float4(a.x, a.y, b.x, b.y);
        }
    }
}

// contiguous tile global -> shared (16-byte loads), conjugated for backward
template <int NC>
__device__ __forceinline__ void load_tile(const float2 *x, float2 *buf, long long nt, bool conj_in) {
    for (int i = threadIdx.x; i < kElems / 2; i += kThreads) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (2 * i < nt * NC) {
            v = reinterpret_cast<const float4 *>(x)[i];
        }
        if (conj_in) {
            v.y = -v.y;
            v.w = -v.w;
        }
        buf[pad<NC>(2 * i)] = mk<float>(v.x, v.y);
        buf[pad<NC>(2 * i + 1)] = mk<float>(v.z, v.w);
    }
}

// Split-TF32 form, c2c float, M = 1, packed: 64 = 32 x 2, 256 = 16 x 16, 512 = 32 x 16, the
// radix-16 / 32 stages on the tensor cores, the radix-2 stage on the CUDA cores.
template <int NC> __global__ void __launch_bounds__(kThreads, 3) fft_tc32_kernel(const __grid_constant__ fft_params p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int tiles = kElems / NC;
    float2 *buf0 = reinterpret_cast<float2 *>(smem_raw);
    float2 *buf1 = buf0 + kBufElems;
    const float2 *tw = static_cast<const float2 *>(p.tw);
    const bool conj_in = p.flags & flag_conj_in, conj_out = p.flags & flag_conj_out;
    const long long t0 = static_cast<long long>(blockIdx.x) * tiles;
    const long long nt = (p.K - t0) < tiles ? (p.K - t0) : tiles;
    const float2 *x = static_cast<const float2 *>(p.in) + t0 * NC;
    float2 *y = static_cast<float2 *>(p.out);
    load_tile<NC>(x, buf0, nt, conj_in);
    __syncthreads();
    if constexpr (NC == 64) {
        stage_tf32<32, NC>(buf0, buf1, 1, tw, tiles);
        __syncthreads();
        stage_last<2, NC>(buf1, y, 32, tw, tiles, t0, p.K, conj_out);
    } else {
        constexpr int P0 = NC == 256 ? 16 : 32;
        stage_tf32<P0, NC>(buf0, buf1, 1, tw, tiles);
        __syncthreads();
        stage_tf32<16, NC>(buf1, buf0, P0, tw, tiles);
        __syncthreads();
        store_tile<NC>(buf0, y + t0 * NC, nt, conj_out);
    }
}

// c2c float, M = 1, packed: tiles of kElems / NC transforms per CTA.
template <int PIECES, int NC> __global__ void __launch_bounds__(kThreads, 3) fft_tc_kernel(const __grid_constant__ fft_params p) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int tiles = kElems / NC;
    float2 *buf0 = reinterpret_cast<float2 *>(smem_raw);
    float2 *buf1 = buf0 + kBufElems;
    const float2 *tw = static_cast<const float2 *>(p.tw);
    const bool conj_in = p.flags & flag_conj_in, conj_out = p.flags & flag_conj_out;
    const long long t0 = static_cast<long long>(blockIdx.x) * tiles;
    const long long nt = (p.K - t0) < tiles ? (p.K - t0) : tiles;
    const float2 *x = static_cast<const float2 *>(p.in) + t0 * NC;
    float2 *y = static_cast<float2 *>(p.out);
    dft16_b<PIECES> B;
    B.init(threadIdx.x & 31);
    // load: the tile is contiguous; 16-byte loads
    for (int i = threadIdx.x; i < kElems / 2; i += kThreads) {
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (2 * i < nt * NC) {
            v = reinterpret_cast<const float4 *>(x)[i];
        }
        if (conj_in) {
            v.y = -v.y;
            v.w = -v.w;
        }
        buf0[pad<NC>(2 * i)] = mk<float>(v.x, v.y);
        buf0[pad<NC>(2 * i + 1)] = mk<float>(v.z, v.w);
    }
    __syncthreads();
    stage16<PIECES, NC>(buf0, buf1, 1, tw, B, tiles);
    __syncthreads();
    if constexpr (NC == 64) {
        stage_last<4, NC>(buf1, y, 16, tw, tiles, t0, p.K, conj_out);
    } else {
        stage16<PIECES, NC>(buf1, buf0, 16, tw, B, tiles);
        __syncthreads();
        if constexpr (NC == 512) {
            stage_last<2, NC>(buf0, y, 256, tw, tiles, t0, p.K, conj_out);
        } else {
            float2 *yt = y + t0 * NC;
            for (int i = threadIdx.x; i < kElems / 2; i += kThreads) {
                if (2 * i < nt * NC) {
                    float2 a = buf0[pad<NC>(2 * i)], b = buf0[pad<NC>(2 * i + 1)];
                    if (conj_out) {
                        a.y = -a.y;
                        b.y = -b.y;
                    }
                    reinterpret_cast<float4 *>(yt)[i] = make_float4(a.x, a.y, b.x, b.y);
                }
            }
        }
    }
}

} // namespace tc

std::size_t tc_shared_bytes() { return 2 * static_cast<std::size_t>(tc::kBufElems) * 8; }
int tc_tile_transforms(int nc) { return tc::kElems / nc; }

const void *tc_kernel(int pieces, int nc) {
#define GBFFT_TC(PC, NCV)                                                                          \
    if (pieces == PC && nc == NCV) {                                                               \
        return reinterpret_cast<const void *>(&tc::fft_tc_kernel<PC, NCV>);                        \
    }
    GBFFT_TC(1, 64)
    GBFFT_TC(1, 256)
    GBFFT_TC(1, 512)
    GBFFT_TC(2, 64)
    GBFFT_TC(2, 256)
    GBFFT_TC(2, 512)
    GBFFT_TC(3, 64)
    GBFFT_TC(3, 256)
    GBFFT_TC(3, 512)
#undef GBFFT_TC
    // pieces == 0: the split-TF32 form
    if (pieces == 0) {
        switch (nc) {
        case 64:
            return reinterpret_cast<const void *>(&tc::fft_tc32_kernel<64>);
        case 256:
            return reinterpret_cast<const void *>(&tc::fft_tc32_kernel<256>);
        case 512:
            return reinterpret_cast<const void *>(&tc::fft_tc32_kernel<512>);
        }
    }
    return nullptr;
}

} // namespace gbfft
