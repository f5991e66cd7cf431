// Kernel parameter block shared by the host library and the device engine.
// Plain C++ (no CUDA types) so that the host compiler, nvcc and NVRTC agree on the layout.
#pragma once

namespace gbfft {

constexpr int max_stages = 12;

// generic odd radices up to gen_table_max_p use a shared k-major coefficient table with
// rows padded to a multiple of gen_group (output pairs per sweep)
constexpr int gen_table_max_p = 61;
constexpr int gen_group = 8;

enum kind : int {
    kind_c2c = 0,
    kind_r2c_half = 1, // even N: N/2-point complex FFT + post-process
    kind_r2c_full = 2, // odd N: N-point complex FFT of real data
    kind_c2r_half = 3, // even N: pre-process + N/2-point complex FFT
    kind_c2r_full = 4, // odd N: N-point complex FFT of the Hermitian extension
};

// flags
constexpr int flag_conj_in = 1;   // c2c: conjugate on load (backward)
constexpr int flag_conj_out = 2;  // c2c: conjugate on store (backward)
constexpr int flag_adj_r2c = 4;   // adjoint of r2c, run as a c2r kernel (Hermitian weights)
constexpr int flag_adj_c2r = 8;   // adjoint of c2r, run as a r2c kernel (Hermitian weights)
constexpr int flag_scale_out = 16; // multiply the output by params.scale
constexpr int flag_vec_in = 32;   // real input pairs x[2n], x[2n+1] are adjacent and aligned
constexpr int flag_vec_out = 64;  // real output pairs are adjacent and aligned
constexpr int flag_pair = 128;    // odd real N: the transforms k and k + 1 share one complex FFT

struct fft_params {
    const void *in;
    void *out;
    const void *tw;        // w_Nt^{-i}, i = 0..Nt-1, complex of the plan precision
    long long M;           // left batch
    long long K;           // right batch
    long long is2, os2;    // input / output strides of the K mode (elements)
    int is1, os1;          // input / output strides of the N mode (elements)
    int N;                 // logical FFT length
    int Nc;                // complex FFT length (N or N/2)
    int Nt;                // twiddle table length
    int L;                 // number of stages
    int radix[max_stages]; // radix per stage; 1 = copy stage
    int T;                 // threads per transform
    int Mb, Kb;            // tile
    int m_tiles;           // ceil(M / Mb)
    int flags;
    int nbuf;              // shared buffers (1 or 2)
    int buf_elems;         // padded elements per buffer
    int pad_shift, pad_add; // shared index i -> i + (i >> pad_shift) * pad_add
    // compile-time kernels with 16-byte lane vectors: 16-byte chunk c of plane q lives at
    // q * plane_chunks + (c ^ (((c >> sw_a) & sw_mask) << sw_b))
    int sw_a, sw_b, sw_mask, plane_chunks;
    double scale;          // used with flag_scale_out
    // Bluestein kernels (bluestein.cu): table {chirp (Nc), FFT_L(conj chirp) / L (bL),
    // stage twiddles} and the convolution length bL (0 for the other kernels)
    const void *bs;
    int bL;
};

} // namespace gbfft

namespace gbfft {

// One transform of a ragged batch: the launch parameters of its pass and the kernel kind.
struct ragged_item_dev {
    fft_params p;
    int kind;
    int vid; // compile-time-size tile function (ragged_ct_call), or -1: runtime-size engine
};

} // namespace gbfft
