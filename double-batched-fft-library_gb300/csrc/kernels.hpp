// Host-visible handles of the AOT-compiled kernels.
#pragma once

#include <cstddef>

namespace gbfft {

// runtime-size kernels, one per transform kind
const void *kernel_f32(int kind);
const void *kernel_f64(int kind);

// compile-time-size kernels (generated by gen_specializations.py)
struct ct_entry {
    int prec;    // bytes per real
    int kind;    // gbfft::kind
    int nc;      // complex FFT length
    int T;       // threads per transform
    int V;       // transforms per thread along M
    int L;       // number of stages
    int rad[12]; // radices
    const void *fn;
    int minb;    // resident CTAs of 256 threads the register allocation is sized for
};
const ct_entry *ct_lookup(int prec, int kind, int nc, int T, int V, const int *rad, int L,
                          int minb);
// compile-time-size tiles of the persistent ragged kernel: index into ragged_ct_table or -1
extern const ct_entry ragged_ct_table[];
int ragged_ct_lookup(int prec, int kind, int nc, int T, int V, const int *rad, int L);
// compile-time-size tiles (V = 1) of the other float lengths with prime factors <= 61:
// index into cover_ct_table or -1, and the plan kernel of an index
extern const ct_entry cover_ct_table[];
int cover_ct_lookup(int prec, int kind, int nc, int T, const int *rad, int L);
const void *cover_ct_kernel(int i);

// Bluestein's algorithm for float lengths with a prime factor above 61 (bluestein.cu)
// pair: odd real N, two real transforms (k, k + 1) per complex transform; mb: transforms
// along M per tile (1, 2 or 4)
const void *bluestein_kernel(int kind, bool pair, int mb);
int bluestein_pad(int L, int mb); // spare shared elements after every 16
int bluestein_threads(int L); // threads per transform of the length-L tile
int bluestein_stages(int L);  // Stockham stages of the length-L transform
int bluestein_radix(int L, int s);

// tensor-core DFT stages (tc.cu)
const void *tc_kernel(int pieces, int nc);
std::size_t tc_shared_bytes();
int tc_tile_transforms(int nc);

// persistent kernel of ragged batches (ragged.cu)
const void *ragged_kernel_ptr(int prec, bool persistent);

// strided gather / scatter of nd plans with non-default layouts (strided_copy.cu)
constexpr int copy_max_rank = 5;
struct copy_params {
    const void *src;
    void *dst;
    long long total;                  // elements
    long long shape[copy_max_rank];   // packed side, mode 0 fastest
    long long stride[copy_max_rank];  // strided side (elements)
    int rank;
    int gather;                       // 1: strided src -> packed dst; 0: packed src -> strided dst
};
const void *strided_copy_kernel_ptr(int elem_bytes);
// class form of ragged batches: kernel(items, units) over the units of one class
const void *ragged_class_kernel(int vid);
// plan kernel (fft_params by value, one CTA per tile) of a ragged tile function
const void *ragged_plan_kernel(int vid);
const void *ragged_class_runtime_kernel(int prec, int kind);

} // namespace gbfft
