// Allocation-free 2d c2r transform.
//
// Some callers cannot allocate device memory at the point where they need a transform: a
// process whose memory manager reserves the device memory at start-up and forbids
// cudaMalloc afterwards (cudaMalloc would then fail, or silently take memory the manager
// has promised elsewhere), or a host that must not grow its device footprint after
// start-up.  The regular nd c2r
// plan allocates a temporary buffer (the reference's nd_fft does the same,
// src/common/algorithm/nd_fft.hpp:114-125) and twiddle tables at plan creation.  The entry
// point below instead keeps its temporary and its twiddles in file-scope device arrays
// that are part of the loaded library: every GPU that loads the library holds them until
// the process exits, and no call allocates anything.
#include "bbfft_gb300.h"
#include "kernels.hpp"
#include "params.h"

#include <cuda_runtime.h>

#include <mutex>

namespace gbfft {

const char *plan_pass_fixed(int prec, int type, int dir, long long M, long long N, long long K,
                            long long is1, long long is2, long long os1, long long os2,
                            int device, fft_params &p, unsigned &grid, unsigned &block,
                            std::size_t &smem, const void *&func);
void set_fixed_error(const char *msg);
void clear_fixed_error();

// Largest temporary: M * (N1/2 + 1) * N2 * K complex floats = 2^21 (16 MiB).
constexpr unsigned long long kNoAllocScratchComplex = 1ull << 21;
constexpr int kNoAllocMaxN = 512;

static __device__ __align__(256) float2 g_noalloc_scratch[kNoAllocScratchComplex];
static __device__ __align__(256) float2 g_noalloc_twiddles[2][kNoAllocMaxN];

constexpr int kMaxDevices = 64;

// Device addresses of the arrays, one set per device, filled on the first call on that
// device with the device current (host code may not take the address of a __device__
// array directly: on the host its name denotes a host-side stand-in).
struct noalloc_device_state {
    bool ready = false;
    float2 *scratch = nullptr;
    float2 *twiddles = nullptr;
};
static noalloc_device_state g_state[kMaxDevices];
static std::mutex g_state_mu;

static const char *setup_device(int device, noalloc_device_state *&out) {
    if (device < 0 || device >= kMaxDevices) {
        return "device ordinal out of range for the allocation-free entry point";
    }
    std::lock_guard<std::mutex> lock(g_state_mu);
    noalloc_device_state &st = g_state[device];
    if (!st.ready) {
        void *scratch = nullptr;
        void *tw = nullptr;
        if (cudaGetSymbolAddress(&scratch, g_noalloc_scratch) != cudaSuccess ||
            cudaGetSymbolAddress(&tw, g_noalloc_twiddles) != cudaSuccess) {
            (void)cudaGetLastError();
            return "cudaGetSymbolAddress failed for the static scratch arrays";
        }
        st.scratch = static_cast<float2 *>(scratch);
        st.twiddles = static_cast<float2 *>(tw);
        st.ready = true;
    }
    out = &st;
    return "";
}

// w_Nt^{-i} = exp(-2 pi i i / Nt), evaluated in double precision and rounded once to float.
__global__ void noalloc_twiddle_kernel(float2 *tw, int Nt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < Nt) {
        double s, c;
        sincospi(2.0 * static_cast<double>(i) / static_cast<double>(Nt), &s, &c);
        tw[i] = make_float2(static_cast<float>(c), static_cast<float>(-s));
    }
}

} // namespace gbfft

extern "C" int bbfft_c2r_2d_noalloc_f32(const void *in, void *out, size_t M, size_t N1, size_t N2,
                                        size_t K, cudaStream_t stream) {
    using namespace gbfft;
    clear_fixed_error();
    // an error left on this thread by earlier, unrelated work must not be reported as a
    // failure of this call
    (void)cudaGetLastError();
    if (!in || !out) {
        set_fixed_error("null tensor pointer");
        return BBFFT_INVALID_ARGUMENT;
    }
    if (in == out) {
        set_fixed_error("the allocation-free c2r is out-of-place only");
        return BBFFT_BAD_CONFIGURATION;
    }
    if (M == 0 || N1 == 0 || N2 == 0 || K == 0) {
        set_fixed_error("tensor shape entries must be positive");
        return BBFFT_BAD_CONFIGURATION;
    }
    if (N1 > static_cast<size_t>(kNoAllocMaxN) || N2 > static_cast<size_t>(kNoAllocMaxN)) {
        set_fixed_error("allocation-free c2r: N1 and N2 must not exceed 512");
        return BBFFT_BAD_CONFIGURATION;
    }
    const unsigned long long h = N1 / 2 + 1;
    const unsigned long long need = static_cast<unsigned long long>(M) * h * N2 * K;
    if (need > kNoAllocScratchComplex || need / K / N2 / h != M) {
        set_fixed_error("allocation-free c2r: M * (N1/2+1) * N2 * K exceeds the static scratch of "
                        "2^21 complex floats (16 MiB); use a plan instead");
        return BBFFT_BAD_CONFIGURATION;
    }
    int device = 0;
    if (cudaGetDevice(&device) != cudaSuccess) {
        (void)cudaGetLastError();
        set_fixed_error("cudaGetDevice failed");
        return BBFFT_CUDA_ERROR;
    }
    noalloc_device_state *st = nullptr;
    const char *err = setup_device(device, st);
    if (*err) {
        set_fixed_error(err);
        return BBFFT_CUDA_ERROR;
    }
    // pass 0: c2c backward along N2 on M' = M (N1/2+1) interleaved transforms, in -> scratch;
    // pass 1: c2r along N1 on M transforms, K' = N2 K, scratch -> out
    // (the chain of the reference's nd_fft for c2r, nd_fft.hpp:63-108)
    const long long Mp = static_cast<long long>(M * h);
    fft_params p[2];
    unsigned grid[2], block[2];
    size_t smem[2];
    const void *func[2];
    err = plan_pass_fixed(4, BBFFT_C2C, BBFFT_BACKWARD, Mp, static_cast<long long>(N2),
                          static_cast<long long>(K), Mp, Mp * static_cast<long long>(N2), Mp,
                          Mp * static_cast<long long>(N2), device, p[0], grid[0], block[0], smem[0],
                          func[0]);
    if (!*err) {
        err = plan_pass_fixed(4, BBFFT_C2R, BBFFT_BACKWARD, static_cast<long long>(M),
                              static_cast<long long>(N1), static_cast<long long>(N2 * K),
                              static_cast<long long>(M), static_cast<long long>(M * h),
                              static_cast<long long>(M), static_cast<long long>(M * N1), device,
                              p[1], grid[1], block[1], smem[1], func[1]);
    }
    if (*err) {
        set_fixed_error(err);
        return BBFFT_BAD_CONFIGURATION;
    }
    float2 *tw0 = st->twiddles;
    float2 *tw1 = st->twiddles + kNoAllocMaxN;
    for (int i = 0; i < 2; ++i) {
        noalloc_twiddle_kernel<<<(p[i].Nt + 127) / 128, 128, 0, stream>>>(i ? tw1 : tw0, p[i].Nt);
        if (cudaGetLastError() != cudaSuccess) {
            set_fixed_error("twiddle kernel launch failed in the allocation-free c2r");
            return BBFFT_CUDA_ERROR;
        }
    }
    p[0].in = in;
    p[0].out = st->scratch;
    p[0].tw = tw0;
    p[1].in = st->scratch;
    p[1].out = out;
    p[1].tw = tw1;
    for (int i = 0; i < 2; ++i) {
        void *args[] = {&p[i]};
        cudaError_t e = cudaLaunchKernel(func[i], dim3(grid[i]), dim3(block[i]), args, smem[i], stream);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            set_fixed_error("kernel launch failed in the allocation-free c2r");
            return BBFFT_CUDA_ERROR;
        }
    }
    return BBFFT_SUCCESS;
}
