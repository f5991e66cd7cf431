// Throughput probes for roofline denominators that a copy kernel and a cuBLAS GEMM do not
// give: the FP64 FMA pipe (the bound of the double-precision transforms) and the
// warp-level tensor-core MMA rates (mma.sync TF32 m16n8k8 and BF16 m16n8k16) that the
// tensor-core DFT stages issue.  Benchmark plumbing only (libbbfft_probes.so); the FFT
// library does not link it.
//
// Every kernel runs a fixed number of iterations of independent FMA / MMA chains in
// registers and writes one value per thread, so the work cannot be removed; there are no
// waits, no shared memory and no data-dependent control flow.
#include <cuda_runtime.h>

namespace {

constexpr int kChains = 8;

__global__ void dfma_kernel(double *out, int iters, double b, double c) {
    double a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) {
        a[i] = 1.0 + 1e-9 * threadIdx.x + 1e-3 * i;
    }
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) {
            a[i] = fma(a[i], b, c);
        }
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < kChains; ++i) {
        s += a[i];
    }
    out[static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x] = s;
}

__global__ void ffma_kernel(float *out, int iters, float b, float c) {
    float a[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) {
        a[i] = 1.0f + 1e-6f * threadIdx.x + 1e-3f * i;
    }
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < kChains; ++i) {
            a[i] = fmaf(a[i], b, c);
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < kChains; ++i) {
        s += a[i];
    }
    out[static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x] = s;
}

constexpr int kAcc = 4; // independent accumulator tiles per warp

__global__ void mma_tf32_kernel(float *out, int iters) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned a0 = __float_as_uint(1.0f + lane * 1e-3f), a1 = __float_as_uint(0.5f);
    const unsigned a2 = __float_as_uint(0.25f), a3 = __float_as_uint(-0.125f);
    const unsigned b0 = __float_as_uint(1e-3f), b1 = __float_as_uint(-1e-3f);
    float d[kAcc][4] = {};
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int t = 0; t < kAcc; ++t) {
            asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, "
                         "{%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                         : "+f"(d[t][0]), "+f"(d[t][1]), "+f"(d[t][2]), "+f"(d[t][3])
                         : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int t = 0; t < kAcc; ++t) {
        s += d[t][0] + d[t][1] + d[t][2] + d[t][3];
    }
    out[static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x] = s;
}

__global__ void mma_bf16_kernel(float *out, int iters) {
    const unsigned lane = threadIdx.x & 31u;
    const unsigned a0 = 0x3f803f80u + lane, a1 = 0x3f003f00u, a2 = 0x3e803e80u, a3 = 0xbe00be00u;
    const unsigned b0 = 0x3a833a83u, b1 = 0xba83ba83u;
    float d[kAcc][4] = {};
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int t = 0; t < kAcc; ++t) {
            asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, "
                         "{%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
                         : "+f"(d[t][0]), "+f"(d[t][1]), "+f"(d[t][2]), "+f"(d[t][3])
                         : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
        }
    }
    float s = 0.0f;
#pragma unroll
    for (int t = 0; t < kAcc; ++t) {
        s += d[t][0] + d[t][1] + d[t][2] + d[t][3];
    }
    out[static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x] = s;
}

} // namespace

// Each entry point launches blocks x threads threads (out must hold that many values) and
// returns the cudaError_t of the launch.  Flops per launch:
//   dfma / ffma: 2 * kChains * iters per thread;
//   mma tf32:    2 * 16 * 8 * 8  * kAcc * iters per warp;
//   mma bf16:    2 * 16 * 8 * 16 * kAcc * iters per warp.
extern "C" {

__attribute__((visibility("default"))) int gbfft_probe_chains(void) { return kChains; }
__attribute__((visibility("default"))) int gbfft_probe_mma_acc(void) { return kAcc; }

__attribute__((visibility("default"))) int gbfft_probe_dfma(int blocks, int threads, int iters,
                                                            double *out, cudaStream_t stream) {
    dfma_kernel<<<blocks, threads, 0, stream>>>(out, iters, 0.999999999, 1e-12);
    return static_cast<int>(cudaGetLastError());
}

__attribute__((visibility("default"))) int gbfft_probe_ffma(int blocks, int threads, int iters,
                                                            float *out, cudaStream_t stream) {
    ffma_kernel<<<blocks, threads, 0, stream>>>(out, iters, 0.9999999f, 1e-9f);
    return static_cast<int>(cudaGetLastError());
}

__attribute__((visibility("default"))) int gbfft_probe_mma_tf32(int blocks, int threads, int iters,
                                                                float *out, cudaStream_t stream) {
    if (threads % 32 != 0) { // the MMAs are warp-wide
        return static_cast<int>(cudaErrorInvalidValue);
    }
    mma_tf32_kernel<<<blocks, threads, 0, stream>>>(out, iters);
    return static_cast<int>(cudaGetLastError());
}

__attribute__((visibility("default"))) int gbfft_probe_mma_bf16(int blocks, int threads, int iters,
                                                                float *out, cudaStream_t stream) {
    if (threads % 32 != 0) {
        return static_cast<int>(cudaErrorInvalidValue);
    }
    mma_bf16_kernel<<<blocks, threads, 0, stream>>>(out, iters);
    return static_cast<int>(cudaGetLastError());
}

} // extern "C"
