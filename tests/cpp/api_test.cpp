// Exercises the C++ API (include/bbfft/*.hpp) the way the reference's callers use it.
// "host": configuration, strides, descriptors, tensor_indexer, bad_configuration (no GPU).
// "gpu":  make_plan / execute with events, in-place round trip, unmanaged-event plan.
#include "bbfft/configuration.hpp"
#include "bbfft/cuda/make_plan.hpp"
#include "bbfft/parser.hpp"
#include "bbfft/tensor_indexer.hpp"

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <random>
#include <vector>

using namespace bbfft;

#define EXPECT(c)                                                                                \
    do {                                                                                         \
        if (!(c)) {                                                                              \
            std::fprintf(stderr, "FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);                  \
            return 1;                                                                            \
        }                                                                                        \
    } while (0)

static int host_tests() {
    // configuration aggregate initialisation with default in-place strides
    configuration cfg = {1, {8, 64, 100}, precision::f32, direction::forward, transform_type::r2c};
    EXPECT((cfg.istride == std::array<std::size_t, 5>{1, 8, 8 * 66, 0, 0}));
    EXPECT((cfg.ostride == std::array<std::size_t, 5>{1, 8, 8 * 33, 0, 0}));
    cfg.set_strides_default(false);
    EXPECT(cfg.istride[2] == 8 * 64);
    EXPECT(cfg.to_string() == "srfo8.64*100");
    auto p = parse_fft_descriptor("dcbi4.5");
    EXPECT(p.dim == 1 && p.shape[0] == 4 && p.shape[1] == 5 && p.fp == precision::f64);
    EXPECT(p.dir == direction::backward && p.to_string() == "dcbi4.5");
    bool threw = false;
    try {
        parse_fft_descriptor("srb4x5*6x7");
    } catch (std::runtime_error const &) {
        threw = true;
    }
    EXPECT(threw);
    // tensor_indexer
    auto xi = tensor_indexer<std::size_t, 3u, layout::col_major>({4, 5, 6});
    EXPECT(xi(1, 2, 3) == 1 + 4 * 2 + 20 * 3);
    EXPECT(xi.size() == 120);
    EXPECT((xi.may_fuse<1u, 2u>()));
    auto xf = xi.fused<1u, 2u>();
    EXPECT(xf.shape(1) == 30 && xf(1, 7) == 1 + 4 * 7);
    EXPECT(!xi.may_reshape_mode(1, std::array<std::size_t, 2u>{2, 3}));
    auto yi = tensor_indexer<std::size_t, 3u, layout::col_major>({4, 6, 6});
    auto yr = yi.reshaped_mode(1, std::array<std::size_t, 2u>{2, 3});
    EXPECT(yr(1, 1, 2, 3) == yi(1, 1 + 2 * 2, 3));
    auto ri = tensor_indexer<int, 2u, layout::row_major>({3, 4});
    EXPECT(ri(1, 2) == 6 && ri.stride(1) == 1);
    auto padded = tensor_indexer<std::size_t, 3u, layout::col_major>({2, 5, 3}, {1, 3, 20});
    EXPECT(!(padded.may_fuse<0u, 1u>()) && padded(1, 4, 2) == 1 + 12 + 40);
    // unsupported dimension -> bad_configuration (reference test/error.cpp:13-21)
    threw = false;
    try {
        configuration bad = {4, {1, 8, 8, 8, 1}, precision::f32};
        make_plan(bad, nullptr);
    } catch (bad_configuration const &) {
        threw = true;
    }
    EXPECT(threw);
    std::puts("host ok");
    return 0;
}

static int gpu_tests() {
    std::size_t M = 3, N = 63, K = 16;
    std::size_t n = M * N * K;
    std::vector<std::complex<float>> x(n), y(n);
    std::mt19937 gen(11);
    std::uniform_real_distribution<float> U(0.0f, 1.0f);
    for (auto &v : x) {
        v = {U(gen), U(gen)};
    }
    void *d = nullptr;
    EXPECT(cudaMalloc(&d, n * sizeof(std::complex<float>)) == cudaSuccess);
    EXPECT(cudaMemcpy(d, x.data(), n * sizeof(x[0]), cudaMemcpyHostToDevice) == cudaSuccess);
    cudaStream_t s;
    EXPECT(cudaStreamCreate(&s) == cudaSuccess);
    configuration cfg = {1, {M, N, K}, precision::f32, direction::forward};
    auto plan = make_plan(cfg, s);
    cfg.dir = direction::backward;
    auto iplan = make_plan(cfg, s);
    cudaEvent_t e1 = plan.execute(d);
    cudaEvent_t e2 = iplan.execute(d, e1);
    EXPECT(cudaEventSynchronize(e2) == cudaSuccess);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    EXPECT(cudaMemcpy(y.data(), d, n * sizeof(y[0]), cudaMemcpyDeviceToHost) == cudaSuccess);
    double tol = 100.0 * 1.1920929e-7 * std::sqrt(double(N));
    for (std::size_t i = 0; i < n; ++i) {
        EXPECT(std::abs(y[i] / float(N) - x[i]) < tol * (1.0 + std::abs(x[i])));
    }
    // unmanaged events: caller-owned signal and wait events
    auto uplan = make_plan_unmanaged(configuration{1, {M, N, K}, precision::f32}, s);
    cudaEvent_t sig, dep;
    EXPECT(cudaEventCreate(&sig) == cudaSuccess && cudaEventCreate(&dep) == cudaSuccess);
    EXPECT(cudaEventRecord(dep, s) == cudaSuccess);
    uplan.execute(d, sig, 1, &dep);
    EXPECT(cudaEventSynchronize(sig) == cudaSuccess);
    // copies share the plan (reference plan.hpp:24-48)
    auto copy = plan;
    EXPECT(bool(copy));
    cudaEvent_t e3 = copy.execute(d);
    EXPECT(cudaEventSynchronize(e3) == cudaSuccess);
    cudaEventDestroy(e3);
    cudaEventDestroy(sig);
    cudaEventDestroy(dep);
    cudaStreamDestroy(s);
    cudaFree(d);
    std::puts("gpu ok");
    return 0;
}

int main(int argc, char **argv) {
    if (argc > 1 && std::strcmp(argv[1], "gpu") == 0) {
        return gpu_tests();
    }
    return host_tests();
}
