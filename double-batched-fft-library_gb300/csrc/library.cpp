// Host side of the GB300 double-batched FFT library: plan creation (algorithm
// selection and blocking), nd chaining, execution, plan caches and the NVRTC path for
// user callbacks.  Everything is exported through the C ABI of bbfft_gb300.h.
//
// Correspondence with the reference (intel/double-batched-fft-library 0.5.1):
//   select_fft_algorithm           src/common/algorithm.hpp:20-30      -> make_plan_impl
//   select_1d_fft_algorithm        src/common/algorithm_1d.hpp:19-36   -> make_1d_pass
//   small_batch_fft / factor2_slm  src/common/algorithm/*.hpp          -> one engine, blocking below
//   nd_fft                         src/common/algorithm/nd_fft.hpp     -> make_nd
//   jit_cache / jit_cache_all      src/base/jit_cache*.cpp             -> bbfft_cache_s
//   aot_cache                      src/base/aot_cache.cpp              -> bbfft_cache_s (aot)
#include "config.hpp"
#include "kernels.hpp"
#include "params.h"

#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <set>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "engine_src.inc" // kEngineSource: the device engine as text, for NVRTC

namespace gbfft {

// ------------------------------------------------------------------------------------------
// errors

thread_local std::string tl_error;
// fixed-size message buffer for the allocation-free entry point (no string allocation)
thread_local char tl_fixed_error[256];
thread_local bool tl_fixed_active = false;
void set_fixed_error(const char *msg) {
    std::strncpy(tl_fixed_error, msg, sizeof(tl_fixed_error) - 1);
    tl_fixed_error[sizeof(tl_fixed_error) - 1] = '\0';
    tl_fixed_active = true;
}
void clear_fixed_error() { tl_fixed_active = false; }

#define GB_CUDA(call)                                                                            \
    do {                                                                                         \
        cudaError_t e_ = (call);                                                                 \
        if (e_ != cudaSuccess) {                                                                 \
            (void)cudaGetLastError(); /* do not leave a non-sticky error behind */              \
            throw status_error(BBFFT_CUDA_ERROR,                                                 \
                               std::string(#call) + " failed: " + cudaGetErrorString(e_));       \
        }                                                                                        \
    } while (0)

[[noreturn]] void bad_config(std::string const &what) {
    throw status_error(BBFFT_BAD_CONFIGURATION, what);
}

template <class F> int guarded(F &&f) {
    try {
        f();
        return BBFFT_SUCCESS;
    } catch (status_error const &e) {
        tl_fixed_active = false;
        tl_error = e.what();
        return e.status();
    } catch (std::bad_alloc const &) {
        tl_error = "out of host memory";
        return BBFFT_OUT_OF_MEMORY;
    } catch (std::exception const &e) {
        tl_error = e.what();
        return BBFFT_INTERNAL_ERROR;
    } catch (...) {
        tl_error = "unknown error";
        return BBFFT_INTERNAL_ERROR;
    }
}

// ------------------------------------------------------------------------------------------
// device memory

struct device_buffer {
    void *ptr = nullptr;
    std::size_t bytes = 0;
    device_buffer(std::size_t n) : bytes(n) {
        if (n) {
            cudaError_t e = cudaMalloc(&ptr, n);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                throw status_error(BBFFT_OUT_OF_MEMORY,
                                   "cudaMalloc(" + std::to_string(n) + ") failed: " +
                                       cudaGetErrorString(e));
            }
        }
    }
    ~device_buffer() {
        if (ptr) {
            cudaFree(ptr);
        }
    }
    device_buffer(device_buffer const &) = delete;
    device_buffer &operator=(device_buffer const &) = delete;
};

// Twiddle tables w_Nt^{-i} = exp(-2 pi i i / Nt), i = 0..Nt-1, evaluated in long double
// and rounded once to the plan precision.  Shared between plans of one device.
static void twiddle_value(int i, int Nt, long double &c, long double &s) {
    // exact values at multiples of pi/2
    int q = i % Nt;
    if ((4LL * q) % Nt == 0) {
        int quad = static_cast<int>((4LL * q) / Nt);
        static const int cs[4][2] = {{1, 0}, {0, 1}, {-1, 0}, {0, -1}};
        c = cs[quad][0];
        s = cs[quad][1];
        return;
    }
    long double const tau = 6.283185307179586476925286766559005768L;
    long double a = tau * static_cast<long double>(q) / static_cast<long double>(Nt);
    c = std::cos(a);
    s = std::sin(a);
}

std::shared_ptr<device_buffer> get_twiddles(int device, int prec, int Nt) {
    static std::mutex mu;
    static std::map<std::tuple<int, int, int>, std::weak_ptr<device_buffer>> tables;
    std::lock_guard<std::mutex> lock(mu);
    auto key = std::make_tuple(device, prec, Nt);
    auto it = tables.find(key);
    if (it != tables.end()) {
        if (auto sp = it->second.lock()) {
            return sp;
        }
    }
    auto buf = std::make_shared<device_buffer>(static_cast<std::size_t>(Nt) * 2 * prec);
    if (prec == 4) {
        std::vector<float> h(2 * Nt);
        for (int i = 0; i < Nt; ++i) {
            long double c, s;
            twiddle_value(i, Nt, c, s);
            h[2 * i] = static_cast<float>(c);
            h[2 * i + 1] = static_cast<float>(-s);
        }
        GB_CUDA(cudaMemcpy(buf->ptr, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    } else {
        std::vector<double> h(2 * Nt);
        for (int i = 0; i < Nt; ++i) {
            long double c, s;
            twiddle_value(i, Nt, c, s);
            h[2 * i] = static_cast<double>(c);
            h[2 * i + 1] = static_cast<double>(-s);
        }
        GB_CUDA(cudaMemcpy(buf->ptr, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    tables[key] = buf;
    return buf;
}

// ------------------------------------------------------------------------------------------
// modules (NVRTC output or registered AOT images)

struct module {
    cudaLibrary_t lib = nullptr;
    ~module() {
        if (lib) {
            cudaLibraryUnload(lib);
        }
    }
    cudaKernel_t kernel(std::string const &name) const {
        cudaKernel_t k = nullptr;
        cudaError_t e = cudaLibraryGetKernel(&k, lib, name.c_str());
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            return nullptr;
        }
        return k;
    }
};

} // namespace gbfft

struct bbfft_cache_s {
    bool aot = false;
    std::mutex mu;
    std::unordered_map<std::string, std::shared_ptr<gbfft::module>> jit; // key: name@device
    struct aot_module {
        std::shared_ptr<gbfft::module> mod;
        std::set<std::string> names;
        int device;
    };
    std::vector<aot_module> aot_modules;
    std::atomic<uint64_t> hits{0}, misses{0};

    std::shared_ptr<gbfft::module> get(std::string const &name, int device) {
        std::lock_guard<std::mutex> lock(mu);
        std::shared_ptr<gbfft::module> r;
        if (aot) {
            for (auto const &m : aot_modules) {
                if (m.device == device && m.names.count(name)) {
                    r = m.mod;
                    break;
                }
            }
        } else {
            auto it = jit.find(name + "@" + std::to_string(device));
            if (it != jit.end()) {
                r = it->second;
            }
        }
        (r ? hits : misses)++;
        return r;
    }
    void store(std::string const &name, int device, std::shared_ptr<gbfft::module> m) {
        if (aot) {
            return; // reference aot_cache::store is a no-op (src/base/aot_cache.cpp:24)
        }
        std::lock_guard<std::mutex> lock(mu);
        jit[name + "@" + std::to_string(device)] = std::move(m);
    }
};

namespace gbfft {

static std::string nvrtc_arch(int device) {
    // device < 0: ahead-of-time compilation without a GPU, for BBFFT_GB300_AOT_ARCH
    // (e.g. sm_103a), the counterpart of the reference tool's device option
    if (device < 0) {
        const char *a = std::getenv("BBFFT_GB300_AOT_ARCH");
        return std::string("--gpu-architecture=") + (a && *a ? a : "sm_103a");
    }
    cudaDeviceProp prop;
    GB_CUDA(cudaGetDeviceProperties(&prop, device));
    std::string arch = "sm_" + std::to_string(prop.major) + std::to_string(prop.minor);
    if (prop.major >= 9) {
        arch += "a";
    }
    return "--gpu-architecture=" + arch;
}

std::vector<char> nvrtc_compile(std::string const &source, std::string const &name, int device);

std::shared_ptr<module> nvrtc_build(std::string const &source, std::string const &name,
                                    int device) {
    std::vector<char> cubin = nvrtc_compile(source, name, device);
    auto m = std::make_shared<module>();
    GB_CUDA(cudaLibraryLoadData(&m->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
    return m;
}

std::vector<char> nvrtc_compile(std::string const &source, std::string const &name, int device) {
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, source.c_str(), (name + ".cu").c_str(), 0, nullptr, nullptr) !=
        NVRTC_SUCCESS) {
        throw status_error(BBFFT_COMPILE_ERROR, "nvrtcCreateProgram failed");
    }
    std::string arch = nvrtc_arch(device);
    // -default-device: user callbacks may be written without __device__, like the
    // reference's OpenCL-C functions
    const char *opts[] = {arch.c_str(), "-std=c++17", "-lineinfo", "-default-device",
                          "-DGBFFT_JIT=1"};
    nvrtcResult rc = nvrtcCompileProgram(prog, 5, opts);
    std::size_t log_size = 0;
    nvrtcGetProgramLogSize(prog, &log_size);
    std::string log(log_size, '\0');
    if (log_size) {
        nvrtcGetProgramLog(prog, &log[0]);
    }
    if (rc != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        throw status_error(BBFFT_COMPILE_ERROR, "NVRTC compilation of " + name + " failed:\n" + log);
    }
    std::size_t cubin_size = 0;
    nvrtcGetCUBINSize(prog, &cubin_size);
    std::vector<char> cubin(cubin_size);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    return cubin;
}

// ------------------------------------------------------------------------------------------
// algorithm selection and blocking

static bool unrolled(int P) { return P == 1 || (P >= 2 && P <= 13) || P == 16; }
// Generic (non-unrolled) odd radix with the coefficient table of run_stage_generic
// (engine.cuh): one thread per group of gen_group output pairs of a butterfly.
static bool table_generic(int P) { return !unrolled(P) && P % 2 == 1 && P <= gen_table_max_p; }
static bool ptc_supported_host(int P) {
    return P == 17 || P == 19 || P == 23 || P == 29 || P == 31 || P == 37 || P == 41 || P == 43 ||
           P == 47 || P == 53 || P == 59 || P == 61;
}
// Float prime radices 17..61 run on the tensor cores (prime_tc.cuh): no shared table,
// and every warp of the block must be full.  NVRTC kernels (user callbacks) keep the
// CUDA-core stage and its table.
static bool tc_prime(int prec, int P) { return prec == 4 && ptc_supported_host(P); }
// A complex length k * P (P the smallest prime factor >= 17, P <= 61, k <= 32 without a
// prime factor >= 17) runs its radix-P butterflies in registers on the compile-time tiles
// of the other lengths (cover tiles): the prime stage first, one butterfly per thread on
// k threads per transform, then the stages of k, no copy stages (same rule as
// reg_prime_of() in gen_specializations.py).  Returns P or 0.
static int reg_prime_length(int nc) {
    for (int P = 17; P <= 61; ++P) {
        if (nc % P != 0 || !ptc_supported_host(P)) {
            continue; // P: the smallest prime factor >= 17 of nc
        }
        int const k = nc / P;
        if (k > 32) {
            return 0;
        }
        for (int q = 17; q <= k; ++q) {
            if (ptc_supported_host(q) && k % q == 0) {
                return 0; // k has a prime factor >= 17 (k <= 32: 17..31)
            }
        }
        return P;
    }
    return 0;
}
// shared-memory elements the generic stage of radix P needs after the data buffers
// (`tc_ok`: the kernel has the tensor-core stages, i.e. it is not an NVRTC kernel)
static int gen_shared_elems(int prec, int P, bool tc_ok) {
    if (unrolled(P) || (tc_ok && tc_prime(prec, P))) {
        return 0;
    }
    if (P <= gen_table_max_p) {
        int H = (P - 1) / 2;
        return (H + gen_group - 1) / gen_group * gen_group * H;
    }
    return P;
}

// Radices for an Nc-point complex FFT: few stages, unrolled butterflies where possible.
// Writes at most 32 radices to `out` and returns their number (no allocation).
int choose_radices_core(int Nc, int *out) {
    if (Nc == 1) {
        out[0] = 1;
        return 1;
    }
    int c2 = 0, c3 = 0, nodd = 0, nbig = 0;
    int odd[32], big[32];
    for (int n = Nc, f = 2; n > 1;) {
        if (n % f == 0) {
            if (f == 2) {
                ++c2;
            } else if (f == 3) {
                ++c3;
            } else if (f <= 13) {
                odd[nodd++] = f;
            } else {
                big[nbig++] = f;
            }
            n /= f;
        } else {
            ++f;
        }
    }
    int r[32];
    int nr = 0;
    while (c3 >= 2) {
        r[nr++] = 9;
        c3 -= 2;
    }
    if (c3 == 1) {
        if (c2 >= 2 && c2 != 3 && c2 != 6) { // keep 8 / 8x8 for the power-of-two part
            r[nr++] = 12;
            c2 -= 2;
        } else if (c2 >= 1) {
            r[nr++] = 6;
            c2 -= 1;
        } else {
            r[nr++] = 3;
        }
    }
    for (int i = 0; i < nodd; ++i) {
        if (odd[i] == 5 && c2 >= 1 && c2 % 3 == 1) {
            r[nr++] = 10;
            c2 -= 1;
        } else {
            r[nr++] = odd[i];
        }
    }
    if (c2 > 0) {
        int chunks = (c2 + 3) / 4;
        for (int i = 0; i < chunks; ++i) {
            int bits = c2 / chunks + (i < c2 % chunks ? 1 : 0);
            r[nr++] = 1 << bits;
        }
    }
    std::sort(r, r + nr, [](int x, int y) { return x > y; });
    int n = 0;
    for (int i = 0; i < nr; ++i) {
        out[n++] = r[i];
    }
    for (int i = 0; i < nbig; ++i) {
        out[n++] = big[i]; // generic radices last: they need a shared-memory source
    }
    return n;
}

std::vector<int> choose_radices(int Nc) {
    int r[32];
    int n = choose_radices_core(Nc, r);
    return std::vector<int>(r, r + n);
}

struct pass {
    int prec = 4;
    int kind = kind_c2c;
    fft_params p = {};
    unsigned grid = 0;
    unsigned block = 0;
    std::size_t smem = 0;
    const void *func = nullptr;
    std::shared_ptr<module> mod;
    std::shared_ptr<device_buffer> tw;
    std::shared_ptr<device_buffer> extra; // Bluestein tables (chirp, FFT of the chirp, stage twiddles)
    bool inplace_ok = true;
    bool specialized = false; // compile-time-size kernel
    bool tc = false;          // tensor-core DFT stages
    int V = 1;                // transforms per thread along M
    std::shared_ptr<pass> scalar_alt; // V = 1 variant for pointers not aligned to 16 bytes
    int ragged_vid = -1;              // compile-time-size tile of the ragged kernel, or -1
    int min_blocks = 0;               // register budget of the compile-time kernel (0: none)
    std::string identifier;
    int in_sel = 0;  // 0: user input, 2: temporary, 3: packed input, 4: packed output
    int out_sel = 1; // 1: user output, 2: temporary, 3: packed input, 4: packed output
    bool copy = false; // strided gather / scatter of an nd plan with a non-default layout
    copy_params cp = {};
};

struct pass_request {
    int prec, type, dir;
    bool adjoint = false;
    long long M, N, K;
    long long is1, is2, os1, os2;
    const char *cb_source = nullptr;
    std::size_t cb_length = 0;
    const char *load_fn = nullptr;
    const char *store_fn = nullptr;
    // tuning overrides
    std::vector<int> radices;
    int T = 0, Mb = 0, Kb = 0;
    int V = 0; // 0: automatic, 1: no vectorisation along M, > 1: requested width
    int occ = 0; // resident CTAs of the compile-time kernel's register budget (0: automatic)
    bool force_v1 = false;
    bool runtime_only = false; // runtime-size kernel (ragged batches)
    int compute = BBFFT_COMPUTE_NATIVE;
    int max_block = 0;         // threads per CTA limit (0: kernel default)
};

// ------------------------------------------------------------------------------------------
// tuning table written by the autotuner (bbfft_gb300/autotune.py): one line per
//   <prec bytes> <kind> <N> <M or -1> <V> <Mb> <Kb>
// chosen by timing candidate blockings on the device.  Loaded once from
// $BBFFT_GB300_TUNING ("off" disables) or <package>/tuning/gb300.tune.

struct tune_entry {
    int V, Mb, Kb;
    int occ;              // resident CTAs the kernel's registers are sized for (2 or 3)
    int T;                // threads per transform (0: the heuristic's)
    std::vector<int> rad; // radices (empty: the heuristic's)
};

static std::string library_dir() {
    Dl_info info;
    if (dladdr(reinterpret_cast<void *>(&library_dir), &info) && info.dli_fname) {
        std::string f = info.dli_fname;
        auto pos = f.rfind('/');
        return pos == std::string::npos ? std::string(".") : f.substr(0, pos);
    }
    return ".";
}

static std::map<std::tuple<int, std::string, int, long long>, tune_entry> const &tuning_table() {
    static std::map<std::tuple<int, std::string, int, long long>, tune_entry> table;
    static std::once_flag once;
    std::call_once(once, [] {
        const char *env = std::getenv("BBFFT_GB300_TUNING");
        std::string path = env ? env : library_dir() + "/../../tuning/gb300.tune";
        if (path == "off") {
            return;
        }
        std::ifstream in(path);
        std::string line;
        while (std::getline(in, line)) {
            auto hash = line.find('#');
            if (hash != std::string::npos) {
                line = line.substr(0, hash);
            }
            std::istringstream ls(line);
            int prec, N, V, Mb, Kb, occ = 2, T = 0;
            long long M;
            std::string kind, rads;
            if (ls >> prec >> kind >> N >> M >> V >> Mb >> Kb) {
                // optional columns: CTAs per SM, threads per transform, radices (AxBxC)
                if (!(ls >> occ) || (occ != 2 && occ != 3 && occ != 12 && occ != 13)) {
                    occ = 2;
                }
                std::vector<int> rad;
                if (ls >> T >> rads) {
                    std::istringstream rs(rads);
                    std::string tok;
                    while (std::getline(rs, tok, 'x')) {
                        rad.push_back(std::atoi(tok.c_str()));
                    }
                } else {
                    T = 0;
                }
                table[std::make_tuple(prec, kind, N, M)] = tune_entry{V, Mb, Kb, occ, T, rad};
            }
        }
    });
    return table;
}

static int max_optin_smem(int device) {
    int v = 0;
    GB_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    return v;
}

// The dynamic shared-memory limit is a property of the kernel, shared by every plan that
// launches it: raise it once per kernel and device to the device maximum (lowering it for
// one plan would break the launches of another).
// Whether `smem` dynamic bytes need the opt-in limit: the default limit is 48 KiB minus the
// kernel's static shared memory (1 KiB of margin covers the library's kernels, whose static
// shared memory is a parameter block of a few hundred bytes).
static bool needs_smem_optin(std::size_t smem) { return smem > 47 * 1024; }

// Raise a kernel's dynamic shared-memory limit to the device maximum.  Kernels compiled
// into the library are set once per device; kernels of NVRTC modules (module_kernel) are
// set every time, since a handle of an unloaded module can be reused by a new one.
static void allow_max_smem(const void *func, int device, bool module_kernel = false) {
    static std::mutex mu;
    static std::set<std::pair<const void *, int>> done;
    std::lock_guard<std::mutex> lock(mu);
    if (!module_kernel && done.count({func, device})) {
        return;
    }
    cudaFuncAttributes attr;
    GB_CUDA(cudaFuncGetAttributes(&attr, func));
    GB_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 max_optin_smem(device) - static_cast<int>(attr.sharedSizeBytes)));
    if (!module_kernel) {
        done.insert({func, device});
    }
}

static std::string c_ident(std::string s) {
    for (auto &ch : s) {
        if (!std::isalnum(static_cast<unsigned char>(ch)) && ch != '_') {
            ch = '_';
        }
    }
    return s;
}

static uint64_t fnv1a(const char *data, std::size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (std::size_t i = 0; i < n; ++i) {
        h ^= static_cast<unsigned char>(data[i]);
        h *= 1099511628211ull;
    }
    return h;
}

static char const *kind_name(int kind);

static tune_entry const *find_tuning(int prec, int kind, int N, long long M) {
    auto const &t = tuning_table();
    auto it = t.find(std::make_tuple(prec, std::string(kind_name(kind)), N, M));
    if (it == t.end()) {
        it = t.find(std::make_tuple(prec, std::string(kind_name(kind)), N, -1LL));
    }
    return it == t.end() ? nullptr : &it->second;
}

static char const *kind_name(int kind) {
    switch (kind) {
    case kind_c2c:
        return "c2c";
    case kind_r2c_half:
        return "r2ch";
    case kind_r2c_full:
        return "r2cf";
    case kind_c2r_half:
        return "c2rh";
    case kind_c2r_full:
        return "c2rf";
    }
    return "?";
}

// Transforms per thread along M for the compile-time kernels: V * max radix complex
// values stay within 32 (float) / 16 (double) register pairs (gen_specializations.py
// instantiates the same widths).
static int vector_width(int prec, std::vector<int> const &rad) {
    int pmax = *std::max_element(rad.begin(), rad.end());
    int v = prec == 4 ? 4 : 2;
    int budget = prec == 4 ? 32 : 16;
    while (v > 1 && v * pmax > budget) {
        v /= 2;
    }
    return v;
}

// Threads per transform of a compile-time tile (the ragged tiles and the tiles of the
// other lengths; gen_specializations.py tile_threads() is the same rule): the count that
// leaves the fewest thread slots idle over the stages (a stage of nb butterflies runs
// ceil(nb / T) rounds on T threads), with at most 32 complex values per thread (V
// transforms each) in any stage and at least 4 threads where a stage has 4 butterflies
// (consecutive threads load consecutive elements: 32-byte sectors when M = 1); ties go to
// more threads.  The tensor-core prime stages use every warp of the block and do not count,
// but with one of them T is at most 4 x its butterflies per transform where possible, so
// that a block of 256 threads holds at least 64 of its butterflies (8 per warp).  `reg`:
// the prime stage runs in registers, one butterfly per thread: nc / P threads
// (reg_prime_length).
static int tile_threads(int nc, const int *rad, int L, int V, bool reg = false) {
    if (reg || (L == 2 && rad[1] == 1)) {
        // a register prime stage, or one butterfly stage and the copy stage: one butterfly
        // per thread in the first stage
        return nc / rad[0];
    }
    auto counts = [](int r) { return !(r > 16 && ptc_supported_host(r)); };
    int nbmax = 1;
    int tcap = 256;
    for (int s = 0; s < L; ++s) {
        if (counts(rad[s])) {
            nbmax = std::max(nbmax, nc / rad[s]);
        } else {
            tcap = std::min(tcap, 4 * (nc / rad[s]));
        }
    }
    int const his[2] = {std::min({nc, 256, tcap}), std::min(nc, 256)};
    for (int hi : his) {
        int best_t = -1;
        long best_cost = -1;
        for (int t = std::min(4, nbmax); t <= hi; ++t) {
            long cost = 0;
            bool ok = true;
            for (int s = 0; s < L && ok; ++s) {
                int const r = rad[s];
                if (!counts(r)) {
                    continue;
                }
                int const rounds = (nc / r + t - 1) / t;
                ok = rounds * r * V <= 32;
                cost += static_cast<long>(rounds) * t;
            }
            if (ok && (best_cost < 0 || cost <= best_cost)) {
                best_t = t;
                best_cost = cost;
            }
        }
        if (best_t > 0) {
            return best_t;
        }
    }
    return 1;
}

// Shared-memory bank model.  One warp instruction in which every lane moves `w` bytes
// (8 or 16) is served in wavefronts of 128 / w lanes; within a wavefront a bank serves one
// 4-byte word at a time, so the cost of a wavefront is the largest number of distinct words
// that its lanes touch in one bank.
static long instr_cost(long const *addr, int w) {
    int per = 128 / w;
    long total = 0;
    for (int g = 0; g < 32; g += per) {
        int worst = 1;
        long words[32][8];
        int nw[32] = {0};
        for (int l = g; l < g + per; ++l) {
            if (addr[l] < 0) {
                continue;
            }
            for (int k = 0; k < w / 4; ++k) {
                long word = addr[l] / 4 + k;
                int bank = static_cast<int>(word % 32);
                bool seen = false;
                for (int d = 0; d < nw[bank]; ++d) {
                    seen = seen || words[bank][d] == word;
                }
                if (!seen && nw[bank] < 8) {
                    words[bank][nw[bank]++] = word;
                }
                worst = std::max(worst, nw[bank]);
            }
        }
        total += worst;
    }
    return total;
}

struct layout_choice {
    bool planes = false;
    int sh = 30, ad = 0;          // linear: i -> i + (i >> sh) * ad
    int a = 30, b = 0, mask = 0;  // planes: c -> c ^ (((c >> a) & mask) << b)
};

// Modelled cost of all shared accesses of the first warp of a tile (Stockham reads and
// writes of every shared stage and the r2c post-process) under a layout.
static long layout_cost(fft_params const &p, int prec, bool post, int V, layout_choice const &L) {
    int const eb = 2 * prec;
    int const mvb = p.Mb / V;
    int const nq = L.planes ? std::max(1, eb * V / 16) : 1;
    int const w = L.planes ? 16 : eb * V; // bytes per lane per instruction (LIN: V * eb <= 16)
    long const plane = 1L << 20;          // planes far apart: no interaction modelled
    auto addr = [&](int k_l, int n, int mv, int q) -> long {
        if (!L.planes) {
            long i = (static_cast<long>(k_l) * p.Nc + n) * p.Mb + mv * V;
            i = i + (i >> L.sh) * L.ad;
            return i * eb;
        }
        long c = (static_cast<long>(k_l) * p.Nc + n) * mvb + mv;
        c = c ^ (((c >> L.a) & L.mask) << L.b);
        return (q * plane + c) * 16;
    };
    long cost = 0;
    int Ns = 1;
    long rd[32], wr[32];
    for (int s = 0; s < p.L; ++s) {
        int P = p.radix[s];
        bool src_g = s == 0;
        bool dst_g = s == p.L - 1 && !post;
        int nb = p.Nc / P;
        for (int r = 0; r < P; ++r) {
            for (int q = 0; q < nq; ++q) {
                for (int l = 0; l < 32; ++l) {
                    int mv = l % mvb, j = (l / mvb) % p.T, k_l = l / (mvb * p.T);
                    rd[l] = wr[l] = -1;
                    if (k_l >= p.Kb || j >= nb) {
                        continue;
                    }
                    int o = j + (j / Ns) * Ns * (P - 1);
                    rd[l] = addr(k_l, j + r * nb, mv, q);
                    wr[l] = addr(k_l, o + r * Ns, mv, q);
                }
                if (!src_g) {
                    cost += instr_cost(rd, w);
                }
                if (!dst_g) {
                    cost += instr_cost(wr, w);
                }
            }
        }
        Ns *= P;
    }
    if (post) {
        for (int q = 0; q < nq; ++q) {
            for (int l = 0; l < 32; ++l) {
                int mv = l % mvb, j = (l / mvb) % p.T, k_l = l / (mvb * p.T);
                rd[l] = wr[l] = -1;
                if (k_l >= p.Kb || 2 * j > p.Nc) {
                    continue;
                }
                rd[l] = addr(k_l, j, mv, q);
                wr[l] = addr(k_l, (p.Nc - j) % p.Nc, mv, q);
            }
            cost += instr_cost(rd, w) + instr_cost(wr, w);
        }
    }
    return cost;
}

// Pick the shared layout with the fewest modelled wavefronts; fills the layout fields of
// p and returns the bytes of one buffer.
std::size_t choose_layout(fft_params &p, int prec, bool post, int V, bool planes_kernel) {
    int const eb = 2 * prec;
    std::vector<layout_choice> cands;
    if (!planes_kernel) {
        static const int lin[][2] = {{30, 0}, {4, 1}, {3, 1}, {5, 1}, {6, 8}, {5, 8}, {7, 8},
                                     {4, 2}, {5, 2}, {6, 4}};
        for (auto const &c : lin) {
            if (V > 1 && ((1 << c[0]) < V || (c[1] % V) != 0)) {
                continue;
            }
            layout_choice L;
            L.sh = c[0];
            L.ad = c[1];
            cands.push_back(L);
        }
    } else {
        layout_choice none;
        none.planes = true;
        cands.push_back(none);
        for (int a = 2; a <= 8; ++a) {
            for (int b = 0; b <= 2; ++b) {
                for (int bits = 1; bits <= 3; ++bits) {
                    if (b + bits > a) {
                        continue;
                    }
                    layout_choice L;
                    L.planes = true;
                    L.a = a;
                    L.b = b;
                    L.mask = (1 << bits) - 1;
                    cands.push_back(L);
                }
            }
        }
    }
    long best_cost = -1;
    layout_choice best;
    for (auto const &L : cands) {
        long c = layout_cost(p, prec, post, V, L);
        if (best_cost < 0 || c < best_cost) {
            best_cost = c;
            best = L;
        }
    }
    p.pad_shift = best.sh;
    p.pad_add = best.ad;
    p.sw_a = best.a;
    p.sw_b = best.b;
    p.sw_mask = best.mask;
    long const n = static_cast<long>(p.Kb) * p.Nc * p.Mb; // complex elements per buffer
    if (!best.planes) {
        long last = n - 1;
        p.buf_elems = static_cast<int>(last + (last >> best.sh) * best.ad + 1);
        p.plane_chunks = 0;
        return static_cast<std::size_t>(p.buf_elems) * eb;
    }
    int nq = std::max(1, eb * V / 16);
    long chunks = n * eb / nq / 16; // chunks per plane
    int bits = 0;
    while ((1 << bits) <= best.mask) {
        ++bits;
    }
    long gran = 1L << (best.b + bits); // the swizzle permutes within aligned blocks of gran
    chunks = (chunks + gran - 1) / gran * gran;
    p.plane_chunks = static_cast<int>(chunks);
    p.buf_elems = static_cast<int>(nq * chunks * 16 / eb);
    return static_cast<std::size_t>(nq) * chunks * 16;
}

// Name of the callback kernel: the compiled code depends on the precision, the kernel kind
// and the user module only, so plans of different shapes share one module.
std::string callback_kernel_name(int prec, int kind, const char *src, std::size_t len,
                                 const char *load_fn, const char *store_fn) {
    std::ostringstream key;
    key << "gbfft_cb_f" << prec * 8 << "_" << kind_name(kind) << "_" << (load_fn ? load_fn : "")
        << "_" << (store_fn ? store_fn : "") << "_" << std::hex << fnv1a(src, len);
    return c_ident(key.str());
}

// NVRTC program: the engine, the user module and one kernel per (name, precision, kind,
// io).  io selects which of the user's functions the kernel calls (bit 0: load, bit 1:
// store); the passes of an nd plan call the load function in the first pass only and the
// store function in the last pass only.  The user's load / store functions are called with
// the element offset of the tensor (reference callback_accessor,
// src/base/generator/tensor_accessor.cpp:34-55).
std::string callback_program(const char *cb, std::size_t len, const char *load_fn,
                             const char *store_fn,
                             std::vector<std::tuple<std::string, int, int, int>> const &kernels) {
    std::ostringstream src;
    src << "typedef decltype(sizeof(0)) size_t;\n";
    // NVRTC kernels keep the CUDA-core odd-radix stages (the tensor-core stages'
    // coefficient tables are not part of the embedded engine source)
    src << "#define GBFFT_NVRTC 1\n";
    src << kEngineSource << "\n";
    src << std::string(cb, len) << "\n";
    std::set<int> ios;
    for (auto const &k : kernels) {
        ios.insert(std::get<3>(k));
    }
    for (int io : ios) {
        bool user_load = (io & 1) && load_fn && *load_fn;
        bool user_store = (io & 2) && store_fn && *store_fn;
        src << "struct gbfft_user_io_" << io << " {\n"
            << "  static constexpr bool direct = false;\n"
            << "  template <class T> static __device__ __forceinline__ T load(const T *t, long long "
               "base, int off) {\n";
        if (user_load) {
            src << "    return " << load_fn << "(const_cast<T *>(t), (size_t)(base + off));\n";
        } else {
            src << "    return (t + base)[off];\n";
        }
        src << "  }\n  template <class T> static __device__ __forceinline__ void store(T *t, long long "
               "base, int off, T v) {\n";
        if (user_store) {
            src << "    " << store_fn << "(t, (size_t)(base + off), v);\n";
        } else {
            src << "    (t + base)[off] = v;\n";
        }
        src << "  }\n};\n";
    }
    for (auto const &k : kernels) {
        src << "extern \"C\" __global__ void __launch_bounds__(512) " << std::get<0>(k)
            << "(const __grid_constant__ gbfft::fft_params p) {\n"
            << "  gbfft::fft_tile<" << (std::get<1>(k) == 4 ? "float" : "double") << ", "
            << std::get<2>(k) << ", gbfft_user_io_" << std::get<3>(k) << ">(p);\n}\n";
    }
    return src.str();
}

// Which user functions a pass with these load / store names calls (the io of
// callback_program).
int callback_io(const char *load_fn, const char *store_fn) {
    return ((load_fn && *load_fn) ? 1 : 0) | ((store_fn && *store_fn) ? 2 : 0);
}

static int largest_prime_factor(int n) {
    int f = 1;
    for (int p = 2; n > 1;) {
        if (n % p == 0) {
            f = p;
            n /= p;
        } else {
            ++p;
        }
    }
    return f;
}

// Bluestein pass (bluestein.cu) for a float length Nc whose largest prime factor is above
// 61: one CTA per tile of Mb x Kb transforms (4 per CTA, 64 threads each), the convolution
// of length L (the power of two >= 2 Nc - 1) in shared memory.  Tables in long double,
// rounded once: chirp c_n = exp(-i pi (n^2 mod 2 Nc) / Nc), FFT_L(b) / L with b_m =
// conj(c_|m|) at m mod L, and w_L^{-i}.
static pass make_bluestein_pass(pass_request const &q, pass ps, int flags, int N, int Nc, int Nt,
                                int device) {
    int L = 256;
    while (L < 2 * Nc - 1) {
        L *= 2;
    }
    if (L > 1024) {
        throw status_error(BBFFT_INTERNAL_ERROR, "Bluestein length above 1024");
    }
    // T threads per transform, 256 threads per tile
    int const T = bluestein_threads(L);
    long long const M = q.M, K = q.K;
    // odd real N: two real transforms along K per complex transform (not for the adjoint
    // forms, whose Hermitian weights the pairing does not apply)
    bool const pair = (ps.kind == kind_r2c_full || ps.kind == kind_c2r_full) && K >= 2 &&
                      (flags & (flag_adj_r2c | flag_adj_c2r)) == 0;
    long long const Kt = pair ? (K + 1) / 2 : K; // transforms along K of the tiles
    // compile-time tile widths 1, 2, 4 (M = 3 in one tile of 4, as before in-place real
    // transforms need the whole M range in one tile)
    int const Mb = M >= 3 ? 4 : static_cast<int>(M);
    int const Kb =
        static_cast<int>(std::max<long long>(1, std::min<long long>(256 / T / Mb, Kt)));
    fft_params &p = ps.p;
    p.M = M;
    p.K = K;
    if ((N + 1) * std::max(std::llabs(q.is1), std::llabs(q.os1)) > 0x7fffffffLL) {
        bad_config("stride of the FFT mode too large");
    }
    p.is1 = static_cast<int>(q.is1);
    p.is2 = q.is2;
    p.os1 = static_cast<int>(q.os1);
    p.os2 = q.os2;
    p.N = N;
    p.Nc = Nc;
    p.Nt = Nt;
    p.L = 0;
    p.T = T;
    p.Mb = Mb;
    p.Kb = Kb;
    p.m_tiles = static_cast<int>((M + Mb - 1) / Mb);
    p.flags = flags;
    if (ps.kind == kind_r2c_half && q.is1 == 1 && M == 1 && q.is2 % 2 == 0) {
        p.flags |= flag_vec_in;
    }
    if (ps.kind == kind_c2r_half && q.os1 == 1 && M == 1 && q.os2 % 2 == 0) {
        p.flags |= flag_vec_out;
    }
    p.nbuf = 1;
    // spare elements after every 16: the stages write with strides of Ns * Mb elements;
    // these gaps (searched per L and Mb with a model of the 32 banks, 8-byte elements in
    // half-warp phases) leave one wavefront per 16 lanes except for L = 512, Mb = 1 (+20 %)
    int const E = Mb * Kb * L;
    p.pad_shift = 4;
    p.pad_add = bluestein_pad(L, Mb);
    p.buf_elems = E + (E >> 4) * p.pad_add + p.pad_add;
    p.sw_a = 30;
    p.scale = 1.0;
    p.bL = L;
    ps.tw = get_twiddles(device, 4, Nt);
    p.tw = ps.tw->ptr;
    // stage twiddles of the length-L transform, per stage s >= 1 as [r - 1][kk]:
    // w_L^{-r kk L / (Ns R)}, kk < Ns
    std::vector<int> tw_e;
    for (int s = 1, Ns = bluestein_radix(L, 0); s < bluestein_stages(L); ++s) {
        int const R = bluestein_radix(L, s);
        for (int r = 1; r < R; ++r) {
            for (int kk = 0; kk < Ns; ++kk) {
                tw_e.push_back(r * kk * (L / (Ns * R)));
            }
        }
        Ns *= R;
    }
    int const TW = static_cast<int>(tw_e.size());
    std::vector<float> h(2 * static_cast<std::size_t>(Nc + L + TW));
    long double const pi = 3.141592653589793238462643383279502884L;
    std::vector<long double> cr(Nc), ci(Nc);
    for (int n = 0; n < Nc; ++n) {
        long long const qn = (static_cast<long long>(n) * n) % (2LL * Nc);
        long double const a = pi * static_cast<long double>(qn) / static_cast<long double>(Nc);
        cr[n] = std::cos(a);
        ci[n] = -std::sin(a);
        h[2 * n] = static_cast<float>(cr[n]);
        h[2 * n + 1] = static_cast<float>(ci[n]);
    }
    std::vector<long double> wc(L), ws(L); // w_L^{-i} = (cos, -sin)(2 pi i / L)
    for (int i = 0; i < L; ++i) {
        long double c, sn;
        twiddle_value(i, L, c, sn);
        wc[i] = c;
        ws[i] = -sn;
    }
    for (int i = 0; i < TW; ++i) {
        h[2 * (Nc + L + i)] = static_cast<float>(wc[tw_e[i]]);
        h[2 * (Nc + L + i) + 1] = static_cast<float>(ws[tw_e[i]]);
    }
    std::vector<long double> br(L, 0.0L), bi(L, 0.0L);
    for (int m = 0; m < Nc; ++m) { // b_m = conj(c_m) at m and at L - m
        br[m] = cr[m];
        bi[m] = -ci[m];
        if (m > 0) {
            br[L - m] = cr[m];
            bi[L - m] = -ci[m];
        }
    }
    for (int k = 0; k < L; ++k) {
        long double sr = 0.0L, si = 0.0L;
        for (int m = 0; m < L; ++m) {
            if (br[m] == 0.0L && bi[m] == 0.0L) {
                continue;
            }
            int const e = static_cast<int>((static_cast<long long>(m) * k) % L);
            sr += br[m] * wc[e] - bi[m] * ws[e];
            si += br[m] * ws[e] + bi[m] * wc[e];
        }
        h[2 * (Nc + k)] = static_cast<float>(sr / L);
        h[2 * (Nc + k) + 1] = static_cast<float>(si / L);
    }
    ps.extra = std::make_shared<device_buffer>(h.size() * sizeof(float));
    GB_CUDA(cudaMemcpy(ps.extra->ptr, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
    p.bs = ps.extra->ptr;
    long long const k_tiles = (Kt + Kb - 1) / Kb;
    if (static_cast<long long>(p.m_tiles) * k_tiles > 0x7fffffffLL) {
        bad_config("tensor too large for one launch");
    }
    ps.block = static_cast<unsigned>(Mb * T * Kb);
    ps.smem = static_cast<std::size_t>(p.buf_elems + TW) * 8; // tile buffer + stage twiddles
    ps.V = 1;
    ps.inplace_ok = q.type == BBFFT_C2C || Mb >= M;
    ps.func = bluestein_kernel(ps.kind, pair, Mb);
    if (!ps.func) {
        throw status_error(BBFFT_INTERNAL_ERROR, "Bluestein kernel not found");
    }
    if (needs_smem_optin(ps.smem)) {
        allow_max_smem(ps.func, device);
    }
    ps.grid = static_cast<unsigned>(p.m_tiles * k_tiles);
    std::ostringstream id;
    id << "gbfft_f32_" << kind_name(ps.kind) << "_fl" << flags << "_bluestein_L" << L
       << (pair ? "_pair" : "") << "_M" << M
       << "_N" << N << "_Mb" << Mb << "_Kb" << Kb << "_is" << q.is1 << "_" << q.is2 << "_os" << q.os1
       << "_" << q.os2;
    ps.identifier = c_ident(id.str());
    return ps;
}

pass make_1d_pass(pass_request const &q, int device, bbfft_cache_s *cache) {
    pass ps;
    ps.prec = q.prec;
    bool is_real = q.type != BBFFT_C2C;
    int N = static_cast<int>(q.N);
    bool even = N % 2 == 0;
    // kernel kind; the adjoint of r2c runs the c2r engine and vice versa
    int eff_type = q.type;
    int flags = 0;
    if (q.adjoint) {
        if (q.type == BBFFT_R2C) {
            eff_type = BBFFT_C2R;
            flags |= flag_adj_r2c;
        } else if (q.type == BBFFT_C2R) {
            eff_type = BBFFT_R2C;
            flags |= flag_adj_c2r;
        }
    }
    int dir = q.adjoint && q.type == BBFFT_C2C ? -q.dir : q.dir;
    switch (eff_type) {
    case BBFFT_C2C:
        ps.kind = kind_c2c;
        if (dir == BBFFT_BACKWARD) {
            flags |= flag_conj_in | flag_conj_out;
        }
        break;
    case BBFFT_R2C:
        ps.kind = even ? kind_r2c_half : kind_r2c_full;
        break;
    case BBFFT_C2R:
        ps.kind = even ? kind_c2r_half : kind_c2r_full;
        break;
    }
    int Nc = (is_real && even) ? N / 2 : N;
    int Nt = (is_real && even) ? N : Nc;
    // float lengths with a prime factor above 61: Bluestein's algorithm in one kernel
    bool const has_cb0 = (q.load_fn && *q.load_fn) || (q.store_fn && *q.store_fn);
    if (q.prec == 4 && !has_cb0 && !q.runtime_only && q.compute == BBFFT_COMPUTE_NATIVE &&
        q.radices.empty() && q.T == 0 && largest_prime_factor(Nc) > gen_table_max_p) {
        return make_bluestein_pass(q, ps, flags, N, Nc, Nt, device);
    }

    // autotuned blocking (radices, threads per transform, V, Mb, Kb, register budget)
    tune_entry const *te = nullptr;
    if (q.radices.empty() && q.T == 0 && q.V == 0 && q.Mb == 0 && q.Kb == 0 && q.occ == 0 &&
        !q.force_v1 && !q.runtime_only && q.compute == BBFFT_COMPUTE_NATIVE) {
        te = find_tuning(q.prec, ps.kind, N, q.M);
    }
    bool te_rad = false;
    if (te && !te->rad.empty()) {
        long long prod = 1;
        for (int r : te->rad) {
            prod *= r > 0 ? r : 0;
        }
        te_rad = prod == Nc; // a table line for another length is ignored
    }
    std::vector<int> rad = !q.radices.empty() ? q.radices : te_rad ? te->rad : choose_radices(Nc);
    {
        long long prod = 1;
        for (int r : rad) {
            if (r < 1) {
                bad_config("radix must be positive");
            }
            prod *= r;
        }
        if (prod != Nc) {
            bad_config("product of radices must equal the complex FFT length " + std::to_string(Nc));
        }
        for (int r : rad) {
            if (!unrolled(r) && r % 2 == 0) {
                bad_config("radix " + std::to_string(r) + " has no butterfly (even radices up to "
                           "16 only)");
            }
        }
    }
    bool post = ps.kind == kind_r2c_half;
    if (q.compute != BBFFT_COMPUTE_NATIVE) {
        // tensor-core DFT stages (tc.cu): fixed tiles of whole transforms
        // BF16 pieces per operand; 0 selects the split-TF32 kernels
        int pieces = q.compute == BBFFT_COMPUTE_BF16               ? 1
                     : q.compute == BBFFT_COMPUTE_SPLIT_BF16_3TERM ? 2
                     : q.compute == BBFFT_COMPUTE_SPLIT_TF32       ? 0
                                                                   : 3;
        fft_params &p = ps.p;
        p.M = 1;
        p.K = q.K;
        p.is1 = p.os1 = 1;
        p.is2 = q.is2;
        p.os2 = q.os2;
        p.N = p.Nc = p.Nt = N;
        p.flags = flags;
        p.scale = 1.0;
        int tiles = tc_tile_transforms(N);
        ps.grid = static_cast<unsigned>((q.K + tiles - 1) / tiles);
        ps.block = 256;
        ps.smem = tc_shared_bytes();
        ps.func = tc_kernel(pieces, N);
        ps.tc = true;
        ps.inplace_ok = true;
        ps.tw = get_twiddles(device, q.prec, N);
        p.tw = ps.tw->ptr;
        ps.identifier = "gbfft_tc_p" + std::to_string(pieces) + "_N" + std::to_string(N) + "_K" +
                        std::to_string(q.K);
        if (!ps.func) {
            throw status_error(BBFFT_INTERNAL_ERROR, "tensor-core kernel not found");
        }
        return ps;
    }
    // a generic (non-unrolled) first stage needs a shared-memory source
    if (!unrolled(rad.front())) {
        rad.insert(rad.begin(), 1);
    }
    // the compile-time prime stages write shared memory only, so a prime last stage is
    // followed by a copy stage (the same radices for the runtime engine)
    if (!post && table_generic(rad.back())) {
        rad.push_back(1);
    }
    // real transforms must finish all global reads of a tile before the first global write
    // (in-place safety): with a single global->global stage, add a shared round trip
    if (is_real && !post && rad.size() == 1) {
        rad.push_back(1);
    }
    if (rad.size() > static_cast<std::size_t>(max_stages)) {
        bad_config("too many stages");
    }
    int L = static_cast<int>(rad.size());
    int pu = 1;
    for (int r : rad) {
        if (unrolled(r)) {
            pu = std::max(pu, r);
        }
    }
    int const reqT = q.T > 0 ? q.T : (te && (te_rad || te->rad.empty()) ? te->T : 0);
    int T = reqT > 0 ? reqT : std::max(1, Nc / pu);
    if (pu == 1) {
        T = std::min(Nc, 64);
    }
    // with a table-driven generic stage: one thread per task (a group of gen_group output
    // pairs of one butterfly) of the largest one
    int ptg = 0;
    for (int r : rad) {
        if (table_generic(r)) {
            ptg = std::max(ptg, r);
        }
    }
    if (ptg > 0 && reqT <= 0) {
        int H = (ptg - 1) / 2;
        T = Nc / ptg * ((H + gen_group - 1) / gen_group);
    }
    T = std::min(T, 512);

    long long M = q.M, K = q.K;
    bool has_cb = (q.load_fn && *q.load_fn) || (q.store_fn && *q.store_fn);
    int reqV = q.V, reqMb = q.Mb, reqKb = q.Kb, reqOcc = q.occ;
    if (te) {
        reqV = te->V;
        reqMb = te->Mb;
        reqKb = te->Kb;
        reqOcc = te->occ;
    }
    // kernel variant: 2 / 3 resident CTAs, + 10 for the paired c2r pre-process
    int minb = (reqOcc == 3 || reqOcc == 13) ? 3 : 2;
    if ((reqOcc == 12 || reqOcc == 13) && ps.kind == kind_c2r_half && q.prec == 4) {
        minb += 10;
    }
    // compile-time-size kernel, vectorised over M when the layout allows it
    const ct_entry *ct = nullptr;
    int V = 1;
    if (!has_cb && !q.runtime_only) {
        int vw = vector_width(q.prec, rad);
        if (reqV > 0) {
            vw = std::min(vw, reqV);
        }
        bool v_ok = !q.force_v1 && vw > 1 && M % vw == 0 && q.is1 % vw == 0 && q.os1 % vw == 0 &&
                    q.is2 % vw == 0 && q.os2 % vw == 0;
        if (v_ok) {
            ct = ct_lookup(q.prec, ps.kind, Nc, T, vw, rad.data(), L, minb);
            V = ct ? vw : 1;
        }
        if (!ct) {
            ct = ct_lookup(q.prec, ps.kind, Nc, T, 1, rad.data(), L, minb);
        }
    }
    // compile-time-size tile functions of the ragged set (float, V = 1): the tiles of
    // ragged batches, and plans of lengths without a compile-time plan kernel
    int ragged_vid = -1;
    int cover_id = -1;
    // a length whose prime stage runs in registers (reg_prime_length): the prime stage
    // first, then the radices of Nc / P (no copy stages; real single stages keep theirs)
    int const Preg = (q.radices.empty() && !te_rad && reqT <= 0) ? reg_prime_length(Nc) : 0;
    std::vector<int> rad_reg;
    if (Preg > 0) {
        rad_reg.push_back(Preg);
        if (Nc > Preg) {
            std::vector<int> rest = choose_radices(Nc / Preg);
            rad_reg.insert(rad_reg.end(), rest.begin(), rest.end());
        }
        if (is_real && !post && rad_reg.size() == 1) {
            rad_reg.push_back(1);
        }
    }
    int const L_reg = static_cast<int>(rad_reg.size());
    int const T_reg = Preg > 0 ? tile_threads(Nc, rad_reg.data(), L_reg, 1, true) : 0;
    if (!has_cb && !ct && q.prec == 4 && Preg > 0 && Preg <= 47) {
        // the ragged tiles run the prime stage in registers up to P = 47
        ragged_vid = ragged_ct_lookup(q.prec, ps.kind, Nc, T_reg, 1, rad_reg.data(), L_reg);
        if (ragged_vid >= 0) {
            rad = rad_reg;
            L = L_reg;
            T = T_reg;
            V = 1;
            ct = &ragged_ct_table[ragged_vid];
        }
    }
    if (!has_cb && !ct && q.prec == 4) {
        // compile-time tiles choose their own threads per transform (tile_threads)
        int const Tt = reqT > 0 ? T : tile_threads(Nc, rad.data(), L, 1);
        int vw = vector_width(q.prec, rad);
        if (reqV > 0) {
            vw = std::min(vw, reqV);
        }
        bool v_ok = !q.force_v1 && vw > 1 && M % vw == 0 && q.is1 % vw == 0 && q.os1 % vw == 0 &&
                    q.is2 % vw == 0 && q.os2 % vw == 0;
        if (v_ok) {
            int const Tv = reqT > 0 ? T : tile_threads(Nc, rad.data(), L, vw);
            ragged_vid = ragged_ct_lookup(q.prec, ps.kind, Nc, Tv, vw, rad.data(), L);
            V = ragged_vid >= 0 ? vw : 1;
            if (ragged_vid >= 0) {
                T = Tv;
            }
        }
        if (ragged_vid < 0) {
            ragged_vid = ragged_ct_lookup(q.prec, ps.kind, Nc, Tt, 1, rad.data(), L);
            V = 1;
            if (ragged_vid >= 0) {
                T = Tt;
            }
        }
        if (ragged_vid >= 0) {
            ct = &ragged_ct_table[ragged_vid];
        } else if (!q.runtime_only) {
            // plans of the other lengths (not ragged items: the persistent kernel cannot
            // call these tiles, and the runtime engine needs its own blocking)
            if (Preg > 0) {
                cover_id = cover_ct_lookup(q.prec, ps.kind, Nc, T_reg, rad_reg.data(), L_reg);
                if (cover_id >= 0) {
                    rad = rad_reg;
                    L = L_reg;
                    T = T_reg;
                }
            }
            if (cover_id < 0) {
                cover_id = cover_ct_lookup(q.prec, ps.kind, Nc, Tt, rad.data(), L);
                if (cover_id >= 0) {
                    T = Tt;
                }
            }
            if (cover_id >= 0) {
                ct = &cover_ct_table[cover_id];
            }
        }
    }
    // odd real N on a compile-time cover tile: the transforms k and k + 1 share one complex
    // FFT (not for the adjoint forms, whose Hermitian weights the pairing does not apply)
    bool const pair = cover_id >= 0 && (ps.kind == kind_r2c_full || ps.kind == kind_c2r_full) &&
                      K >= 2 && (flags & (flag_adj_r2c | flag_adj_c2r)) == 0;
    if (pair) {
        flags |= flag_pair;
    }
    long long const Kt = pair ? (K + 1) / 2 : K; // transforms along K of the tiles
    int const max_block = q.max_block > 0 ? q.max_block : (ct ? 256 : 512);
    // the runtime kernel ping-pongs between two buffers when a stage goes shared->shared;
    // compile-time kernels run their stages in place in one buffer
    int nbuf = 1;
    for (int s = 0; s < L && !ct; ++s) {
        bool src_g = s == 0;
        bool dst_g = s == L - 1 && !post;
        if (!src_g && !dst_g) {
            nbuf = 2;
        }
    }

    int Mb;
    if (reqMb > 0) {
        Mb = static_cast<int>(std::min<long long>(reqMb, M));
        if (Mb % V != 0) {
            Mb = std::max(V, Mb / V * V);
        }
    } else if (M == 1) {
        Mb = 1;
    } else if (is_real && M <= 64 && (M / V) * T <= max_block) {
        Mb = static_cast<int>(M);
    } else {
        Mb = static_cast<int>(std::min<long long>(M, 32));
    }
    while (Mb > V && (Mb / V) * T > max_block) {
        Mb = std::max(V, (Mb / 2) / V * V);
    }
    if (Mb % V != 0) {
        Mb = std::max(V, Mb / V * V);
    }
    int const lanes_per_k = (Mb / V) * T;
    std::size_t celem = 2 * static_cast<std::size_t>(q.prec);
    int pgen = 0; // generic stages keep their coefficient tables in shared memory
    for (int r : rad) {
        pgen = std::max(pgen, gen_shared_elems(q.prec, r, !has_cb));
    }
    // (compile-time kernels keep their prime coefficients in the code)
    std::size_t const gen_extra = ct ? 0 : static_cast<std::size_t>(pgen) * celem;
    // shared padding i -> i + (i >> shift) * add adds at most a quarter (choose_padding)
    auto buf_elems = [&](int kb, int mb) {
        long long last = static_cast<long long>(kb) * Nc * mb - 1;
        return last + (last >> 2) + 1;
    };
    int Kb = reqKb > 0 ? reqKb : std::max(1, std::min(256, max_block) / lanes_per_k);
    Kb = static_cast<int>(std::min<long long>(Kb, Kt));
    Kb = std::max(Kb, 1);
    while (Kb * lanes_per_k > max_block && Kb > 1) {
        Kb /= 2;
    }
    std::size_t const soft_limit = 96 * 1024;
    while (Kb > 1 && nbuf * buf_elems(Kb, Mb) * celem > soft_limit) {
        Kb /= 2;
    }
    // a tile of Mb transforms that does not fit is split along M (in-place real
    // transforms then become unsupported, as in the reference when Mb < M)
    while (Mb > V && nbuf * buf_elems(Kb, Mb) * celem > soft_limit) {
        Mb = std::max(V, (Mb / 2) / V * V);
    }
    std::size_t smem = nbuf * buf_elems(Kb, Mb) * celem + gen_extra;
    if (smem > static_cast<std::size_t>(max_optin_smem(device))) {
        bad_config("FFT length " + std::to_string(N) + " needs " + std::to_string(smem) +
                   " bytes of shared memory per block, more than the device provides");
    }

    fft_params &p = ps.p;
    p.M = M;
    p.K = K;
    if ((N + 1) * std::max(std::llabs(q.is1), std::llabs(q.os1)) > 0x7fffffffLL) {
        bad_config("stride of the FFT mode too large");
    }
    p.is1 = static_cast<int>(q.is1);
    p.is2 = q.is2;
    p.os1 = static_cast<int>(q.os1);
    p.os2 = q.os2;
    p.N = N;
    p.Nc = Nc;
    p.Nt = Nt;
    p.L = L;
    for (int s = 0; s < L; ++s) {
        p.radix[s] = rad[s];
    }
    p.T = T;
    p.Mb = Mb;
    p.Kb = Kb;
    p.m_tiles = static_cast<int>((M + Mb - 1) / Mb);
    p.flags = flags;
    p.nbuf = nbuf;
    p.scale = 1.0;
    // compile-time kernels store lane vectors of 16 bytes or more as swizzled 16-byte planes
    bool planes_kernel = ct != nullptr && celem * V >= 16;
    smem = static_cast<std::size_t>(nbuf) * choose_layout(p, q.prec, post, V, planes_kernel) + gen_extra;
    // paired real loads / stores: adjacent (unit N-stride, one transform per M) and aligned
    if (ps.kind == kind_r2c_half && q.is1 == 1 && M == 1 && q.is2 % 2 == 0) {
        p.flags |= flag_vec_in;
    }
    if (ps.kind == kind_c2r_half && q.os1 == 1 && M == 1 && q.os2 % 2 == 0) {
        p.flags |= flag_vec_out;
    }
    long long k_tiles = (Kt + Kb - 1) / Kb;
    if (static_cast<long long>(p.m_tiles) * k_tiles > 0x7fffffffLL) {
        bad_config("tensor too large for one launch");
    }
    ps.grid = static_cast<unsigned>(p.m_tiles * k_tiles);
    ps.block = static_cast<unsigned>((Mb / V) * T * Kb);
    if (!has_cb && std::any_of(rad.begin(), rad.end(), [&](int r) { return tc_prime(q.prec, r); })) {
        // tensor-core prime stages run on full warps; the extra threads only take part in
        // the barriers (both engines support threads beyond the tile)
        ps.block = (ps.block + 31) / 32 * 32;
    }
    ps.V = V;
    ps.smem = smem;
    ps.inplace_ok = !is_real || Mb >= M;
    ps.tw = get_twiddles(device, q.prec, Nt);
    p.tw = ps.tw->ptr;

    std::ostringstream id;
    id << "gbfft_f" << q.prec * 8 << "_" << kind_name(ps.kind) << "_fl" << flags << "_M" << M
       << "_Mb" << Mb << "_N" << N << "_r";
    for (int s = 0; s < L; ++s) {
        id << (s ? "x" : "") << rad[s];
    }
    id << "_T" << T << "_V" << V << "_Kb" << Kb << (pair ? "_pair" : "") << "_is" << q.is1 << "_"
       << q.is2 << "_os" << q.os1 << "_" << q.os2;
    if (q.load_fn && *q.load_fn) {
        id << "_" << q.load_fn;
    }
    if (q.store_fn && *q.store_fn) {
        id << "_" << q.store_fn;
    }
    ps.identifier = c_ident(id.str());

    if (!has_cb) {
        ps.func = (ct && ct->fn) ? ct->fn
                  : ragged_vid >= 0 ? ragged_plan_kernel(ragged_vid)
                  : cover_id >= 0   ? cover_ct_kernel(cover_id)
                                    : (q.prec == 4 ? kernel_f32(ps.kind) : kernel_f64(ps.kind));
        ps.specialized = ct != nullptr;
        ps.min_blocks = ct ? ct->minb : 0; // (+ 10: paired c2r variant)
        ps.ragged_vid = ragged_vid;
        if (V > 1) {
            pass_request q1 = q;
            q1.force_v1 = true;
            q1.Mb = Mb;
            q1.Kb = std::max(1, Kb / V);
            ps.scalar_alt = std::make_shared<pass>(make_1d_pass(q1, device, cache));
        }
        if (!ps.func) {
            throw status_error(BBFFT_INTERNAL_ERROR, "kernel not found");
        }
    } else {
        if (!q.cb_source || q.cb_length == 0) {
            bad_config("callback function named but no callback source given");
        }
        std::string kname = callback_kernel_name(q.prec, ps.kind, q.cb_source, q.cb_length,
                                                 q.load_fn, q.store_fn);
        std::shared_ptr<module> mod;
        if (cache) {
            mod = cache->get(kname, device);
        }
        if (!mod) {
            std::string src = callback_program(
                q.cb_source, q.cb_length, q.load_fn, q.store_fn,
                {std::make_tuple(kname, q.prec, ps.kind, callback_io(q.load_fn, q.store_fn))});
            mod = nvrtc_build(src, kname, device);
            if (cache) {
                cache->store(kname, device, mod);
            }
        }
        cudaKernel_t k = mod->kernel(kname);
        if (!k) {
            throw status_error(BBFFT_INTERNAL_ERROR, "kernel " + kname + " not in module");
        }
        ps.mod = mod;
        ps.func = reinterpret_cast<const void *>(k);
    }
    if (needs_smem_optin(smem)) {
        allow_max_smem(ps.func, device, static_cast<bool>(ps.mod));
    }
    return ps;
}

// Launch geometry of one 1d pass computed without any allocation: heuristic radices and
// blocking, one transform per thread along M, compile-time kernel when one exists, padded
// linear shared layout.  The caller provides the twiddle table.  Returns an empty string
// on success, else the reason the pass is not supported this way.
const char *plan_pass_fixed(int prec, int type, int dir, long long M, long long N, long long K,
                            long long is1, long long is2, long long os1, long long os2,
                            int device, fft_params &p, unsigned &grid, unsigned &block,
                            std::size_t &smem, const void *&func) {
    bool is_real = type != BBFFT_C2C;
    bool even = N % 2 == 0;
    int kind = type == BBFFT_C2C ? kind_c2c
               : type == BBFFT_R2C ? (even ? kind_r2c_half : kind_r2c_full)
                                   : (even ? kind_c2r_half : kind_c2r_full);
    int flags = (type == BBFFT_C2C && dir == BBFFT_BACKWARD) ? (flag_conj_in | flag_conj_out) : 0;
    int Nc = static_cast<int>((is_real && even) ? N / 2 : N);
    int Nt = (is_real && even) ? static_cast<int>(N) : Nc;
    int rad[max_stages + 2];
    int r0[32];
    int n0 = choose_radices_core(Nc, r0);
    int L = 0;
    if (!unrolled(r0[0])) {
        rad[L++] = 1;
    }
    for (int i = 0; i < n0; ++i) {
        if (L >= max_stages) {
            return "too many stages";
        }
        rad[L++] = r0[i];
    }
    bool post = kind == kind_r2c_half;
    // a generic odd-radix stage reads and writes shared memory only (its tensor-core form
    // writes the butterflies of several transforms per warp): a copy stage follows it, as
    // in make_1d_pass
    if (!post && table_generic(rad[L - 1])) {
        if (L >= max_stages) {
            return "too many stages";
        }
        rad[L++] = 1;
    }
    if (is_real && !post && L == 1) {
        rad[L++] = 1;
    }
    if (L > max_stages) {
        return "too many stages";
    }
    int pu = 1;
    for (int i = 0; i < L; ++i) {
        if (unrolled(rad[i])) {
            pu = std::max(pu, rad[i]);
        }
    }
    int T = pu == 1 ? std::min(Nc, 64) : std::max(1, Nc / pu);
    T = std::min(T, 512);
    const ct_entry *ct = ct_lookup(prec, kind, Nc, T, 1, rad, L, 2);
    int const max_block = ct ? 256 : 512;
    int nbuf = 1;
    for (int s2 = 0; s2 < L && !ct; ++s2) {
        if (s2 != 0 && !(s2 == L - 1 && !post)) {
            nbuf = 2;
        }
    }
    int Mb = M == 1 ? 1 : static_cast<int>(std::min<long long>(M, 32));
    while (Mb > 1 && Mb * T > max_block) {
        Mb /= 2;
    }
    std::size_t celem = 2 * static_cast<std::size_t>(prec);
    auto bytes = [&](int kb) {
        long long last = static_cast<long long>(kb) * Nc * Mb - 1;
        return static_cast<std::size_t>(nbuf) * static_cast<std::size_t>(last + (last >> 2) + 1) * celem;
    };
    int Kb = static_cast<int>(std::max<long long>(1, std::min<long long>(256 / (Mb * T), K)));
    while (Kb > 1 && (Kb * Mb * T > max_block || bytes(Kb) > 96 * 1024)) {
        Kb /= 2;
    }
    if ((N + 1) * std::max(std::llabs(is1), std::llabs(os1)) > 0x7fffffffLL) {
        return "stride of the FFT mode too large";
    }
    p = fft_params{};
    p.M = M;
    p.K = K;
    p.is1 = static_cast<int>(is1);
    p.is2 = is2;
    p.os1 = static_cast<int>(os1);
    p.os2 = os2;
    p.N = static_cast<int>(N);
    p.Nc = Nc;
    p.Nt = Nt;
    p.L = L;
    for (int i = 0; i < L; ++i) {
        p.radix[i] = rad[i];
    }
    p.T = T;
    p.Mb = Mb;
    p.Kb = Kb;
    p.m_tiles = static_cast<int>((M + Mb - 1) / Mb);
    p.flags = flags;
    p.nbuf = nbuf;
    p.scale = 1.0;
    static const int lin[][2] = {{30, 0}, {4, 1}, {3, 1}, {5, 1}, {6, 8}, {5, 8}, {7, 8},
                                 {4, 2}, {5, 2}, {6, 4}};
    long best_cost = -1;
    layout_choice best;
    for (auto const &c : lin) {
        layout_choice Lc;
        Lc.sh = c[0];
        Lc.ad = c[1];
        long cost = layout_cost(p, prec, post, 1, Lc);
        if (best_cost < 0 || cost < best_cost) {
            best_cost = cost;
            best = Lc;
        }
    }
    p.pad_shift = best.sh;
    p.pad_add = best.ad;
    p.sw_a = 30;
    long long last = static_cast<long long>(Kb) * Nc * Mb - 1;
    p.buf_elems = static_cast<int>(last + (last >> best.sh) * best.ad + 1);
    int pgen = 0;
    for (int i = 0; i < L; ++i) {
        pgen = std::max(pgen, gen_shared_elems(prec, rad[i], true));
    }
    smem = static_cast<std::size_t>(nbuf) * p.buf_elems * celem + static_cast<std::size_t>(pgen) * celem;
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device) != cudaSuccess) {
        return "cudaDeviceGetAttribute failed";
    }
    if (smem > static_cast<std::size_t>(optin)) {
        return "FFT length needs more shared memory than the device provides";
    }
    long long k_tiles = (K + Kb - 1) / Kb;
    if (static_cast<long long>(p.m_tiles) * k_tiles > 0x7fffffffLL) {
        return "tensor too large for one launch";
    }
    grid = static_cast<unsigned>(p.m_tiles * k_tiles);
    block = static_cast<unsigned>(Mb * T * Kb);
    for (int i = 0; i < L; ++i) {
        if (tc_prime(prec, rad[i])) { // tensor-core prime stages run on full warps
            block = (block + 31) / 32 * 32;
            break;
        }
    }
    func = ct ? ct->fn : (prec == 4 ? kernel_f32(kind) : kernel_f64(kind));
    if (needs_smem_optin(smem) &&
        cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess) {
        return "cudaFuncSetAttribute failed";
    }
    return "";
}

} // namespace gbfft

// ------------------------------------------------------------------------------------------
// plans

struct bbfft_plan_s {
    std::atomic<int> refs{1};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<gbfft::pass> passes;
    std::shared_ptr<gbfft::device_buffer> tmp;
    // nd plans with non-default layouts run on packed copies of the input and output
    std::shared_ptr<gbfft::device_buffer> packed_in, packed_out;
    bool inplace_ok = true;
    bool jit = false;
    // nd plans whose intermediate tensor does not fit in a share of the L2 cache run slab by
    // slab along the K mode: every pass over one slab of slab_k transforms, then the next
    // slab, so that the intermediate stays in L2 between the passes (0: one slab)
    long long slab_k = 0;
    long long slab_count = 0;                // slabs of slab_k transforms
    std::vector<gbfft::pass> tail_passes;    // passes of a last, shorter slab (if any)
    std::size_t slab_in_bytes = 0, slab_out_bytes = 0; // pointer advance per slab
};

namespace gbfft {

static void validate(bbfft_configuration const &cfg) {
    if (cfg.dim < 1 || cfg.dim > max_fft_dim) {
        bad_config("Unsupported FFT dimension: " + std::to_string(cfg.dim));
    }
    if (cfg.precision != BBFFT_PRECISION_F32 && cfg.precision != BBFFT_PRECISION_F64) {
        bad_config("Unsupported precision");
    }
    if (cfg.type != BBFFT_C2C && cfg.type != BBFFT_R2C && cfg.type != BBFFT_C2R) {
        bad_config("Unsupported transform type");
    }
    if (cfg.direction != BBFFT_FORWARD && cfg.direction != BBFFT_BACKWARD) {
        bad_config("Unsupported direction");
    }
    if ((cfg.type == BBFFT_R2C && cfg.direction != BBFFT_FORWARD) ||
        (cfg.type == BBFFT_C2R && cfg.direction != BBFFT_BACKWARD)) {
        bad_config("r2c direction must be forward and c2r direction must be backward");
    }
    for (unsigned d = 0; d < cfg.dim + 2; ++d) {
        if (cfg.shape[d] == 0) {
            bad_config("tensor shape entries must be positive");
        }
    }
    if (cfg.istride[0] != 1 || cfg.ostride[0] != 1) {
        bad_config("stride s0 != 1 is not supported");
    }
    if (cfg.compute != BBFFT_COMPUTE_NATIVE) {
        bool ok = cfg.compute == BBFFT_COMPUTE_BF16 || cfg.compute == BBFFT_COMPUTE_SPLIT_BF16 ||
                  cfg.compute == BBFFT_COMPUTE_SPLIT_BF16_3TERM || cfg.compute == BBFFT_COMPUTE_SPLIT_TF32;
        std::size_t N = cfg.shape[1];
        ok = ok && cfg.dim == 1 && cfg.type == BBFFT_C2C && cfg.precision == BBFFT_PRECISION_F32 &&
             (N == 64 || N == 256 || N == 512) && cfg.shape[0] == 1 && cfg.istride[1] == 1 &&
             cfg.ostride[1] == 1 && cfg.istride[2] == N && cfg.ostride[2] == N &&
             !(cfg.load_function && *cfg.load_function) &&
             !(cfg.store_function && *cfg.store_function);
        if (!ok) {
            bad_config("tensor-core compute modes support 1d c2c float transforms of length 64, "
                       "256 or 512 with M = 1 and the packed layout, without callbacks");
        }
    }
}

static void make_plan_impl(bbfft_configuration const &cfg, cudaStream_t stream,
                           bbfft_cache_s *cache, bool adjoint, bbfft_plan_s &plan,
                           pass_request const *tuning) {
    validate(cfg);
    bool has_cb = (cfg.load_function && *cfg.load_function) ||
                  (cfg.store_function && *cfg.store_function);
    stride_t shape = to_array(cfg.shape);
    auto is_default = [&](bool inplace) {
        stride_t di = default_istride(cfg.dim, shape, cfg.type, inplace);
        stride_t dout = default_ostride(cfg.dim, shape, cfg.type, inplace);
        for (unsigned d = 0; d < cfg.dim + 2; ++d) {
            if (cfg.istride[d] != di[d] || cfg.ostride[d] != dout[d]) {
                return false;
            }
        }
        return true;
    };
    // nd with a layout other than the two defaults: gather the input into the packed
    // out-of-place layout, run the chain there and scatter the result (the reference rejects
    // such layouts, src/common/algorithm/nd_fft.hpp:47-49)
    bool strided_nd = false;
    if (cfg.dim > 1) {
        if (!is_default(false) && !is_default(true)) {
            if (adjoint) {
                bad_config("adjoint plans of nd transforms need a default tensor layout");
            }
            if (has_cb) {
                bad_config("callbacks of nd transforms need a default tensor layout");
            }
            strided_nd = true;
        }
    }
    if (adjoint && has_cb) {
        bad_config("callbacks are not supported for adjoint plans");
    }
    GB_CUDA(cudaGetDevice(&plan.device));
    plan.stream = stream;
    if (cfg.dim == 1) {
        pass_request q = tuning ? *tuning : pass_request{};
        q.prec = cfg.precision;
        q.type = cfg.type;
        q.dir = cfg.direction;
        q.adjoint = adjoint;
        q.M = static_cast<long long>(cfg.shape[0]);
        q.N = static_cast<long long>(cfg.shape[1]);
        q.K = static_cast<long long>(cfg.shape[2]);
        if (!adjoint) {
            q.is1 = cfg.istride[1];
            q.is2 = cfg.istride[2];
            q.os1 = cfg.ostride[1];
            q.os2 = cfg.ostride[2];
        } else { // the adjoint maps the output layout back to the input layout
            q.is1 = cfg.ostride[1];
            q.is2 = cfg.ostride[2];
            q.os1 = cfg.istride[1];
            q.os2 = cfg.istride[2];
        }
        q.cb_source = cfg.callback_source;
        q.cb_length = cfg.callback_length;
        q.load_fn = cfg.load_function;
        q.store_fn = cfg.store_function;
        q.compute = adjoint ? BBFFT_COMPUTE_NATIVE : cfg.compute;
        plan.passes.push_back(make_1d_pass(q, plan.device, cache));
        plan.inplace_ok = plan.passes.back().inplace_ok;
        plan.jit = has_cb;
        return;
    }
    // ---- nd: chain of 1d passes (reference src/common/algorithm/nd_fft.hpp:27-130) ----
    bool inplace_layout = !strided_nd && is_default(true);
    bool is_real = cfg.type != BBFFT_C2C;
    unsigned dim = cfg.dim;
    auto nd_complex = [&](unsigned d) -> long long {
        return d == 0 && is_real ? cfg.shape[1] / 2 + 1 : cfg.shape[d + 1];
    };
    auto nd_real = [&](unsigned d) -> long long {
        return d == 0 && is_real && inplace_layout ? 2 * (cfg.shape[1] / 2 + 1) : cfg.shape[d + 1];
    };
    long long Ntot = 1;
    for (unsigned d = 0; d < dim; ++d) {
        Ntot *= nd_complex(d);
    }
    std::vector<pass_request> reqs(dim);
    long long M = cfg.shape[0];
    long long K = Ntot * static_cast<long long>(cfg.shape[dim + 1]);
    for (unsigned d = 0; d < dim; ++d) {
        long long Nd = cfg.shape[d + 1];
        long long Ndc = nd_complex(d);
        K /= Ndc;
        pass_request &q = reqs[d];
        q.prec = cfg.precision;
        q.type = d == 0 ? cfg.type : BBFFT_C2C;
        q.dir = cfg.direction;
        q.adjoint = adjoint;
        q.M = M;
        q.N = Nd;
        q.K = K;
        q.is1 = M;
        q.is2 = M * nd_real(d);
        q.os1 = M;
        q.os2 = M * Ndc;
        M *= Ndc;
    }
    // forward execution order: c2r starts with the outer dimensions and swaps the layouts
    // of every pass (nd_fft.hpp:100-108)
    std::vector<pass_request> order;
    bool reverse = cfg.type == BBFFT_C2R;
    for (unsigned d = 0; d < dim; ++d) {
        pass_request q = reverse ? reqs[dim - 1 - d] : reqs[d];
        q.adjoint = false;
        if (reverse) {
            std::swap(q.is1, q.os1);
            std::swap(q.is2, q.os2);
        }
        order.push_back(q);
    }
    // the adjoint runs the adjoints of the passes in reverse order, each mapping the
    // layout of its forward output back to the layout of its forward input
    if (adjoint) {
        std::reverse(order.begin(), order.end());
        for (auto &q : order) {
            q.adjoint = true;
            std::swap(q.is1, q.os1);
            std::swap(q.is2, q.os2);
        }
    }
    // user callbacks (the reference takes none for dim > 1, nd_fft.hpp:29-31): the first
    // pass reads the input tensor in its own layout and the last pass writes the output
    // tensor in its own layout, so the load function runs in the first pass and the store
    // function in the last, each with the element offset of its tensor
    for (std::size_t i = 0; i < order.size(); ++i) {
        pass_request &q = order[i];
        if (has_cb) {
            q.cb_source = cfg.callback_source;
            q.cb_length = cfg.callback_length;
            q.load_fn = i == 0 ? cfg.load_function : nullptr;
            q.store_fn = i + 1 == order.size() ? cfg.store_function : nullptr;
        }
    }
    plan.jit = has_cb;
    // temporary buffer if the input is larger than the output (nd_fft.hpp:114-125)
    std::size_t real_b = cfg.precision, cplx_b = 2 * real_b;
    bool in_real = adjoint ? cfg.type == BBFFT_C2R : cfg.type == BBFFT_R2C;
    bool out_real = adjoint ? cfg.type == BBFFT_R2C : cfg.type == BBFFT_C2R;
    stride_t pis = default_istride(dim, shape, cfg.type, false);
    stride_t pos = default_ostride(dim, shape, cfg.type, false);
    std::size_t const *ist = strided_nd ? pis.data() : adjoint ? cfg.ostride : cfg.istride;
    std::size_t const *ost = strided_nd ? pos.data() : adjoint ? cfg.istride : cfg.ostride;
    std::size_t isize = ist[dim + 1] * cfg.shape[dim + 1] * (in_real ? real_b : cplx_b);
    std::size_t osize = ost[dim + 1] * cfg.shape[dim + 1] * (out_real ? real_b : cplx_b);
    // L2-resident chaining (no counterpart in the reference, which runs each pass over the
    // whole tensor, nd_fft.hpp:140-152): with BBFFT_GB300_ND_SLAB_BYTES = B > 0 and an
    // intermediate tensor larger than B, the passes run slab by slab along K (slabs of at
    // most B intermediate bytes), so the intermediate written by one pass can still be in
    // L2 when the next pass reads it.  Off by default: on GB300 the 2d 128 x 128 and 3d 64^3
    // benchmark plans ran slower in slabs of L2/4 or 64 MB (more, shorter launches) than
    // over the whole tensor.  Not with callbacks (their offsets are relative to the whole
    // tensor) or custom layouts (packed copies).
    long long const Kimg = static_cast<long long>(cfg.shape[dim + 1]);
    std::size_t const inter_per_k = std::max(isize, osize) / static_cast<std::size_t>(Kimg);
    std::size_t budget = 0;
    if (const char *e = std::getenv("BBFFT_GB300_ND_SLAB_BYTES")) {
        budget = static_cast<std::size_t>(std::strtoull(e, nullptr, 10));
    }
    long long slab_k = 0;
    if (!has_cb && !strided_nd && budget > 0 && inter_per_k * Kimg > budget) {
        slab_k = std::max<long long>(1, static_cast<long long>(budget / inter_per_k));
        if (slab_k >= Kimg) {
            slab_k = 0;
        }
    }
    auto make_passes = [&](long long kk, std::vector<pass> &out) {
        for (pass_request q : order) {
            q.K = q.K / Kimg * kk; // the K mode of every pass is (outer modes) x Kimg
            out.push_back(make_1d_pass(q, plan.device, cache));
        }
    };
    make_passes(slab_k > 0 ? slab_k : Kimg, plan.passes);
    if (slab_k > 0) {
        plan.slab_k = slab_k;
        plan.slab_count = Kimg / slab_k;
        plan.slab_in_bytes = ist[dim + 1] * slab_k * (in_real ? real_b : cplx_b);
        plan.slab_out_bytes = ost[dim + 1] * slab_k * (out_real ? real_b : cplx_b);
        if (Kimg % slab_k != 0) {
            make_passes(Kimg % slab_k, plan.tail_passes);
        }
        // a separate temporary is reused by every slab (the next slab overwrites it while it
        // is still in L2, so it is never written back to HBM)
        isize = isize / static_cast<std::size_t>(Kimg) * static_cast<std::size_t>(slab_k);
        osize = osize / static_cast<std::size_t>(Kimg) * static_cast<std::size_t>(slab_k);
    }
    if (isize > osize) {
        plan.tmp = std::make_shared<device_buffer>(isize);
    }
    for (auto *pl : {&plan.passes, &plan.tail_passes}) {
        for (std::size_t i = 0; i < pl->size(); ++i) {
            (*pl)[i].in_sel = i == 0 ? (strided_nd ? 3 : 0) : 2;
            (*pl)[i].out_sel = i + 1 == pl->size() ? (strided_nd ? 4 : 1) : 2;
        }
    }
    if (strided_nd) {
        auto copy_pass = [&](bool gather) {
            pass cpass;
            cpass.copy = true;
            cpass.prec = cfg.precision;
            copy_params &c = cpass.cp;
            c.rank = static_cast<int>(dim) + 2;
            c.gather = gather ? 1 : 0;
            c.total = 1;
            bool side_real = gather ? in_real : out_real;
            bool half = gather ? cfg.type == BBFFT_C2R : cfg.type == BBFFT_R2C;
            for (unsigned d = 0; d < dim + 2; ++d) {
                long long e = static_cast<long long>(cfg.shape[d]);
                if (d == 1 && half) {
                    e = e / 2 + 1;
                }
                c.shape[d] = e;
                c.stride[d] = static_cast<long long>(gather ? cfg.istride[d] : cfg.ostride[d]);
                c.total *= e;
            }
            std::size_t eb = side_real ? real_b : cplx_b;
            cpass.func = strided_copy_kernel_ptr(static_cast<int>(eb));
            cpass.block = 256;
            long long blocks = (c.total + 255) / 256;
            cpass.grid = static_cast<unsigned>(std::min<long long>(blocks, 152LL * 16));
            cpass.in_sel = gather ? 0 : 4;
            cpass.out_sel = gather ? 3 : 1;
            cpass.identifier = gather ? "gbfft_strided_gather" : "gbfft_strided_scatter";
            (gather ? plan.packed_in : plan.packed_out) =
                std::make_shared<device_buffer>(static_cast<std::size_t>(c.total) * eb);
            return cpass;
        };
        plan.passes.insert(plan.passes.begin(), copy_pass(true));
        plan.passes.push_back(copy_pass(false));
    }
    plan.inplace_ok = true;
    for (auto *pl : {&plan.passes, &plan.tail_passes}) {
        for (auto const &ps : *pl) {
            plan.inplace_ok = plan.inplace_ok && ps.inplace_ok;
        }
    }
}

static void run_passes(bbfft_plan_s &plan, std::vector<pass> const &passes, const void *in,
                       void *out, cudaStream_t stream);

static void execute_impl(bbfft_plan_s &plan, const void *in, void *out, cudaStream_t stream) {
    if (in == out && !plan.inplace_ok) {
        bad_config("The plan does not support in-place transform on the current device. Please "
                   "use the out-of-place transform.");
    }
    int cur = -1;
    GB_CUDA(cudaGetDevice(&cur));
    // the caller's device is current again on every way out, errors included
    struct restore_device {
        int cur, dev;
        ~restore_device() {
            if (cur != dev) {
                cudaSetDevice(cur);
            }
        }
    } restore{cur, cur};
    if (cur != plan.device) {
        GB_CUDA(cudaSetDevice(plan.device));
        restore.dev = plan.device;
    }
    if (plan.slab_k > 0) {
        // L2-resident chaining: every pass over one slab of K, slab after slab; the
        // temporary aliases the slab's output unless the plan has its own (reused)
        char const *ib = static_cast<char const *>(in);
        char *ob = static_cast<char *>(out);
        for (long long sl = 0; sl < plan.slab_count; ++sl) {
            run_passes(plan, plan.passes, ib + sl * plan.slab_in_bytes, ob + sl * plan.slab_out_bytes,
                       stream);
        }
        if (!plan.tail_passes.empty()) {
            run_passes(plan, plan.tail_passes, ib + plan.slab_count * plan.slab_in_bytes,
                       ob + plan.slab_count * plan.slab_out_bytes, stream);
        }
        return;
    }
    run_passes(plan, plan.passes, in, out, stream);
}

static void run_passes(bbfft_plan_s &plan, std::vector<pass> const &passes, const void *in,
                       void *out, cudaStream_t stream) {
    void *packed_in = plan.packed_in ? plan.packed_in->ptr : nullptr;
    void *packed_out = plan.packed_out ? plan.packed_out->ptr : nullptr;
    void *tmp = plan.tmp ? plan.tmp->ptr : (packed_out ? packed_out : out);
    auto select = [&](int sel) -> void * {
        switch (sel) {
        case 0:
            return const_cast<void *>(in);
        case 1:
            return out;
        case 3:
            return packed_in;
        case 4:
            return packed_out;
        default:
            return tmp;
        }
    };
    for (auto &pass0 : passes) {
        const void *pin = select(pass0.in_sel);
        void *pout = select(pass0.out_sel);
        if (pass0.copy) {
            copy_params cp = pass0.cp;
            cp.src = pin;
            cp.dst = pout;
            void *cargs[] = {&cp};
            cudaError_t e = cudaLaunchKernel(pass0.func, dim3(pass0.grid), dim3(pass0.block), cargs, 0, stream);
            if (e != cudaSuccess) {
                throw status_error(BBFFT_CUDA_ERROR,
                                   std::string("kernel launch failed: ") + cudaGetErrorString(e));
            }
            continue;
        }
        bool misaligned = ((reinterpret_cast<std::uintptr_t>(pin) |
                            reinterpret_cast<std::uintptr_t>(pout)) % 16) != 0;
        if (pass0.tc && misaligned) {
            throw status_error(BBFFT_INVALID_ARGUMENT,
                               "tensor-core plans need 16-byte aligned tensors");
        }
        pass const &ps = (pass0.V > 1 && misaligned) ? *pass0.scalar_alt : pass0;
        fft_params p = ps.p;
        p.in = pin;
        p.out = pout;
        // paired real accesses need pointers aligned to one complex element
        std::uintptr_t const align = 2 * static_cast<std::uintptr_t>(ps.prec);
        if (reinterpret_cast<std::uintptr_t>(p.in) % align) {
            p.flags &= ~flag_vec_in;
        }
        if (reinterpret_cast<std::uintptr_t>(p.out) % align) {
            p.flags &= ~flag_vec_out;
        }
        void *args[] = {&p};
        cudaError_t e = cudaLaunchKernel(ps.func, dim3(ps.grid), dim3(ps.block), args, ps.smem, stream);
        if (e != cudaSuccess) {
            throw status_error(BBFFT_CUDA_ERROR,
                               std::string("kernel launch failed: ") + cudaGetErrorString(e));
        }
    }
}

} // namespace gbfft

// ------------------------------------------------------------------------------------------
// ragged batches

struct bbfft_ragged_s {
    int device = 0;
    int prec = 4;
    std::vector<gbfft::pass> passes; // keep the twiddle tables alive
    std::unique_ptr<gbfft::device_buffer> items, units, counter;
    int n_units = 0;
    unsigned grid = 0, block = 256;
    std::size_t smem = 0;
    const void *func = nullptr;      // persistent kernel
    const void *grid_func = nullptr; // one CTA per unit
    int form = BBFFT_RAGGED_PERSISTENT;
    // class form: one kernel per class of units (same tile function); as a graph, the
    // kernels form four chains of nodes
    struct unit_class {
        const void *func;
        int offset, count; // units class_units[offset, offset + count)
        unsigned block;
        std::size_t smem;
    };
    std::vector<unit_class> classes;
    std::unique_ptr<gbfft::device_buffer> class_units;
    uint64_t bytes = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~bbfft_ragged_s() {
        if (exec) {
            cudaGraphExecDestroy(exec);
        }
        if (graph) {
            cudaGraphDestroy(graph);
        }
    }
};

namespace gbfft {

static void make_ragged(bbfft_ragged_item const *items, std::size_t n, bbfft_ragged_s &r) {
    if (!items || n == 0) {
        throw status_error(BBFFT_INVALID_ARGUMENT, "empty ragged batch");
    }
    r.prec = items[0].precision;
    for (std::size_t i = 0; i < n; ++i) {
        auto const &it = items[i];
        if (it.precision != r.prec) {
            bad_config("all transforms of a ragged batch share one precision");
        }
        if (it.N == 0 || it.M == 0 || it.K == 0) {
            bad_config("ragged item with an empty shape");
        }
        if (!it.in || !it.out) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "ragged item without tensor pointers");
        }
        bbfft_configuration c = {};
        c.dim = 1;
        c.shape[0] = it.M;
        c.shape[1] = it.N;
        c.shape[2] = it.K;
        c.precision = it.precision;
        c.type = it.type;
        c.direction = it.direction;
        c.istride[0] = c.ostride[0] = 1;
        validate(c);
    }
    GB_CUDA(cudaGetDevice(&r.device));
    std::vector<ragged_item_dev> dev(n);
    std::vector<std::pair<double, std::pair<int, int>>> units;
    int const block = 256;
    std::size_t smem = 0;
    for (std::size_t i = 0; i < n; ++i) {
        auto const &it = items[i];
        long long N = it.N;
        long long nin = it.type == BBFFT_C2R ? N / 2 + 1 : N;
        long long nout = it.type == BBFFT_R2C ? N / 2 + 1 : N;
        pass_request q{};
        q.prec = it.precision;
        q.type = it.type;
        q.dir = it.direction;
        q.M = static_cast<long long>(it.M);
        q.N = N;
        q.K = static_cast<long long>(it.K);
        q.is1 = q.M;
        q.is2 = q.M * nin;
        q.os1 = q.M;
        q.os2 = q.M * nout;
        q.runtime_only = true;
        q.max_block = block;
        // tiles vectorised over M need 16-byte aligned tensors
        q.force_v1 = ((reinterpret_cast<std::uintptr_t>(it.in) | reinterpret_cast<std::uintptr_t>(it.out)) % 16) != 0;
        r.passes.push_back(make_1d_pass(q, r.device, nullptr));
        pass const &ps = r.passes.back();
        dev[i].p = ps.p;
        dev[i].p.in = it.in;
        dev[i].p.out = it.out;
        dev[i].kind = ps.kind;
        dev[i].vid = ps.ragged_vid;
        smem = std::max(smem, ps.smem);
        std::size_t ib = it.type == BBFFT_R2C ? it.precision : 2 * it.precision;
        std::size_t ob = it.type == BBFFT_C2R ? it.precision : 2 * it.precision;
        r.bytes += (nin * ib + nout * ob) * it.M * it.K;
        // cost of one tile ~ elements x (sum of radices): largest first (LPT order)
        double work = 0;
        for (int s2 = 0; s2 < ps.p.L; ++s2) {
            work += ps.p.radix[s2];
        }
        double cost = static_cast<double>(ps.p.Mb) * ps.p.Kb * N * (work + 4);
        for (unsigned t = 0; t < ps.grid; ++t) {
            units.push_back({cost, {static_cast<int>(i), static_cast<int>(t)}});
        }
    }
    // order: classes of units with the same tile function together (the CTAs running at the
    // same time then execute the same code, which keeps the instruction cache warm), the
    // class with the most work first, largest tiles first inside a class
    {
        auto key_of = [&](int i) { return dev[i].vid >= 0 ? dev[i].vid : -1 - (r.prec * 8 + dev[i].kind); };
        std::map<int, double> class_cost;
        for (auto const &u : units) {
            class_cost[key_of(u.second.first)] += u.first;
        }
        std::stable_sort(units.begin(), units.end(), [&](auto const &a, auto const &b) {
            int ka = key_of(a.second.first), kb = key_of(b.second.first);
            if (ka != kb) {
                double ca = class_cost[ka], cb = class_cost[kb];
                return ca != cb ? ca > cb : ka < kb;
            }
            return a.first > b.first;
        });
    }
    // class form: units grouped by tile function, LPT order kept inside a class
    {
        std::map<int, std::vector<int>> by_class; // key: vid, or -1 - (prec * 8 + kind)
        for (std::size_t u = 0; u < units.size(); ++u) {
            int i = units[u].second.first;
            int key = dev[i].vid >= 0 ? dev[i].vid : -1 - (r.prec * 8 + dev[i].kind);
            by_class[key].push_back(static_cast<int>(u));
        }
        std::vector<int> cflat;
        for (auto const &kv : by_class) {
            bbfft_ragged_s::unit_class c{};
            c.func = kv.first >= 0 ? ragged_class_kernel(kv.first)
                                   : ragged_class_runtime_kernel(r.prec, dev[units[kv.second[0]].second.first].kind);
            if (!c.func) {
                throw status_error(BBFFT_INTERNAL_ERROR, "ragged class kernel not found");
            }
            c.offset = static_cast<int>(cflat.size() / 2);
            c.count = static_cast<int>(kv.second.size());
            c.block = 32;
            c.smem = 0;
            for (int u : kv.second) {
                int i = units[u].second.first;
                pass const &ps = r.passes[i];
                c.block = std::max(c.block, (ps.block + 31) / 32 * 32);
                c.smem = std::max(c.smem, ps.smem);
                cflat.push_back(units[u].second.first);
                cflat.push_back(units[u].second.second);
            }
            if (needs_smem_optin(c.smem)) {
                allow_max_smem(c.func, r.device);
            }
            r.classes.push_back(c);
        }
        r.class_units = std::make_unique<device_buffer>(cflat.size() * sizeof(int));
        GB_CUDA(cudaMemcpy(r.class_units->ptr, cflat.data(), cflat.size() * sizeof(int),
                           cudaMemcpyHostToDevice));
    }
    std::vector<int> flat(2 * units.size());
    for (std::size_t u = 0; u < units.size(); ++u) {
        flat[2 * u] = units[u].second.first;
        flat[2 * u + 1] = units[u].second.second;
    }
    r.n_units = static_cast<int>(units.size());
    r.items = std::make_unique<device_buffer>(dev.size() * sizeof(ragged_item_dev));
    r.units = std::make_unique<device_buffer>(flat.size() * sizeof(int));
    r.counter = std::make_unique<device_buffer>(sizeof(unsigned));
    GB_CUDA(cudaMemcpy(r.items->ptr, dev.data(), dev.size() * sizeof(ragged_item_dev),
                       cudaMemcpyHostToDevice));
    GB_CUDA(cudaMemcpy(r.units->ptr, flat.data(), flat.size() * sizeof(int),
                       cudaMemcpyHostToDevice));
    r.func = ragged_kernel_ptr(r.prec, true);
    r.grid_func = ragged_kernel_ptr(r.prec, false);
    r.block = block;
    r.smem = smem;
    if (needs_smem_optin(smem)) {
        allow_max_smem(r.func, r.device);
        allow_max_smem(r.grid_func, r.device);
    }
    int per_sm = 0, sms = 0;
    GB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, r.func, block, smem));
    GB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, r.device));
    if (per_sm < 1) {
        cudaFuncAttributes fa;
        GB_CUDA(cudaFuncGetAttributes(&fa, r.func));
        bad_config("ragged batch: a unit does not fit on a multiprocessor (block " +
                   std::to_string(block) + ", dynamic shared " + std::to_string(smem) +
                   " B, static " + std::to_string(fa.sharedSizeBytes) + " B, max dynamic " +
                   std::to_string(fa.maxDynamicSharedSizeBytes) + " B, registers " +
                   std::to_string(fa.numRegs) + ")");
    }
    r.grid = static_cast<unsigned>(std::min<long long>(static_cast<long long>(per_sm) * sms,
                                                       std::max(1, r.n_units)));
}

static void launch_ragged(bbfft_ragged_s &r, cudaStream_t stream) {
    const void *items = r.items->ptr;
    const void *units = r.units->ptr;
    int n = r.n_units;
    void *counter = r.counter->ptr;
    void *args[] = {&items, &units, &n, &counter};
    if (r.form == BBFFT_RAGGED_GRID) {
        GB_CUDA(cudaLaunchKernel(r.grid_func, dim3(static_cast<unsigned>(std::max(1, n))),
                                 dim3(r.block), args, r.smem, stream));
        return;
    }
    if (r.form == BBFFT_RAGGED_CLASSES) {
        for (auto const &c : r.classes) {
            const void *cu = static_cast<const int2 *>(r.class_units->ptr) + c.offset;
            void *cargs[] = {&items, &cu};
            cudaError_t e = cudaLaunchKernel(c.func, dim3(static_cast<unsigned>(c.count)),
                                             dim3(c.block), cargs, c.smem, stream);
            if (e != cudaSuccess) {
                (void)cudaGetLastError();
                cudaFuncAttributes fa = {};
                cudaFuncGetAttributes(&fa, c.func);
                throw status_error(BBFFT_CUDA_ERROR,
                                   std::string("ragged class launch failed: ") + cudaGetErrorString(e) +
                                       " (block " + std::to_string(c.block) + ", dynamic shared " +
                                       std::to_string(c.smem) + " B, max dynamic " +
                                       std::to_string(fa.maxDynamicSharedSizeBytes) + " B, max threads " +
                                       std::to_string(fa.maxThreadsPerBlock) + ", registers " +
                                       std::to_string(fa.numRegs) + ")");
            }
        }
        return;
    }
    GB_CUDA(cudaMemsetAsync(r.counter->ptr, 0, sizeof(unsigned), stream));
    GB_CUDA(cudaLaunchKernel(r.func, dim3(r.grid), dim3(r.block), args, r.smem, stream));
}

} // namespace gbfft

// ------------------------------------------------------------------------------------------
// C ABI

using gbfft::guarded;
using gbfft::status_error;

extern "C" {

const char *bbfft_last_error(void) {
    return gbfft::tl_fixed_active ? gbfft::tl_fixed_error : gbfft::tl_error.c_str();
}
const char *bbfft_version(void) { return "bbfft-gb300 0.1.0 (sm_103a)"; }

// Internal (no header): the prime P of a length whose radix-P stage the compile-time tiles
// run in registers, or 0 — for the check that the host and the kernel generator agree.
BBFFT_GB300_API int gbfft_internal_reg_prime(int nc) { return gbfft::reg_prime_length(nc); }

int bbfft_default_istride(uint32_t dim, const size_t shape[BBFFT_MAX_TENSOR_DIM], int32_t type,
                          int inplace, size_t stride_out[BBFFT_MAX_TENSOR_DIM]) {
    return guarded([&] {
        if (!shape || !stride_out) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null pointer");
        }
        gbfft::from_array(gbfft::default_istride(dim, gbfft::to_array(shape), type, inplace != 0),
                          stride_out);
    });
}

int bbfft_default_ostride(uint32_t dim, const size_t shape[BBFFT_MAX_TENSOR_DIM], int32_t type,
                          int inplace, size_t stride_out[BBFFT_MAX_TENSOR_DIM]) {
    return guarded([&] {
        if (!shape || !stride_out) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null pointer");
        }
        gbfft::from_array(gbfft::default_ostride(dim, gbfft::to_array(shape), type, inplace != 0),
                          stride_out);
    });
}

static void copy_string(std::string const &s, char *buf, size_t buf_len, size_t *needed) {
    if (needed) {
        *needed = s.size() + 1;
    }
    if (buf && buf_len) {
        size_t n = std::min(buf_len - 1, s.size());
        std::memcpy(buf, s.data(), n);
        buf[n] = '\0';
    }
}

int bbfft_configuration_to_string(const bbfft_configuration *cfg, char *buf, size_t buf_len,
                                  size_t *needed) {
    return guarded([&] {
        if (!cfg) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null configuration");
        }
        copy_string(gbfft::to_descriptor(*cfg), buf, buf_len, needed);
    });
}

int bbfft_parse_fft_descriptor(const char *desc, bbfft_configuration *cfg) {
    return guarded([&] {
        if (!desc || !cfg) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null pointer");
        }
        *cfg = gbfft::parse_descriptor(desc);
    });
}

int bbfft_jit_cache_create(bbfft_cache_t *cache) {
    return guarded([&] {
        if (!cache) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null pointer");
        }
        *cache = new bbfft_cache_s();
    });
}

int bbfft_aot_cache_create(bbfft_cache_t *cache) {
    return guarded([&] {
        if (!cache) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null pointer");
        }
        auto c = new bbfft_cache_s();
        c->aot = true;
        *cache = c;
    });
}

int bbfft_aot_cache_register_module(bbfft_cache_t cache, const void *image, size_t image_size,
                                    const char *const *kernel_names, size_t num_kernel_names,
                                    int device) {
    return guarded([&] {
        if (!cache || !cache->aot || !image || image_size == 0) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "invalid aot module registration");
        }
        int cur = 0;
        GB_CUDA(cudaGetDevice(&cur));
        if (cur != device) {
            GB_CUDA(cudaSetDevice(device));
        }
        auto m = std::make_shared<gbfft::module>();
        cudaError_t e =
            cudaLibraryLoadData(&m->lib, image, nullptr, nullptr, 0, nullptr, nullptr, 0);
        if (cur != device) {
            cudaSetDevice(cur);
        }
        if (e != cudaSuccess) {
            throw status_error(BBFFT_CUDA_ERROR,
                               std::string("cudaLibraryLoadData failed: ") + cudaGetErrorString(e));
        }
        bbfft_cache_s::aot_module am;
        am.mod = m;
        am.device = device;
        for (size_t i = 0; i < num_kernel_names; ++i) {
            am.names.insert(kernel_names[i]);
        }
        std::lock_guard<std::mutex> lock(cache->mu);
        cache->aot_modules.push_back(std::move(am));
    });
}

int bbfft_aot_generate(const bbfft_configuration *cfgs, size_t num_cfgs, void *image,
                       size_t image_len, size_t *image_needed, char *names, size_t names_len,
                       size_t *names_needed) {
    return guarded([&] {
        if (!cfgs || num_cfgs == 0) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "no configurations");
        }
        const bbfft_configuration &c0 = cfgs[0];
        std::vector<std::tuple<std::string, int, int, int>> kernels;
        std::set<std::string> seen;
        for (size_t i = 0; i < num_cfgs; ++i) {
            const bbfft_configuration &c = cfgs[i];
            gbfft::validate(c);
            bool has_cb = (c.load_function && *c.load_function) ||
                          (c.store_function && *c.store_function);
            if (!has_cb) {
                throw status_error(BBFFT_BAD_CONFIGURATION,
                                   "only configurations with callbacks need generated "
                                   "kernels; the others are built into the library");
            }
            if (c.callback_length != c0.callback_length ||
                std::memcmp(c.callback_source, c0.callback_source, c.callback_length) != 0 ||
                std::strcmp(c.load_function ? c.load_function : "",
                            c0.load_function ? c0.load_function : "") != 0 ||
                std::strcmp(c.store_function ? c.store_function : "",
                            c0.store_function ? c0.store_function : "") != 0) {
                throw status_error(BBFFT_BAD_CONFIGURATION,
                                   "all configurations of one image must share the user module");
            }
            bool even = c.shape[1] % 2 == 0;
            int kind = c.type == BBFFT_C2C ? gbfft::kind_c2c
                       : c.type == BBFFT_R2C
                           ? (even ? gbfft::kind_r2c_half : gbfft::kind_r2c_full)
                           : (even ? gbfft::kind_c2r_half : gbfft::kind_c2r_full);
            auto add = [&](int k, const char *load_fn, const char *store_fn) {
                if (gbfft::callback_io(load_fn, store_fn) == 0) {
                    return;
                }
                std::string name = gbfft::callback_kernel_name(
                    c.precision, k, c.callback_source, c.callback_length, load_fn, store_fn);
                if (seen.insert(name).second) {
                    kernels.emplace_back(name, c.precision, k,
                                         gbfft::callback_io(load_fn, store_fn));
                }
            };
            if (c.dim == 1) {
                add(kind, c.load_function, c.store_function);
            } else {
                // the passes of an nd plan that call user functions: the first (load) and
                // the last (store); c2r runs the outer modes first and its real pass last.
                // An nd plan always has dim >= 2 passes (make_plan_impl keeps modes of
                // size 1), so no pass calls both functions.
                bool c2r = c.type == BBFFT_C2R;
                add(c2r ? gbfft::kind_c2c : kind, c.load_function, nullptr);
                add(c2r ? kind : gbfft::kind_c2c, nullptr, c.store_function);
            }
        }
        // the current device's architecture, or BBFFT_GB300_AOT_ARCH when it is set (also
        // the only way without a GPU)
        int device = -1;
        const char *arch = std::getenv("BBFFT_GB300_AOT_ARCH");
        if (!(arch && *arch)) {
            GB_CUDA(cudaGetDevice(&device));
        }
        std::string src = gbfft::callback_program(c0.callback_source, c0.callback_length,
                                                  c0.load_function, c0.store_function, kernels);
        std::vector<char> cubin = gbfft::nvrtc_compile(src, "gbfft_aot", device);
        if (image_needed) {
            *image_needed = cubin.size();
        }
        if (image && image_len >= cubin.size()) {
            std::memcpy(image, cubin.data(), cubin.size());
        } else if (image) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "image buffer too small");
        }
        std::string all;
        for (auto const &k : kernels) {
            all += std::get<0>(k) + "\n";
        }
        copy_string(all, names, names_len, names_needed);
    });
}

int bbfft_cache_destroy(bbfft_cache_t cache) {
    return guarded([&] { delete cache; });
}

int bbfft_cache_kernel_names(bbfft_cache_t cache, char *buf, size_t buf_len, size_t *needed) {
    return guarded([&] {
        if (!cache) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null cache");
        }
        std::string s;
        std::lock_guard<std::mutex> lock(cache->mu);
        std::vector<std::string> names;
        if (cache->aot) {
            for (auto const &m : cache->aot_modules) {
                names.insert(names.end(), m.names.begin(), m.names.end());
            }
        } else {
            for (auto const &kv : cache->jit) {
                names.push_back(kv.first.substr(0, kv.first.rfind('@')));
            }
        }
        std::sort(names.begin(), names.end());
        for (auto const &n : names) {
            s += n + "\n";
        }
        copy_string(s, buf, buf_len, needed);
    });
}

int bbfft_cache_stats(bbfft_cache_t cache, uint64_t *hits, uint64_t *misses) {
    return guarded([&] {
        if (!cache) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null cache");
        }
        if (hits) {
            *hits = cache->hits.load();
        }
        if (misses) {
            *misses = cache->misses.load();
        }
    });
}

static int create_common(const bbfft_configuration *cfg, cudaStream_t stream, bbfft_cache_t cache,
                         bool adjoint, bbfft_plan_t *plan, gbfft::pass_request const *tuning) {
    return guarded([&] {
        if (!cfg || !plan) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null pointer");
        }
        *plan = nullptr;
        std::unique_ptr<bbfft_plan_s> p(new bbfft_plan_s());
        gbfft::make_plan_impl(*cfg, stream, cache, adjoint, *p, tuning);
        *plan = p.release();
    });
}

int bbfft_plan_create(const bbfft_configuration *cfg, cudaStream_t stream, bbfft_cache_t cache,
                      bbfft_plan_t *plan) {
    return create_common(cfg, stream, cache, false, plan, nullptr);
}

int bbfft_plan_create_adjoint(const bbfft_configuration *cfg, cudaStream_t stream,
                              bbfft_cache_t cache, bbfft_plan_t *plan) {
    return create_common(cfg, stream, cache, true, plan, nullptr);
}

int bbfft_plan_create_tuned(const bbfft_configuration *cfg, cudaStream_t stream,
                            const uint32_t *radices, uint32_t num_radices,
                            uint32_t threads_per_transform, uint32_t vector_width, uint32_t mb,
                            uint32_t kb, uint32_t min_blocks, bbfft_plan_t *plan) {
    gbfft::pass_request t{};
    if (radices) {
        for (uint32_t i = 0; i < num_radices && radices[i] != 0; ++i) {
            t.radices.push_back(static_cast<int>(radices[i]));
        }
    }
    t.T = static_cast<int>(threads_per_transform);
    t.V = static_cast<int>(vector_width);
    t.force_v1 = vector_width == 1;
    t.Mb = static_cast<int>(mb);
    t.Kb = static_cast<int>(kb);
    t.occ = static_cast<int>(min_blocks);
    if (cfg && cfg->dim != 1) {
        gbfft::tl_error = "tuned plans are 1d only";
        return BBFFT_BAD_CONFIGURATION;
    }
    return create_common(cfg, stream, nullptr, false, plan, &t);
}

int bbfft_plan_execute(bbfft_plan_t plan, const void *in, void *out, uint32_t num_wait_events,
                       const cudaEvent_t *wait_events, cudaEvent_t signal_event) {
    return guarded([&] {
        if (!plan) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null plan");
        }
        if (num_wait_events && !wait_events) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "num_wait_events > 0 but no events");
        }
        for (uint32_t i = 0; i < num_wait_events; ++i) {
            GB_CUDA(cudaStreamWaitEvent(plan->stream, wait_events[i], 0));
        }
        gbfft::execute_impl(*plan, in, out, plan->stream);
        if (signal_event) {
            GB_CUDA(cudaEventRecord(signal_event, plan->stream));
        }
    });
}

int bbfft_plan_execute_on(bbfft_plan_t plan, const void *in, void *out, cudaStream_t stream) {
    return guarded([&] {
        if (!plan) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null plan");
        }
        gbfft::execute_impl(*plan, in, out, stream);
    });
}

int bbfft_plan_retain(bbfft_plan_t plan) {
    return guarded([&] {
        if (!plan) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null plan");
        }
        plan->refs++;
    });
}

int bbfft_plan_destroy(bbfft_plan_t plan) {
    return guarded([&] {
        if (plan && --plan->refs == 0) {
            delete plan;
        }
    });
}

int bbfft_ragged_create(const bbfft_ragged_item *items, size_t num_items, bbfft_ragged_t *ragged) {
    return guarded([&] {
        if (!ragged) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null pointer");
        }
        *ragged = nullptr;
        std::unique_ptr<bbfft_ragged_s> r(new bbfft_ragged_s());
        gbfft::make_ragged(items, num_items, *r);
        *ragged = r.release();
    });
}

int bbfft_ragged_execute(bbfft_ragged_t ragged, cudaStream_t stream, int use_graph) {
    return guarded([&] {
        if (!ragged) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null ragged batch");
        }
        if (!use_graph) {
            gbfft::launch_ragged(*ragged, stream);
            return;
        }
        if (!ragged->exec && ragged->form == BBFFT_RAGGED_CLASSES) {
            // one kernel node per class in kChains chains (largest classes first, dealt
            // round robin): the chains run concurrently, the kernels of a chain back to back
            // (hundreds of independent nodes measured slower than a few chains);
            // BBFFT_GB300_RAGGED_CHAINS overrides the number of chains
            std::size_t kChains = 4;
            if (const char *e = std::getenv("BBFFT_GB300_RAGGED_CHAINS")) {
                kChains = std::max<std::size_t>(1, std::strtoul(e, nullptr, 10));
            }
            GB_CUDA(cudaGraphCreate(&ragged->graph, 0));
            const void *items = ragged->items->ptr;
            std::vector<std::size_t> order(ragged->classes.size());
            for (std::size_t c = 0; c < order.size(); ++c) {
                order[c] = c;
            }
            std::stable_sort(order.begin(), order.end(), [&](std::size_t a, std::size_t b) {
                return ragged->classes[a].count > ragged->classes[b].count;
            });
            std::vector<const void *> cus(ragged->classes.size());
            std::vector<cudaGraphNode_t> nodes(order.size());
            for (std::size_t n = 0; n < order.size(); ++n) {
                std::size_t c = order[n];
                auto const &uc = ragged->classes[c];
                cus[c] = static_cast<const int2 *>(ragged->class_units->ptr) + uc.offset;
                void *cargs[] = {&items, &cus[c]};
                cudaKernelNodeParams kp = {};
                kp.func = const_cast<void *>(uc.func);
                kp.gridDim = dim3(static_cast<unsigned>(uc.count));
                kp.blockDim = dim3(uc.block);
                kp.sharedMemBytes = static_cast<unsigned>(uc.smem);
                kp.kernelParams = cargs;
                cudaGraphNode_t const *dep = n >= kChains ? &nodes[n - kChains] : nullptr;
                GB_CUDA(cudaGraphAddKernelNode(&nodes[n], ragged->graph, dep, dep ? 1 : 0, &kp));
            }
            GB_CUDA(cudaGraphInstantiate(&ragged->exec, ragged->graph, 0));
        }
        if (!ragged->exec) {
            cudaStream_t cs;
            GB_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
            cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                try {
                    gbfft::launch_ragged(*ragged, cs);
                } catch (...) {
                    cudaGraph_t g = nullptr;
                    cudaStreamEndCapture(cs, &g);
                    if (g) {
                        cudaGraphDestroy(g);
                    }
                    cudaStreamDestroy(cs);
                    throw;
                }
                e = cudaStreamEndCapture(cs, &ragged->graph);
            }
            cudaStreamDestroy(cs);
            if (e != cudaSuccess) {
                throw status_error(BBFFT_CUDA_ERROR,
                                   std::string("graph capture failed: ") + cudaGetErrorString(e));
            }
            GB_CUDA(cudaGraphInstantiate(&ragged->exec, ragged->graph, 0));
        }
        GB_CUDA(cudaGraphLaunch(ragged->exec, stream));
    });
}

int bbfft_ragged_set_launch_form(bbfft_ragged_t ragged, int form) {
    return guarded([&] {
        if (!ragged || (form != BBFFT_RAGGED_PERSISTENT && form != BBFFT_RAGGED_GRID &&
                        form != BBFFT_RAGGED_CLASSES)) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null ragged batch or unknown launch form");
        }
        if (form != ragged->form) {
            ragged->form = form;
            if (ragged->exec) { // the captured graph holds the other form
                cudaGraphExecDestroy(ragged->exec);
                ragged->exec = nullptr;
            }
            if (ragged->graph) {
                cudaGraphDestroy(ragged->graph);
                ragged->graph = nullptr;
            }
        }
    });
}

int bbfft_ragged_get_info(bbfft_ragged_t ragged, bbfft_ragged_info *info) {
    return guarded([&] {
        if (!ragged || !info) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null pointer");
        }
        info->num_units = static_cast<uint64_t>(ragged->n_units);
        info->grid = ragged->grid;
        info->block = ragged->block;
        info->shared_bytes = ragged->smem;
        info->bytes_moved = ragged->bytes;
    });
}

int bbfft_ragged_destroy(bbfft_ragged_t ragged) {
    return guarded([&] { delete ragged; });
}

int bbfft_plan_get_info(bbfft_plan_t plan, bbfft_plan_info *info) {
    return guarded([&] {
        if (!plan || !info) {
            throw status_error(BBFFT_INVALID_ARGUMENT, "null pointer");
        }
        std::memset(info, 0, sizeof(*info));
        auto const *first = &plan->passes.front();
        for (auto const &q : plan->passes) {
            if (!q.copy) { // the first transform pass (after a strided gather)
                first = &q;
                break;
            }
        }
        auto const &ps = *first;
        std::strncpy(info->identifier, ps.identifier.c_str(), sizeof(info->identifier) - 1);
        info->num_launches = static_cast<uint32_t>(
            plan->slab_k > 0 ? plan->passes.size() * plan->slab_count + plan->tail_passes.size()
                             : plan->passes.size());
        info->inplace_supported = plan->inplace_ok;
        info->jit_compiled = plan->jit;
        info->num_stages = static_cast<uint32_t>(ps.p.L);
        for (int s = 0; s < ps.p.L && s < 12; ++s) {
            info->radix[s] = static_cast<uint32_t>(ps.p.radix[s]);
        }
        info->threads_per_transform = static_cast<uint32_t>(ps.p.T);
        info->mb = static_cast<uint32_t>(ps.p.Mb);
        info->kb = static_cast<uint32_t>(ps.p.Kb);
        info->block_threads = ps.block;
        info->shared_bytes = ps.smem;
        info->workspace_bytes = (plan->tmp ? plan->tmp->bytes : 0) +
                                (plan->packed_in ? plan->packed_in->bytes : 0) +
                                (plan->packed_out ? plan->packed_out->bytes : 0);
        info->vector_width = static_cast<uint32_t>(ps.V);
        info->specialized = ps.specialized ? 1u : 0u;
        info->min_blocks = static_cast<uint32_t>(ps.min_blocks);
    });
}

} // extern "C"
