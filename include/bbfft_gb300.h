/*
 * bbfft_gb300.h - C ABI of the GB300 (sm_103a) double-batched FFT library.
 *
 * This is the drop-in boundary for the hot path of Intel's double-batched FFT
 * library (bbfft 0.5.1): many small FFTs over an M x N1..Nd x K tensor.  Every
 * entry point names the reference interface it replaces.  The C++ API of the
 * reference (bbfft::configuration, bbfft::make_plan, bbfft::plan<E>::execute, the
 * jit/aot caches) is provided header-only on top of this ABI in include/bbfft/.
 *
 * Conventions
 *  - Functions return BBFFT_SUCCESS (0) or a negative status; the message of the last
 *    failure on the calling thread is returned by bbfft_last_error().
 *  - Pointers to tensors are device pointers (cudaMalloc'd or managed).  Offsets and
 *    strides are counted in elements: real elements for real tensors, complex
 *    elements for complex tensors (reference include/bbfft/configuration.hpp:162-179).
 *  - Streams and events are the CUDA runtime's cudaStream_t / cudaEvent_t; a null
 *    stream is the legacy default stream.
 *  - No entry point synchronises the device unless stated.
 */
#ifndef BBFFT_GB300_H
#define BBFFT_GB300_H

#include <stddef.h>
#include <stdint.h>

#include <cuda_runtime_api.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define BBFFT_GB300_API __declspec(dllexport)
#else
#define BBFFT_GB300_API __attribute__((visibility("default")))
#endif

/* ---- status codes (reference: exceptions bad_configuration / cl::error / ze::error /
 *      std::runtime_error, include/bbfft/bad_configuration.hpp:17-40) ---- */
typedef enum bbfft_status {
    BBFFT_SUCCESS = 0,
    BBFFT_BAD_CONFIGURATION = -1, /* bbfft::bad_configuration */
    BBFFT_INVALID_ARGUMENT = -2,  /* null pointers, bad sizes */
    BBFFT_CUDA_ERROR = -3,        /* a CUDA runtime call failed */
    BBFFT_COMPILE_ERROR = -4,     /* NVRTC could not compile user callbacks */
    BBFFT_PARSE_ERROR = -5,       /* malformed descriptor (std::runtime_error in the reference) */
    BBFFT_OUT_OF_MEMORY = -6,
    BBFFT_INTERNAL_ERROR = -7,
    BBFFT_DEVICE_ERROR = -8 /* a kernel reported an error status (e.g. a bounded wait ran out) */
} bbfft_status;

#define BBFFT_MAX_FFT_DIM 3
#define BBFFT_MAX_TENSOR_DIM 5

/* reference: enum class precision (configuration.hpp:22-25): value = bytes per real */
#define BBFFT_PRECISION_F32 4
#define BBFFT_PRECISION_F64 8
/* reference: enum class direction (configuration.hpp:67-70) */
#define BBFFT_FORWARD (-1)
#define BBFFT_BACKWARD 1
/* reference: enum class transform_type (configuration.hpp:79-83) */
#define BBFFT_C2C 0
#define BBFFT_R2C 1
#define BBFFT_C2R 2

/* Arithmetic used by the DFT stages (no counterpart in the reference, which computes in
 * the plan precision only).  F32 plans only; F64 plans always use BBFFT_COMPUTE_NATIVE. */
#define BBFFT_COMPUTE_NATIVE 0     /* plain FP32 / FP64 on CUDA cores */
#define BBFFT_COMPUTE_BF16 1       /* tensor-core radix-16 stages, BF16 operands, FP32 accumulate */
#define BBFFT_COMPUTE_SPLIT_BF16 2 /* operands split in 3 BF16 pieces, 6 product terms (~FP32) */
#define BBFFT_COMPUTE_SPLIT_BF16_3TERM 3 /* operands split in 2 BF16 pieces, 3 product terms */
#define BBFFT_COMPUTE_SPLIT_TF32 4 /* radix-16 / 32 stages as TF32 products of the pair sums and
                                    * differences, operands in 2 TF32 pieces, 3 product terms
                                    * (~FP32) */
/* The tensor-core modes apply to 1d c2c float plans with N in {64, 256, 512}, M = 1 and the
 * packed layout; other configurations reject them with BBFFT_BAD_CONFIGURATION. */

/*
 * FFT configuration; mirrors bbfft::configuration (reference
 * include/bbfft/configuration.hpp:151-192) and bbfft::user_module
 * (include/bbfft/user_module.hpp:24-37).  Callbacks are CUDA C++ source defining
 *   T load(const T* in, size_t offset)          -- T = float2/double2 or float/double
 *   void store(T* out, size_t offset, T value)
 * compiled for sm_103a with NVRTC at plan creation (the reference compiles OpenCL-C).
 * offset counts elements of the input (load) or output (store) tensor.  For dim > 1 (the
 * reference rejects callbacks there, src/common/algorithm/nd_fft.hpp:29-31) the tensors
 * need one of the default layouts: load is called for every element read from the input
 * tensor, store for every element written to the output tensor.
 */
typedef struct bbfft_configuration {
    uint32_t dim;                             /* 1..3 */
    size_t shape[BBFFT_MAX_TENSOR_DIM];       /* {M, N1, .., Nd, K} */
    int32_t precision;                        /* BBFFT_PRECISION_F32 / _F64 */
    int32_t direction;                        /* BBFFT_FORWARD / BBFFT_BACKWARD */
    int32_t type;                             /* BBFFT_C2C / _R2C / _C2R */
    size_t istride[BBFFT_MAX_TENSOR_DIM];     /* s0..s_{d+1}; s0 must be 1 */
    size_t ostride[BBFFT_MAX_TENSOR_DIM];
    const char *callback_source;              /* user_module::data (may be NULL) */
    size_t callback_length;                   /* user_module::length */
    const char *load_function;                /* user_module::load_function (may be NULL) */
    const char *store_function;               /* user_module::store_function (may be NULL) */
    int32_t compute;                          /* BBFFT_COMPUTE_*; 0 for the reference behaviour */
} bbfft_configuration;

typedef struct bbfft_plan_s *bbfft_plan_t;
typedef struct bbfft_cache_s *bbfft_cache_t;

/* ---- configuration helpers ---- */

/* reference: default_istride (src/base/configuration.cpp:24-43) */
BBFFT_GB300_API int bbfft_default_istride(uint32_t dim, const size_t shape[BBFFT_MAX_TENSOR_DIM],
                                          int32_t type, int inplace,
                                          size_t stride_out[BBFFT_MAX_TENSOR_DIM]);
/* reference: default_ostride (src/base/configuration.cpp:45-56) */
BBFFT_GB300_API int bbfft_default_ostride(uint32_t dim, const size_t shape[BBFFT_MAX_TENSOR_DIM],
                                          int32_t type, int inplace,
                                          size_t stride_out[BBFFT_MAX_TENSOR_DIM]);
/* reference: configuration::to_string / operator<< (src/base/configuration.cpp:63-160).
 * Writes at most buf_len bytes including the terminating zero; *needed receives the full
 * length + 1 (may be NULL). */
BBFFT_GB300_API int bbfft_configuration_to_string(const bbfft_configuration *cfg, char *buf,
                                                  size_t buf_len, size_t *needed);
/* reference: parse_fft_descriptor (src/base/parser.cpp:59-211) */
BBFFT_GB300_API int bbfft_parse_fft_descriptor(const char *desc, bbfft_configuration *cfg);

/* ---- caches (reference include/bbfft/jit_cache.hpp:23-69, jit_cache_all.hpp:20-37,
 *      aot_cache.hpp:21-48) ---- */

/* reference: jit_cache_all (src/base/jit_cache_all.cpp:10-26): stores every module that
 * plan creation compiles, keyed by (kernel identifier, device id). */
BBFFT_GB300_API int bbfft_jit_cache_create(bbfft_cache_t *cache);
/* reference: aot_cache (src/base/aot_cache.cpp:12-28): look-up only; modules are
 * registered with bbfft_aot_cache_register_module. */
BBFFT_GB300_API int bbfft_aot_cache_create(bbfft_cache_t *cache);
/* reference: aot_cache::register_module (src/base/aot_cache.cpp:26-28).  `image` is a
 * cubin / fatbin for sm_103a holding kernels named by `kernel_names`. */
BBFFT_GB300_API int bbfft_aot_cache_register_module(bbfft_cache_t cache, const void *image,
                                                    size_t image_size,
                                                    const char *const *kernel_names,
                                                    size_t num_kernel_names, int device);
/* reference: bbfft-aot-generate (tools/aot/main.cpp:22-60) over generate_fft_kernels
 * (src/base/generator.cpp:16-25).  Compiles the kernels that configurations with user
 * callbacks need (all sharing one user module) into one cubin for the current device (or,
 * when the environment variable BBFFT_GB300_AOT_ARCH names one, e.g. sm_103a, for that
 * architecture without touching a GPU), to be registered with
 * bbfft_aot_cache_register_module; kernels of configurations without callbacks are compiled
 * into this library and need no image.  image may be NULL to query *image_needed; `names`
 * receives the kernel names, one per line. */
BBFFT_GB300_API int bbfft_aot_generate(const bbfft_configuration *cfgs, size_t num_cfgs,
                                       void *image, size_t image_len, size_t *image_needed,
                                       char *names, size_t names_len, size_t *names_needed);
BBFFT_GB300_API int bbfft_cache_destroy(bbfft_cache_t cache);
/* reference: jit_cache_all::kernel_names (jit_cache_all.hpp:33) */
BBFFT_GB300_API int bbfft_cache_kernel_names(bbfft_cache_t cache, char *buf, size_t buf_len,
                                             size_t *needed);
/* number of cache look-ups that hit / missed since creation (no counterpart; test hook) */
BBFFT_GB300_API int bbfft_cache_stats(bbfft_cache_t cache, uint64_t *hits, uint64_t *misses);

/* ---- plans ---- */

/* reference: make_plan(cfg, queue, cache) (include/bbfft/sycl/make_plan.hpp:27,40;
 * cl/make_plan.hpp:27,40; ze/make_plan.hpp:29) -> select_fft_algorithm
 * (src/common/algorithm.hpp:20-30).  The plan is bound to the current CUDA device and to
 * `stream`; `cache` may be NULL. */
BBFFT_GB300_API int bbfft_plan_create(const bbfft_configuration *cfg, cudaStream_t stream,
                                      bbfft_cache_t cache, bbfft_plan_t *plan);

/* Adjoint of the transform described by cfg (no counterpart in the reference): c2c
 * forward -> unnormalised backward; r2c -> c2r with Hermitian weights (interior bins
 * halved, imaginary parts of DC and Nyquist dropped); c2r -> r2c with interior bins
 * doubled.  The plan maps tensors laid out like cfg's OUTPUT to tensors laid out like
 * cfg's INPUT. */
BBFFT_GB300_API int bbfft_plan_create_adjoint(const bbfft_configuration *cfg, cudaStream_t stream,
                                              bbfft_cache_t cache, bbfft_plan_t *plan);

/* reference: plan<E>::execute(in, out, dep_events) (include/bbfft/plan.hpp:77-131) and
 * plan_unmanaged_event::execute(in, out, signal, n_wait, wait) (plan.hpp:165-183).
 * Waits on `wait_events` (cudaStreamWaitEvent), launches on the plan's stream and, if
 * `signal_event` is not NULL, records it after the launch.  in == out is in-place. */
BBFFT_GB300_API int bbfft_plan_execute(bbfft_plan_t plan, const void *in, void *out,
                                       uint32_t num_wait_events, const cudaEvent_t *wait_events,
                                       cudaEvent_t signal_event);
/* Same, on an explicit stream instead of the plan's stream. */
BBFFT_GB300_API int bbfft_plan_execute_on(bbfft_plan_t plan, const void *in, void *out,
                                          cudaStream_t stream);
/* Copies of plans share the implementation (reference plan.hpp:24-48: shared_ptr). */
BBFFT_GB300_API int bbfft_plan_retain(bbfft_plan_t plan);
BBFFT_GB300_API int bbfft_plan_destroy(bbfft_plan_t plan);

/* Plan introspection (no counterpart; the reference exposes the kernel identifier only
 * through the cache key, src/common/algorithm/small_batch_fft.hpp:64-67). */
typedef struct bbfft_plan_info {
    char identifier[256];  /* kernel identifier used as cache key */
    uint32_t num_launches; /* kernels per execute (d for an nd plan) */
    uint32_t inplace_supported;
    uint32_t jit_compiled; /* 1 if a kernel of this plan came from NVRTC or the cache */
    uint32_t radix[12];    /* radices of the first pass */
    uint32_t num_stages;
    uint32_t threads_per_transform;
    uint32_t mb, kb;        /* tile of the first pass */
    uint32_t block_threads; /* threads per CTA of the first pass */
    size_t shared_bytes;    /* dynamic shared memory of the first pass */
    size_t workspace_bytes; /* device scratch owned by the plan (nd temporaries) */
    uint32_t vector_width;  /* transforms per thread along M (first pass) */
    uint32_t specialized;   /* 1 if the first pass runs a compile-time-size kernel */
    uint32_t min_blocks;    /* its register budget: resident CTAs of 256 threads (0: none) */
} bbfft_plan_info;
BBFFT_GB300_API int bbfft_plan_get_info(bbfft_plan_t plan, bbfft_plan_info *info);

/* Override the automatic blocking of a 1d plan (autotuner hook; no counterpart in the
 * reference).  radices: list whose product is the complex FFT length (NULL / 0 entries =
 * automatic); threads_per_transform, mb, kb: 0 = automatic; vector_width: transforms per
 * thread along M (0 = automatic, 1 = none); min_blocks: 2 or 3 resident CTAs of 256
 * threads that the compile-time kernel's registers are sized for (0 = automatic, float
 * only for 3).  Plans made with bbfft_plan_create consult the tuning table
 * (BBFFT_GB300_TUNING or the package's tuning/gb300.tune) written by the autotuner. */
BBFFT_GB300_API int bbfft_plan_create_tuned(const bbfft_configuration *cfg, cudaStream_t stream,
                                            const uint32_t *radices, uint32_t num_radices,
                                            uint32_t threads_per_transform,
                                            uint32_t vector_width, uint32_t mb, uint32_t kb,
                                            uint32_t min_blocks, bbfft_plan_t *plan);

/* ---- ragged batches (no counterpart in the reference, which launches one kernel per plan,
 *      src/common/algorithm/small_batch_fft.hpp:111) ---- */

/* One independent 1d transform of a ragged batch: default packed layout (c2c: M*N*K
 * complex in and out; r2c: M*N*K real in, M*(N/2+1)*K complex out; c2r the reverse). */
typedef struct bbfft_ragged_item {
    int32_t precision; /* all items of a batch share the precision */
    int32_t direction;
    int32_t type;
    uint32_t N;
    size_t M, K;
    const void *in;
    void *out; /* must not alias another item's input */
} bbfft_ragged_item;
typedef struct bbfft_ragged_s *bbfft_ragged_t;

typedef struct bbfft_ragged_info {
    uint64_t num_units;   /* CTA tiles over all transforms */
    uint32_t grid, block; /* persistent launch geometry */
    size_t shared_bytes;  /* dynamic shared memory per CTA */
    uint64_t bytes_moved; /* algorithmic bytes: one read + one write of every tensor */
} bbfft_ragged_info;

/* Plans all transforms of the batch for ONE persistent launch on the current device. */
BBFFT_GB300_API int bbfft_ragged_create(const bbfft_ragged_item *items, size_t num_items,
                                        bbfft_ragged_t *ragged);
/* Runs the whole batch in one kernel launch.  Persistent form (default): a reset of the
 * work counter and one persistent kernel whose CTAs take tiles from the counter.  Grid
 * form: one CTA per tile.  With use_graph != 0 the launch is captured once into a CUDA
 * graph that is replayed on `stream`. */
BBFFT_GB300_API int bbfft_ragged_execute(bbfft_ragged_t ragged, cudaStream_t stream,
                                         int use_graph);
#define BBFFT_RAGGED_PERSISTENT 0
#define BBFFT_RAGGED_GRID 1
#define BBFFT_RAGGED_CLASSES 2
/* Selects the launch form of bbfft_ragged_execute: BBFFT_RAGGED_PERSISTENT or
 * BBFFT_RAGGED_GRID (one launch), or BBFFT_RAGGED_CLASSES (one kernel per class of
 * tiles with the same tile function, each sized for that class; as a graph the classes
 * are independent nodes that may run concurrently).  Drops a graph made for another
 * form. */
BBFFT_GB300_API int bbfft_ragged_set_launch_form(bbfft_ragged_t ragged, int form);
BBFFT_GB300_API int bbfft_ragged_get_info(bbfft_ragged_t ragged, bbfft_ragged_info *info);
BBFFT_GB300_API int bbfft_ragged_destroy(bbfft_ragged_t ragged);

/* Allocation-free 2d c2r, float precision.  No counterpart in the reference: it exists for
 * callers that cannot allocate device memory when they transform -- a process whose
 * memory manager reserves the device memory at start-up and forbids cudaMalloc later, or
 * a host that must keep a fixed device footprint -- while a plan allocates its
 * temporary and twiddle tables.  The result equals that of a plan of {dim 2, shape
 * {M, N1, N2, K}, f32, backward, c2r} with the default out-of-place layout within float
 * rounding (rel-L2 <= 2e-6), but the temporary between the two passes and the twiddle
 * tables live in static device arrays of the library (16 MiB + 8 KiB held on every GPU
 * that loads the library until the process exits).  Limits: N1, N2 <= 512 and
 * M * (N1/2+1) * N2 * K <= 2^21; larger problems return BBFFT_BAD_CONFIGURATION.  It
 * calls no cudaMalloc, cudaFree or other allocating routine.  The first call on a device
 * resolves the device addresses of the static arrays (cudaGetSymbolAddress) with that
 * device current; make that first call before any stream capture begins.  All calls
 * share the arrays and every call rewrites what it uses, so calls that may overlap on
 * the GPU (different streams, different host threads) race; serialise them.
 * Out-of-place only (in != out). */
BBFFT_GB300_API int bbfft_c2r_2d_noalloc_f32(const void *in, void *out, size_t M, size_t N1,
                                             size_t N2, size_t K, cudaStream_t stream);

/* Thread-local message of the last failure (empty string if none). */
BBFFT_GB300_API const char *bbfft_last_error(void);
/* Library version string. */
BBFFT_GB300_API const char *bbfft_version(void);

#ifdef __cplusplus
}
#endif

#endif /* BBFFT_GB300_H */
