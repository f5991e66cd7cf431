// bbfft::user_module for the GB300 library.
// Mirrors the reference's include/bbfft/user_module.hpp:24-37.  The source is CUDA C++
// (compiled with NVRTC for sm_103a) defining
//   T load(T *in, size_t offset)  /  void store(T *out, size_t offset, T value)
// with T = float2 / double2 for complex and float / double for real tensors; the functions
// may omit __device__, as OpenCL-C functions do in the reference.
#ifndef BBFFT_GB300_USER_MODULE_HPP
#define BBFFT_GB300_USER_MODULE_HPP

#include <cstddef>

namespace bbfft {

enum class kernel_language {
    opencl_c, ///< accepted for source compatibility; the GB300 library compiles CUDA C++
    cuda_cpp  ///< CUDA C++ (NVRTC)
};

struct user_module {
    char const *data = nullptr;           ///< source code
    std::size_t length = 0;               ///< length of the source
    char const *load_function = nullptr;  ///< name of the load function or nullptr
    char const *store_function = nullptr; ///< name of the store function or nullptr
    kernel_language language = kernel_language::cuda_cpp;

    explicit operator bool() const noexcept {
        return data && length > 0 && (load_function || store_function);
    }
};

} // namespace bbfft

#endif
