// bbfft::shared_handle: a reference-counted opaque handle with a deleter.  Mirrors the
// reference's include/bbfft/shared_handle.hpp:18-52 (pointer-sized handle, shared ownership).
#ifndef BBFFT_GB300_SHARED_HANDLE_HPP
#define BBFFT_GB300_SHARED_HANDLE_HPP

#include <memory>
#include <type_traits>

namespace bbfft {

template <typename T, typename Enable = void> class shared_handle;

template <typename T>
class shared_handle<T, std::enable_if_t<sizeof(T) <= sizeof(void *) && alignof(T) <= sizeof(void *)>> {
  public:
    shared_handle() = default;
    shared_handle(T t, void (*deleter)(T))
        : handle_(reinterpret_cast<void *>(t), [deleter](void *p) { deleter(reinterpret_cast<T>(p)); }) {}
    T get() const { return reinterpret_cast<T>(handle_.get()); }
    explicit operator bool() const noexcept { return bool(handle_); }

  private:
    std::shared_ptr<void> handle_;
};

} // namespace bbfft

#endif
