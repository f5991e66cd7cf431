// Host-visible handles of the AOT-compiled kernels.
#pragma once

namespace gbfft {
const void *kernel_f32(int kind);
const void *kernel_f64(int kind);
} // namespace gbfft
