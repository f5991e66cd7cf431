// Same declarations as the reference header of this name (see jit_cache.hpp).
#include "bbfft/jit_cache.hpp"
