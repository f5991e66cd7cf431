"""Thin Python binding of the bbfft GB300 C ABI (include/bbfft_gb300.h).

This module is test and benchmark plumbing: it loads the in-tree shared library
with ctypes and exposes the reference's plan interface (configuration, make_plan,
plan.execute) with the same names and argument meaning as the reference's C++ API
(include/bbfft/configuration.hpp, include/bbfft/plan.hpp of bbfft 0.5.1).  Device
memory is passed as integer device pointers (e.g. torch.Tensor.data_ptr()).

There is no CPU fallback: if the library cannot be loaded, import fails loudly.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, '_lib', 'libbbfft_gb300.so')

MAX_TENSOR_DIM = 5
F32, F64 = 4, 8
FORWARD, BACKWARD = -1, 1
C2C, R2C, C2R = 0, 1, 2
COMPUTE_NATIVE, COMPUTE_BF16, COMPUTE_SPLIT_BF16, COMPUTE_SPLIT_BF16_3TERM = 0, 1, 2, 3
COMPUTE_SPLIT_TF32 = 4

STATUS = {
    0: 'SUCCESS', -1: 'BAD_CONFIGURATION', -2: 'INVALID_ARGUMENT', -3: 'CUDA_ERROR',
    -4: 'COMPILE_ERROR', -5: 'PARSE_ERROR', -6: 'OUT_OF_MEMORY', -7: 'INTERNAL_ERROR',
    -8: 'DEVICE_ERROR',
}


class BBFFTError(RuntimeError):
    def __init__(self, status, message):
        super().__init__('%s: %s' % (STATUS.get(status, status), message))
        self.status = status
        self.message = message


class BadConfiguration(BBFFTError):
    """Raised where the reference throws bbfft::bad_configuration."""


class ParseError(BBFFTError):
    """Raised where the reference's descriptor parser throws std::runtime_error."""


class CompileError(BBFFTError):
    """NVRTC could not compile the user callbacks."""


class Configuration(ctypes.Structure):
    _fields_ = [
        ('dim', ctypes.c_uint32),
        ('shape', ctypes.c_size_t * MAX_TENSOR_DIM),
        ('precision', ctypes.c_int32),
        ('direction', ctypes.c_int32),
        ('type', ctypes.c_int32),
        ('istride', ctypes.c_size_t * MAX_TENSOR_DIM),
        ('ostride', ctypes.c_size_t * MAX_TENSOR_DIM),
        ('callback_source', ctypes.c_char_p),
        ('callback_length', ctypes.c_size_t),
        ('load_function', ctypes.c_char_p),
        ('store_function', ctypes.c_char_p),
        ('compute', ctypes.c_int32),
    ]

    def __repr__(self):
        return 'Configuration(%s)' % to_string(self)


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ('identifier', ctypes.c_char * 256),
        ('num_launches', ctypes.c_uint32),
        ('inplace_supported', ctypes.c_uint32),
        ('jit_compiled', ctypes.c_uint32),
        ('radix', ctypes.c_uint32 * 12),
        ('num_stages', ctypes.c_uint32),
        ('threads_per_transform', ctypes.c_uint32),
        ('mb', ctypes.c_uint32),
        ('kb', ctypes.c_uint32),
        ('block_threads', ctypes.c_uint32),
        ('shared_bytes', ctypes.c_size_t),
        ('workspace_bytes', ctypes.c_size_t),
        ('vector_width', ctypes.c_uint32),
        ('specialized', ctypes.c_uint32),
        ('min_blocks', ctypes.c_uint32),
    ]


class RaggedItem(ctypes.Structure):
    _fields_ = [
        ('precision', ctypes.c_int32),
        ('direction', ctypes.c_int32),
        ('type', ctypes.c_int32),
        ('N', ctypes.c_uint32),
        ('M', ctypes.c_size_t),
        ('K', ctypes.c_size_t),
        ('in_', ctypes.c_void_p),
        ('out', ctypes.c_void_p),
    ]


class RaggedInfo(ctypes.Structure):
    _fields_ = [
        ('num_units', ctypes.c_uint64),
        ('grid', ctypes.c_uint32),
        ('block', ctypes.c_uint32),
        ('shared_bytes', ctypes.c_size_t),
        ('bytes_moved', ctypes.c_uint64),
    ]


# Every symbol declared in include/bbfft_gb300.h with its ctypes signature.
_vp = ctypes.c_void_p
_SIGNATURES = {
    'bbfft_default_istride': (ctypes.c_int, [ctypes.c_uint32, ctypes.POINTER(ctypes.c_size_t),
                                             ctypes.c_int32, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_size_t)]),
    'bbfft_default_ostride': (ctypes.c_int, [ctypes.c_uint32, ctypes.POINTER(ctypes.c_size_t),
                                             ctypes.c_int32, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_size_t)]),
    'bbfft_configuration_to_string': (ctypes.c_int, [ctypes.POINTER(Configuration), ctypes.c_char_p,
                                                     ctypes.c_size_t,
                                                     ctypes.POINTER(ctypes.c_size_t)]),
    'bbfft_parse_fft_descriptor': (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(Configuration)]),
    'bbfft_jit_cache_create': (ctypes.c_int, [ctypes.POINTER(_vp)]),
    'bbfft_aot_cache_create': (ctypes.c_int, [ctypes.POINTER(_vp)]),
    'bbfft_aot_cache_register_module': (ctypes.c_int, [_vp, _vp, ctypes.c_size_t,
                                                       ctypes.POINTER(ctypes.c_char_p),
                                                       ctypes.c_size_t, ctypes.c_int]),
    'bbfft_aot_generate': (ctypes.c_int, [ctypes.POINTER(Configuration), ctypes.c_size_t, _vp,
                                          ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                          ctypes.c_char_p, ctypes.c_size_t,
                                          ctypes.POINTER(ctypes.c_size_t)]),
    'bbfft_cache_destroy': (ctypes.c_int, [_vp]),
    'bbfft_cache_kernel_names': (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_size_t,
                                                ctypes.POINTER(ctypes.c_size_t)]),
    'bbfft_cache_stats': (ctypes.c_int, [_vp, ctypes.POINTER(ctypes.c_uint64),
                                         ctypes.POINTER(ctypes.c_uint64)]),
    'bbfft_plan_create': (ctypes.c_int, [ctypes.POINTER(Configuration), _vp, _vp,
                                         ctypes.POINTER(_vp)]),
    'bbfft_plan_create_adjoint': (ctypes.c_int, [ctypes.POINTER(Configuration), _vp, _vp,
                                                 ctypes.POINTER(_vp)]),
    'bbfft_plan_create_tuned': (ctypes.c_int, [ctypes.POINTER(Configuration), _vp,
                                               ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint32,
                                               ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                               ctypes.c_uint32, ctypes.c_uint32,
                                               ctypes.POINTER(_vp)]),
    'bbfft_plan_execute': (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_uint32, ctypes.POINTER(_vp), _vp]),
    'bbfft_plan_execute_on': (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    'bbfft_plan_retain': (ctypes.c_int, [_vp]),
    'bbfft_plan_destroy': (ctypes.c_int, [_vp]),
    'bbfft_plan_get_info': (ctypes.c_int, [_vp, ctypes.POINTER(PlanInfo)]),
    'bbfft_ragged_create': (ctypes.c_int, [ctypes.POINTER(RaggedItem), ctypes.c_size_t,
                                           ctypes.POINTER(_vp)]),
    'bbfft_ragged_execute': (ctypes.c_int, [_vp, _vp, ctypes.c_int]),
    'bbfft_ragged_get_info': (ctypes.c_int, [_vp, ctypes.POINTER(RaggedInfo)]),
    'bbfft_ragged_set_launch_form': (ctypes.c_int, [_vp, ctypes.c_int]),
    'bbfft_ragged_destroy': (ctypes.c_int, [_vp]),
    'bbfft_c2r_2d_noalloc_f32': (ctypes.c_int, [_vp, _vp, ctypes.c_size_t, ctypes.c_size_t,
                                                ctypes.c_size_t, ctypes.c_size_t, _vp]),
    'bbfft_last_error': (ctypes.c_char_p, []),
    'bbfft_version': (ctypes.c_char_p, []),
}

_lib = None


def lib():
    """Load the shared library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError('bbfft GB300 library not built: %s (run build())' % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return sorted(_SIGNATURES)


def _check(status):
    if status != 0:
        msg = lib().bbfft_last_error().decode(errors='replace')
        cls = {-1: BadConfiguration, -5: ParseError, -4: CompileError}.get(status, BBFFTError)
        raise cls(status, msg)


def _arr(values):
    a = (ctypes.c_size_t * MAX_TENSOR_DIM)()
    for i, v in enumerate(values):
        a[i] = int(v)
    return a


def default_istride(dim, shape, type=C2C, inplace=False):
    out = (ctypes.c_size_t * MAX_TENSOR_DIM)()
    _check(lib().bbfft_default_istride(dim, _arr(shape), type, int(inplace), out))
    return list(out)


def default_ostride(dim, shape, type=C2C, inplace=False):
    out = (ctypes.c_size_t * MAX_TENSOR_DIM)()
    _check(lib().bbfft_default_ostride(dim, _arr(shape), type, int(inplace), out))
    return list(out)


def configuration(dim, shape, precision=F32, direction=FORWARD, type=C2C, istride=None,
                  ostride=None, inplace=False, callbacks=None, compute=COMPUTE_NATIVE):
    """Build a configuration like the reference's aggregate initialisation.

    shape = [M, N1, .., Nd, K]; strides default to the reference's defaults
    (in-place layout if inplace=True).  callbacks = (source, load_name, store_name).
    """
    shape = list(shape) + [0] * (MAX_TENSOR_DIM - len(shape))
    cfg = Configuration()
    cfg.dim = dim
    cfg.shape = _arr(shape)
    cfg.precision = precision
    cfg.direction = direction
    cfg.type = type
    cfg.istride = _arr(istride if istride is not None else default_istride(dim, shape, type, inplace))
    cfg.ostride = _arr(ostride if ostride is not None else default_ostride(dim, shape, type, inplace))
    if callbacks:
        src, load, store = callbacks
        data = src.encode() if isinstance(src, str) else src
        cfg._keep = data  # keep the buffer alive
        cfg.callback_source = data
        cfg.callback_length = len(data)
        cfg.load_function = load.encode() if load else None
        cfg.store_function = store.encode() if store else None
    cfg.compute = compute
    return cfg


def to_string(cfg):
    needed = ctypes.c_size_t()
    buf = ctypes.create_string_buffer(512)
    _check(lib().bbfft_configuration_to_string(ctypes.byref(cfg), buf, 512, ctypes.byref(needed)))
    return buf.value.decode()


def parse_fft_descriptor(desc):
    cfg = Configuration()
    _check(lib().bbfft_parse_fft_descriptor(desc.encode(), ctypes.byref(cfg)))
    return cfg


def aot_generate(cfgs, max_image=64 << 20):
    """Compile the callback kernels of `cfgs` into one cubin; returns (image bytes, names)."""
    arr = (Configuration * len(cfgs))(*cfgs)
    buf = ctypes.create_string_buffer(max_image)
    need = ctypes.c_size_t()
    names = ctypes.create_string_buffer(8192)
    _check(lib().bbfft_aot_generate(arr, len(cfgs), ctypes.cast(buf, _vp), max_image,
                                    ctypes.byref(need), names, 8192, None))
    return buf.raw[:need.value], [n for n in names.value.decode().split('\n') if n]


class Cache:
    """jit_cache_all (aot=False) or aot_cache (aot=True)."""

    def __init__(self, aot=False):
        h = _vp()
        _check((lib().bbfft_aot_cache_create if aot else lib().bbfft_jit_cache_create)(ctypes.byref(h)))
        self.handle = h

    def register_module(self, image, kernel_names, device=0):
        arr = (ctypes.c_char_p * len(kernel_names))(*[n.encode() for n in kernel_names])
        buf = ctypes.create_string_buffer(bytes(image), len(image))
        _check(lib().bbfft_aot_cache_register_module(self.handle, ctypes.cast(buf, _vp), len(image),
                                                     arr, len(kernel_names), device))

    def kernel_names(self):
        needed = ctypes.c_size_t()
        _check(lib().bbfft_cache_kernel_names(self.handle, None, 0, ctypes.byref(needed)))
        buf = ctypes.create_string_buffer(needed.value)
        _check(lib().bbfft_cache_kernel_names(self.handle, buf, needed.value, None))
        return [n for n in buf.value.decode().split('\n') if n]

    def stats(self):
        h, m = ctypes.c_uint64(), ctypes.c_uint64()
        _check(lib().bbfft_cache_stats(self.handle, ctypes.byref(h), ctypes.byref(m)))
        return h.value, m.value

    def __del__(self):
        if getattr(self, 'handle', None) and _lib is not None:
            _lib.bbfft_cache_destroy(self.handle)
            self.handle = None


def _stream_ptr(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(getattr(stream, 'cuda_stream', stream))


class Plan:
    """A plan (reference: bbfft::plan<E>, include/bbfft/plan.hpp:60-132)."""

    def __init__(self, cfg, stream=None, cache=None, adjoint=False, tuning=None):
        h = _vp()
        L = lib()
        s = _stream_ptr(stream)
        if tuning is not None:
            rad, T, V, mb, kb = tuning[:5]
            occ = tuning[5] if len(tuning) > 5 else 0
            arr = (ctypes.c_uint32 * max(1, len(rad)))(*rad) if rad else None
            _check(L.bbfft_plan_create_tuned(ctypes.byref(cfg), s, arr, len(rad) if rad else 0,
                                             T or 0, V or 0, mb or 0, kb or 0, occ or 0,
                                             ctypes.byref(h)))
        else:
            fn = L.bbfft_plan_create_adjoint if adjoint else L.bbfft_plan_create
            _check(fn(ctypes.byref(cfg), s, cache.handle if cache else None, ctypes.byref(h)))
        self.handle = h
        self.cfg = cfg
        self.stream = s

    def execute(self, inp, out=None, wait_events=(), signal_event=None):
        """execute(in, out) out-of-place; execute(inout) in-place.  Pointers are ints."""
        if out is None:
            out = inp
        n = len(wait_events)
        arr = (_vp * max(1, n))(*[int(e) for e in wait_events]) if n else None
        _check(lib().bbfft_plan_execute(self.handle, int(inp), int(out), n, arr,
                                        int(signal_event) if signal_event else None))

    def execute_on(self, inp, out, stream):
        _check(lib().bbfft_plan_execute_on(self.handle, int(inp), int(out), _stream_ptr(stream)))

    def info(self):
        i = PlanInfo()
        _check(lib().bbfft_plan_get_info(self.handle, ctypes.byref(i)))
        return i

    def destroy(self):
        if getattr(self, 'handle', None) and _lib is not None:
            _lib.bbfft_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.destroy()


class Ragged:
    """A ragged batch of independent 1d transforms run by one kernel launch.

    items: list of (precision, direction, type, N, M, K, in_ptr, out_ptr) with default
    packed layouts (include/bbfft_gb300.h: bbfft_ragged_item)."""

    def __init__(self, items):
        arr = (RaggedItem * len(items))()
        for i, (prec, d, t, N, M, K, ip, op) in enumerate(items):
            arr[i] = RaggedItem(prec, d, t, N, M, K, int(ip), int(op))
        h = _vp()
        _check(lib().bbfft_ragged_create(arr, len(items), ctypes.byref(h)))
        self.handle = h

    PERSISTENT, GRID, CLASSES = 0, 1, 2

    def execute(self, stream=None, use_graph=False):
        _check(lib().bbfft_ragged_execute(self.handle, _stream_ptr(stream), int(bool(use_graph))))

    def set_launch_form(self, form):
        """Ragged.PERSISTENT (CTAs take tiles from a counter), Ragged.GRID (one CTA per
        tile) or Ragged.CLASSES (one kernel per class of tiles with the same tile
        function); include/bbfft_gb300.h: bbfft_ragged_set_launch_form."""
        _check(lib().bbfft_ragged_set_launch_form(self.handle, int(form)))

    def info(self):
        i = RaggedInfo()
        _check(lib().bbfft_ragged_get_info(self.handle, ctypes.byref(i)))
        return i

    def __del__(self):
        if getattr(self, 'handle', None) and _lib is not None:
            _lib.bbfft_ragged_destroy(self.handle)
            self.handle = None


def make_plan(cfg, stream=None, cache=None):
    """reference: bbfft::make_plan(cfg, queue, cache) (include/bbfft/sycl/make_plan.hpp:27,40)."""
    return Plan(cfg, stream=stream, cache=cache)


def make_adjoint_plan(cfg, stream=None, cache=None):
    return Plan(cfg, stream=stream, cache=cache, adjoint=True)


def c2r_2d_noalloc_f32(inp, out, M, N1, N2, K, stream=None):
    """Allocation-free 2d c2r (include/bbfft_gb300.h: bbfft_c2r_2d_noalloc_f32)."""
    _check(lib().bbfft_c2r_2d_noalloc_f32(int(inp), int(out), M, N1, N2, K, _stream_ptr(stream)))


def shard_k(cfg, world, rank):
    """K slab of one rank when a transform is split over `world` GPUs.

    Every (m, k) transform of the tensor is independent, so the tensor is cut along K
    (shape[dim + 1]) into `world` contiguous slabs, one per rank, with no exchange between
    ranks.  Returns (k0, k1, in_offset, out_offset, slab): the rank's K range, the byte
    offsets of its first input and output element (k0 * stride[dim + 1] elements), and a
    configuration of the slab with the caller's strides (None when the rank gets no
    transform).  Plans of the slab run on the rank's own GPU on `in + in_offset`,
    `out + out_offset`."""
    dim = cfg.dim
    K = int(cfg.shape[dim + 1])
    k0 = rank * K // world
    k1 = (rank + 1) * K // world
    real = 4 if cfg.precision == F32 else 8
    isz = real if cfg.type == R2C else 2 * real
    osz = real if cfg.type == C2R else 2 * real
    in_off = k0 * int(cfg.istride[dim + 1]) * isz
    out_off = k0 * int(cfg.ostride[dim + 1]) * osz
    if k1 == k0:
        return k0, k1, in_off, out_off, None
    slab = Configuration()
    ctypes.memmove(ctypes.byref(slab), ctypes.byref(cfg), ctypes.sizeof(Configuration))
    if hasattr(cfg, '_keep'):
        slab._keep = cfg._keep
    slab.shape[dim + 1] = k1 - k0
    return k0, k1, in_off, out_off, slab


def version():
    return lib().bbfft_version().decode()
