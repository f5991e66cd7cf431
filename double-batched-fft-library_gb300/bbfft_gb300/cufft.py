"""cuFFT comparator over the double-batched layout (benchmark plumbing, not the product).

The reference's cuFFT benchmark (benchmark/test-cufft.cpp:38-45) transforms an M x N x K
column-major tensor with one cufftPlanMany plan over K (signal stride M, distance M*N) and
loops over the M offsets, since cuFFT has a single batch mode.  This module does the same
through ctypes on libcufft, on the caller's stream.  Real transforms cannot take the
per-m offsets (cuFFT rejects a real pointer offset by one element), so the benchmark runs
them through torch.fft instead.
"""
import ctypes
import ctypes.util
import os

CUFFT_FORWARD, CUFFT_INVERSE = -1, 1
_TYPES = {  # (precision bytes, type) -> cufftType
    (4, 'c2c'): 0x29, (4, 'r2c'): 0x2a, (4, 'c2r'): 0x2c,
    (8, 'c2c'): 0x69, (8, 'r2c'): 0x6a, (8, 'c2r'): 0x6c,
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        cands = []
        for d in (os.environ.get('CUDA_HOME'), '/usr/local/cuda'):
            if d:
                cands += [os.path.join(d, 'lib64', 'libcufft.so'), os.path.join(d, 'lib64', 'libcufft.so.12')]
        found = ctypes.util.find_library('cufft')
        if found:
            cands.append(found)
        for c in cands:
            try:
                _lib = ctypes.CDLL(c)
                break
            except OSError:
                continue
        if _lib is None:
            raise OSError('libcufft not found')
        L = _lib
        L.cufftPlanMany.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                    ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int]
        L.cufftSetStream.argtypes = [ctypes.c_int, ctypes.c_void_p]
        for f in ('cufftExecC2C', 'cufftExecZ2Z'):
            getattr(L, f).argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        for f in ('cufftExecR2C', 'cufftExecC2R', 'cufftExecD2Z', 'cufftExecZ2D'):
            getattr(L, f).argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.cufftDestroy.argtypes = [ctypes.c_int]
    return _lib


def _check(r, what):
    if r != 0:
        raise RuntimeError('%s failed with cufftResult %d' % (what, r))


class Plan:
    """1d transform of every (m, k) of an M x N x K tensor with the default (packed)
    layout: one plan over K, executed once per m (the reference's cuFFT loop)."""

    def __init__(self, prec, kind, M, N, K, stream=0, direction=CUFFT_FORWARD):
        L = lib()
        self.prec, self.kind, self.M, self.N, self.K = prec, kind, M, N, K
        self.direction = direction
        nin = N if kind in ('c2c', 'r2c') else N // 2 + 1
        nout = N if kind in ('c2c', 'c2r') else N // 2 + 1
        # element sizes of the input and output in bytes (for the per-m pointer offsets)
        self.isz = prec * (1 if kind == 'r2c' else 2)
        self.osz = prec * (1 if kind == 'c2r' else 2)
        h = ctypes.c_int(0)
        n = (ctypes.c_int * 1)(N)
        inem = (ctypes.c_int * 1)(nin)
        onem = (ctypes.c_int * 1)(nout)
        _check(L.cufftPlanMany(ctypes.byref(h), 1, n, inem, M, M * nin, onem, M, M * nout,
                               _TYPES[(prec, kind)], K), 'cufftPlanMany')
        self.h = h.value
        _check(L.cufftSetStream(self.h, ctypes.c_void_p(stream)), 'cufftSetStream')
        self._exec = {
            (4, 'c2c'): lambda i, o: L.cufftExecC2C(self.h, i, o, self.direction),
            (8, 'c2c'): lambda i, o: L.cufftExecZ2Z(self.h, i, o, self.direction),
            (4, 'r2c'): lambda i, o: L.cufftExecR2C(self.h, i, o),
            (8, 'r2c'): lambda i, o: L.cufftExecD2Z(self.h, i, o),
            (4, 'c2r'): lambda i, o: L.cufftExecC2R(self.h, i, o),
            (8, 'c2r'): lambda i, o: L.cufftExecZ2D(self.h, i, o),
        }[(prec, kind)]

    def execute(self, inp, out):
        for m in range(self.M):
            _check(self._exec(ctypes.c_void_p(inp + m * self.isz), ctypes.c_void_p(out + m * self.osz)),
                   'cufftExec')

    def destroy(self):
        if self.h:
            lib().cufftDestroy(self.h)
            self.h = 0

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass
