"""TEST INFRASTRUCTURE ONLY -- CPU oracle for the double-batched FFT.

Two independent references:
  * `oracle_fft`: the C restatement of the reference's algorithm (bbfft_oracle.c),
    in the plan precision or FP64, with the reference's nd chaining
    (src/common/algorithm/nd_fft.hpp:27-176);
  * `dft64`: an FP64 DFT (numpy pocketfft in float64) with the reference's c2r
    semantics, used to measure rel-L2 errors.
Plus the analytic known-answer signals of the reference's device tests
(test/c2c.cpp:17-51, test/r2c.cpp:28-135), reimplemented.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, 'liboracle.so')

C2C, R2C, C2R = 0, 1, 2
FORWARD, BACKWARD = -1, 1

_lib = None


def build():
    subprocess.run(['make', '-s', '-C', HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(
                os.path.join(HERE, 'bbfft_oracle.c')):
            build()
        L = ctypes.CDLL(LIB)
        for sfx in ('f32', 'f64'):
            fn = getattr(L, 'oracle_fft1d_' + sfx)
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, ctypes.c_long, ctypes.c_long,
                           ctypes.c_void_p, ctypes.c_long, ctypes.c_long, ctypes.c_void_p,
                           ctypes.c_long, ctypes.c_long, ctypes.c_int]
        _lib = L
    return _lib


def _real_dtype(prec):
    return np.float32 if prec == 4 else np.float64


def _cplx_dtype(prec):
    return np.complex64 if prec == 4 else np.complex128


def fft1d(type, direction, M, N, K, x, is1, is2, out, os1, os2, prec=8, threads=1):
    """One double-batched 1d pass on flat numpy arrays (strides in elements, s0 = 1)."""
    fn = lib().oracle_fft1d_f32 if prec == 4 else lib().oracle_fft1d_f64
    assert x.flags['C_CONTIGUOUS'] and out.flags['C_CONTIGUOUS']
    rc = fn(type, direction, M, N, K, x.ctypes.data, is1, is2, out.ctypes.data, os1, os2, threads)
    if rc != 0:
        raise ValueError('oracle rejected the pass')
    return out


def default_istride(dim, shape, type, inplace):
    """reference src/base/configuration.cpp:24-43"""
    n1 = shape[1]
    if type == R2C:
        n1 = 2 * (shape[1] // 2 + 1) if inplace else shape[1]
    elif type == C2R:
        n1 = shape[1] // 2 + 1
    s = [1, shape[0], n1 * shape[0], 0, 0]
    for d in range(1, dim):
        s[d + 2] = shape[d + 1] * s[d + 1]
    return s


def default_ostride(dim, shape, type, inplace):
    """reference src/base/configuration.cpp:45-56"""
    sw = {R2C: C2R, C2R: R2C, C2C: C2C}[type]
    return default_istride(dim, shape, sw, inplace)


def tensor_size(dim, shape, stride):
    """Elements spanned by the tensor: offset of the last element + 1."""
    last = sum((shape[d] - 1) * stride[d] for d in range(dim + 2))
    return last + 1


def oracle_fft(dim, shape, type, direction, x, istride=None, ostride=None, inplace=False, prec=8,
               threads=1, out=None):
    """Reference semantics of a plan execute() on flat arrays.

    x: flat numpy array (real for r2c input, complex otherwise) in the plan precision or FP64.
    For dim > 1 only default layouts are allowed (reference nd_fft.hpp:47-49) and the
    passes are chained exactly like nd_fft (M grows by N_d^complex)."""
    shape = list(shape)
    if istride is None:
        istride = default_istride(dim, shape, type, inplace)
    if ostride is None:
        ostride = default_ostride(dim, shape, type, inplace)
    rdt, cdt = _real_dtype(prec), _cplx_dtype(prec)
    out_is_real = type == C2R
    n1out = shape[1] // 2 + 1 if type == R2C else shape[1]
    oshape = [shape[0], n1out] + shape[2:dim + 2]
    osize = tensor_size(dim, oshape, ostride)
    if out is None:
        out = np.zeros(osize, dtype=rdt if out_is_real else cdt)
    x = np.ascontiguousarray(x)
    if dim == 1:
        return fft1d(type, direction, shape[0], shape[1], shape[2], x, istride[1], istride[2],
                     out, ostride[1], ostride[2], prec, threads)
    # nd chaining (nd_fft.hpp:63-112)
    is_real = type != C2C
    inplace_layout = (list(istride[:dim + 2]) == default_istride(dim, shape, type, True)[:dim + 2]
                      and list(ostride[:dim + 2]) == default_ostride(dim, shape, type, True)[:dim + 2])

    def ndc(d):
        return shape[1] // 2 + 1 if d == 0 and is_real else shape[d + 1]

    def ndr(d):
        return 2 * (shape[1] // 2 + 1) if (d == 0 and is_real and inplace_layout) else shape[d + 1]

    Ntot = 1
    for d in range(dim):
        Ntot *= ndc(d)
    M = shape[0]
    K = Ntot * shape[dim + 1]
    passes = []
    for d in range(dim):
        Nd = shape[d + 1]
        K //= ndc(d)
        t = type if d == 0 else C2C
        passes.append([t, M, Nd, K, M, M * ndr(d), M, M * ndc(d)])
        M *= ndc(d)
    if type == C2R:
        passes = passes[::-1]
        for p in passes:
            p[4], p[5], p[6], p[7] = p[6], p[7], p[4], p[5]
    # temporary: complex work array large enough for every intermediate
    work = np.zeros(max(x.size, out.size) + 16, dtype=cdt)
    cur = x
    for i, (t, M_, N_, K_, is1, is2, os1, os2) in enumerate(passes):
        last = i == len(passes) - 1
        if last:
            dst = out
        else:
            dst = np.zeros(work.size, dtype=cdt)
        fft1d(t, direction, M_, N_, K_, np.ascontiguousarray(cur), is1, is2, dst, os1, os2, prec,
              threads)
        cur = dst
    return out


# ------------------------------------------------------------------------------------------
# independent FP64 DFT


def gather(x, dim, shape, stride):
    """Strided flat array -> dense array of shape (K, Nd, ..., N1, M) (C order)."""
    idx = np.zeros([shape[d] for d in range(dim + 2)][::-1], dtype=np.int64)
    grids = np.meshgrid(*[np.arange(shape[d]) for d in range(dim + 2)][::-1], indexing='ij')
    for ax, g in enumerate(grids):
        d = dim + 1 - ax
        idx += g * stride[d]
    return x[idx]


def dft64(dim, shape, type, direction, xdense):
    """FP64 DFT of a dense array laid out (K, Nd..N1, M); returns the dense result.

    r2c returns N1//2+1 bins along N1; c2r takes N1//2+1 bins and returns N1 reals with
    the reference's semantics: the outer dimensions are transformed first (complex,
    backward), then along N1 imag(X[0]) is ignored and, for even N1, imag(X[N1/2]) is
    subtracted from every output sample (the reference's half-length c2r formula,
    src/base/generator/sbfft_gen.cpp:202-247)."""
    axes = tuple(range(1, dim + 1))  # N axes of (K, Nd, .., N1, M); N1 is axis `dim`
    x = np.asarray(xdense)
    if type == C2C:
        x = x.astype(np.complex128)
        if direction == FORWARD:
            return np.fft.fftn(x, axes=axes)
        return np.fft.ifftn(x, axes=axes) * np.prod([x.shape[a] for a in axes])
    if type == R2C:
        return np.fft.rfftn(x.astype(np.float64), axes=axes)
    N1 = shape[1]
    X = x.astype(np.complex128)
    outer = axes[:-1]
    if outer:
        X = np.fft.ifftn(X, axes=outer) * np.prod([X.shape[a] for a in outer])
    sl0 = [slice(None)] * X.ndim
    sl0[dim] = slice(0, 1)
    X = X.copy()
    X[tuple(sl0)] = X[tuple(sl0)].real
    y = np.fft.irfft(X, n=N1, axis=dim) * N1
    if N1 % 2 == 0:
        sln = [slice(None)] * X.ndim
        sln[dim] = slice(N1 // 2, N1 // 2 + 1)
        y = y - X[tuple(sln)].imag
    return y


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128).ravel()
    b = np.asarray(b, dtype=np.complex128).ravel()
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def tol(prec, N):
    """reference test/fft.hpp:17-20: 100 * eps * sqrt(N)"""
    eps = np.finfo(np.float32 if prec == 4 else np.float64).eps
    return 100.0 * eps * np.sqrt(N)


# ------------------------------------------------------------------------------------------
# known-answer signals of the reference's device tests


def c2c_known_answer(M, N, K, prec=8):
    """test/c2c.cpp:17-51: x = (1 + k/K) e^{2 pi i ((m+k) mod N) n / N} / N,
    X = (1 + k/K) delta(n - (m+k) mod N).  Dense arrays (K, N, M)."""
    k = np.arange(K)[:, None, None]
    n = np.arange(N)[None, :, None]
    m = np.arange(M)[None, None, :]
    basis = (m + k) % N
    scale = 1.0 + k / K
    x = scale * np.exp(2j * np.pi * basis * n / N) / N
    X = scale * ((n - basis) % N == 0)
    return x.astype(_cplx_dtype(prec)), X.astype(np.complex128)


def r2c_known_answer(M, Ns, K, prec=8):
    """test/r2c.cpp:28-115 (1d..3d): x = (1+k/K) prod_d cos(2 pi b_d n_d / N_d) / N_d,
    X = (1+k/K) prod_d (delta(n_d - b_d) + delta(n_d + b_d)) / 2 with b_d = (m+k) mod N_d.
    Returns dense x of shape (K, Nd..N1, M) and X of shape (K, Nd..N1//2+1, M)."""
    dim = len(Ns)
    shp = [K] + list(Ns[::-1]) + [M]
    x = np.ones(shp)
    Xf = np.ones([K] + list(Ns[::-1]) + [M])
    k = np.arange(K).reshape([K] + [1] * (dim + 1))
    m = np.arange(M).reshape([1] * (dim + 1) + [M])
    for d, Nd in enumerate(Ns):
        ax = dim - d
        nshape = [1] * (dim + 2)
        nshape[ax] = Nd
        n = np.arange(Nd).reshape(nshape)
        b = (m + k) % Nd
        x = x * np.cos(2 * np.pi * b * n / Nd) / Nd
        Xf = Xf * (((n - b) % Nd == 0).astype(float) + ((n + b) % Nd == 0).astype(float)) / 2
    scale = 1.0 + k / K
    x = x * scale
    Xf = Xf * scale
    sl = [slice(None)] * (dim + 2)
    sl[dim] = slice(0, Ns[0] // 2 + 1)
    return x.astype(_real_dtype(prec)), Xf[tuple(sl)].astype(np.complex128)


def c2r_known_answer(M, Ns, K, prec=8, pollute_0=False):
    """test/r2c.cpp:56-78 and 115-135: the half-delta spectrum and its cosine transform
    (without the 1/N_d factors).  imag(X[0]) is polluted with 1 + m + k when asked
    (test/r2c.cpp:310-324); the result must not change."""
    x, Xf = r2c_known_answer(M, Ns, K, 8)
    dim = len(Ns)
    X = Xf.astype(np.complex128)
    if pollute_0:
        k = np.arange(K).reshape([K] + [1] * (dim + 1))
        m = np.arange(M).reshape([1] * (dim + 1) + [M])
        sl = [slice(None)] * (dim + 2)
        sl[dim] = slice(0, 1)
        X[tuple(sl)] = X[tuple(sl)].real + 1j * np.broadcast_to(1.0 + m + k, X[tuple(sl)].shape)
    y = x * np.prod(Ns)
    return X.astype(_cplx_dtype(prec)), y


def scatter(dense, dim, shape, stride, size, dtype):
    """dense (K, Nd..N1, M) -> strided flat array."""
    out = np.zeros(size, dtype=dtype)
    idx = np.zeros(dense.shape, dtype=np.int64)
    grids = np.meshgrid(*[np.arange(s) for s in dense.shape], indexing='ij')
    for ax, g in enumerate(grids):
        d = dim + 1 - ax
        idx += g * stride[d]
    out[idx] = dense
    return out
