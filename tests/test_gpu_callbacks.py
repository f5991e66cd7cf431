"""User load/store callbacks (NVRTC) and the JIT / AOT plan caches.

Restates the reference's test/callback.cpp:18-202 with callbacks written in CUDA C++ (the
reference writes them in OpenCL-C):
  * a load callback that zero-pads a truncated half spectrum for a c2r of twice the length;
  * a store callback that scales by 1/N and keeps the first N/4 bins of an r2c.
The reference requires bit-exact equality with a plan that reads/writes the padded tensor
through the same generated kernel; here the comparison plan runs the same NVRTC-compiled
kernel with identity callbacks (bit-exact), and the callback-free plan is checked within
the float/double tolerances.  Caches: reference src/base/jit_cache_all.cpp,
src/base/aot_cache.cpp."""
import numpy as np
import pytest

from gpu_helpers import TOL, dtypes, rel_l2, run

pytestmark = pytest.mark.gpu

LOAD_SRC = """
{T2} load_pad({T2} *in, size_t offset) {{
    unsigned n = offset / {M} % {NEXT};
    if (n < {NCUT}) {{
        size_t k = offset / ({M} * {NEXT});
        return in[offset - k * {M} * ({NEXT} - {NCUT})];
    }}
    {T2} z = {{0, 0}};
    return z;
}}
{T2} load_id({T2} *in, size_t offset) {{ return in[offset]; }}
"""

STORE_SRC = """
void store_cut({T2} *out, size_t offset, {T2} value) {{
    unsigned n = offset / {M} % {NH};
    if (n < {NCUT}) {{
        size_t k = offset / ({M} * {NH});
        {T2} v = value;
        v.x = v.x * ({T})({SCALE});
        v.y = v.y * ({T})({SCALE});
        out[offset - k * {M} * ({NH} - {NCUT})] = v;
    }}
}}
void store_id({T2} *out, size_t offset, {T2} value) {{ out[offset] = value; }}
"""


def _types(prec):
    return ('float', 'float2') if prec == 4 else ('double', 'double2')


@pytest.mark.parametrize('prec', [4, 8])
@pytest.mark.parametrize('N', [8, 64, 212])
@pytest.mark.parametrize('M', [1, 32])
def test_load_callback_zero_pads(bb, torch_cuda, prec, N, M):
    """reference test/callback.cpp:18-114"""
    torch = torch_cuda
    K = 16
    N_ext = 2 * N
    next_, ncut = N_ext // 2 + 1, N // 2 + 1
    T, T2 = _types(prec)
    src = LOAD_SRC.format(T2=T2, M=M, NEXT=next_, NCUT=ncut)
    rdt, cdt = dtypes(prec)
    rng = np.random.default_rng(N + M + prec)
    vals = (rng.uniform(0, 1, (K, ncut, M)) + 1j * rng.uniform(0, 1, (K, ncut, M))).astype(cdt)
    X_ref = np.zeros((K, next_, M), dtype=cdt)
    X_ref[:, :ncut, :] = vals
    istride = [1, M, M * next_, 0, 0]
    ostride = [1, M, M * N_ext, 0, 0]
    shape = [M, N_ext, K]
    cfg_id = bb.configuration(1, shape, precision=prec, direction=bb.BACKWARD, type=bb.C2R,
                              istride=istride, ostride=ostride, callbacks=(src, 'load_id', None))
    cfg_cb = bb.configuration(1, shape, precision=prec, direction=bb.BACKWARD, type=bb.C2R,
                              istride=istride, ostride=ostride, callbacks=(src, 'load_pad', None))
    cfg_plain = bb.configuration(1, shape, precision=prec, direction=bb.BACKWARD, type=bb.C2R,
                                 istride=istride, ostride=ostride)
    n_out = M * N_ext * K
    x_id = run(bb, torch, cfg_id, X_ref.ravel(), n_out, rdt)
    x_cb = run(bb, torch, cfg_cb, vals.ravel(), n_out, rdt)
    x_plain = run(bb, torch, cfg_plain, X_ref.ravel(), n_out, rdt)
    assert np.array_equal(x_cb, x_id)
    assert rel_l2(x_cb, x_plain) <= TOL[prec]


@pytest.mark.parametrize('prec', [4, 8])
@pytest.mark.parametrize('N', [8, 64, 212])
@pytest.mark.parametrize('M', [1, 32])
def test_store_callback_scales_and_truncates(bb, torch_cuda, prec, N, M):
    """reference test/callback.cpp:116-202"""
    torch = torch_cuda
    K = 16
    nh, ncut = N // 2 + 1, N // 4
    T, T2 = _types(prec)
    src = STORE_SRC.format(T=T, T2=T2, M=M, NH=nh, NCUT=ncut, SCALE=float.hex(1.0 / N))
    rdt, cdt = dtypes(prec)
    rng = np.random.default_rng(3 * N + M + prec)
    x = rng.uniform(0, 1, M * N * K).astype(rdt)
    istride = [1, M, M * N, 0, 0]
    ostride = [1, M, M * nh, 0, 0]
    shape = [M, N, K]
    cfg_id = bb.configuration(1, shape, precision=prec, type=bb.R2C, istride=istride,
                              ostride=ostride, callbacks=(src, None, 'store_id'))
    cfg_cb = bb.configuration(1, shape, precision=prec, type=bb.R2C, istride=istride,
                              ostride=ostride, callbacks=(src, None, 'store_cut'))
    cfg_plain = bb.configuration(1, shape, precision=prec, type=bb.R2C, istride=istride,
                                 ostride=ostride)
    X_id = run(bb, torch, cfg_id, x, M * nh * K, cdt).reshape(K, nh, M)
    X_cb = run(bb, torch, cfg_cb, x, M * ncut * K, cdt).reshape(K, ncut, M)
    X_plain = run(bb, torch, cfg_plain, x, M * nh * K, cdt).reshape(K, nh, M)
    scale = rdt(1.0 / N)
    ref = (X_id[:, :ncut, :].real * scale) + 1j * (X_id[:, :ncut, :].imag * scale)
    assert np.array_equal(X_cb.real, ref.real.astype(rdt))
    assert np.array_equal(X_cb.imag, ref.imag.astype(rdt))
    assert rel_l2(X_cb, X_plain[:, :ncut, :] * scale) <= TOL[prec]


def _cb_cfg(bb, M, N, K, prec=4):
    src = LOAD_SRC.format(T2='float2' if prec == 4 else 'double2', M=M, NEXT=N // 2 + 1,
                          NCUT=N // 2 + 1)
    return bb.configuration(1, [M, N, K], precision=prec, direction=bb.BACKWARD, type=bb.C2R,
                            callbacks=(src, 'load_id', None))


def test_jit_cache_reuses_modules(bb, torch_cuda):
    """jit_cache_all: the second plan with the same user module hits the cache."""
    torch = torch_cuda
    cache = bb.Cache()
    stream = torch.cuda.current_stream().cuda_stream
    p1 = bb.Plan(_cb_cfg(bb, 4, 64, 8), stream=stream, cache=cache)
    assert cache.stats() == (0, 1)
    assert p1.info().jit_compiled == 1
    src_cfg = _cb_cfg(bb, 4, 64, 8)
    cfg2 = bb.configuration(1, [4, 64, 100], precision=4, direction=bb.BACKWARD, type=bb.C2R,
                            callbacks=(src_cfg._keep.decode(), 'load_id', None))
    bb.Plan(cfg2, stream=stream, cache=cache)
    assert cache.stats() == (1, 1)
    names = cache.kernel_names()
    assert len(names) == 1 and names[0].startswith('gbfft_cb_f32_c2rh_load_id')


def test_aot_cache_serves_generated_image(bb, torch_cuda):
    """aot_cache: a cubin from bbfft_aot_generate registered once serves plan creation."""
    torch = torch_cuda
    cfg = _cb_cfg(bb, 4, 64, 8)
    image, names = bb.aot_generate([cfg])
    assert len(image) > 1000 and len(names) == 1
    aot = bb.Cache(aot=True)
    aot.register_module(image, names, device=torch.cuda.current_device())
    rng = np.random.default_rng(5)
    X = (rng.standard_normal(4 * 33 * 8) + 1j * rng.standard_normal(4 * 33 * 8)).astype(np.complex64)
    stream = torch.cuda.current_stream().cuda_stream
    p_aot = bb.Plan(cfg, stream=stream, cache=aot)
    assert aot.stats() == (1, 0)
    y_aot = run(bb, torch, cfg, X, 4 * 64 * 8, np.float32, plan=p_aot)
    y_jit = run(bb, torch, cfg, X, 4 * 64 * 8, np.float32)
    assert np.array_equal(y_aot, y_jit)


def test_callback_compile_error_is_reported(bb, torch_cuda):
    cfg = bb.configuration(1, [1, 16, 1], precision=4, callbacks=('this is not C++', 'load', None))
    with pytest.raises(bb.CompileError, match='NVRTC'):
        bb.make_plan(cfg)


def test_aot_tool_image_serves_plans(bb, torch_cuda, tmp_path):
    """An image written by the bbfft_gb300.aot tool (offline, --arch of this GPU) and loaded
    with aot.load() serves plan creation without NVRTC; results equal the JIT plan's."""
    torch = torch_cuda
    from bbfft_gb300 import aot

    major, minor = torch.cuda.get_device_capability()
    src = tmp_path / 'user.cu'
    src.write_text(LOAD_SRC.format(T2='float2', M=4, NEXT=64 // 2 + 1, NCUT=20))
    out = tmp_path / 'k.cubin'
    aot.main(['-o', str(out), '--callbacks', str(src), '--load', 'load_id',
              '--arch', 'sm_%d%da' % (major, minor), 'srbo4.64*8'])
    cache = aot.load(str(out), device=torch.cuda.current_device())
    cfg = bb.configuration(1, [4, 64, 8], precision=4, type=bb.C2R, direction=bb.BACKWARD,
                           callbacks=(src.read_text(), 'load_id', None))
    stream = torch.cuda.current_stream().cuda_stream
    p_aot = bb.Plan(cfg, stream=stream, cache=cache)
    assert cache.stats() == (1, 0)
    rng = np.random.default_rng(8)
    X = (rng.standard_normal(4 * 33 * 8) + 1j * rng.standard_normal(4 * 33 * 8)).astype(np.complex64)
    y_aot = run(bb, torch, cfg, X, 4 * 64 * 8, np.float32, plan=p_aot)
    y_jit = run(bb, torch, cfg, X, 4 * 64 * 8, np.float32)
    assert np.array_equal(y_aot, y_jit)


ND_SRC = """
{T2} load_w({T2} *in, size_t offset) {{
    {T2} v = in[offset];
    {T} w = ({T})1 + ({T})(offset % 5) * ({T})0.25;
    v.x = v.x * w;
    v.y = v.y * w;
    return v;
}}
{T} load_w({T} *in, size_t offset) {{
    return in[offset] * (({T})1 + ({T})(offset % 5) * ({T})0.25);
}}
void store_w({T2} *out, size_t offset, {T2} v) {{
    {T} w = ({T})1 + ({T})(offset % 3) * ({T})0.5;
    v.x = v.x * w;
    v.y = v.y * w;
    out[offset] = v;
}}
void store_w({T} *out, size_t offset, {T} v) {{
    out[offset] = v * (({T})1 + ({T})(offset % 3) * ({T})0.5);
}}
"""

ND_CASES = [
    # dim, shape, type, inplace
    (2, [2, 8, 6, 3], 0, False),
    (2, [1, 12, 10, 2], 0, True),
    (2, [2, 16, 6, 3], 1, False),
    (2, [3, 10, 4, 2], 1, True),
    (2, [2, 16, 6, 3], 2, False),
    (2, [1, 12, 5, 2], 2, True),
    (3, [1, 8, 6, 4, 2], 0, False),
    (3, [2, 8, 4, 6, 2], 1, False),
    (3, [1, 6, 4, 4, 3], 2, False),
]


@pytest.fixture(scope='module')
def nd_cache(bb, torch_cuda):
    """One JIT cache for the nd callback tests: they need four distinct kernels per precision
    (c2c with load, c2c with store, r2c with load, c2r with store)."""
    return bb.Cache()


@pytest.mark.parametrize('which', ['both', 'load', 'store'])
@pytest.mark.parametrize('prec', [4, 8])
@pytest.mark.parametrize('case', ND_CASES, ids=['x'.join(map(str, c[1])) + ['-c2c', '-r2c', '-c2r'][c[2]]
                                                + ('-inplace' if c[3] else '') for c in ND_CASES])
def test_nd_callbacks(bb, po, torch_cuda, nd_cache, case, prec, which):
    """nd plans with callbacks (the reference rejects them, src/common/algorithm/nd_fft.hpp:29-31):
    the load function weights every input element by its input-tensor offset, the store
    function every output element by its output-tensor offset; against the FP64 DFT of the
    weighted input, weighted at the output."""
    torch = torch_cuda
    dim, shape, type, inplace = case
    T, T2 = _types(prec)
    src = ND_SRC.format(T=T, T2=T2)
    load = 'load_w' if which in ('both', 'load') else None
    store = 'store_w' if which in ('both', 'store') else None
    d = bb.BACKWARD if type == 2 else bb.FORWARD
    cfg = bb.configuration(dim, shape, precision=prec, type=type, direction=d, inplace=inplace,
                           callbacks=(src, load, store))
    ist, ost = list(cfg.istride), list(cfg.ostride)
    n1in = shape[1] // 2 + 1 if type == 2 else shape[1]
    n1out = shape[1] // 2 + 1 if type == 1 else shape[1]
    ishape = [shape[0], n1in] + shape[2:dim + 2]
    oshape = [shape[0], n1out] + shape[2:dim + 2]
    isize = po.tensor_size(dim, ishape, ist)
    osize = po.tensor_size(dim, oshape, ost)
    rdt, cdt = dtypes(prec)
    rng = np.random.default_rng(sum(shape) * 7 + type + prec)
    if type == 1:
        x = rng.standard_normal(isize).astype(rdt)
    else:
        x = (rng.standard_normal(isize) + 1j * rng.standard_normal(isize)).astype(cdt)
    plan = bb.Plan(cfg, stream=torch.cuda.current_stream().cuda_stream, cache=nd_cache)
    out = run(bb, torch, cfg, x, osize, rdt if type == 2 else cdt, inplace=inplace, plan=plan)
    xw = x.astype(np.float64 if type == 1 else np.complex128)
    if load:
        xw = xw * (1.0 + (np.arange(isize) % 5) * 0.25)
    ref = po.dft64(dim, shape, type, d, po.gather(xw, dim, ishape, ist))
    if store:
        ref = ref * (1.0 + (po.gather(np.arange(osize), dim, oshape, ost) % 3) * 0.5)
    got = po.gather(out, dim, oshape, ost)
    assert rel_l2(got, ref) <= TOL[prec]
    info = plan.info()
    assert info.num_launches == dim and info.jit_compiled == 1
