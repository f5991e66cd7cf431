"""GPU parity of the 1d and nd plans with the reference's own device tests and the oracle.

Known-answer cases restate test/c2c.cpp, test/r2c.cpp (1d..3d) of the reference; random
cases compare with the C restatement of the reference algorithm in FP64 (oracle/) and
require rel-L2 <= 2e-6 (float) / 1e-14 (double) as the benchmark spec's tolerances state.
The element-wise check uses the reference's tolerance tol(N) = 100 eps sqrt(N)
(test/fft.hpp:17-20) with doctest's Approx semantics |a-b| < tol (1 + max(|a|,|b|))."""
import numpy as np
import pytest

from gpu_helpers import TOL, dtypes, rel_l2, run

pytestmark = pytest.mark.gpu

PRECS = [4, 8]


def approx_ok(a, ref, eps):
    a = np.asarray(a)
    ref = np.asarray(ref)
    for part in (np.real, np.imag):
        x, r = part(a).astype(np.float64), part(ref).astype(np.float64)
        bound = eps * (1.0 + np.maximum(np.abs(x), np.abs(r)))
        if not np.all(np.abs(x - r) < bound):
            i = np.argmax(np.abs(x - r) - bound)
            return False, (i, x.ravel()[i], r.ravel()[i])
    return True, None


def tol(prec, N):
    eps = np.finfo(np.float32 if prec == 4 else np.float64).eps
    return 100.0 * eps * np.sqrt(N)


# ---------------------------------------------------------------- c2c (test/c2c.cpp)

C2C_M = [1, 2, 3, 16, 17, 64, 256, 1024]
C2C_N = [2, 3, 5, 7, 11, 13, 4, 8, 16, 32, 128, 256, 512, 27, 63, 105, 363]


@pytest.mark.parametrize('prec', PRECS)
@pytest.mark.parametrize('K', [1, 32])
@pytest.mark.parametrize('N', C2C_N)
def test_c2c_forward_known_answer(bb, po, torch_cuda, prec, K, N):
    """reference test/c2c.cpp:53-66 (in-place, default layout)"""
    torch = torch_cuda
    for M in C2C_M:
        x, X = po.c2c_known_answer(M, N, K, prec)
        cfg = bb.configuration(1, [M, N, K], precision=prec)
        out = run(bb, torch, cfg, x.ravel(), x.size, dtypes(prec)[1], inplace=True)
        ok, where = approx_ok(out.reshape(K, N, M), X, tol(prec, N))
        assert ok, (M, N, K, where)


@pytest.mark.parametrize('prec', PRECS)
@pytest.mark.parametrize('N', [6, 17, 102])
@pytest.mark.parametrize('M', [1, 32])
def test_c2c_non_packed(bb, po, torch_cuda, prec, N, M):
    """reference test/c2c.cpp:68-82: stride {1, M+1, (M+1)(N+1)}, K = 33"""
    torch = torch_cuda
    K = 33
    stride = [1, M + 1, (M + 1) * (N + 1), 0, 0]
    x, X = po.c2c_known_answer(M, N, K, prec)
    size = po.tensor_size(1, [M, N, K], stride)
    xf = po.scatter(x, 1, [M, N, K], stride, size, dtypes(prec)[1])
    cfg = bb.configuration(1, [M, N, K], precision=prec, istride=stride, ostride=stride)
    out = run(bb, torch, cfg, xf, size, dtypes(prec)[1], inplace=True)
    ok, where = approx_ok(po.gather(out, 1, [M, N, K], stride), X, tol(prec, N))
    assert ok, where


@pytest.mark.parametrize('prec', PRECS)
@pytest.mark.parametrize('N', [5, 63, 92])
@pytest.mark.parametrize('M', [1, 32])
def test_c2c_identity(bb, torch_cuda, prec, N, M):
    """reference test/c2c.cpp:84-127: backward(forward(x)) / N == x"""
    torch = torch_cuda
    K = 16
    rng = np.random.default_rng(1000 + N + M)
    x = (rng.uniform(0, 1, M * N * K) + 1j * rng.uniform(0, 1, M * N * K)).astype(dtypes(prec)[1])
    f = bb.configuration(1, [M, N, K], precision=prec, direction=bb.FORWARD)
    b = bb.configuration(1, [M, N, K], precision=prec, direction=bb.BACKWARD)
    y = run(bb, torch, f, x, x.size, dtypes(prec)[1], inplace=True)
    z = run(bb, torch, b, y, x.size, dtypes(prec)[1], inplace=True)
    ok, where = approx_ok(x, z / N, tol(prec, N))
    assert ok, where


# ---------------------------------------------------------------- r2c / c2r (test/r2c.cpp)

def _r2c_case(bb, po, torch, prec, M, Ns, K, inplace):
    dim = len(Ns)
    shape = [M] + list(Ns) + [K]
    cfg = bb.configuration(dim, shape, precision=prec, type=bb.R2C, inplace=inplace)
    ist, ost = list(cfg.istride), list(cfg.ostride)
    x, X = po.r2c_known_answer(M, Ns, K, prec)
    ishape = list(shape)
    if inplace:
        ishape[1] = 2 * (Ns[0] // 2 + 1)
    xs = np.zeros([K] + ([ishape[d + 1] for d in range(dim)][::-1]) + [M], dtype=x.dtype)
    xs[tuple([slice(None)] * dim + [slice(0, Ns[0])] + [slice(None)])] = x
    isize = po.tensor_size(dim, ishape, ist)
    xf = po.scatter(xs, dim, ishape, ist, isize, dtypes(prec)[0])
    oshape = list(shape)
    oshape[1] = Ns[0] // 2 + 1
    osize = po.tensor_size(dim, oshape, ost)
    out = run(bb, torch, cfg, xf, osize, dtypes(prec)[1], inplace=inplace)
    got = po.gather(out, dim, oshape, ost)
    ok, where = approx_ok(got, X, tol(prec, int(np.prod(Ns))))
    assert ok, (M, Ns, K, inplace, where)


def _c2r_case(bb, po, torch, prec, M, Ns, K, inplace, pollute=False):
    dim = len(Ns)
    shape = [M] + list(Ns) + [K]
    cfg = bb.configuration(dim, shape, precision=prec, type=bb.C2R, direction=bb.BACKWARD,
                           inplace=inplace)
    ist, ost = list(cfg.istride), list(cfg.ostride)
    X, y = po.c2r_known_answer(M, Ns, K, prec, pollute_0=pollute)
    ishape = list(shape)
    ishape[1] = Ns[0] // 2 + 1
    isize = po.tensor_size(dim, ishape, ist)
    Xf = po.scatter(X, dim, ishape, ist, isize, dtypes(prec)[1])
    oshape = list(shape)
    if inplace:
        oshape[1] = 2 * (Ns[0] // 2 + 1)
    osize = po.tensor_size(dim, oshape, ost)
    out = run(bb, torch, cfg, Xf, osize, dtypes(prec)[0], inplace=inplace)
    got = po.gather(out, dim, oshape, ost)
    got = got[tuple([slice(None)] * dim + [slice(0, Ns[0])] + [slice(None)])]
    ok, where = approx_ok(got, y, tol(prec, int(np.prod(Ns))))
    assert ok, (M, Ns, K, inplace, where)


@pytest.mark.parametrize('prec', PRECS)
@pytest.mark.parametrize('N', [2, 4, 5, 8, 27, 16, 32, 128, 105, 256, 512, 102, 220, 10, 26])
def test_r2c_1d_out_of_place(bb, po, torch_cuda, prec, N):
    """reference test/r2c.cpp:182-192"""
    for K in (1, 33):
        for M in (1, 3, 32):
            _r2c_case(bb, po, torch_cuda, prec, M, [N], K, False)


@pytest.mark.parametrize('prec', PRECS)
@pytest.mark.parametrize('N', [4, 12, 13, 110])
def test_r2c_1d_in_place(bb, po, torch_cuda, prec, N):
    """reference test/r2c.cpp:194-203"""
    for M in (1, 3):
        _r2c_case(bb, po, torch_cuda, prec, M, [N], 65, True)


@pytest.mark.parametrize('prec', PRECS)
@pytest.mark.parametrize('Ns,inplace', [((4, 8), True), ((8, 5), True), ((5, 4), False),
                                        ((10, 3), False), ((4, 8, 2), True), ((8, 256, 5), True),
                                        ((5, 4, 6), False), ((10, 286, 3), False)])
def test_r2c_nd(bb, po, torch_cuda, prec, Ns, inplace):
    """reference test/r2c.cpp:205-250"""
    for K in (1, 33) if inplace else (1, 65):
        for M in (1, 3) if inplace else (1, 7):
            _r2c_case(bb, po, torch_cuda, prec, M, list(Ns), K, inplace)


@pytest.mark.parametrize('prec', PRECS)
@pytest.mark.parametrize('N', [11, 16, 25, 96, 256, 300, 315])
def test_c2r_1d_out_of_place(bb, po, torch_cuda, prec, N):
    """reference test/r2c.cpp:299-308"""
    for M in (1, 5, 32):
        _c2r_case(bb, po, torch_cuda, prec, M, [N], 33, False)


@pytest.mark.parametrize('prec', PRECS)
@pytest.mark.parametrize('N', [5, 16, 21, 48, 512])
def test_c2r_1d_in_place_polluted_0(bb, po, torch_cuda, prec, N):
    """reference test/r2c.cpp:310-324: imag(X[0]) must be ignored"""
    _c2r_case(bb, po, torch_cuda, prec, 1, [N], 33, True, pollute=True)


@pytest.mark.parametrize('prec', PRECS)
@pytest.mark.parametrize('Ns,inplace', [((4, 2), True), ((96, 96), True), ((4, 8, 2), True),
                                        ((96, 96, 80), True), ((5, 4), False), ((10, 3), False),
                                        ((5, 4, 6), False), ((10, 286, 3), False)])
def test_c2r_nd(bb, po, torch_cuda, prec, Ns, inplace):
    """reference test/r2c.cpp:326-372"""
    for K in ((1, 54) if inplace else (1, 65)):
        for M in ((1, 3) if inplace else (1, 7)):
            if np.prod(Ns) * K * M > 4_000_000:
                continue  # keep the largest 3d case at K=1/M=1..3 within test time
            _c2r_case(bb, po, torch_cuda, prec, M, list(Ns), K, inplace)


@pytest.mark.parametrize('prec', PRECS)
@pytest.mark.parametrize('Ns,K,M,inplace', [((8,), 16, 1, True), ((64,), 16, 8, True),
                                             ((212,), 16, 8, True), ((135,), 7, 8, True),
                                             ((509,), 5, 4, True), ((8,), 16, 1, False),
                                             ((64,), 16, 8, False), ((212,), 16, 1, False),
                                             ((8, 8, 8), 11, 7, True), ((96, 96, 80), 1, 1, True)])
def test_real_identity(bb, po, torch_cuda, prec, Ns, K, M, inplace):
    """reference test/r2c.cpp:376-497: c2r(r2c(x)) / prod(N) == x"""
    torch = torch_cuda
    dim = len(Ns)
    shape = [M] + list(Ns) + [K]
    f = bb.configuration(dim, shape, precision=prec, type=bb.R2C, inplace=inplace)
    b = bb.configuration(dim, shape, precision=prec, type=bb.C2R, direction=bb.BACKWARD,
                         inplace=inplace)
    rng = np.random.default_rng(7 + sum(Ns) + K + M)
    ishape = list(shape)
    if inplace:
        ishape[1] = 2 * (Ns[0] // 2 + 1)
    isize = po.tensor_size(dim, ishape, list(f.istride))
    x = rng.uniform(0, 1, isize).astype(dtypes(prec)[0])
    oshape = list(shape)
    oshape[1] = Ns[0] // 2 + 1
    osize = po.tensor_size(dim, oshape, list(f.ostride))
    X = run(bb, torch, f, x, osize if not inplace else osize, dtypes(prec)[1], inplace=inplace)
    if inplace:
        y = run(bb, torch, b, X, isize, dtypes(prec)[0], inplace=True)
    else:
        y = run(bb, torch, b, X, isize, dtypes(prec)[0])
    xd = po.gather(x, dim, shape, list(f.istride))
    yd = po.gather(y, dim, shape, list(b.ostride))
    ok, where = approx_ok(xd, yd / np.prod(Ns), tol(prec, int(np.prod(Ns))))
    assert ok, where


# ---------------------------------------------------------------- random vs oracle

RANDOM_N = list(range(1, 65)) + [72, 81, 96, 100, 121, 128, 136, 160, 169, 192, 224, 243, 256,
                                 289, 320, 361, 384, 400, 472, 480, 488, 500, 509, 512]


@pytest.mark.parametrize('prec', PRECS)
@pytest.mark.parametrize('type', [0, 1, 2])
def test_random_vs_oracle(bb, po, torch_cuda, prec, type):
    """Every N in 1..64 and a spread of larger N (primes, prime powers, the ragged set),
    random double batching, against the oracle in FP64: rel-L2 within the north-star
    tolerance."""
    torch = torch_cuda
    rng = np.random.default_rng(42 + type + prec)
    rdt, cdt = dtypes(prec)
    worst = 0.0
    for N in RANDOM_N:
        if type != 0 and N == 1:
            continue
        M = int(rng.choice([1, 2, 5, 8, 33]))
        K = int(rng.integers(1, 40))
        for direction in ([bb.FORWARD, bb.BACKWARD] if type == 0 else [None]):
            d = direction if type == 0 else (bb.FORWARD if type == 1 else bb.BACKWARD)
            cfg = bb.configuration(1, [M, N, K], precision=prec, type=type, direction=d)
            nin = N // 2 + 1 if type == 2 else N
            nout = N // 2 + 1 if type == 1 else N
            if type == 1:
                x = rng.standard_normal(M * nin * K).astype(rdt)
            else:
                x = (rng.standard_normal(M * nin * K) + 1j * rng.standard_normal(M * nin * K)).astype(cdt)
            out = run(bb, torch, cfg, x, M * nout * K, rdt if type == 2 else cdt)
            ref = po.oracle_fft(1, [M, N, K], type, d, x.astype(np.complex128 if type != 1 else np.float64), prec=8)
            e = rel_l2(out, ref)
            worst = max(worst, e)
            assert e <= TOL[prec], (N, M, K, direction, e)
    print('worst rel-L2', worst)


# ------------------------------------------------- full benchmark sizes (1 GiB per pass)

SWEEP_N = [16, 32, 64, 128, 256, 512, 48, 96, 160, 224, 384, 7, 11, 13]


@pytest.mark.parametrize('N', SWEEP_N)
def test_full_size_round_trip(bb, po, torch_cuda, N):
    """At the benchmark's full size (float, M=8, K = 2^30 / (4 * 8 * N), 1 GiB real input):
    c2r(r2c(x)) = N x to rel-L2 <= 2e-6, and 24 sampled k-slices of the r2c output equal
    the FP64 transform of those slices (rel-L2 <= 2e-6) and the oracle."""
    torch = torch_cuda
    M, K = 8, (1 << 30) // (4 * 8 * N)
    nc = N // 2 + 1
    stream = torch.cuda.current_stream().cuda_stream
    g = torch.Generator(device='cuda')
    g.manual_seed(N)
    x = torch.randn(M * N * K, device='cuda', generator=g)
    X = torch.empty(2 * M * nc * K, device='cuda')
    y = torch.empty(M * N * K, device='cuda')
    fwd = bb.Plan(bb.configuration(1, [M, N, K], precision=bb.F32, type=bb.R2C), stream=stream)
    bwd = bb.Plan(bb.configuration(1, [M, N, K], precision=bb.F32, type=bb.C2R,
                                   direction=bb.BACKWARD), stream=stream)
    fwd.execute(x.data_ptr(), X.data_ptr())
    bwd.execute(X.data_ptr(), y.data_ptr())
    torch.cuda.synchronize()
    err = float(torch.linalg.vector_norm(y / N - x) / torch.linalg.vector_norm(x))
    assert err <= 2e-6, err
    ks = np.random.default_rng(N).choice(K, 24, replace=False)
    ks = torch.tensor(np.sort(ks), device='cuda')
    xs = x.view(K, N * M)[ks].cpu().numpy()
    Xs = torch.view_as_complex(X.view(K, nc * M, 2)[ks]).cpu().numpy()
    ref = po.dft64(1, [M, N, 24], po.R2C, po.FORWARD, xs.reshape(24, N, M))
    assert rel_l2(Xs.reshape(ref.shape), ref) <= 2e-6
    orc = po.oracle_fft(1, [M, N, 24], po.R2C, po.FORWARD, xs.ravel(), prec=4)
    assert rel_l2(Xs.ravel(), orc) <= 2e-6
    del x, X, y
    torch.cuda.empty_cache()


@pytest.mark.parametrize('type', [0, 1, 2])
def test_plans_of_the_ragged_lengths(bb, po, torch_cuda, type):
    """Float plans of every N in {16, 24, ..., 512} (the lengths the ragged tile functions
    cover, incl. the prime factors 17..61), forward and backward, against the oracle in FP64."""
    torch = torch_cuda
    rng = np.random.default_rng(7 + type)
    for N in range(16, 513, 8):
        M = int(rng.choice([1, 3, 8]))
        K = int(rng.integers(1, 20))
        for d in ([bb.FORWARD, bb.BACKWARD] if type == 0 else [bb.BACKWARD if type == 2 else bb.FORWARD]):
            cfg = bb.configuration(1, [M, N, K], precision=bb.F32, type=type, direction=d)
            nin = N // 2 + 1 if type == 2 else N
            nout = N // 2 + 1 if type == 1 else N
            if type == 1:
                x = rng.standard_normal(M * N * K).astype(np.float32)
            else:
                x = (rng.standard_normal(M * nin * K) + 1j * rng.standard_normal(M * nin * K)).astype(np.complex64)
            out = run(bb, torch, cfg, x, M * nout * K, np.float32 if type == 2 else np.complex64)
            ref = po.oracle_fft(1, [M, N, K], type, d, x.astype(np.complex128 if type != 1 else np.float64), prec=8)
            e = rel_l2(out, ref)
            assert e <= TOL[4], (N, M, K, d, e)


def _largest_prime_factor(n):
    f, p = 1, 2
    while n > 1:
        if n % p == 0:
            f = p
            n //= p
        else:
            p += 1
    return f


# every length up to 512 with a prime factor 17..61 (the tensor-core prime stages of the
# float engines), each once as c2c, r2c and c2r
PRIME_TC_N = [n for n in range(17, 513) if 17 <= _largest_prime_factor(n) <= 61]


@pytest.mark.parametrize('type', [0, 1, 2])
def test_prime_factor_lengths(bb, po, torch_cuda, type):
    """Float plans of every N <= 512 whose largest prime factor is 17..61 (stages on the
    tensor cores with split TF32 operands), random double batching, against the oracle in
    FP64 within the float tolerance."""
    torch = torch_cuda
    rng = np.random.default_rng(11 + type)
    worst = 0.0
    for N in PRIME_TC_N:
        M = int(rng.choice([1, 2, 4, 8, 16]))
        K = int(rng.integers(1, 24))
        d = bb.BACKWARD if type == 2 else (bb.FORWARD if type == 1 else
                                           int(rng.choice([bb.FORWARD, bb.BACKWARD])))
        cfg = bb.configuration(1, [M, N, K], precision=bb.F32, type=type, direction=d)
        nin = N // 2 + 1 if type == 2 else N
        nout = N // 2 + 1 if type == 1 else N
        if type == 1:
            x = rng.standard_normal(M * nin * K).astype(np.float32)
        else:
            x = (rng.standard_normal(M * nin * K) + 1j * rng.standard_normal(M * nin * K)).astype(np.complex64)
        out = run(bb, torch, cfg, x, M * nout * K, np.float32 if type == 2 else np.complex64)
        ref = po.oracle_fft(1, [M, N, K], type, d, x.astype(np.complex128 if type != 1 else np.float64), prec=8)
        e = rel_l2(out, ref)
        worst = max(worst, e)
        assert e <= TOL[4], (N, M, K, d, e)
    print('worst rel-L2', worst)


# every odd length 17..511 with prime factors <= 61 (compile-time tiles that run two real
# transforms along K per complex FFT)
ODD_REAL_N = [n for n in range(17, 512, 2) if _largest_prime_factor(n) <= 61]


@pytest.mark.parametrize('type', [1, 2])
def test_odd_real_lengths_paired(bb, po, torch_cuda, type):
    """Float r2c / c2r of every odd N <= 511 with prime factors <= 61, random double
    batching with odd and even K (the last pair of an odd K has one transform), against
    the oracle in FP64 within the float tolerance."""
    torch = torch_cuda
    rng = np.random.default_rng(31 + type)
    worst = 0.0
    for N in ODD_REAL_N:
        M = int(rng.choice([1, 2, 3, 8]))
        K = int(rng.integers(1, 10))
        d = bb.BACKWARD if type == 2 else bb.FORWARD
        cfg = bb.configuration(1, [M, N, K], precision=bb.F32, type=type, direction=d)
        nin = N // 2 + 1 if type == 2 else N
        nout = N // 2 + 1 if type == 1 else N
        if type == 1:
            x = rng.standard_normal(M * nin * K).astype(np.float32)
        else:
            x = (rng.standard_normal(M * nin * K) + 1j * rng.standard_normal(M * nin * K)).astype(np.complex64)
        out = run(bb, torch, cfg, x, M * nout * K, np.float32 if type == 2 else np.complex64)
        ref = po.oracle_fft(1, [M, N, K], type, d, x.astype(np.complex128 if type != 1 else np.float64), prec=8)
        e = rel_l2(out, ref)
        worst = max(worst, e)
        assert e <= TOL[4], (N, M, K, e)
    print('worst rel-L2', worst)


# every length up to 512 with a prime factor above 61 (float: the Bluestein kernel, one
# shared-memory layout per transforms-per-tile count Mb = 1..4)
BIG_PRIME_N = [n for n in range(67, 513) if _largest_prime_factor(n) > 61]


@pytest.mark.parametrize('type', [0, 1, 2])
def test_big_prime_factor_lengths(bb, po, torch_cuda, type):
    """Float plans of every N <= 512 whose largest prime factor is above 61, random double
    batching, against the oracle in FP64 within the float tolerance."""
    torch = torch_cuda
    rng = np.random.default_rng(21 + type)
    worst = 0.0
    for N in BIG_PRIME_N:
        M = int(rng.choice([1, 2, 3, 8, 16]))
        K = int(rng.integers(1, 12))
        d = bb.BACKWARD if type == 2 else (bb.FORWARD if type == 1 else
                                           int(rng.choice([bb.FORWARD, bb.BACKWARD])))
        cfg = bb.configuration(1, [M, N, K], precision=bb.F32, type=type, direction=d)
        nin = N // 2 + 1 if type == 2 else N
        nout = N // 2 + 1 if type == 1 else N
        if type == 1:
            x = rng.standard_normal(M * nin * K).astype(np.float32)
        else:
            x = (rng.standard_normal(M * nin * K) + 1j * rng.standard_normal(M * nin * K)).astype(np.complex64)
        out = run(bb, torch, cfg, x, M * nout * K, np.float32 if type == 2 else np.complex64)
        ref = po.oracle_fft(1, [M, N, K], type, d, x.astype(np.complex128 if type != 1 else np.float64), prec=8)
        e = rel_l2(out, ref)
        worst = max(worst, e)
        assert e <= TOL[4], (N, M, K, d, e)
    print('worst rel-L2', worst)


@pytest.mark.parametrize('type,N,M', [(1, 160, 8), (2, 160, 8), (0, 64, 1), (2, 384, 8), (1, 96, 8)])
def test_tuned_variants_agree(bb, po, torch_cuda, type, N, M):
    """Every blocking the autotuner may pick (V, Mb, Kb, 2 or 3 resident CTAs) gives the
    FP64 transform within the float tolerance."""
    torch = torch_cuda
    rng = np.random.default_rng(N + type)
    K = 37
    d = bb.BACKWARD if type == 2 else bb.FORWARD
    cfg = bb.configuration(1, [M, N, K], precision=bb.F32, type=type, direction=d)
    nin = N // 2 + 1 if type == 2 else N
    nout = N // 2 + 1 if type == 1 else N
    if type == 1:
        x = rng.standard_normal(M * nin * K).astype(np.float32)
    else:
        x = (rng.standard_normal(M * nin * K) + 1j * rng.standard_normal(M * nin * K)).astype(np.complex64)
    ref = po.oracle_fft(1, [M, N, K], type, d, x.astype(np.float64 if type == 1 else np.complex128), prec=8)
    seen = set()
    stream = torch.cuda.current_stream().cuda_stream
    for V in (1, 2, 4):
        for Mb in (1, 4, 8):
            for Kb in (1, 4):
                for occ in (2, 3):
                    try:
                        plan = bb.Plan(cfg, stream=stream, tuning=(None, 0, V, Mb, Kb, occ))
                    except bb.BBFFTError:
                        continue
                    i = plan.info()
                    key = (i.vector_width, i.mb, i.kb, i.min_blocks)
                    if key in seen:
                        continue
                    seen.add(key)
                    out = run(bb, torch, cfg, x, M * nout * K, np.float32 if type == 2 else np.complex64,
                              plan=plan)
                    assert rel_l2(out, ref) <= TOL[4], key
    assert any(k[3] == 3 for k in seen) and any(k[3] == 2 for k in seen)


ND_STRIDED = [
    # dim, shape, type, istride, ostride
    (2, [1, 8, 8, 2], 0, [1, 1, 9, 80, 0], [1, 1, 9, 80, 0]),           # padded rows
    (2, [3, 12, 10, 4], 0, [1, 40, 3, 600, 0], [1, 3, 36, 360, 0]),     # transposed N1/N2 input
    (2, [2, 16, 6, 3], 1, [1, 2, 40, 260, 0], [1, 2, 18, 120, 0]),      # r2c, padded
    (2, [2, 16, 6, 3], 2, [1, 2, 20, 130, 0], [1, 2, 36, 260, 0]),      # c2r, padded
    (3, [1, 8, 6, 4, 2], 0, [1, 1, 10, 70, 300], [1, 1, 8, 48, 192]),   # 3d c2c
]


@pytest.mark.parametrize('prec', PRECS)
@pytest.mark.parametrize('case', ND_STRIDED, ids=[str(c[1]) + str(c[2]) for c in ND_STRIDED])
def test_nd_custom_layouts(bb, po, torch_cuda, prec, case):
    """nd transforms with custom strides (a strided gather and scatter around the packed
    chain), against the FP64 DFT of the gathered tensor."""
    torch = torch_cuda
    dim, shape, type, ist, ost = case
    d = bb.BACKWARD if type == 2 else bb.FORWARD
    cfg = bb.configuration(dim, shape, precision=prec, type=type, direction=d, istride=ist, ostride=ost)
    n1in = shape[1] // 2 + 1 if type == 2 else shape[1]
    n1out = shape[1] // 2 + 1 if type == 1 else shape[1]
    ishape = [shape[0], n1in] + shape[2:dim + 2]
    oshape = [shape[0], n1out] + shape[2:dim + 2]
    isize = po.tensor_size(dim, ishape, ist)
    osize = po.tensor_size(dim, oshape, ost)
    rdt, cdt = dtypes(prec)
    rng = np.random.default_rng(sum(shape) + type)
    if type == 1:
        x = rng.standard_normal(isize).astype(rdt)
    else:
        x = (rng.standard_normal(isize) + 1j * rng.standard_normal(isize)).astype(cdt)
    out = run(bb, torch, cfg, x, osize, rdt if type == 2 else cdt)
    ref = po.dft64(dim, shape, type, d, po.gather(x.astype(np.float64 if type == 1 else np.complex128), dim, ishape, ist))
    got = po.gather(out, dim, oshape, ost)
    assert rel_l2(got, ref) <= TOL[prec]
    info = bb.Plan(cfg, stream=torch.cuda.current_stream().cuda_stream).info()
    assert info.num_launches == dim + 2 and info.workspace_bytes > 0


def test_transpose_fft_transpose_equals_double_batched(bb, torch_cuda):
    """reference examples/transpose_fft_transpose: transpose -> FFT over contiguous N ->
    transpose equals one double-batched plan over the M x N x K layout."""
    torch = torch_cuda
    M, N, K = 16, 64, 40
    s = torch.cuda.current_stream().cuda_stream
    x = torch.randn(K, N, M, dtype=torch.complex64, device='cuda')
    y = torch.empty_like(x)
    bb.Plan(bb.configuration(1, [M, N, K], precision=bb.F32), stream=s).execute(x.data_ptr(), y.data_ptr())
    xt = x.permute(0, 2, 1).contiguous()
    bb.Plan(bb.configuration(1, [1, N, M * K], precision=bb.F32), stream=s).execute(xt.data_ptr())
    torch.cuda.synchronize()
    y2 = xt.permute(0, 2, 1)
    assert float(torch.linalg.vector_norm(y - y2) / torch.linalg.vector_norm(y2)) <= 1e-6


# ------------------------------------------------- nd plans run slab by slab through L2

# intermediates larger than 32 MB: with BBFFT_GB300_ND_SLAB_BYTES = 32 MB the plan runs its
# passes slab by slab along K (full slabs and a shorter last one for these K)
ND_SLABS = [
    (2, [1, 128, 128, 700], 1, False), (2, [1, 128, 128, 700], 2, False),
    (2, [1, 128, 128, 700], 1, True), (3, [1, 64, 64, 64, 20], 0, False),
    (2, [2, 96, 80, 900], 0, False),
]


@pytest.mark.parametrize('case', ND_SLABS, ids=[str(c) for c in ND_SLABS])
def test_nd_plans_in_l2_slabs(bb, po, torch_cuda, monkeypatch, case):
    """nd float plans run slab by slab along K (BBFFT_GB300_ND_SLAB_BYTES = 32 MB, smaller
    than their intermediate tensors): images at the start, inside and at the end of the
    tensor, around slab boundaries, against the oracle in FP64."""
    torch = torch_cuda
    dim, shape, type, inplace = case
    K = shape[-1]
    rng = np.random.default_rng(sum(shape) + type)
    d = bb.BACKWARD if type == 2 else bb.FORWARD
    cfg = bb.configuration(dim, shape, precision=bb.F32, type=type, direction=d, inplace=inplace)
    monkeypatch.setenv('BBFFT_GB300_ND_SLAB_BYTES', str(32 << 20))
    plan = bb.Plan(cfg, stream=torch.cuda.current_stream().cuda_stream)
    monkeypatch.delenv('BBFFT_GB300_ND_SLAB_BYTES')
    info = plan.info()
    assert info.num_launches > dim, 'expected a slabbed plan'
    ist = list(cfg.istride)[:dim + 2]
    ost = list(cfg.ostride)[:dim + 2]
    in_per_k, out_per_k = ist[dim + 1], ost[dim + 1]
    cplx_in, cplx_out = type != 1, type != 2
    n_in = in_per_k * K
    if cplx_in:
        x = (rng.standard_normal(n_in) + 1j * rng.standard_normal(n_in)).astype(np.complex64)
    else:
        x = rng.standard_normal(n_in).astype(np.float32)
    out_dt = np.complex64 if cplx_out else np.float32
    out = run(bb, torch, cfg, x, out_per_k * K, out_dt, inplace=inplace, plan=plan)
    picks = sorted(set([0, 1, K // 3, K // 2 - 1, K // 2, K - 2, K - 1]))
    sub_shape = list(shape[:-1]) + [len(picks)]
    xs = np.concatenate([x[k * in_per_k:(k + 1) * in_per_k] for k in picks])
    cfg_s = bb.configuration(dim, sub_shape, precision=bb.F32, type=type, direction=d, inplace=inplace)
    ref = po.oracle_fft(dim, sub_shape, type, d, xs.astype(np.complex128 if cplx_in else np.float64),
                        istride=ist[:dim + 1] + [in_per_k], ostride=ost[:dim + 1] + [out_per_k],
                        inplace=inplace, prec=8)
    got = np.concatenate([out[k * out_per_k:(k + 1) * out_per_k] for k in picks])
    e = rel_l2(got, ref)
    assert e <= TOL[4], e
