"""Pins the CPU oracle (oracle/bbfft_oracle.c, the restatement of the reference's algorithm)
against the known answers of the reference's own device tests and an independent FP64 DFT.

Known answers restated from test/c2c.cpp:17-66 (delta spectra of complex exponentials),
test/r2c.cpp:28-135 (cosines <-> half deltas, 1d..3d) and the polluted imag(X[0]) case
(test/r2c.cpp:310-324); tolerance tol(N) = 100 eps sqrt(N) of test/fft.hpp:17-20 with
doctest Approx semantics.  Runs on the CPU only."""
import numpy as np
import pytest


def approx_ok(a, ref, eps):
    for part in (np.real, np.imag):
        x = part(np.asarray(a)).astype(np.float64)
        r = part(np.asarray(ref)).astype(np.float64)
        if not np.all(np.abs(x - r) < eps * (1.0 + np.maximum(np.abs(x), np.abs(r)))):
            return False
    return True


@pytest.mark.parametrize('prec', [4, 8])
@pytest.mark.parametrize('N', [2, 3, 5, 7, 11, 13, 4, 8, 16, 32, 128, 256, 512, 27, 63, 105, 363])
def test_oracle_c2c_known_answer(po, prec, N):
    """reference test/c2c.cpp:53-66 (M subset keeps the CPU run short)"""
    for M in (1, 3, 17):
        for K in (1, 32):
            x, X = po.c2c_known_answer(M, N, K, prec)
            out = po.oracle_fft(1, [M, N, K], po.C2C, po.FORWARD, x.ravel(), prec=prec)
            assert approx_ok(out.reshape(K, N, M), X, po.tol(prec, N)), (M, N, K)


@pytest.mark.parametrize('prec', [4, 8])
@pytest.mark.parametrize('Ns', [(2,), (5,), (27,), (16,), (128,), (105,), (512,), (102,), (220,),
                                (4, 8), (8, 5), (5, 4, 6), (10, 6, 3)])
def test_oracle_r2c_known_answer(po, prec, Ns):
    """reference test/r2c.cpp:182-250"""
    dim = len(Ns)
    for M in (1, 3):
        for K in (1, 33):
            x, X = po.r2c_known_answer(M, list(Ns), K, prec)
            shape = [M] + list(Ns) + [K]
            out = po.oracle_fft(dim, shape, po.R2C, po.FORWARD, x.ravel(), prec=prec)
            assert approx_ok(out.reshape(X.shape), X, po.tol(prec, int(np.prod(Ns)))), (M, Ns, K)


@pytest.mark.parametrize('prec', [4, 8])
@pytest.mark.parametrize('Ns,pollute', [((11,), False), ((16,), False), ((96,), False),
                                        ((300,), False), ((315,), False), ((5,), True),
                                        ((48,), True), ((512,), True), ((4, 2), False),
                                        ((10, 3), False), ((5, 4, 6), False)])
def test_oracle_c2r_known_answer(po, prec, Ns, pollute):
    """reference test/r2c.cpp:299-372, incl. the polluted imag(X[0]) that must be ignored"""
    dim = len(Ns)
    for M in (1, 5):
        K = 33 if dim == 1 else 2
        X, y = po.c2r_known_answer(M, list(Ns), K, prec, pollute_0=pollute)
        shape = [M] + list(Ns) + [K]
        out = po.oracle_fft(dim, shape, po.C2R, po.BACKWARD, X.ravel(), prec=prec)
        assert approx_ok(out.reshape(y.shape), y, po.tol(prec, int(np.prod(Ns)))), (M, Ns)


@pytest.mark.parametrize('type', [0, 1, 2])
def test_oracle_matches_fp64_dft(po, type):
    """Random tensors (incl. random imag(X[N/2]) for c2r) against numpy's FP64 DFT with the
    reference's c2r semantics; float oracle within 2e-6, double within 1e-14 (rel-L2)."""
    rng = np.random.default_rng(100 + type)
    for N in list(range(1, 40)) + [48, 61, 64, 96, 128, 243, 256, 509, 512]:
        if type != 0 and N == 1:
            continue
        M, K = 3, 4
        d = po.BACKWARD if type == 2 else po.FORWARD
        nin = N // 2 + 1 if type == 2 else N
        if type == 1:
            x = rng.standard_normal(M * nin * K)
        else:
            x = rng.standard_normal(M * nin * K) + 1j * rng.standard_normal(M * nin * K)
        ref = po.dft64(1, [M, N, K], type, d, x.reshape(K, nin, M))
        for prec, tol in ((8, 1e-14), (4, 2e-6)):
            xin = x.astype(np.float32 if type == 1 else np.complex64) if prec == 4 else x
            out = po.oracle_fft(1, [M, N, K], type, d, xin, prec=prec)
            assert po.rel_l2(out.reshape(ref.shape), ref) <= tol, (N, prec)


def test_oracle_identity_round_trip(po):
    """reference test/r2c.cpp:376-497 / test/c2c.cpp:84-127: backward(forward(x)) = N x"""
    rng = np.random.default_rng(9)
    for N in (8, 64, 212, 5, 63, 92):
        x = rng.uniform(0, 1, 8 * N * 16)
        X = po.oracle_fft(1, [8, N, 16], po.R2C, po.FORWARD, x)
        y = po.oracle_fft(1, [8, N, 16], po.C2R, po.BACKWARD, X)
        assert np.allclose(y / N, x, rtol=0, atol=1e-13)
