"""CPU emulation of the Bluestein tile (csrc/bluestein.cu) for every length L it runs.

The kernel's stage schedule (radices and threads per transform of each L, the Stockham
read / write indices, the per-stage twiddle table [r - 1][b mod Ns], the zero upper half of
the first stage's inputs and the unused upper half of the last stage's outputs) and the
plan's tables (chirp, FFT_L(b) / L, stage twiddles) are restated in numpy and checked against a
float64 DFT of each complex length Nc with a prime factor above 61 (no GPU)."""
import numpy as np
import pytest

SHAPE = {256: (16, [16, 16]), 512: (64, [8, 8, 8]), 1024: (64, [16, 16, 4])}


def bluestein_length(nc):
    L = 256
    while L < 2 * nc - 1:
        L *= 2
    return L


def tables(nc, L):
    """chirp, FFT_L(b) / L and the stage twiddles (per stage s >= 1, [r - 1][kk])."""
    n = np.arange(nc)
    chirp = np.exp(-1j * np.pi * ((n * n) % (2 * nc)) / nc)
    b = np.zeros(L, dtype=complex)
    b[:nc] = np.conj(chirp)
    b[L - nc + 1:] = np.conj(chirp[1:])[::-1]
    bhat = np.fft.fft(b) / L
    radices = SHAPE[L][1]
    tw, Ns = [], radices[0]
    for R in radices[1:]:
        e = np.outer(np.arange(1, R), np.arange(Ns)) * (L // (Ns * R))
        tw.append(np.exp(-2j * np.pi * e.ravel() / L))
        Ns *= R
    return chirp, bhat, [None] + tw


def stage(x, L, R, Ns, tw, half_in=False, half_out=False):
    """One radix-R stage as the kernel runs it (every butterfly b of nb = L / R)."""
    nb = L // R
    b = np.arange(nb)
    kk = b % Ns
    v = np.zeros((nb, R), dtype=complex)
    for r in range(R):
        if half_in and r >= R // 2:
            continue
        t = x[b + r * nb]
        if Ns > 1 and r > 0:
            t = t * tw[(r - 1) * Ns + kk]
        v[:, r] = t
    V = np.fft.fft(v, axis=1)  # the radix-R butterfly (dft<R>)
    out = np.full(L, np.nan + 0j)
    o = (b // Ns) * Ns * R + kk
    for r in range(R // 2 if half_out else R):
        out[o + r * Ns] = V[:, r]
    return out


def tile(x, nc):
    L = bluestein_length(nc)
    T, radices = SHAPE[L]
    chirp, bhat, tw = tables(nc, L)
    a = np.zeros(L, dtype=complex)
    a[:nc] = x * chirp
    # forward transform: first stage from the loads, last stage times bhat, conjugated
    s, Ns = a, 1
    for i, R in enumerate(radices):
        s = stage(s, L, R, Ns, tw[i], half_in=(i == 0))
        Ns *= R
    s = np.conj(s * bhat)
    Ns = 1
    for i, R in enumerate(radices):
        s = stage(s, L, R, Ns, tw[i], half_out=(i == len(radices) - 1))
        Ns *= R
    return np.conj(s[:nc]) * chirp


def big_prime_nc():
    def lpf(n):
        p, best = 2, 1
        while p * p <= n:
            while n % p == 0:
                best, n = p, n // p
            p += 1
        return max(best, n)
    return [n for n in range(67, 513) if lpf(n) > 61]


def test_shapes_cover_every_length():
    for nc in big_prime_nc():
        L = bluestein_length(nc)
        assert L in SHAPE and L // 2 >= nc
        T, radices = SHAPE[L]
        assert int(np.prod(radices)) == L
        # 256 threads per tile; every stage gives each thread whole rounds of butterflies
        assert 256 % T == 0 and all((L // R) % T == 0 for R in radices)


@pytest.mark.parametrize('nc', [67, 127, 131, 251, 257, 383, 509, 134, 254, 502])
def test_tile_emulation_matches_dft(nc):
    rng = np.random.default_rng(nc)
    x = rng.standard_normal(nc) + 1j * rng.standard_normal(nc)
    got = tile(x, nc)
    ref = np.fft.fft(x)
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12


def test_every_big_prime_length_quick():
    rng = np.random.default_rng(7)
    for nc in big_prime_nc()[::7]:
        x = rng.standard_normal(nc) + 1j * rng.standard_normal(nc)
        got = tile(x, nc)
        ref = np.fft.fft(x)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12, nc


@pytest.mark.parametrize('nc', [67, 131, 509])
def test_paired_real_transforms(nc):
    """Odd real N: the kernel's two-for-one forms (r2c: z = x0 + i x1, spectra split from
    Z_k and conj Z_{N-k}; c2r: forward transform of A - i B with A, B the conjugated
    Hermitian extensions, x0 = Re, x1 = -Im) restated with the emulated tile."""
    rng = np.random.default_rng(nc + 1)
    x0, x1 = rng.standard_normal(nc), rng.standard_normal(nc)
    Z = tile(x0 + 1j * x1, nc)
    k = np.arange(nc // 2 + 1)
    zn = Z[(nc - k) % nc]
    X0 = 0.5 * (Z[k] + np.conj(zn))
    X1 = -0.5j * (Z[k] - np.conj(zn))
    assert np.allclose(X0, np.fft.rfft(x0), atol=1e-10)
    assert np.allclose(X1, np.fft.rfft(x1), atol=1e-10)
    # c2r: Hermitian extensions of X0, X1, conjugated as the engine's load returns them
    ext = lambda X: np.concatenate([X, np.conj(X[1:][::-1][:nc - len(X)])])
    A, B = np.conj(ext(X0)), np.conj(ext(X1))
    Y = tile(A - 1j * B, nc)
    assert np.allclose(Y.real, x0 * nc, atol=1e-9)
    assert np.allclose(-Y.imag, x1 * nc, atol=1e-9)
