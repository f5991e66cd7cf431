"""CPU emulation of the Bluestein tile (csrc/bluestein.cu) for every length L it runs.

The kernel's stage schedule (radices and threads per transform of each L, the Stockham
read / write indices, the twiddle index r (b mod Ns) L / (Ns R), the zero upper half of
the first stage's inputs and the unused upper half of the last stage's outputs) and the
plan's tables (chirp, FFT_L(b) / L, w_L) are restated in numpy and checked against a
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
    n = np.arange(nc)
    chirp = np.exp(-1j * np.pi * ((n * n) % (2 * nc)) / nc)
    b = np.zeros(L, dtype=complex)
    b[:nc] = np.conj(chirp)
    b[L - nc + 1:] = np.conj(chirp[1:])[::-1]
    bhat = np.fft.fft(b) / L
    wL = np.exp(-2j * np.pi * np.arange(L) / L)
    return chirp, bhat, wL


def stage(x, L, R, Ns, wL, half_in=False, half_out=False):
    """One radix-R stage as the kernel runs it (every butterfly b of nb = L / R)."""
    nb = L // R
    b = np.arange(nb)
    kk = b % Ns
    tws = L // (Ns * R)
    v = np.zeros((nb, R), dtype=complex)
    for r in range(R):
        if half_in and r >= R // 2:
            continue
        t = x[b + r * nb]
        if Ns > 1 and r > 0:
            t = t * wL[r * kk * tws]
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
    chirp, bhat, wL = tables(nc, L)
    a = np.zeros(L, dtype=complex)
    a[:nc] = x * chirp
    # forward transform: first stage from the loads, last stage times bhat, conjugated
    s, Ns = a, 1
    for i, R in enumerate(radices):
        s = stage(s, L, R, Ns, wL, half_in=(i == 0))
        Ns *= R
    s = np.conj(s * bhat)
    Ns = 1
    for i, R in enumerate(radices):
        s = stage(s, L, R, Ns, wL, half_out=(i == len(radices) - 1))
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
