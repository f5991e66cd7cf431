"""CPU emulation of the tensor-core radix stage (csrc/prime_tc.cuh) with the generated
coefficient fragments (csrc/gen_prime_frags.py).

Each lane's A fragments (its butterfly's pair sums and differences, split into two TF32
pieces), the per-lane B fragments of the table and the accumulator fragments are placed
into and read out of the 16x8 / 8x8 / 16x8 matrices of mma.m16n8k8 by the fragment
layouts of the PTX ISA, so the test checks the table, the index mapping of the lanes and
the output assembly of the stage against a float64 DFT of each butterfly (no GPU)."""
import os
import sys

import numpy as np
import pytest

CSRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                    'double-batched-fft-library_gb300', 'csrc')
sys.path.insert(0, CSRC)
import gen_prime_frags as gpf  # noqa: E402


def tf32(x):
    """cvt.rna.tf32.f32 of float32 values: nearest, ties away from zero, 10 mantissa bits."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x1000) & 0xFFFFE000).astype(np.uint32)
    return u.view(np.float32)


def split(x):
    x = np.float32(x)
    hi = tf32(x)
    lo = tf32(np.float32(x - hi))
    return hi, lo


def bits(u):
    return np.array([u], dtype=np.uint32).view(np.float32)[0]


def emulate(P, xs):
    """Run the stage for 8 butterflies xs[g, r] (complex64) as the warp does."""
    H = gpf.pairs(P)
    even = P % 2 == 0
    KS = (H + 7) // 8
    frag = gpf.frags(P)  # [ks][nt][lane][2] of 4 bit patterns
    U = np.zeros((KS, 16, 8))
    W = np.zeros((KS, 16, 8))
    xs = xs.astype(np.complex64)
    for ks in range(KS):
        # A matrices (16 x 8) from the lanes: a0 (g, t), a1 (g+8, t), a2 (g, t+4), a3 (g+8, t+4)
        A = {name: np.zeros((16, 8), dtype=np.float32) for name in ('sh', 'sl', 'dh', 'dl')}
        for lane in range(32):
            g, t = lane >> 2, lane & 3
            sv, dv = [], []
            for h in range(2):
                j = 8 * ks + t + 1 + 4 * h
                if j <= H:
                    a, b = xs[g, j], xs[g, P - j]
                else:
                    a = b = np.complex64(0)
                s, d = np.complex64(a + b), np.complex64(a - b)
                sv += [s.real, s.imag]
                dv += [d.real, d.imag]
            for e, (r, c) in enumerate(((g, t), (g + 8, t), (g, t + 4), (g + 8, t + 4))):
                A['sh'][r, c], A['sl'][r, c] = split(sv[e])
                A['dh'][r, c], A['dl'][r, c] = split(dv[e])
        for nt in range(KS):
            B = {name: np.zeros((8, 8), dtype=np.float32) for name in ('ch', 'cl', 'sh', 'sl')}
            for lane in range(32):
                g, t = lane >> 2, lane & 3
                fc = frag[((ks * KS + nt) * 32 + lane) * 2]
                fs = frag[((ks * KS + nt) * 32 + lane) * 2 + 1]
                # b0 (row t, col g), b1 (row t+4, col g)
                B['ch'][t, g], B['ch'][t + 4, g] = bits(fc[0]), bits(fc[1])
                B['cl'][t, g], B['cl'][t + 4, g] = bits(fc[2]), bits(fc[3])
                B['sh'][t, g], B['sh'][t + 4, g] = bits(fs[0]), bits(fs[1])
                B['sl'][t, g], B['sl'][t + 4, g] = bits(fs[2]), bits(fs[3])
            f64 = lambda m: m.astype(np.float64)
            U[nt] += f64(A['sl']) @ f64(B['ch']) + f64(A['sh']) @ f64(B['cl']) + f64(A['sh']) @ f64(B['ch'])
            W[nt] += f64(A['dl']) @ f64(B['sh']) + f64(A['dh']) @ f64(B['sl']) + f64(A['dh']) @ f64(B['sh'])
    out = np.zeros((8, P), dtype=np.complex128)
    for lane in range(32):
        g, t = lane >> 2, lane & 3
        x0 = xs[g, 0]
        xh = xs[g, P // 2] if even else 0
        s = xs[g, 1:H + 1] + xs[g, P - H:][::-1]  # s_j, j = 1..H
        if t == 0:
            out[g, 0] = x0 + xh + s.sum()
        if even and t == 1:
            out[g, P // 2] = x0 + (-1) ** (P // 2) * xh + (s * (-1.0) ** np.arange(1, H + 1)).sum()
        for nt in range(KS):
            for e in range(2):
                k = 8 * nt + 2 * t + 1 + e
                if k <= H:
                    # accumulator entries c_e (g, 2t+e) and c_{2+e} (g+8, 2t+e)
                    ur, ui = U[nt][g, 2 * t + e], U[nt][g + 8, 2 * t + e]
                    wr, wi = W[nt][g, 2 * t + e], W[nt][g + 8, 2 * t + e]
                    b = x0 + (-1) ** k * xh
                    out[g, k] = complex(b.real + ur - wi, b.imag + ui + wr)
                    out[g, P - k] = complex(b.real + ur + wi, b.imag + ui - wr)
    return out


@pytest.mark.parametrize('P', gpf.RADICES)
def test_radix_stage_emulation_matches_dft(P):
    rng = np.random.default_rng(P)
    xs = (rng.standard_normal((8, P)) + 1j * rng.standard_normal((8, P))).astype(np.complex64)
    got = emulate(P, xs)
    ref = np.fft.fft(xs.astype(np.complex128), axis=1)
    err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    # two TF32 pieces per operand, three products: FP32-level accuracy
    assert err <= 2e-7, (P, err)


def test_fragment_pieces_carry_22_bits():
    for P in gpf.RADICES:
        H = gpf.pairs(P)
        for j in range(1, H + 1):
            for k in range(1, H + 1):
                c = np.cos(2 * np.pi * j * k / P)
                hi, lo = gpf.split(c)
                assert abs(float(bits(hi)) + float(bits(lo)) - c) <= 2.0 ** -21 * max(abs(c), 2.0 ** -4)
