"""CPU check of the stage schedules the compile-time tiles run (csrc/engine_ct.cuh
ct_stage): for every c2c cover tile the generator emits (gen_specializations.py), the
Stockham stages over its radices — butterfly b of a radix-R stage reads elements
b + r Nc / R times w_Nc^{-r (b mod Ns) Nc / (Ns R)} and writes (b / Ns) Ns R + b mod Ns +
r Ns; radix 1 is a copy — restated in numpy give the DFT (no GPU).  This covers the
register prime orders (the prime first, then the radices of Nc / P) next to the others."""
import os
import sys

import numpy as np

from conftest import REPO

sys.path.insert(0, os.path.join(REPO, 'double-batched-fft-library_gb300', 'csrc'))
import gen_specializations as gen  # noqa: E402


def stockham(x, radices):
    n = len(x)
    w = np.exp(-2j * np.pi * np.arange(n) / n)
    ns = 1
    for r in radices:
        if r == 1:
            continue
        nb = n // r
        b = np.arange(nb)
        kk = b % ns
        v = np.stack([x[b + q * nb] * (w[(q * kk * (n // (ns * r))) % n] if ns > 1 else 1)
                      for q in range(r)], axis=1)
        y = np.fft.fft(v, axis=1)  # the radix-r butterfly
        out = np.empty(n, dtype=complex)
        o = (b // ns) * ns * r + kk
        for q in range(r):
            out[o + q * ns] = y[:, q]
        x = out
        ns *= r
    return x


def test_every_c2c_cover_schedule_is_a_dft():
    rng = np.random.default_rng(3)
    seen = set()
    for prec, kind, nc, T, rad, V in gen.cover_entries():
        if kind != 0 or tuple(rad) in seen:
            continue
        seen.add(tuple(rad))
        x = rng.standard_normal(nc) + 1j * rng.standard_normal(nc)
        got = stockham(x, rad)
        ref = np.fft.fft(x)
        assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-12, (nc, rad)
    assert len(seen) > 250  # distinct c2c schedules of the cover set
