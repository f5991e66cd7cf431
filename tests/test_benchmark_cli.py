"""The reference-style benchmark CLI (bbfft_gb300.benchmark): argument parsing, K from the
memory footprint and the byte / flop models of benchmark/args.cpp, test.hpp, adapter.hpp.
CPU only; the GPU run is in tests/test_gpu_benchmark_cli.py."""
import math

import pytest


def test_parse_like_the_reference():
    from bbfft_gb300 import benchmark as bm

    a = bm.parse_args(['-o', '-v', '-m', '8', '-m', '16', '-b', '256m', 'dc', '64', '128'])
    assert (a.inplace, a.inverse, a.MM, a.bytes, a.p, a.d, a.NN) == (
        False, True, [8, 16], 256 << 20, 'd', 'c', [64, 128])
    a = bm.parse_args(['s', '48'])
    assert (a.inplace, a.inverse, a.MM, a.bytes, a.p, a.d) == (True, False, [1], 1 << 30, 's', 'r')
    assert bm.parse_args(['-k', '100', 'sr', '7']).K == 100
    with pytest.raises(SystemExit):
        bm.parse_args(['xr', '7'])


def test_k_and_models():
    from bbfft_gb300 import benchmark as bm

    a = bm.parse_args(['sr', '64'])
    assert bm.k_for(a, 8, 64) == (1 << 30) // (8 * 64 * 4)       # test.hpp K_memory_limit
    a = bm.parse_args(['-b', '1k', 'dc', '64'])
    assert bm.k_for(a, 8, 64) == 1                                # at least one
    a = bm.parse_args(['dc', '64'])
    b, f = bm.models(a, 2, 64, 3)                                 # adapter.hpp c2c
    assert b == 2 * 64 * 2 * 3 * 16 and f == 5 * 64 * 6 * 2 * 3
    a = bm.parse_args(['sr', '10'])
    b, f = bm.models(a, 1, 10, 1)                                 # real: N r + (N/2+1) c
    assert b == 10 * 4 + 6 * 8 and math.isclose(f, 2.5 * 10 * math.log2(10))
