"""The stage-list rules that the kernel generator (csrc/gen_specializations.py) and the
host library (csrc/library.cpp) must apply identically: a plan finds its compile-time tile
only when both choose the same radices and threads per transform.  Runs without a GPU."""
import ctypes
import os
import sys

from conftest import REPO

sys.path.insert(0, os.path.join(REPO, 'double-batched-fft-library_gb300', 'csrc'))
import gen_specializations as gen  # noqa: E402


def test_register_prime_rule_matches_generator(bb):
    """Every complex length up to 512: the prime P whose radix-P stage runs in registers
    (0: none) is the same in the host library and in the generator."""
    fn = bb.lib().gbfft_internal_reg_prime
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_int]
    for nc in range(1, 513):
        assert fn(nc) == gen.reg_prime_of(nc), nc


def test_register_prime_stage_lists():
    """Register-prime tiles put the prime first, on nc / P threads per transform, with no
    copy stage (a real single stage keeps its shared round trip)."""
    for nc in range(17, 513):
        p = gen.reg_prime_of(nc)
        if not p:
            continue
        rad, T = gen.stage_list(nc, 0, ragged=True, reg_ok=True)
        assert rad[0] == p and 1 not in rad and T == nc // p, (nc, rad, T)
        prod = 1
        for r in rad:
            prod *= r
        assert prod == nc
    rad, T = gen.stage_list(17, 2, ragged=True, reg_ok=True)
    assert rad == [17, 1] and T == 1


def test_every_generated_tile_is_consistent():
    """Every compile-time tile the generator emits (cover and ragged sets): its radices
    multiply to the complex length (copy stages are radix 1), its threads per transform
    fit a 256-thread block, a register prime tile puts its prime first on nc / P threads,
    and the resident-CTA budget matches the stage kinds."""
    for kind_set, ents in (('cover', gen.cover_entries()), ('ragged', gen.ragged_entries())):
        for prec, kind, nc, T, rad, V in ents:
            prod = 1
            for r in rad:
                prod *= r
            assert prod == nc, (kind_set, kind, nc, rad)
            assert 1 <= T <= 256 and T * V <= 256, (kind_set, kind, nc, T, V)
            reg = gen.reg_prime_tile(nc, rad)
            if reg:
                assert rad[0] == gen.reg_prime_of(nc) and T == nc // rad[0], (kind_set, nc, rad, T)
                assert gen.tile_min_blocks(rad, reg) in (1, 2)
            if kind_set == 'ragged' and reg:
                assert rad[0] <= 47, (nc, rad)  # the ragged units compile for 128 registers
