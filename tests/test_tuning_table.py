"""The autotuner's table format (bbfft_gb300/autotune.py): written lines read back, the
optional columns (resident-CTA variant, threads per transform, radices), and the table
committed with the package parses with stage lists whose product is the FFT length."""
import os

import pytest


def test_roundtrip(bb, tmp_path):
    from bbfft_gb300 import autotune as at

    entries = [((4, 'r2ch', 160, 8, 2, 8, 2, 3, 0, ''), 6197.5),
               ((4, 'c2rh', 384, 8, 2, 8, 1, 13, 16, '4x4x12'), 5709.5),
               ((8, 'c2c', 64, 1, 1, 1, 4, 2, 0, ''), 700.0)]
    path = str(tmp_path / 't.tune')
    at.write_table(path, entries)
    back = at.read_table(path)
    assert back == entries


def test_committed_table_is_consistent(bb):
    from bbfft_gb300 import autotune as at

    path = at.DEFAULT_OUT
    assert os.path.exists(path)
    rows = at.read_table(path)
    assert len(rows) >= 50
    kinds = {'c2c', 'r2ch', 'r2cf', 'c2rh', 'c2rf'}
    for (prec, kind, N, M, V, Mb, Kb, occ, T, rad), gbs in rows:
        assert prec in (4, 8) and kind in kinds and N > 0 and M > 0
        assert V in (1, 2, 4) and Mb >= 1 and Kb >= 1 and occ in (2, 3, 12, 13)
        if rad:
            nc = N // 2 if kind in ('r2ch', 'c2rh') else N
            prod = 1
            for r in rad.split('x'):
                prod *= int(r)
            assert prod == nc and T > 0, (kind, N, rad)


def test_alternative_stages_are_generated(bb):
    """Every (radices, T) the autotuner may pick has compile-time kernels."""
    from bbfft_gb300 import autotune as at

    real, c2c = at.alt_stages()
    import gen_specializations as gs

    ents = {(e[1], e[2], e[3], tuple(e[4])) for e in gs.entries() if e[0] == 4}
    for nc, alts in real.items():
        for rad, T in alts:
            for kind in (1, 3):
                assert (kind, nc, T, tuple(rad)) in ents
    for nc, alts in c2c.items():
        for rad, T in alts:
            assert (0, nc, T, tuple(rad)) in ents
