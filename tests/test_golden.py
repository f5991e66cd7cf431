"""Committed golden fixtures (tests/golden/*.npz, written by tests/golden/make_golden.py).

CPU: the oracle still reproduces every fixture, and the known-answer vectors of the
reference's tests still hold for it.  GPU: the CUDA path, called through the C ABI,
matches the fixtures' FP64 transforms within the path's tolerance (rel-L2 2e-6 float,
1e-14 double) and the oracle's own output within twice that."""
import glob
import os

import numpy as np
import pytest

from gpu_helpers import TOL, rel_l2, run

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(HERE, '*.npz'))
               if not p.endswith('known_answers.npz'))


def load(name):
    z = np.load(os.path.join(HERE, name + '.npz'))
    m = [int(v) for v in z['meta']]
    dim = m[0]
    shape = m[1:dim + 3]
    type, direction, prec, inplace = m[6:10]
    return z, dim, shape, type, direction, prec, bool(inplace)


def test_fixtures_present():
    assert len(CASES) >= 15


@pytest.mark.parametrize('name', CASES)
def test_oracle_reproduces_fixture(po, name):
    z, dim, shape, type, direction, prec, inplace = load(name)
    out = po.oracle_fft(dim, shape, type, direction, z['x'], inplace=inplace, prec=prec)
    assert out.shape == z['out'].shape
    assert rel_l2(out, z['out']) <= (1e-6 if prec == 4 else 1e-13)
    n1out = shape[1] // 2 + 1 if type == po.R2C else shape[1]
    oshape = [shape[0], n1out] + list(shape[2:dim + 2])
    dense = po.gather(out, dim, oshape, po.default_ostride(dim, shape, type, inplace))
    assert rel_l2(dense, z['ref']) <= TOL[prec]


def test_known_answer_vectors(po):
    from test_oracle import approx_ok

    z = np.load(os.path.join(HERE, 'known_answers.npz'))
    for prec in (4, 8):
        for N in (8, 13, 64):
            x, X = z[f'c2c_{prec}_{N}_x'], z[f'c2c_{prec}_{N}_X']
            out = po.oracle_fft(1, [3, N, 2], po.C2C, po.FORWARD, x.ravel(), prec=prec)
            assert approx_ok(out.reshape(X.shape), X, po.tol(prec, N))
        for N in (16, 27):
            x, X = z[f'r2c_{prec}_{N}_x'], z[f'r2c_{prec}_{N}_X']
            out = po.oracle_fft(1, [2, N, 3], po.R2C, po.FORWARD, x.ravel(), prec=prec)
            assert approx_ok(out.reshape(X.shape), X, po.tol(prec, N))
        X, y = z[f'c2r_{prec}_48_X'], z[f'c2r_{prec}_48_y']
        out = po.oracle_fft(1, [2, 48, 3], po.C2R, po.BACKWARD, X.ravel(), prec=prec)
        assert approx_ok(out.reshape(y.shape), y, po.tol(prec, 48))


@pytest.mark.gpu
@pytest.mark.parametrize('name', CASES)
def test_cuda_matches_fixture(bb, po, torch_cuda, name):
    z, dim, shape, type, direction, prec, inplace = load(name)
    cfg = bb.configuration(dim, shape, precision=prec, type=type, direction=direction,
                           inplace=inplace)
    out_ref = z['out']
    got = run(bb, torch_cuda, cfg, z['x'], out_ref.size, out_ref.dtype, inplace=inplace)
    n1out = shape[1] // 2 + 1 if type == po.R2C else shape[1]
    oshape = [shape[0], n1out] + list(shape[2:dim + 2])
    dense = po.gather(got, dim, oshape, list(cfg.ostride))
    assert rel_l2(dense, z['ref']) <= TOL[prec], name
    assert rel_l2(got, out_ref) <= 2 * TOL[prec], name


@pytest.mark.gpu
def test_cuda_known_answer_vectors(bb, po, torch_cuda):
    from test_oracle import approx_ok

    z = np.load(os.path.join(HERE, 'known_answers.npz'))
    for prec in (4, 8):
        rdt, cdt = (np.float32, np.complex64) if prec == 4 else (np.float64, np.complex128)
        for N in (8, 13, 64):
            x, X = z[f'c2c_{prec}_{N}_x'], z[f'c2c_{prec}_{N}_X']
            cfg = bb.configuration(1, [3, N, 2], precision=prec)
            got = run(bb, torch_cuda, cfg, x.ravel().astype(cdt), X.size, cdt)
            assert approx_ok(got.reshape(X.shape), X, po.tol(prec, N)), (prec, N)
        for N in (16, 27):
            x, X = z[f'r2c_{prec}_{N}_x'], z[f'r2c_{prec}_{N}_X']
            cfg = bb.configuration(1, [2, N, 3], precision=prec, type=bb.R2C)
            got = run(bb, torch_cuda, cfg, x.ravel().astype(rdt), X.size, cdt)
            assert approx_ok(got.reshape(X.shape), X, po.tol(prec, N)), (prec, N)
        X, y = z[f'c2r_{prec}_48_X'], z[f'c2r_{prec}_48_y']
        cfg = bb.configuration(1, [2, 48, 3], precision=prec, type=bb.C2R, direction=bb.BACKWARD)
        got = run(bb, torch_cuda, cfg, X.ravel().astype(cdt), y.size, rdt)
        assert approx_ok(got.reshape(y.shape), y, po.tol(prec, 48)), prec
