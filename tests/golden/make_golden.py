"""Writes the golden fixtures of this directory (run from the repository root:
`python tests/golden/make_golden.py`).

Each case of CASES becomes `<name>.npz` with
  x     the seeded input tensor (flat, plan precision, the configuration's layout),
  ref   its FP64 transform (numpy float64 DFT with the reference's c2r semantics),
  out   the CPU oracle's output in the plan precision (oracle/bbfft_oracle.c),
  meta  dim, shape, type, direction, precision, inplace;
plus `known_answers.npz`: the analytic known-answer signals of the reference's device
tests (test/c2c.cpp:17-51, test/r2c.cpp:28-135, polluted imag X[0] of
test/r2c.cpp:310-324) at a few sizes, with their exact spectra.

The oracle is pinned against those known answers by tests/test_oracle.py before it is
trusted to write `out`."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
from oracle import pyoracle as po  # noqa: E402

# name: (dim, shape, type, direction, prec, inplace)
CASES = {
    'c2c_f32_n64_m1_k64_fwd': (1, [1, 64, 64], 0, -1, 4, False),
    'c2c_f32_n13_m3_k16_bwd': (1, [3, 13, 16], 0, 1, 4, False),
    'c2c_f64_n105_m2_k8_fwd': (1, [2, 105, 8], 0, -1, 8, False),
    'c2c_f32_n512_m1_k8_fwd': (1, [1, 512, 8], 0, -1, 4, False),
    'r2c_f32_n16_m8_k64': (1, [8, 16, 64], 1, -1, 4, False),
    'r2c_f32_n160_m8_k8': (1, [8, 160, 8], 1, -1, 4, False),
    'r2c_f32_n7_m8_k64': (1, [8, 7, 64], 1, -1, 4, False),
    'r2c_f64_n384_m2_k4': (1, [2, 384, 4], 1, -1, 8, False),
    'r2c_f32_n12_m4_k8_inplace': (1, [4, 12, 8], 1, -1, 4, True),
    'c2r_f32_n224_m8_k8': (1, [8, 224, 8], 2, 1, 4, False),
    'c2r_f32_n11_m8_k32': (1, [8, 11, 32], 2, 1, 4, False),
    'c2r_f64_n48_m3_k8': (1, [3, 48, 8], 2, 1, 8, False),
    'r2c_2d_f32_16x12_k4': (2, [1, 16, 12, 4], 1, -1, 4, False),
    'c2r_2d_f32_10x6_k3': (2, [2, 10, 6, 3], 2, 1, 4, False),
    'c2c_3d_f64_8x6x4_k2': (3, [1, 8, 6, 4, 2], 0, -1, 8, False),
}


def make_case(i, dim, shape, type, direction, prec, inplace):
    rng = np.random.default_rng(4242 + i)
    rdt, cdt = (np.float32, np.complex64) if prec == 4 else (np.float64, np.complex128)
    ist = po.default_istride(dim, shape, type, inplace)
    ost = po.default_ostride(dim, shape, type, inplace)
    n1in = shape[1] // 2 + 1 if type == po.C2R else shape[1]
    n1out = shape[1] // 2 + 1 if type == po.R2C else shape[1]
    ishape = [shape[0], n1in] + list(shape[2:dim + 2])
    oshape = [shape[0], n1out] + list(shape[2:dim + 2])
    isize = po.tensor_size(dim, ishape, ist)
    if type == po.R2C:
        x = rng.standard_normal(isize).astype(rdt)
    else:
        x = (rng.standard_normal(isize) + 1j * rng.standard_normal(isize)).astype(cdt)
    dense = po.gather(x, dim, ishape, ist)
    ref = po.dft64(dim, shape, type, direction, dense)
    out = po.oracle_fft(dim, shape, type, direction, x, istride=ist, ostride=ost,
                        inplace=inplace, prec=prec)
    out_dense = po.gather(out, dim, oshape, ost)
    assert po.rel_l2(out_dense, ref) <= (2e-6 if prec == 4 else 1e-14)
    meta = np.array([dim] + list(shape) + [0] * (5 - len(shape)) + [type, direction, prec,
                                                                      int(inplace)])
    return dict(x=x, ref=ref, out=out, meta=meta)


def main():
    po.lib()
    for i, (name, c) in enumerate(sorted(CASES.items())):
        np.savez_compressed(os.path.join(HERE, name + '.npz'), **make_case(i, *c))
    ka = {}
    for prec in (4, 8):
        for N in (8, 13, 64):
            x, X = po.c2c_known_answer(3, N, 2, prec)
            ka[f'c2c_{prec}_{N}_x'], ka[f'c2c_{prec}_{N}_X'] = x, X
        for N in (16, 27):
            x, X = po.r2c_known_answer(2, [N], 3, prec)
            ka[f'r2c_{prec}_{N}_x'], ka[f'r2c_{prec}_{N}_X'] = x, X
        X, y = po.c2r_known_answer(2, [48], 3, prec, pollute_0=True)
        ka[f'c2r_{prec}_48_X'], ka[f'c2r_{prec}_48_y'] = X, y
    np.savez_compressed(os.path.join(HERE, 'known_answers.npz'), **ka)


if __name__ == '__main__':
    main()
