"""Tensor-core DFT stages (compute modes of c2c float plans, N in {64, 256, 512}).

Inputs follow the benchmark's tensor-core workload: iid N(0,1) complex values with a 1e-3
fraction scaled by 1e4.  rel-L2 against the FP64 DFT: the 3-term split-TF32 form (two TF32
pieces of about 11 bits each per operand) and the 6-term split-BF16 form (three BF16 pieces)
must meet 1e-6.  The 3-term split-BF16 form keeps two BF16 pieces (16 significant bits per
operand), so its error is about 4e-6 and it is held to 1e-5; plain BF16 to 2e-2."""
import numpy as np
import pytest

from gpu_helpers import rel_l2, run

pytestmark = pytest.mark.gpu

MODES = {'native': (0, 2e-6), 'bf16': (1, 2e-2), 'split6': (2, 1e-6), 'split3': (3, 1e-5),
         'split_tf32': (4, 1e-6)}


def tc_input(N, K, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(N * K) + 1j * rng.standard_normal(N * K)
    mask = rng.random(N * K) < 1e-3
    x[mask] *= 1e4
    return x.astype(np.complex64)


@pytest.mark.parametrize('N', [64, 256, 512])
@pytest.mark.parametrize('direction', [-1, 1])
def test_tensor_core_modes_accuracy(bb, po, torch_cuda, N, direction):
    torch = torch_cuda
    K = 2051  # not a multiple of the tile
    x = tc_input(N, K, N + direction)
    ref = po.dft64(1, [1, N, K], po.C2C, direction, x.astype(np.complex128).reshape(K, N, 1))
    errs = {}
    for name, (mode, tol) in MODES.items():
        cfg = bb.configuration(1, [1, N, K], precision=bb.F32, direction=direction, compute=mode)
        out = run(bb, torch, cfg, x, N * K, np.complex64)
        errs[name] = rel_l2(out.reshape(ref.shape), ref)
        assert errs[name] <= tol, (name, errs[name])
    print('N=%d dir=%d rel-L2 %s' % (N, direction, {k: '%.2e' % v for k, v in errs.items()}))


@pytest.mark.parametrize('mode', [2, 4])
@pytest.mark.parametrize('N', [64, 256, 512])
def test_tensor_core_mode_in_place(bb, po, torch_cuda, mode, N):
    torch = torch_cuda
    K = 300
    x = tc_input(N, K, 1)
    cfg = bb.configuration(1, [1, N, K], precision=bb.F32, compute=mode)
    out = run(bb, torch, cfg, x, N * K, np.complex64, inplace=True)
    ref = po.dft64(1, [1, N, K], po.C2C, -1, x.astype(np.complex128).reshape(K, N, 1))
    assert rel_l2(out.reshape(ref.shape), ref) <= 1e-6


@pytest.mark.parametrize('kw', [dict(shape=[1, 128, 8]), dict(shape=[2, 64, 8]),
                                dict(shape=[1, 64, 8], precision=8), dict(shape=[1, 64, 8], type=1)])
def test_tensor_core_modes_reject_other_configurations(bb, torch_cuda, kw):
    kw = dict(kw)
    shape = kw.pop('shape')
    cfg = bb.configuration(1, shape, compute=2, **kw)
    with pytest.raises(bb.BadConfiguration, match='tensor-core'):
        bb.make_plan(cfg)
