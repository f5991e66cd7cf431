"""Adjoint kernels (bbfft_plan_create_adjoint) and the autograd binding.

The adjoint has no counterpart in the reference; it is checked
  * analytically: <F x, g> = <x, F^H g> in the real inner product, in FP64 (the maps are
    real-linear: r2c takes reals, c2r ignores imag(X[0]) like the reference does);
  * by finite differences of the spectral layer's loss sum(y^2) in FP64 along 64 random
    directions (relative error <= 1e-6), and
  * against the FP64 result of the float32 layer at the benchmark's shape.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rand(torch, n, dtype, seed):
    g = torch.Generator(device='cuda')
    g.manual_seed(seed)
    if dtype.is_complex:
        r = torch.randn(2 * n, generator=g, device='cuda', dtype=torch.float64)
        return torch.view_as_complex(r.view(n, 2)).to(dtype)
    return torch.randn(n, generator=g, device='cuda', dtype=torch.float64).to(dtype)


def _rdot(a, b):
    if a.is_complex():
        a = torch_view_real(a)
        b = torch_view_real(b)
    return float((a.double() * b.double()).sum())


def torch_view_real(z):
    import torch

    return torch.view_as_real(z.contiguous())


ADJ_CASES = [
    (1, [1, 64, 7], 0, -1), (1, [3, 63, 5], 0, 1), (1, [4, 64, 5], 1, -1), (1, [2, 15, 4], 1, -1),
    (1, [4, 64, 5], 2, 1), (1, [2, 15, 4], 2, 1), (1, [8, 2, 3], 1, -1), (1, [5, 96, 3], 2, 1),
    (2, [1, 16, 12, 3], 1, -1), (2, [2, 10, 6, 2], 2, 1), (2, [1, 9, 8, 2], 1, -1),
    (3, [1, 8, 6, 4, 2], 0, -1), (3, [1, 8, 6, 4, 2], 2, 1), (3, [2, 6, 4, 5, 1], 1, -1),
]


@pytest.mark.parametrize('case', ADJ_CASES, ids=[str(c) for c in ADJ_CASES])
def test_adjoint_identity_fp64(bb, torch_cuda, case):
    torch = torch_cuda
    from bbfft_gb300.autograd import FFT

    dim, shape, type, direction = case
    cfg = bb.configuration(dim, shape, precision=bb.F64, type=type, direction=direction)
    op = FFT(cfg)
    x = _rand(torch, op.in_numel, op.in_dtype, 1)
    g = _rand(torch, op.out_numel, op.out_dtype, 2)
    y = torch.empty(op.out_numel, dtype=op.out_dtype, device='cuda')
    h = torch.empty(op.in_numel, dtype=op.in_dtype, device='cuda')
    op.fwd.execute(x.data_ptr(), y.data_ptr())
    op.adj.execute(g.data_ptr(), h.data_ptr())
    torch.cuda.synchronize()
    lhs = _rdot(y, g)
    rhs = _rdot(x, h)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0) * 10, (lhs, rhs)


def _spectral_fd(bb, torch, N1, N2, batch, channels, m1, m2, ndir=64):
    """Central differences of sum(y^2) in FP64 along `ndir` random directions (exact for
    the polynomial loss up to O(eps^2) and rounding) against the autograd gradient through
    the adjoint kernels; returns the worst relative error."""
    from bbfft_gb300.autograd import SpectralLayer2d

    layer = SpectralLayer2d(N1, N2, batch, channels, m1, m2, prec=bb.F64)
    gen = torch.Generator(device='cuda')
    gen.manual_seed(7)
    x = torch.randn(batch, channels, N2, N1, generator=gen, device='cuda', dtype=torch.float64,
                    requires_grad=True)
    w = (torch.randn(channels, m2, m1, generator=gen, device='cuda', dtype=torch.float64) * 0.02 +
         1j * torch.randn(channels, m2, m1, generator=gen, device='cuda', dtype=torch.float64) * 0.02)
    w = w.requires_grad_(True)
    loss = (layer(x, w) ** 2).sum()
    gx, gw = torch.autograd.grad(loss, (x, w))
    worst = 0.0
    for i in range(ndir):
        vx = torch.randn(x.shape, generator=gen, device='cuda', dtype=torch.float64)
        # directions on the scale of each variable (weights ~ 0.02); the loss is quartic in
        # the step, so the central difference carries a relative error ~ (eps |v| / |w|)^2
        vw = (torch.randn(w.shape, generator=gen, device='cuda', dtype=torch.float64) + 1j *
              torch.randn(w.shape, generator=gen, device='cuda', dtype=torch.float64)) * 0.02
        eps = 1e-5
        with torch.no_grad():
            lp = (layer(x + eps * vx, w + eps * vw) ** 2).sum()
            lm = (layer(x - eps * vx, w - eps * vw) ** 2).sum()
        fd = float((lp - lm) / (2 * eps))
        an = float((gx * vx).sum() + (torch.view_as_real(gw) * torch.view_as_real(vw)).sum())
        rel = abs(fd - an) / max(abs(an), 1e-30)
        worst = max(worst, rel)
    return worst


def test_spectral_layer_finite_differences_fp64(bb, torch_cuda):
    """A small layer (16 x 12, K = 2 x 3, 5 x 4 modes): 64 directions, FP64, 1e-6."""
    assert _spectral_fd(bb, torch_cuda, 16, 12, 2, 3, 5, 4) <= 1e-6


def test_spectral_layer_finite_differences_fp64_benchmark_shape(bb, torch_cuda):
    """The benchmark's layer: 2d r2c / c2r over 128 x 128, K = 64 batch x 32 channels,
    lowest 32 x 32 modes, 64 random directions in FP64, relative error <= 1e-6."""
    worst = _spectral_fd(bb, torch_cuda, 128, 128, 64, 32, 32, 32)
    print('worst FD relative error', worst)
    assert worst <= 1e-6, worst


def test_spectral_layer_fp32_at_benchmark_shape(bb, torch_cuda):
    """2d r2c 128x128, K = 64 batch x 32 channels, lowest 32x32 modes, N(0, 0.02) weights:
    float32 forward and backward against the same layer in FP64."""
    torch = torch_cuda
    from bbfft_gb300.autograd import SpectralLayer2d

    gen = torch.Generator(device='cuda')
    gen.manual_seed(3)
    x64 = torch.randn(64, 32, 128, 128, generator=gen, device='cuda', dtype=torch.float64)
    w64 = torch.complex(torch.randn(32, 32, 32, generator=gen, device='cuda', dtype=torch.float64),
                        torch.randn(32, 32, 32, generator=gen, device='cuda', dtype=torch.float64)) * 0.02
    res = {}
    for prec, rdt, cdt in ((bb.F32, torch.float32, torch.complex64), (bb.F64, torch.float64, torch.complex128)):
        layer = SpectralLayer2d(128, 128, 64, 32, 32, 32, prec=prec)
        x = x64.to(rdt).requires_grad_(True)
        w = w64.to(cdt).requires_grad_(True)
        y = layer(x, w)
        loss = (y ** 2).sum()
        gx, gw = torch.autograd.grad(loss, (x, w))
        res[prec] = (y.detach().double(), gx.double(), gw.to(torch.complex128))
    for a, b in zip(res[bb.F32], res[bb.F64]):
        err = float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
        assert err <= 2e-5, err
