"""torch.autograd binding of the forward and adjoint FFT plans (test binding).

`FFT(cfg)` holds a forward plan and its adjoint (bbfft_plan_create_adjoint: unnormalised
backward transform for c2c, Hermitian-weighted c2r / r2c kernels for r2c / c2r) and is
applied to flat contiguous tensors laid out as the configuration describes.  Gradients use
PyTorch's convention for complex tensors (dL/dRe + i dL/dIm), for which the gradient of a
linear map is its adjoint applied to the incoming gradient.

`SpectralLayer2d` is the differentiable spectral layer of the benchmark: a 2d r2c over
N1 x N2, a complex multiply of the lowest m1 x m2 modes (all other modes dropped) by
per-channel weights, and a 2d c2r back.
"""
import torch

import bbfft_gb300 as bb


def _dtypes(prec):
    return (torch.float32, torch.complex64) if prec == bb.F32 else (torch.float64, torch.complex128)


def _numel(dim, shape, stride, n1):
    s = list(shape)
    s[1] = n1
    return sum((s[d] - 1) * stride[d] for d in range(dim + 2)) + 1


class FFT:
    """A configuration's forward plan and adjoint plan on the current CUDA stream."""

    def __init__(self, cfg, stream=None):
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        self.cfg = cfg
        self.fwd = bb.Plan(cfg, stream=stream)
        self.adj = bb.Plan(cfg, stream=stream, adjoint=True)
        rdt, cdt = _dtypes(cfg.precision)
        N1 = cfg.shape[1]
        in_n1 = N1 // 2 + 1 if cfg.type == bb.C2R else N1
        out_n1 = N1 // 2 + 1 if cfg.type == bb.R2C else N1
        self.in_numel = _numel(cfg.dim, list(cfg.shape), list(cfg.istride), in_n1)
        self.out_numel = _numel(cfg.dim, list(cfg.shape), list(cfg.ostride), out_n1)
        self.in_dtype = rdt if cfg.type == bb.R2C else cdt
        self.out_dtype = rdt if cfg.type == bb.C2R else cdt

    def __call__(self, x):
        return _Apply.apply(x, self)


class _Apply(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, op):
        x = x.contiguous()
        assert x.dtype == op.in_dtype and x.numel() == op.in_numel, 'layout mismatch'
        y = torch.empty(op.out_numel, dtype=op.out_dtype, device=x.device)
        op.fwd.execute(x.data_ptr(), y.data_ptr())
        ctx.op = op
        return y

    @staticmethod
    def backward(ctx, g):
        op = ctx.op
        g = g.contiguous()
        gx = torch.empty(op.in_numel, dtype=op.in_dtype, device=g.device)
        op.adj.execute(g.data_ptr(), gx.data_ptr())
        return gx, None


class SpectralLayer2d:
    """y = c2r( W * mask * r2c(x) ) over N1 x N2 (N1 fastest), K = batch * channels.

    x: real tensor (batch, channels, N2, N1); weights: complex (channels, m2, m1), applied
    to modes k1 < m1 (of the N1/2+1 half spectrum) and k2 < m2; all other modes are zero."""

    def __init__(self, N1, N2, batch, channels, m1, m2, prec=bb.F32):
        K = batch * channels
        self.shape = (batch, channels, N2, N1)
        self.m1, self.m2 = m1, m2
        self.r2c = FFT(bb.configuration(2, [1, N1, N2, K], precision=prec, type=bb.R2C))
        self.c2r = FFT(bb.configuration(2, [1, N1, N2, K], precision=prec, type=bb.C2R,
                                        direction=bb.BACKWARD))
        self.N1, self.N2, self.batch, self.channels = N1, N2, batch, channels

    def __call__(self, x, weights):
        b, c, N2, N1 = self.shape
        X = self.r2c(x.reshape(-1)).reshape(b, c, N2, N1 // 2 + 1)
        Y = torch.zeros_like(X)
        Y[:, :, :self.m2, :self.m1] = X[:, :, :self.m2, :self.m1] * weights
        y = self.c2r(Y.reshape(-1))
        return y.reshape(b, c, N2, N1)
