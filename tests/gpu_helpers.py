"""Helpers for GPU tests: run a plan through the C ABI on host numpy arrays."""
import numpy as np


def to_device(torch, arr, nbytes=None):
    raw = np.ascontiguousarray(arr).view(np.uint8).ravel()
    n = max(raw.size, nbytes or 0)
    t = torch.zeros(n + 64, dtype=torch.uint8, device='cuda')
    t[:raw.size].copy_(torch.from_numpy(raw.copy()))
    return t


def from_device(torch, t, dtype, count):
    torch.cuda.synchronize()
    b = t[:count * np.dtype(dtype).itemsize].cpu().numpy()
    return b.view(dtype).copy()


def dtypes(prec):
    return (np.float32, np.complex64) if prec == 4 else (np.float64, np.complex128)


def run(bb, torch, cfg, x, out_count, out_dtype, inplace=False, plan=None, adjoint=False,
        out_init=None):
    """Execute `cfg` on flat numpy input x; returns the flat numpy output."""
    stream = torch.cuda.current_stream().cuda_stream
    if plan is None:
        plan = bb.Plan(cfg, stream=stream, adjoint=adjoint)
    out_bytes = out_count * np.dtype(out_dtype).itemsize
    if inplace:
        d = to_device(torch, x, nbytes=out_bytes)
        plan.execute(d.data_ptr())
        res = from_device(torch, d, out_dtype, out_count)
    else:
        d = to_device(torch, x)
        if out_init is not None:
            o = to_device(torch, out_init)
        else:
            o = torch.zeros(out_bytes + 64, dtype=torch.uint8, device='cuda')
        plan.execute(d.data_ptr(), o.data_ptr())
        res = from_device(torch, o, out_dtype, out_count)
    return res


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.complex128).ravel()
    b = np.asarray(b, dtype=np.complex128).ravel()
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


# rel-L2 tolerances of the FP32 / FP64 paths against an FP64 DFT
TOL = {4: 2e-6, 8: 1e-14}
