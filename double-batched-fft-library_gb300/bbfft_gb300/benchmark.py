"""Command-line benchmark with the reference benchmark's interface and CSV columns.

    python -m bbfft_gb300.benchmark [-i|-o] [-v] [-m M]... [-k K | -b BYTES] (s|d)(r|c) N...

mirrors benchmark/args.cpp (options), benchmark/test.hpp (K from the input-tensor
footprint, default 1 GiB), benchmark/adapter.hpp (bytes and flop models) and
benchmark/result.hpp (columns p, N, inplace, M, K, domain, inverse, time, bw, flops):
a 1d FFT over the second mode of an M x N x K tensor, timed as the minimum of 10 runs,
bandwidth and flops in GB/s and GFLOP/s.  Each configuration is checked first against an
FP64 DFT of a K-sample (rel-L2 2e-6 float, 1e-14 double).  ``--cufft`` adds the same
measurement for cuFFT (through torch.fft, one call over the whole tensor) as a labelled
comparator column.
"""
import argparse
import math
import sys

import numpy as np

import bbfft_gb300 as bb


def parse_bytes(b):
    scale = {'k': 1 << 10, 'm': 1 << 20, 'g': 1 << 30}.get(b[-1].lower(), 1)
    return int(b[:-1] if scale != 1 else b) * scale


def parse_args(argv):
    ap = argparse.ArgumentParser(description=__doc__.split('\n\n')[0], add_help=True)
    ap.add_argument('-i', dest='inplace', action='store_true', default=True, help='in-place [default]')
    ap.add_argument('-o', dest='inplace', action='store_false', help='out-of-place')
    ap.add_argument('-v', dest='inverse', action='store_true', help='backward transform')
    ap.add_argument('-m', dest='MM', type=int, action='append', help='size of the first mode (repeatable)')
    ap.add_argument('-k', dest='K', type=int, help='fixed size of the third mode')
    ap.add_argument('-b', dest='bytes', type=parse_bytes, default=1 << 30,
                    help='input tensor footprint that sets K (k/m/g suffixes); ignored with -k')
    ap.add_argument('--cufft', action='store_true', help='also time cuFFT (torch.fft) as a comparator')
    ap.add_argument('pd', help='(s|d)(r|c): single / double precision, real / complex')
    ap.add_argument('NN', type=int, nargs='+', help='sizes of the second mode')
    a = ap.parse_args(argv)
    if a.pd[0] not in 'sd' or (len(a.pd) > 1 and a.pd[1] not in 'rc'):
        ap.error('precision/domain must be (s|d)(r|c)')
    a.p = a.pd[0]
    a.d = a.pd[1] if len(a.pd) > 1 else 'r'
    a.MM = a.MM or [1]
    return a


def k_for(a, M, N):
    """benchmark/test.hpp K_memory_limit: bytes / (M N sizeof(number)), at least 1."""
    if a.K:
        return a.K
    size = (8 if a.p == 'd' else 4) * (2 if a.d == 'c' else 1)
    return max(1, a.bytes // (M * N * size))


def models(a, M, N, K):
    """benchmark/adapter.hpp: bytes moved and flop model of one transform pass."""
    real = 8 if a.p == 'd' else 4
    if a.d == 'c':
        return 2 * N * M * K * 2 * real, 5.0 * N * math.log2(N) * M * K
    return (N * real + (N // 2 + 1) * 2 * real) * M * K, 2.5 * N * math.log2(N) * M * K


def run_one(torch, a, M, N, K):
    prec = bb.F64 if a.p == 'd' else bb.F32
    rdt, cdt = (torch.float64, torch.complex128) if prec == bb.F64 else (torch.float32, torch.complex64)
    if a.d == 'c':
        type = bb.C2C
        direction = bb.BACKWARD if a.inverse else bb.FORWARD
    else:
        type = bb.C2R if a.inverse else bb.R2C
        direction = bb.BACKWARD if a.inverse else bb.FORWARD
    cfg = bb.configuration(1, [M, N, K], precision=prec, type=type, direction=direction,
                           inplace=a.inplace)
    n_in = N // 2 + 1 if type == bb.C2R else N
    n_out = N // 2 + 1 if type == bb.R2C else N
    in_c = type != bb.R2C
    out_c = type != bb.C2R
    ist, ost = list(cfg.istride), list(cfg.ostride)
    in_elems = (M - 1) * ist[0] + (n_in - 1) * ist[1] + (K - 1) * ist[2] + 1
    out_elems = (M - 1) * ost[0] + (n_out - 1) * ost[1] + (K - 1) * ost[2] + 1
    real = 8 if prec == bb.F64 else 4
    in_bytes = in_elems * real * (2 if in_c else 1)
    out_bytes = out_elems * real * (2 if out_c else 1)
    g = torch.Generator(device='cuda')
    g.manual_seed(N * 131 + M)
    buf_in = torch.randn((max(in_bytes, out_bytes if a.inplace else 0) + 15) // real, device='cuda',
                         dtype=rdt, generator=g)
    buf_out = buf_in if a.inplace else torch.empty((out_bytes + 15) // real, device='cuda', dtype=rdt)
    stream = torch.cuda.current_stream()
    plan = bb.Plan(cfg, stream=stream.cuda_stream)
    # check a K-sample against an FP64 DFT (the reference checks every run against its signal)
    x_host = buf_in[:in_bytes // real].double().cpu().numpy()
    plan.execute(buf_in.data_ptr(), buf_out.data_ptr())
    torch.cuda.synchronize()
    y_host = buf_out[:out_bytes // real].double().cpu().numpy()
    err = check(a, cfg, type, direction, M, N, K, x_host, y_host, ist, ost)
    # timing: minimum of 10 runs (benchmark/common.hpp), CUDA events on the plan's stream
    times = []
    for _ in range(11):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.execute(buf_in.data_ptr(), buf_out.data_ptr())
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    t = min(times[1:])
    nbytes, nflops = models(a, M, N, K)
    row = {'p': a.p, 'N': N, 'inplace': int(a.inplace), 'M': M, 'K': K, 'domain': a.d,
           'inverse': int(a.inverse), 'time': t, 'bw': nbytes / t / 1e9, 'flops': nflops / t / 1e9,
           'rel_l2': err}
    if a.cufft:
        row['cufft_bw'] = nbytes / time_cufft(torch, a, M, N, K, rdt, cdt) / 1e9
    return row


def check(a, cfg, type, direction, M, N, K, x, y, ist, ost):
    """rel-L2 of the first min(K, 8) transforms of every m against numpy's FP64 FFT."""
    ks = min(K, 8)
    n_in = N // 2 + 1 if type == bb.C2R else N
    n_out = N // 2 + 1 if type == bb.R2C else N
    idx_in = (np.arange(M)[None, None, :] * ist[0] + np.arange(n_in)[None, :, None] * ist[1]
              + np.arange(ks)[:, None, None] * ist[2])
    idx_out = (np.arange(M)[None, None, :] * ost[0] + np.arange(n_out)[None, :, None] * ost[1]
               + np.arange(ks)[:, None, None] * ost[2])
    xc = x.view(np.complex128) if type != bb.R2C else x
    yc = y.view(np.complex128) if type != bb.C2R else y
    xs = xc[idx_in]
    got = yc[idx_out]
    if type == bb.C2C:
        ref = np.fft.fft(xs, axis=1) if direction == bb.FORWARD else np.fft.ifft(xs, axis=1) * N
    elif type == bb.R2C:
        ref = np.fft.rfft(xs, axis=1)
    else:
        # the reference's c2r: imag X[0] ignored, imag X[N/2] enters every sample (even N)
        X = xs.copy()
        X[:, 0, :] = X[:, 0, :].real
        ref = np.fft.irfft(X, n=N, axis=1) * N
        if N % 2 == 0:
            ref = ref - X[:, N // 2:N // 2 + 1, :].imag
    err = float(np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300))
    tol = 1e-14 if a.p == 'd' else 2e-6
    if err > tol:
        raise SystemExit('check failed: N=%d M=%d K=%d rel-L2 %.3g > %g' % (N, M, K, err, tol))
    return err


def time_cufft(torch, a, M, N, K, rdt, cdt):
    """cuFFT through torch.fft over the N mode of a (K, N, M) tensor, minimum of 10 runs."""
    if a.d == 'c':
        x = torch.randn(K, N, M, dtype=cdt, device='cuda')
        f = (lambda: torch.fft.ifft(x, dim=1, norm='forward')) if a.inverse else (lambda: torch.fft.fft(x, dim=1))
    elif a.inverse:
        x = torch.randn(K, N // 2 + 1, M, dtype=cdt, device='cuda')
        f = lambda: torch.fft.irfft(x, n=N, dim=1, norm='forward')
    else:
        x = torch.randn(K, N, M, dtype=rdt, device='cuda')
        f = lambda: torch.fft.rfft(x, dim=1)
    f()
    times = []
    for _ in range(10):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        f()
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    return min(times)


def main(argv=None):
    a = parse_args(sys.argv[1:] if argv is None else argv)
    import torch

    cols = ['p', 'N', 'inplace', 'M', 'K', 'domain', 'inverse', 'time', 'bw', 'flops', 'rel_l2']
    if a.cufft:
        cols.append('cufft_bw')
    print(','.join(cols))
    for M in a.MM:
        for N in a.NN:
            K = k_for(a, M, N)
            r = run_one(torch, a, M, N, K)
            print(','.join(('%.6g' % r[c]) if isinstance(r[c], float) else str(r[c]) for c in cols),
                  flush=True)


if __name__ == '__main__':
    main()
