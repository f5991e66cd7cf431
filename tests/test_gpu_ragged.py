"""Ragged batches: many independent 1d transforms of mixed N, kind and batch sizes in one
launch (persistent CTAs or one CTA per tile, optionally replayed from a CUDA graph),
against the FP64 DFT."""
import numpy as np
import pytest

from gpu_helpers import TOL, rel_l2

pytestmark = pytest.mark.gpu


def make_batch(bb, torch, n, seed, Ns=None):
    """Seeded batch like the benchmark's: N in {16, 24, ..., 512}, c2c complex64 or r2c
    float32 50/50, M in {1, 4, 16}, K in [1, 64], data iid U[-1, 1]."""
    rng = np.random.default_rng(seed)
    Ns = Ns or list(range(16, 513, 8))
    specs = []
    in_off = out_off = 0
    for _ in range(n):
        N = int(rng.choice(Ns))
        t = bb.C2C if rng.random() < 0.5 else bb.R2C
        M = int(rng.choice([1, 4, 16]))
        K = int(rng.integers(1, 65))
        nin = M * N * K * (2 if t == bb.C2C else 1)
        nout = M * (N if t == bb.C2C else N // 2 + 1) * K * 2
        specs.append((t, N, M, K, in_off, nin, out_off, nout))
        in_off += (nin + 3) // 4 * 4      # keep every tensor 16-byte aligned
        out_off += (nout + 3) // 4 * 4
    x = torch.empty(in_off, dtype=torch.float32, device='cuda').uniform_(-1, 1)
    y = torch.zeros(out_off, dtype=torch.float32, device='cuda')
    items = [(bb.F32, bb.FORWARD, t, N, M, K, x.data_ptr() + 4 * io, y.data_ptr() + 4 * oo)
             for (t, N, M, K, io, _, oo, _) in specs]
    return specs, x, y, items


def check_items(bb, po, specs, x, y, idx):
    xh = x.cpu().numpy()
    yh = y.cpu().numpy()
    worst = 0.0
    for i in idx:
        t, N, M, K, io, nin, oo, nout = specs[i]
        if t == bb.C2C:
            xi = xh[io:io + nin].view(np.complex64).reshape(K, N, M)
        else:
            xi = xh[io:io + nin].reshape(K, N, M)
        ref = po.dft64(1, [M, N, K], t, bb.FORWARD, xi)
        got = yh[oo:oo + nout].view(np.complex64).reshape(ref.shape)
        e = rel_l2(got, ref)
        worst = max(worst, e)
        assert e <= TOL[4], (i, t, N, M, K, e)
    return worst


@pytest.mark.parametrize('form', [0, 1, 2])
@pytest.mark.parametrize('use_graph', [False, True])
def test_ragged_small_batch(bb, po, torch_cuda, use_graph, form):
    torch = torch_cuda
    specs, x, y, items = make_batch(bb, torch, 300, seed=11)
    r = bb.Ragged(items)
    r.set_launch_form(form)
    info = r.info()
    assert info.num_units >= len(items) and info.grid >= 1
    r.execute(torch.cuda.current_stream().cuda_stream, use_graph=use_graph)
    torch.cuda.synchronize()
    check_items(bb, po, specs, x, y, range(len(specs)))


def test_ragged_benchmark_batch_graph_replay(bb, po, torch_cuda):
    """The 10^4-transform batch: two graph replays give identical results, the grid form
    the same bits, the class form the same to rounding; every one of the 10^4 transforms
    of the persistent form (bit-equal to the grid form's) and a seeded sample of 400 of
    the class form's match the FP64 DFT."""
    torch = torch_cuda
    specs, x, y, items = make_batch(bb, torch, 10000, seed=4)
    r = bb.Ragged(items)
    s = torch.cuda.current_stream().cuda_stream
    r.execute(s, use_graph=True)
    torch.cuda.synchronize()
    first = y.clone()
    y.zero_()
    r.execute(s, use_graph=True)
    torch.cuda.synchronize()
    assert torch.equal(first, y)
    # the grid form (one CTA per tile) runs the same compiled tile functions: same bits
    y.zero_()
    r.set_launch_form(r.GRID)
    r.execute(s, use_graph=True)
    torch.cuda.synchronize()
    assert torch.equal(first, y)
    # the class form compiles each tile function into its own kernel (the compiler may
    # contract multiply-adds differently): equal to rounding
    y.zero_()
    r.set_launch_form(r.CLASSES)
    r.execute(s, use_graph=True)
    torch.cuda.synchronize()
    assert float(torch.linalg.vector_norm(y - first) / torch.linalg.vector_norm(first)) <= 1e-6
    check_items(bb, po, specs, x, first, range(len(specs)))
    rng = np.random.default_rng(5)
    check_items(bb, po, specs, x, y, rng.choice(len(specs), 400, replace=False))


def test_ragged_rejects_mixed_precision(bb, torch_cuda):
    torch = torch_cuda
    a = torch.zeros(1024, device='cuda')
    items = [(bb.F32, bb.FORWARD, bb.C2C, 16, 1, 1, a.data_ptr(), a.data_ptr() + 512),
             (bb.F64, bb.FORWARD, bb.C2C, 16, 1, 1, a.data_ptr(), a.data_ptr() + 512)]
    with pytest.raises(bb.BadConfiguration):
        bb.Ragged(items)


@pytest.mark.parametrize('prec', [4, 8])
@pytest.mark.parametrize('form', [0, 1, 2])
def test_ragged_every_kind(bb, po, torch_cuda, prec, form):
    """c2c forward and backward, r2c and c2r items, even and odd N, in one batch of each
    precision and launch form, against the FP64 DFT (the reference's c2r semantics)."""
    torch = torch_cuda
    rng = np.random.default_rng(31 + prec + form)
    rdt, cdt = (np.float32, np.complex64) if prec == 4 else (np.float64, np.complex128)
    specs, xs = [], []
    in_off = out_off = 0
    for i in range(120):
        N = int(rng.choice([7, 12, 16, 40, 61, 96, 136, 250, 488, 512]))
        t = int(rng.choice([bb.C2C, bb.R2C, bb.C2R]))
        d = bb.BACKWARD if t == bb.C2R else (int(rng.choice([bb.FORWARD, bb.BACKWARD])) if t == bb.C2C else bb.FORWARD)
        M = int(rng.choice([1, 3, 8]))
        K = int(rng.integers(1, 12))
        nin = N // 2 + 1 if t == bb.C2R else N
        nout = N // 2 + 1 if t == bb.R2C else N
        if t == bb.R2C:
            x = rng.standard_normal(M * nin * K).astype(rdt)
        else:
            x = (rng.standard_normal(M * nin * K) + 1j * rng.standard_normal(M * nin * K)).astype(cdt)
        ib = x.nbytes
        ob = M * nout * K * (np.dtype(rdt).itemsize if t == bb.C2R else np.dtype(cdt).itemsize)
        specs.append((t, d, N, M, K, in_off, out_off, x, nout))
        in_off += (ib + 15) // 16 * 16
        out_off += (ob + 15) // 16 * 16
    xin = torch.zeros(in_off, dtype=torch.uint8, device='cuda')
    yout = torch.zeros(out_off, dtype=torch.uint8, device='cuda')
    for (t, d, N, M, K, io, oo, x, nout) in specs:
        raw = torch.from_numpy(x.view(np.uint8).copy())
        xin[io:io + raw.numel()].copy_(raw)
    items = [(prec, d, t, N, M, K, xin.data_ptr() + io, yout.data_ptr() + oo)
             for (t, d, N, M, K, io, oo, x, nout) in specs]
    r = bb.Ragged(items)
    r.set_launch_form(form)
    r.execute(torch.cuda.current_stream().cuda_stream, use_graph=True)
    torch.cuda.synchronize()
    yh = yout.cpu().numpy()
    for (t, d, N, M, K, io, oo, x, nout) in specs:
        odt = rdt if t == bb.C2R else cdt
        got = yh[oo:oo + M * nout * K * np.dtype(odt).itemsize].view(odt)
        nin = N // 2 + 1 if t == bb.C2R else N
        ref = po.dft64(1, [M, N, K], t, d, x.astype(np.float64 if t == bb.R2C else np.complex128).reshape(K, nin, M))
        e = rel_l2(got.reshape(ref.shape), ref)
        assert e <= TOL[prec], (t, d, N, M, K, e)
