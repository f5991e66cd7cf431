"""Multi-rank path on the CPU: world-size-2 (and 3) gloo process groups.

Each rank takes its K slab of the tensor (bbfft_gb300.shard_k: offsets and slab
configuration), transforms it with the oracle standing in for its GPU, and the slabs are
gathered on rank 0, which checks that they equal the unsharded transform exactly (the
transforms of different k never interact, so no collective is needed on the data path)."""
import os
import socket

import numpy as np
import pytest

CASES = [
    (1, [8, 64, 37], 1, -1, 4),   # r2c float, K = 37 split unevenly
    (1, [1, 48, 5], 0, 1, 8),     # c2c double backward
    (1, [4, 30, 2], 2, 1, 4),     # c2r float, K = 2
    (2, [1, 16, 12, 9], 1, -1, 4),  # 2d r2c
]


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _input(po, dim, shape, type, prec):
    rng = np.random.default_rng(11)
    n1 = shape[1] // 2 + 1 if type == po.C2R else shape[1]
    ishape = [shape[0], n1] + list(shape[2:dim + 2])
    n = po.tensor_size(dim, ishape, po.default_istride(dim, shape, type, False))
    rdt, cdt = (np.float32, np.complex64) if prec == 4 else (np.float64, np.complex128)
    if type == po.R2C:
        return rng.standard_normal(n).astype(rdt)
    return (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(cdt)


def _rank_main(rank, world, port, results):
    import torch.distributed as dist

    import bbfft_gb300 as bb
    from oracle import pyoracle as po

    dist.init_process_group('gloo', init_method=f'tcp://127.0.0.1:{port}', rank=rank,
                            world_size=world)
    try:
        for ci, (dim, shape, type, direction, prec) in enumerate(CASES):
            cfg = bb.configuration(dim, shape, precision=prec, type=type, direction=direction)
            x = _input(po, dim, shape, type, prec)
            k0, k1, ioff, ooff, slab = bb.shard_k(cfg, world, rank)
            piece = None
            if slab is not None:
                sh = [int(slab.shape[d]) for d in range(dim + 2)]
                xs = x[ioff // x.itemsize:]
                out = po.oracle_fft(dim, sh, type, direction, xs, istride=list(slab.istride),
                                    ostride=list(slab.ostride), prec=prec)
                piece = (ooff, out)
            gathered = [None] * world if rank == 0 else None
            dist.gather_object(piece, gathered, dst=0)
            if rank == 0:
                full = po.oracle_fft(dim, shape, type, direction, x, prec=prec)
                got = np.zeros_like(full)
                covered = 0
                for p in gathered:
                    if p is None:
                        continue
                    off, out = p
                    o = off // full.itemsize
                    n = min(out.size, got.size - o)
                    got[o:o + n] = out[:n]
                    covered += 1
                ok = np.array_equal(got, full)
                results.put((ci, ok, covered))
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize('world', [2, 3])
def test_k_slab_sharding_matches_unsharded(po, world):
    import torch.multiprocessing as mp

    ctx = mp.get_context('spawn')
    q = ctx.SimpleQueue()
    port = _free_port()
    os.environ.setdefault('GLOO_SOCKET_IFNAME', 'lo')
    mp.start_processes(_rank_main, args=(world, port, q), nprocs=world, join=True,
                       start_method='spawn')
    res = []
    while not q.empty():
        res.append(q.get())
    assert len(res) == len(CASES)
    for ci, ok, covered in res:
        assert ok, CASES[ci]
        assert covered == min(world, CASES[ci][1][CASES[ci][0] + 1])


def test_shard_k_offsets(bb):
    cfg = bb.configuration(1, [8, 64, 10], precision=bb.F32, type=bb.R2C)
    slabs = [bb.shard_k(cfg, 4, r) for r in range(4)]
    assert [(a, b) for a, b, *_ in slabs] == [(0, 2), (2, 5), (5, 7), (7, 10)]
    # istride[2] = 8 * 64 reals, ostride[2] = 8 * 33 complex
    assert slabs[1][2] == 2 * 8 * 64 * 4 and slabs[1][3] == 2 * 8 * 33 * 8
    assert int(slabs[1][4].shape[2]) == 3 and int(slabs[1][4].shape[1]) == 64
    assert bb.shard_k(bb.configuration(1, [1, 8, 1]), 2, 0)[4] is None  # K = 1: rank 1 has it
