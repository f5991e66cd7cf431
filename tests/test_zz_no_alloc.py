"""The allocation-free 2d c2r entry point (bbfft_c2r_2d_noalloc_f32) against a regular plan.

Callers that cannot allocate device memory when they transform -- a process whose memory
manager reserves the device at start-up and forbids cudaMalloc later, or a host that must
keep a fixed device footprint -- use this entry point: its temporary and twiddles live in
static device arrays of the library instead of buffers that a plan allocates.  The test
calls it through the C ABI several times in a row (each call reuses the shared static
arrays with another shape and other data) and requires the result of the regular nd c2r
plan within the float tolerance of the parity tests (rel-L2 <= 2e-6).  The shapes cover
even and odd N1 (the two c2r kernels), a length with the prime factor 61 (the generic
odd-radix stage) and a shape at the size limit (N1 = N2 = 512, M * 257 * 512 * K just
under 2^21 complex floats).
"""
import numpy as np
import pytest

from gpu_helpers import from_device, rel_l2, run, to_device

pytestmark = pytest.mark.gpu


def _noalloc(bb, torch, X, M, N1, N2, K):
    d_in = to_device(torch, X)
    d_out = torch.zeros(M * N1 * N2 * K * 4 + 64, dtype=torch.uint8, device='cuda')
    stream = torch.cuda.current_stream().cuda_stream
    bb.c2r_2d_noalloc_f32(d_in.data_ptr(), d_out.data_ptr(), M, N1, N2, K, stream)
    return from_device(torch, d_out, np.float32, M * N1 * N2 * K)


def test_noalloc_c2r_2d_matches_plan_on_two_calls(bb, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(2024)
    for M, N1, N2, K in [(3, 32, 24, 5), (1, 128, 128, 9), (2, 15, 13, 4), (1, 122, 61, 3),
                         (1, 512, 512, 15)]:
        h = N1 // 2 + 1
        n = M * h * N2 * K
        X = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
        cfg = bb.configuration(2, [M, N1, N2, K], precision=bb.F32, type=bb.C2R,
                               direction=bb.BACKWARD)
        ref = run(bb, torch, cfg, X, M * N1 * N2 * K, np.float32)
        got = _noalloc(bb, torch, X, M, N1, N2, K)
        err = rel_l2(got, ref)
        assert err <= 2e-6, (M, N1, N2, K, err)


def test_noalloc_c2r_2d_rejects_sizes_beyond_the_scratch(bb, torch_cuda):
    torch = torch_cuda
    d = torch.zeros(64, dtype=torch.uint8, device='cuda')
    e = torch.zeros(64, dtype=torch.uint8, device='cuda')
    with pytest.raises(bb.BadConfiguration, match='static scratch'):
        bb.c2r_2d_noalloc_f32(d.data_ptr(), e.data_ptr(), 1, 128, 128, 2048)
    with pytest.raises(bb.BadConfiguration, match='512'):
        bb.c2r_2d_noalloc_f32(d.data_ptr(), e.data_ptr(), 1, 1024, 4, 1)
