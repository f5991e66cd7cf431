#!/usr/bin/env python3
"""Benchmark of the double-batched FFT hot path on GB300.

Workload (the configuration the headline metric is quoted on): a double-batched 1d r2c
followed by a c2r over an M x N x K float32 tensor, M = 8 (unit stride), K chosen so the
real input is 1 GiB, for every N of the sweep {16,32,64,128,256,512,48,96,160,224,384,7,
11,13}.  One step = the r2c and the c2r pass for every N of the sweep (28 launches).

value  = algorithmic bytes of all passes / device time of the step (GB/s), where a pass
         moves (N * 4 + (N/2+1) * 8) * M * K bytes (one read + one write, the reference's
         benchmark/adapter.hpp:21-25,51-52 byte model); inputs are resident in HBM and are
         1 GiB per pass, far larger than the 129 MB L2, so no flush is needed.
e2e    = the same metric through the C ABI from pinned host memory (1/8 of K per N): each
         step copies the inputs host->device, runs the passes and copies the results
         device->host, in K-chunks pipelined over two copy streams and a compute stream.
roofline = the engine kernels (every launch of the step): algorithmic bytes / summed
         CUDA-event duration of the launches, against the measured HBM copy bandwidth.
cpu_baseline = the oracle (C restatement of the reference's algorithm) on all host cores,
         on a K-subset of the same workload.

--impl reference times the reference's CPU implementation of the path (the oracle port;
the reference's own kernels need an OpenCL/SYCL/Level Zero runtime that is not present)
on the host cores with the same metric.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, 'double-batched-fft-library_gb300')
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

SWEEP_N = [16, 32, 64, 128, 256, 512, 48, 96, 160, 224, 384, 7, 11, 13]
# secondary legs, in the order they run (the peaks first: later legs use them)
LEGS = ['peaks', 'c2c_n64_k16384', 'ragged_10k', 'spectral_layer_2d', 'c2c_3d_64',
        'tft_vs_double_batched', 'sweep_f64', 'tensor_core_c2c', 'cufft', 'sweep_all_n']
M_BATCH = 8
REAL_BYTES = 1 << 30
METRIC = 'GB/s vs HBM peak per N; plain vs split-TC form at rel-L2<=1e-6 vs FP64'


def k_for(N, prec):
    return REAL_BYTES // (prec * M_BATCH * N)


def pass_bytes(N, K, prec, M=M_BATCH):
    return (N * prec + (N // 2 + 1) * 2 * prec) * M * K


def pass_flops(N, K, M=M_BATCH, real=True):
    """The reference's flop model (benchmark/adapter.hpp:21-25,51-52): 5 N log2 N per
    complex transform, 2.5 N log2 N per real one."""
    return (2.5 if real else 5.0) * N * math.log2(N) * M * K


def measured_peaks():
    p = os.path.join(REPO, 'MEASURED_PEAKS.json')
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    return 6800.0, 'fallback'


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
              'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
              'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.FIELDS,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(',')]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == 'active':
                    reasons.add(nm)
        return {'sm_mhz': float(np.median(sm)) if sm else None,
                'sm_max_mhz': float(max(smax)) if smax else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


def dist_env():
    ws = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    return ws, rank, local


# ------------------------------------------------------------------------------------------
# CPU baseline (oracle port)


def cpu_sample_k(N, threads):
    """Slices of the CPU sample for length N: 2^20 / N of them (about 64 MB per pass, the
    same bytes for every N), at least two per host thread, at most the full tensor."""
    return max(2 * threads, min(k_for(N, 4), (1 << 20) // N))


class CpuSample:
    """The oracle's r2c + c2r (the C restatement of the reference's algorithm) on all host
    cores over a fixed K-subset of every N of the sweep.  The buffers are allocated and
    touched once (an untimed sweep), so every timed sweep does the same work."""

    def __init__(self, prec=4, threads=None):
        from oracle import pyoracle as po

        self.po = po
        self.prec = prec
        self.threads = threads or os.cpu_count() or 1
        rng = np.random.default_rng(0)
        rdt = np.float32 if prec == 4 else np.float64
        cdt = np.complex64 if prec == 4 else np.complex128
        self.cases = []
        for N in SWEEP_N:
            K = cpu_sample_k(N, self.threads)
            x = rng.standard_normal(M_BATCH * N * K).astype(rdt)
            X = np.zeros(M_BATCH * (N // 2 + 1) * K, dtype=cdt)
            y = np.zeros(M_BATCH * N * K, dtype=rdt)
            self.cases.append((N, K, x, X, y))
        self.bytes = sum(2 * pass_bytes(N, K, prec) for (N, K, _, _, _) in self.cases)
        self.sweep()  # first touch of every page

    def sweep(self):
        """One timed pass over the sample; returns seconds."""
        po, prec, th = self.po, self.prec, self.threads
        t0 = time.perf_counter()
        for N, K, x, X, y in self.cases:
            po.fft1d(po.R2C, po.FORWARD, M_BATCH, N, K, x, M_BATCH, M_BATCH * N, X, M_BATCH,
                     M_BATCH * (N // 2 + 1), prec, th)
            po.fft1d(po.C2R, po.BACKWARD, M_BATCH, N, K, X, M_BATCH, M_BATCH * (N // 2 + 1), y,
                     M_BATCH, M_BATCH * N, prec, th)
        return time.perf_counter() - t0

    def describe(self, secs):
        ks = [K for (_, K, _, _, _) in self.cases]
        return ('oracle r2c+c2r, M=8, every N of the sweep, K-subset of %d..%d slices per N '
                '(2^20 / N, %.2f GB per sweep), %.1f s timed' % (min(ks), max(ks), self.bytes / 1e9,
                                                                 secs))


def cpu_baseline(prec=4, sweeps=3, threads=None):
    """GB/s of the CPU sample over `sweeps` timed sweeps (the reference arm times the same
    sample, one sweep per step)."""
    smp = CpuSample(prec, threads)
    t = sum(smp.sweep() for _ in range(sweeps))
    return {'value': smp.bytes * sweeps / t / 1e9, 'unit': 'GB/s', 'cores': smp.threads,
            'kind': 'port', 'sample': smp.describe(t)}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    prec = 4
    smp = CpuSample(prec)
    for _ in range(max(0, args.warmup)):
        smp.sweep()
    t = 0.0
    for _ in range(args.steps):
        t += smp.sweep()
    value = smp.bytes * args.steps / t / 1e9
    line = {
        'impl': 'reference', 'metric': METRIC, 'value': value, 'unit': 'GB/s', 'n_gpus': ws,
        'steps': args.steps, 'warmup': args.warmup,
        'ms_per_step': t / args.steps * 1e3, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic: iid N(0,1) reals, seeded',
        'config': {'workload': 'r2c+c2r round trip, M=8, 1 GiB real input per N, f32, '
                               'N in ' + str(SWEEP_N) + ' (K-subset on the CPU)'},
        'cpu_baseline': {'value': value, 'unit': 'GB/s', 'cores': smp.threads, 'kind': 'port',
                         'sample': smp.describe(t)},
        'e2e': {'value': value, 'unit': 'GB/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
        'note': 'reference CPU path = C restatement of the reference kernels (oracle/); the '
                'reference library itself needs an OpenCL/SYCL/Level Zero runtime; the GPU '
                'line\'s cpu_baseline times the same sample',
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------
# GPU arm


def run_ours(args):
    import torch

    import bbfft_gb300 as bb

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group('nccl')
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    prec = 4
    hbm_peak, peak_kind = measured_peaks()

    # one pair of buffers sized for the largest pass; K-slab per rank (weak scaling: every
    # rank transforms a full 1 GiB tensor per N)
    max_real = max(M_BATCH * N * k_for(N, prec) for N in SWEEP_N) * prec
    max_cplx = max(M_BATCH * (N // 2 + 1) * k_for(N, prec) for N in SWEEP_N) * 2 * prec
    xbuf = torch.empty(max_real // 4, dtype=torch.float32, device='cuda')
    Xbuf = torch.empty(max_cplx // 4, dtype=torch.float32, device='cuda')
    ybuf = torch.empty(max_real // 4, dtype=torch.float32, device='cuda')
    g = torch.Generator(device='cuda')
    g.manual_seed(1234 + rank)
    xbuf.normal_(generator=g)

    plans = []
    total_bytes = 0
    for N in SWEEP_N:
        K = k_for(N, prec)
        f = bb.configuration(1, [M_BATCH, N, K], precision=bb.F32, type=bb.R2C)
        b = bb.configuration(1, [M_BATCH, N, K], precision=bb.F32, type=bb.C2R,
                             direction=bb.BACKWARD)
        plans.append((N, K, bb.Plan(f, stream=sptr), bb.Plan(b, stream=sptr)))
        total_bytes += 2 * pass_bytes(N, K, prec)

    xp, Xp, yp = xbuf.data_ptr(), Xbuf.data_ptr(), ybuf.data_ptr()

    def step(events=None):
        for i, (N, K, pf, pb) in enumerate(plans):
            if events is not None:
                events[4 * i].record(stream)
            pf.execute(xp, Xp)
            if events is not None:
                events[4 * i + 1].record(stream)
                events[4 * i + 2].record(stream)
            pb.execute(Xp, yp)
            if events is not None:
                events[4 * i + 3].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4 * len(plans))]
          for _ in range(args.steps)]
    start = torch.cuda.Event(enable_timing=True)
    stop = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for s in range(args.steps):
        step(ev[s])
    stop.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    t_ms = start.elapsed_time(stop)
    if dist:
        tt = torch.tensor([t_ms], device='cuda')
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_ms = float(tt.item())
        dist.barrier()
    ms_per_step = t_ms / args.steps
    value = total_bytes * ws / (ms_per_step * 1e-3) / 1e9
    total_flops = sum(2 * pass_flops(N, K) for (N, K, _, _) in plans)
    gflops = total_flops * ws / (ms_per_step * 1e-3) / 1e9

    # per-launch durations (events around each launch inside the timed region)
    per_n = []
    kernel_ms = 0.0
    for i, (N, K, _, _) in enumerate(plans):
        tf = np.mean([ev[s][4 * i].elapsed_time(ev[s][4 * i + 1]) for s in range(args.steps)])
        tb = np.mean([ev[s][4 * i + 2].elapsed_time(ev[s][4 * i + 3]) for s in range(args.steps)])
        kernel_ms += tf + tb
        pbytes = pass_bytes(N, K, prec)
        pfl = pass_flops(N, K)
        per_n.append({'N': N, 'K': K, 'r2c_gbs': round(pbytes / tf / 1e6, 1),
                      'c2r_gbs': round(pbytes / tb / 1e6, 1),
                      'r2c_gflops': round(pfl / tf / 1e6, 1), 'c2r_gflops': round(pfl / tb / 1e6, 1),
                      'r2c_frac': round(pbytes / tf / 1e6 / hbm_peak, 3),
                      'c2r_frac': round(pbytes / tb / 1e6 / hbm_peak, 3)})
    achieved = total_bytes / (kernel_ms * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(REPO, 'profiles', 'traffic.json')
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic = json.load(f).get('bytes_per_step')

    # end-to-end through the C ABI with pinned host buffers (rank-local)
    e2e = run_e2e(bb, torch, plans, prec, sptr, stream, args)
    del xbuf, Xbuf, ybuf
    torch.cuda.empty_cache()
    legs = {}
    wanted = LEGS if args.legs == 'all' else [w for w in args.legs.split(',') if w]
    if not args.no_legs and rank == 0:
        peaks = None
        runners = {
            'peaks': lambda: leg_peaks(torch, stream),
            'c2c_n64_k16384': lambda: leg_c2c_cfg1(bb, torch, stream, hbm_peak, args.steps, args.warmup),
            'ragged_10k': lambda: leg_ragged(bb, torch, stream, hbm_peak, args.steps, args.warmup),
            'spectral_layer_2d': lambda: leg_spectral(bb, torch, stream, args.steps, args.warmup),
            'c2c_3d_64': lambda: leg_c2c_3d(bb, torch, stream, hbm_peak, args.steps, args.warmup),
            'tft_vs_double_batched': lambda: leg_tft(bb, torch, stream, hbm_peak, args.steps, args.warmup),
            'sweep_f64': lambda: leg_sweep_f64(bb, torch, stream, hbm_peak, max(2, args.steps // 2), 1,
                                               peaks),
            'tensor_core_c2c': lambda: leg_tensor_core(bb, torch, stream, hbm_peak, args.steps,
                                                       args.warmup, peaks),
            'cufft': lambda: leg_cufft(bb, torch, stream, hbm_peak, plans),
            'sweep_all_n': lambda: leg_sweep_all_n(bb, torch, stream, hbm_peak),
        }
        for name in wanted:
            if name not in runners:
                raise SystemExit('unknown leg ' + name)
            try:
                legs[name] = runners[name]()
            except (RuntimeError, OSError) as e:  # one failing leg does not lose the line
                legs[name] = {'error': str(e)[:300]}
            if name == 'peaks' and 'error' not in legs[name]:
                peaks = legs[name]
            torch.cuda.empty_cache()

    line = {
        'metric': METRIC, 'value': round(value, 1), 'unit': 'GB/s', 'n_gpus': ws,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(ms_per_step, 4),
        'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
        'data': 'synthetic: iid N(0,1) float32 reals from a seeded generator',
        'config': {'workload': 'r2c+c2r round trip, M=8, 1 GiB real input per N, f32',
                   'N': SWEEP_N, 'M': M_BATCH, 'l2': 'inputs of 1 GiB per pass > L2, no flush',
                   'parallelism': 'K-slab per rank, no collectives' if ws > 1 else 'single GPU'},
        'roofline': {'bound': 'hbm', 'achieved': round(achieved, 1), 'peak': hbm_peak,
                     'unit': 'GB/s', 'frac': round(achieved / hbm_peak, 4), 'traffic': traffic,
                     'algorithmic_bytes': total_bytes, 'per': 'step (28 launches)',
                     'peak_kind': peak_kind, 'kernel': 'fft_kernel_ct<float, kind, ...> (all '
                     'launches of the step; algorithmic bytes = one read + one write)'},
        'gflops': {'value': round(gflops, 1), 'unit': 'GFLOP/s',
                   'model': '2.5 N log2 N per real transform (reference benchmark/adapter.hpp:51-52)'},
        'per_n': per_n,
        'clocks': clk,
        'e2e': e2e,
        'gpu_launches': 2 * len(plans) * args.steps,
        'legs': legs,
    }
    if rank == 0 and not args.no_cpu:
        line['cpu_baseline'] = cpu_baseline(prec, sweeps=args.cpu_sweeps)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def event_time(torch, stream, fn, reps):
    """Average device time of fn() over reps launches (CUDA events on `stream`)."""
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def leg_sweep_f64(bb, torch, stream, hbm_peak, steps, warmup, peaks=None):
    """Same r2c+c2r sweep in float64.  Each launch is also reported against its roofline
    min(HBM, FP64 peak / flop-per-byte) with the reference's flop model (2.5 N log2 N per
    real transform) and the FP64 FMA peak measured by the peaks leg."""
    sptr = stream.cuda_stream
    fp64 = peaks['fp64_tflops'] if peaks else None
    out = []
    tot_b, tot_ms = 0, 0.0
    x = torch.randn((1 << 30) // 8, dtype=torch.float64, device='cuda')
    maxc = max(M_BATCH * (N // 2 + 1) * k_for(N, 8) for N in SWEEP_N)
    X = torch.empty(2 * maxc, dtype=torch.float64, device='cuda')
    y = torch.empty_like(x)
    for N in SWEEP_N:
        K = k_for(N, 8)
        f = bb.Plan(bb.configuration(1, [M_BATCH, N, K], precision=bb.F64, type=bb.R2C), stream=sptr)
        b = bb.Plan(bb.configuration(1, [M_BATCH, N, K], precision=bb.F64, type=bb.C2R,
                                     direction=bb.BACKWARD), stream=sptr)
        for _ in range(warmup):
            f.execute(x.data_ptr(), X.data_ptr())
            b.execute(X.data_ptr(), y.data_ptr())
        tf = event_time(torch, stream, lambda: f.execute(x.data_ptr(), X.data_ptr()), steps)
        tb = event_time(torch, stream, lambda: b.execute(X.data_ptr(), y.data_ptr()), steps)
        pb = pass_bytes(N, K, 8)
        pf = pass_flops(N, K)
        tot_b += 2 * pb
        tot_ms += tf + tb
        rec = {'N': N, 'r2c_gbs': round(pb / tf / 1e6, 1), 'c2r_gbs': round(pb / tb / 1e6, 1),
               'r2c_gflops': round(pf / tf / 1e6, 1), 'c2r_gflops': round(pf / tb / 1e6, 1)}
        if fp64:
            # attainable GB/s of this launch: min(HBM, FP64 peak / (flops per byte))
            bound = min(hbm_peak, fp64 * 1e3 * pb / pf)
            rec['roofline_gbs'] = round(bound, 1)
            rec['r2c_frac'] = round(pb / tf / 1e6 / bound, 3)
            rec['c2r_frac'] = round(pb / tb / 1e6 / bound, 3)
        out.append(rec)
    res = {'value': round(tot_b / tot_ms / 1e6, 1), 'unit': 'GB/s',
           'frac_of_hbm': round(tot_b / tot_ms / 1e6 / hbm_peak, 3),
           'note': 'r2c+c2r M=8, 1 GiB real input per N, float64',
           'per_n': out}
    if fp64:
        tot_bound_ms = sum(2 * pass_bytes(r['N'], k_for(r['N'], 8), 8) / r['roofline_gbs'] / 1e6
                           for r in out)
        res['fp64_peak_tflops'] = fp64
        res['frac_of_roofline'] = round(tot_bound_ms / tot_ms, 3)
        res['roofline'] = ('per launch min(HBM, FP64 FMA peak x bytes / model flops), model flops '
                           '2.5 N log2 N per real transform')
    return res


def probes_lib():
    import ctypes

    lib = ctypes.CDLL(os.path.join(PKG, 'bbfft_gb300', '_lib', 'libbbfft_probes.so'))
    for f in ('gbfft_probe_dfma', 'gbfft_probe_ffma', 'gbfft_probe_mma_tf32', 'gbfft_probe_mma_bf16'):
        getattr(lib, f).argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                    ctypes.c_void_p]
    return lib


def leg_peaks(torch, stream, seconds=0.6):
    """Measured throughput of the pipes the transforms can be bound by, besides HBM: the
    FP64 and FP32 FMA pipes (independent FMA chains in registers) and the warp-level MMAs
    of the tensor-core stages (mma.sync TF32 m16n8k8, BF16 m16n8k16), each timed with CUDA
    events over about `seconds` of back-to-back work, SM clock sampled meanwhile."""
    lib = probes_lib()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks, threads = sms * 8, 256
    out = torch.empty(blocks * threads, dtype=torch.float64, device='cuda')
    sptr = stream.cuda_stream
    chains, acc = 8, 4
    kinds = {
        # name: (entry, flops per iteration per thread)
        'fp64_tflops': (lib.gbfft_probe_dfma, 2 * chains),
        'fp32_tflops': (lib.gbfft_probe_ffma, 2 * chains),
        'mma_tf32_tflops': (lib.gbfft_probe_mma_tf32, 2 * 16 * 8 * 8 * acc / 32),
        'mma_bf16_tflops': (lib.gbfft_probe_mma_bf16, 2 * 16 * 8 * 16 * acc / 32),
    }
    res = {}
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    for name, (fn, fpi) in kinds.items():
        iters = 256
        for _ in range(12):  # calibrate: grow until one launch takes >= 20 ms
            ms = event_time(torch, stream, lambda: fn(blocks, threads, iters, out.data_ptr(), sptr), 1)
            if ms >= 20.0 or iters >= (1 << 24):
                break
            iters = int(iters * min(16.0, max(2.0, 25.0 / max(ms, 1e-3))))
        reps = max(1, int(seconds * 1e3 / ms))
        ms = event_time(torch, stream, lambda: fn(blocks, threads, iters, out.data_ptr(), sptr), reps)
        res[name] = round(blocks * threads * iters * fpi / (ms * 1e-3) / 1e12, 2)
    clk = clocks.stop()
    res['clocks'] = clk
    res['how'] = ('%d CTAs x %d threads; FMA: %d independent chains per thread; MMA: %d '
                  'independent accumulator tiles per warp; CUDA events' % (blocks, threads, chains, acc))
    return res


def leg_cufft(bb, torch, stream, hbm_peak, plans):
    """cuFFT on the headline shapes beside this library's launches: r2c + c2r, M = 8,
    1 GiB real input per N, float32, through torch.fft over the N mode of the (K, N, M)
    tensor (cuFFT rejects the reference's per-m loop, benchmark/test-cufft.cpp:38-45, for
    real data: a real tensor offset by one float is not a valid cuFFT pointer); and c2c
    M = 8 the reference's way, one cufftPlanMany over K executed once per m."""
    from bbfft_gb300 import cufft

    sptr = stream.cuda_stream
    maxr = max(M_BATCH * N * k_for(N, 4) for N in SWEEP_N)
    maxc = max(M_BATCH * (N // 2 + 1) * k_for(N, 4) for N in SWEEP_N)
    x = torch.randn(maxr, device='cuda')
    X = torch.empty(2 * maxc, device='cuda')
    y = torch.empty(maxr, device='cuda')
    rows, tot_b, tot_ours, tot_cu = [], 0, 0.0, 0.0
    for (N, K, pf, pb) in plans:
        xv = x[:M_BATCH * N * K].view(K, N, M_BATCH)
        Xv = torch.view_as_complex(X[:2 * M_BATCH * (N // 2 + 1) * K].view(K, N // 2 + 1, M_BATCH, 2))
        yv = y[:M_BATCH * N * K].view(K, N, M_BATCH)

        def tfft():
            torch.fft.rfft(xv, dim=1, out=Xv)
            torch.fft.irfft(Xv, n=N, dim=1, norm='forward', out=yv)

        tfft()
        t_cu = event_time(torch, stream, tfft, 3)
        t_ours = event_time(torch, stream, lambda: (pf.execute(x.data_ptr(), X.data_ptr()),
                                                    pb.execute(X.data_ptr(), y.data_ptr())), 3)
        b = 2 * pass_bytes(N, K, 4)
        tot_b += b
        tot_ours += t_ours
        tot_cu += t_cu
        # c2c, M = 8, the reference's cuFFT loop over m (complex offsets are valid pointers)
        Kc = (1 << 30) // (8 * M_BATCH * N)
        cp = cufft.Plan(4, 'c2c', M_BATCH, N, Kc, sptr)
        op = bb.Plan(bb.configuration(1, [M_BATCH, N, Kc], precision=bb.F32), stream=sptr)
        cp.execute(x.data_ptr(), y.data_ptr())
        op.execute(x.data_ptr(), y.data_ptr())
        t_cc = event_time(torch, stream, lambda: cp.execute(x.data_ptr(), y.data_ptr()), 3)
        t_oc = event_time(torch, stream, lambda: op.execute(x.data_ptr(), y.data_ptr()), 3)
        cp.destroy()
        bc = 2 * M_BATCH * N * Kc * 8
        rows.append({'N': N, 'r2c_c2r_torch_fft_gbs': round(b / t_cu / 1e6, 1),
                     'r2c_c2r_ours_gbs': round(b / t_ours / 1e6, 1),
                     'c2c_cufft_loop_gbs': round(bc / t_cc / 1e6, 1),
                     'c2c_ours_gbs': round(bc / t_oc / 1e6, 1)})
    return {'r2c_c2r_torch_fft_gbs': round(tot_b / tot_cu / 1e6, 1),
            'r2c_c2r_ours_gbs': round(tot_b / tot_ours / 1e6, 1),
            'speedup_vs_torch_fft': round(tot_cu / tot_ours, 2), 'per_n': rows,
            'how': 'r2c+c2r: torch.fft.rfft / irfft over dim 1 of the (K, N, 8) tensor (cuFFT), '
                   '1 GiB real input per N; c2c: cufftPlanMany over K (stride 8, distance 8N) '
                   'executed once per m, 1 GiB complex input per N; float32, CUDA events'}


ALL_N = list(range(16, 513))


def leg_sweep_all_n(bb, torch, stream, hbm_peak, reps=2):
    """Every N in 16..512, float32, each launch on a 1 GiB input: c2c forward at M = 1 and
    M = 8, r2c and c2r at M = 8; GB/s (one read + one write) as fractions of the measured
    HBM bandwidth, and cuFFT's c2c M = 1 beside them."""
    from bbfft_gb300 import cufft

    sptr = stream.cuda_stream
    cap = (1 << 28) + (1 << 25)  # floats: 1.125 GiB covers every input and output
    x = torch.randn(cap, device='cuda')
    y = torch.empty(cap, device='cuda')
    z = torch.empty(cap, device='cuda')
    res = {k: [] for k in ('c2c_m1', 'c2c_m8', 'r2c_m8', 'c2r_m8', 'cufft_c2c_m1')}
    t0 = time.perf_counter()
    for N in ALL_N:
        cases = [
            ('c2c_m1', bb.configuration(1, [1, N, (1 << 30) // (8 * N)], precision=bb.F32), x, y,
             2 * N * 8 * ((1 << 30) // (8 * N))),
            ('c2c_m8', bb.configuration(1, [8, N, (1 << 30) // (64 * N)], precision=bb.F32), x, y,
             2 * 8 * N * 8 * ((1 << 30) // (64 * N))),
        ]
        K = (1 << 30) // (32 * N)
        cases.append(('r2c_m8', bb.configuration(1, [8, N, K], precision=bb.F32, type=bb.R2C), x, y,
                      pass_bytes(N, K, 4)))
        cases.append(('c2r_m8', bb.configuration(1, [8, N, K], precision=bb.F32, type=bb.C2R,
                                                 direction=bb.BACKWARD), y, z, pass_bytes(N, K, 4)))
        for name, cfg, a, b, nbytes in cases:
            plan = bb.Plan(cfg, stream=sptr)
            plan.execute(a.data_ptr(), b.data_ptr())
            ms = event_time(torch, stream, lambda: plan.execute(a.data_ptr(), b.data_ptr()), reps)
            res[name].append(round(nbytes / ms / 1e6 / hbm_peak, 3))
            del plan
        Kc = (1 << 30) // (8 * N)
        cp = cufft.Plan(4, 'c2c', 1, N, Kc, sptr)
        cp.execute(x.data_ptr(), y.data_ptr())
        ms = event_time(torch, stream, lambda: cp.execute(x.data_ptr(), y.data_ptr()), reps)
        res['cufft_c2c_m1'].append(round(2 * N * 8 * Kc / ms / 1e6 / hbm_peak, 3))
        cp.destroy()
    summary = {}
    for k, v in res.items():
        arr = np.array(v)
        worst = np.argsort(arr)[:8]
        summary[k] = {'at_least_0.8': int((arr >= 0.8).sum()), 'of': len(v),
                      'min': float(arr.min()), 'median': float(np.median(arr)),
                      'worst': [[ALL_N[i], float(arr[i])] for i in worst]}
    mult8 = [i for i, N in enumerate(ALL_N) if N % 8 == 0]
    for k in ('c2c_m1', 'c2c_m8', 'r2c_m8', 'c2r_m8'):
        summary[k]['multiples_of_8_at_least_0.8'] = int(sum(res[k][i] >= 0.8 for i in mult8))
        summary[k]['multiples_of_8'] = len(mult8)
    return {'unit': 'fraction of measured HBM bandwidth', 'N': [ALL_N[0], ALL_N[-1]],
            'summary': summary, 'frac': res, 'seconds': round(time.perf_counter() - t0, 1),
            'how': 'plan per (N, kind), 1 warm-up launch, %d timed (CUDA events); inputs 1 GiB '
                   '(> L2)' % reps}


def leg_c2c_cfg1(bb, torch, stream, hbm_peak, steps, warmup):
    """c2c forward complex64, M=1, N=64, K=16384 (8 MiB in + 8 MiB out): 24 rotating
    input/output pairs (384 MiB) so that consecutive launches miss in L2."""
    sptr = stream.cuda_stream
    M, N, K = 1, 64, 16384
    nb = 24
    xs = [torch.randn(2 * M * N * K, device='cuda') for _ in range(nb)]
    ys = [torch.empty(2 * M * N * K, device='cuda') for _ in range(nb)]
    plan = bb.Plan(bb.configuration(1, [M, N, K], precision=bb.F32), stream=sptr)
    state = {'i': 0}

    def one():
        i = state['i'] % nb
        plan.execute(xs[i].data_ptr(), ys[i].data_ptr())
        state['i'] += 1

    for _ in range(warmup * nb):
        one()
    ms = event_time(torch, stream, one, max(steps, 4) * nb)
    b = 2 * M * N * K * 8
    # the same 24 launches captured once in a CUDA graph and replayed (no per-launch host
    # work between the kernels)
    g = torch.cuda.CUDAGraph()
    cs = torch.cuda.Stream()
    cs.wait_stream(stream)
    with torch.cuda.graph(g, stream=cs):
        for i in range(nb):
            plan.execute_on(xs[i].data_ptr(), ys[i].data_ptr(), cs.cuda_stream)
    stream.wait_stream(cs)
    for _ in range(warmup):
        g.replay()
    msg = event_time(torch, torch.cuda.current_stream(), g.replay, max(steps, 4)) / nb
    best = min(ms, msg)
    # the floor at this size: a device copy of the same 8 MiB per launch (same bytes read
    # and written), 24 rotating buffer pairs in one graph
    gc = torch.cuda.CUDAGraph()
    with torch.cuda.graph(gc, stream=cs):
        for i in range(nb):
            ys[i].copy_(xs[i])
    stream.wait_stream(cs)
    for _ in range(warmup):
        gc.replay()
    msc = event_time(torch, torch.cuda.current_stream(), gc.replay, max(steps, 4)) / nb
    return {'value': round(b / best / 1e6, 1), 'unit': 'GB/s',
            'frac_of_hbm': round(b / best / 1e6 / hbm_peak, 3),
            'us_per_launch_stream': round(ms * 1e3, 2), 'us_per_launch_graph': round(msg * 1e3, 2),
            'gbs_stream': round(b / ms / 1e6, 1), 'gbs_graph': round(b / msg / 1e6, 1),
            'copy_us_per_launch_graph': round(msc * 1e3, 2), 'copy_gbs_graph': round(b / msc / 1e6, 1),
            'frac_of_copy_at_this_size': round(msc / best, 3),
            'l2': '24 rotating buffer pairs, 384 MiB'}


def ragged_specs(bb, n=10000, seed=4):
    """The ragged workload: N in {16,...,512} step 8, c2c complex64 / r2c float32 50/50,
    M in {1,4,16}, K in [1,64]; offsets keep every tensor 16-byte aligned."""
    rng = np.random.default_rng(seed)
    specs = []
    in_off = out_off = 0
    for _ in range(n):
        N = int(rng.choice(list(range(16, 513, 8))))
        t = bb.C2C if rng.random() < 0.5 else bb.R2C
        M = int(rng.choice([1, 4, 16]))
        K = int(rng.integers(1, 65))
        nin = M * N * K * (2 if t == bb.C2C else 1)
        nout = M * (N if t == bb.C2C else N // 2 + 1) * K * 2
        specs.append((t, N, M, K, in_off, out_off))
        in_off += (nin + 3) // 4 * 4
        out_off += (nout + 3) // 4 * 4
    return specs, in_off, out_off


def leg_ragged(bb, torch, stream, hbm_peak, steps, warmup):
    """10^4 transforms with U[-1,1] data replayed from a graph: one launch (persistent CTAs
    taking tiles from a counter, or one CTA per tile) and one kernel node per tile
    function (class form)."""
    specs, nin, nout = ragged_specs(bb)
    x = torch.empty(nin, dtype=torch.float32, device='cuda').uniform_(-1, 1)
    y = torch.empty(nout, dtype=torch.float32, device='cuda')
    items = [(bb.F32, bb.FORWARD, t, N, M, K, x.data_ptr() + 4 * io, y.data_ptr() + 4 * oo)
             for (t, N, M, K, io, oo) in specs]
    r = bb.Ragged(items)
    info = r.info()
    sptr = stream.cuda_stream
    forms = {}
    for name, form in (('persistent', r.PERSISTENT), ('grid', r.GRID), ('classes', r.CLASSES)):
        r.set_launch_form(form)
        for _ in range(warmup):
            r.execute(sptr, use_graph=True)
        ms = event_time(torch, stream, lambda: r.execute(sptr, use_graph=True), max(steps, 5))
        gbs = info.bytes_moved / ms / 1e6
        forms[name] = {'value': round(gbs, 1), 'frac_of_hbm': round(gbs / hbm_peak, 3),
                       'ms_per_batch': round(ms, 3),
                       'ctas': int(info.grid) if form == r.PERSISTENT else int(info.num_units),
                       'launches': 1 if form != r.CLASSES else 'one kernel node per tile function'}
    best = max(forms, key=lambda k: forms[k]['value'])
    return {'value': forms[best]['value'], 'unit': 'GB/s', 'form': best,
            'frac_of_hbm': forms[best]['frac_of_hbm'], 'forms': forms,
            'bytes_moved': int(info.bytes_moved), 'units': int(info.num_units),
            'launches_per_batch': forms[best]['launches']}


def leg_spectral(bb, torch, stream, steps, warmup):
    """2d r2c 128x128, K = 64 x 32, complex weights on the lowest 32x32 modes, c2r,
    loss sum(y^2): float32 forward + backward time."""
    from bbfft_gb300.autograd import SpectralLayer2d

    layer = SpectralLayer2d(128, 128, 64, 32, 32, 32, prec=bb.F32)
    x = torch.randn(64, 32, 128, 128, device='cuda', requires_grad=True)
    w = (torch.randn(32, 32, 32, dtype=torch.complex64, device='cuda') * 0.02).requires_grad_(True)

    def step():
        loss = (layer(x, w) ** 2).sum()
        loss.backward()

    for _ in range(warmup):
        step()
    ms = event_time(torch, stream, step, max(steps, 3))
    # four 2d transforms per step (r2c and c2r forward, their adjoints backward), each one
    # read and one write of a real (128x128) and a half-spectrum (65x128) tensor of K images
    K = 64 * 32
    b = 4 * K * (128 * 128 * 4 + 65 * 128 * 8)
    return {'ms_fwd_bwd': round(ms, 3), 'gbs_transforms': round(b / ms / 1e6, 1),
            'transform_bytes': b,
            'note': 'bytes of the four 2d transforms (one read + one write each); the mode '
                    'multiply, slicing and zero fill run as torch ops in the same time',
            'shape': 'r2c/c2r 128x128, K=2048, modes 32x32, f32'}


def leg_tft(bb, torch, stream, hbm_peak, steps, warmup):
    """The reference's transpose-FFT-transpose example (examples/transpose_fft_transpose):
    c2c float over the N mode of an M x N x K tensor (M = 64, N = 64, 512 MB), either as
    transpose -> contiguous FFT (M = 1) -> transpose, or as one double-batched plan that
    reads the M x N x K layout directly (the transposes folded into its loads and stores)."""
    sptr = stream.cuda_stream
    M, N = 64, 64
    K = (512 * 1000 * 1000) // (8 * M * N)
    x = torch.randn(K, N, M, dtype=torch.complex64, device='cuda')
    y = torch.empty_like(x)
    direct = bb.Plan(bb.configuration(1, [M, N, K], precision=bb.F32), stream=sptr)
    inner = bb.Plan(bb.configuration(1, [1, N, M * K], precision=bb.F32), stream=sptr)
    xt = torch.empty(K, M, N, dtype=torch.complex64, device='cuda')

    def tft():
        xt.copy_(x.permute(0, 2, 1))                      # (K, M, N): N contiguous
        inner.execute(xt.data_ptr())                      # in place, M = 1
        y.copy_(xt.permute(0, 2, 1))                      # back to (K, N, M)

    def dbl():
        direct.execute(x.data_ptr(), y.data_ptr())

    for _ in range(warmup):
        tft()
        dbl()
    ms_tft = event_time(torch, stream, tft, max(steps, 3))
    ms_dbl = event_time(torch, stream, dbl, max(steps, 3))
    b = 2 * M * N * K * 8
    return {'ms_transpose_fft_transpose': round(ms_tft, 3), 'ms_double_batched': round(ms_dbl, 3),
            'gbs_double_batched': round(b / ms_dbl / 1e6, 1), 'speedup': round(ms_tft / ms_dbl, 2),
            'shape': 'c2c f32 M=64 N=64 K=%d' % K}


def leg_c2c_3d(bb, torch, stream, hbm_peak, steps, warmup):
    """3d c2c 64^3 complex64, K=64 (128 MiB), forward and backward (3 passes each)."""
    sptr = stream.cuda_stream
    shape = [1, 64, 64, 64, 64]
    n = 64 ** 4
    x = torch.randn(2 * n, device='cuda')
    y = torch.empty_like(x)
    f = bb.Plan(bb.configuration(3, shape, precision=bb.F32, direction=bb.FORWARD), stream=sptr)
    b = bb.Plan(bb.configuration(3, shape, precision=bb.F32, direction=bb.BACKWARD), stream=sptr)
    for _ in range(warmup):
        f.execute(x.data_ptr(), y.data_ptr())
        b.execute(y.data_ptr(), x.data_ptr())

    def both():
        f.execute(x.data_ptr(), y.data_ptr())
        b.execute(y.data_ptr(), x.data_ptr())

    ms = event_time(torch, stream, both, max(steps, 3))
    bytes_ = 2 * 3 * 2 * n * 8  # 2 transforms x 3 passes x (read + write)
    once = 2 * 2 * n * 8        # 2 transforms x one read + one write of the tensor
    return {'ms_fwd_bwd': round(ms, 3), 'gbs_all_passes': round(bytes_ / ms / 1e6, 1),
            'gbs_one_read_one_write': round(once / ms / 1e6, 1),
            'frac_of_hbm': round(bytes_ / ms / 1e6 / hbm_peak, 3),
            'note': 'gbs_all_passes and frac_of_hbm count one read + one write per pass (three '
                    'passes per transform); gbs_one_read_one_write counts one per transform'}


# MMAs (mma.sync m16n8k8 TF32, 2048 flops each with the padding) per transform of the
# split-TF32 form: a radix-P stage on the tensor cores runs 2 (cosine, sine) x KS^2 x 3
# (split products) MMAs per 8 butterflies, KS = ceil((P/2 - 1) / 8): 3 per radix-32
# butterfly, 0.75 per radix-16 one.  64 = 32 x 2, 256 = 16 x 16, 512 = 32 x 16.
TF32_MMAS_PER_TRANSFORM = {64: 2 * 3, 256: 32 * 0.75, 512: 16 * 3 + 32 * 0.75}


def leg_tensor_core(bb, torch, stream, hbm_peak, steps, warmup, peaks=None):
    """c2c forward, M=1, K=2^20, N in {64, 256, 512}, N(0,1) inputs with a 1e-3 fraction
    scaled by 1e4: plain FP32 against the tensor-core forms, GB/s and rel-L2 against FP64
    on a 4096-transform slice; for the split-TF32 form also its MMA throughput against the
    measured mma.sync TF32 peak."""
    from oracle import pyoracle as po

    sptr = stream.cuda_stream
    K = 1 << 20
    out = {}
    tf32_peak = peaks.get('mma_tf32_tflops') if peaks else None
    for N in (64, 256, 512):
        g = torch.Generator(device='cuda')
        g.manual_seed(N)
        x = torch.randn(2 * N * K, device='cuda', generator=g)
        sel = torch.rand(2 * N * K, device='cuda', generator=g) < 1e-3
        x[sel] *= 1e4
        y = torch.empty_like(x)
        xs = x[:2 * N * 4096].cpu().numpy().view(np.complex64).astype(np.complex128)
        ref = po.dft64(1, [1, N, 4096], po.C2C, po.FORWARD, xs.reshape(4096, N, 1))
        row = {}
        for name, mode in (('fp32', 0), ('bf16', 1), ('split_bf16_3term', 3), ('split_bf16_6term', 2),
                           ('split_tf32_3term', 4)):
            plan = bb.Plan(bb.configuration(1, [1, N, K], precision=bb.F32, compute=mode), stream=sptr)
            for _ in range(warmup):
                plan.execute(x.data_ptr(), y.data_ptr())
            ms = event_time(torch, stream, lambda: plan.execute(x.data_ptr(), y.data_ptr()), max(steps, 3))
            got = y[:2 * N * 4096].cpu().numpy().view(np.complex64).reshape(ref.shape)
            err = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
            gbs = 2 * N * K * 8 / ms / 1e6
            row[name] = {'gbs': round(gbs, 1), 'frac_of_hbm': round(gbs / hbm_peak, 3),
                         'rel_l2': float('%.3g' % err)}
            if mode == 4:
                tfl = TF32_MMAS_PER_TRANSFORM[N] * 2048 * K / ms / 1e9
                row[name]['mma_tflops'] = round(tfl, 1)
                if tf32_peak:
                    row[name]['frac_of_mma_tf32_peak'] = round(tfl / tf32_peak, 3)
        out['N%d' % N] = row
        del x, y
    return out


def run_e2e(bb, torch, plans, prec, sptr, stream, args):
    """Same workload through the C ABI from pinned host memory: per N, K-chunks flow
    host -> device (copy stream), r2c + c2r (compute stream, bbfft_plan_execute_on) and
    device -> host (copy stream back), double-buffered so that the copies of one chunk
    overlap the transforms of the next.  All copies are inside the timed region."""
    # a reduced sweep keeps the host buffers small: every N, K-slab of 1/8 of the tensor
    frac, nchunk = 8, 4
    total_bytes, h2d, d2h = 0, 0, 0
    chunks = []  # (forward plan, backward plan, host offset in reals, reals, complexes)
    off = 0
    for (N, K, _, _) in plans:
        Ks = max(1, K // frac)
        Kc = (Ks + nchunk - 1) // nchunk
        made = {}
        k0 = 0
        while k0 < Ks:
            kc = min(Kc, Ks - k0)
            if kc not in made:
                f = bb.configuration(1, [M_BATCH, N, kc], precision=bb.F32, type=bb.R2C)
                b = bb.configuration(1, [M_BATCH, N, kc], precision=bb.F32, type=bb.C2R,
                                     direction=bb.BACKWARD)
                made[kc] = (bb.Plan(f, stream=sptr), bb.Plan(b, stream=sptr))
            nreal = M_BATCH * N * kc
            chunks.append(made[kc] + (off, nreal, M_BATCH * (N // 2 + 1) * kc))
            off += nreal
            k0 += kc
        total_bytes += 2 * pass_bytes(N, Ks, prec)
        h2d += M_BATCH * N * Ks * prec
        d2h += M_BATCH * N * Ks * prec
    maxr = max(c[3] for c in chunks)
    maxc = max(c[4] for c in chunks)
    host_in = torch.empty(off, dtype=torch.float32, pin_memory=True)
    host_in.normal_()
    host_out = torch.empty(off, dtype=torch.float32, pin_memory=True)
    d_in = [torch.empty(maxr, dtype=torch.float32, device='cuda') for _ in range(2)]
    d_X = [torch.empty(2 * maxc, dtype=torch.float32, device='cuda') for _ in range(2)]
    d_out = [torch.empty(maxr, dtype=torch.float32, device='cuda') for _ in range(2)]
    s_in, s_comp, s_out = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
    ev = {k: [torch.cuda.Event() for _ in range(2)] for k in ('in', 'comp', 'out')}

    def step():
        for st in (s_in, s_comp, s_out):
            st.wait_stream(stream)
        for i, (pf, pb, o, nreal, _) in enumerate(chunks):
            sl = i % 2
            if i >= 2:
                s_in.wait_event(ev['comp'][sl])   # d_in[sl] consumed by chunk i - 2
            with torch.cuda.stream(s_in):
                d_in[sl][:nreal].copy_(host_in[o:o + nreal], non_blocking=True)
            ev['in'][sl].record(s_in)
            s_comp.wait_event(ev['in'][sl])
            if i >= 2:
                s_comp.wait_event(ev['out'][sl])  # d_out[sl] drained by chunk i - 2
            pf.execute_on(d_in[sl].data_ptr(), d_X[sl].data_ptr(), s_comp.cuda_stream)
            pb.execute_on(d_X[sl].data_ptr(), d_out[sl].data_ptr(), s_comp.cuda_stream)
            ev['comp'][sl].record(s_comp)
            s_out.wait_event(ev['comp'][sl])
            with torch.cuda.stream(s_out):
                host_out[o:o + nreal].copy_(d_out[sl][:nreal], non_blocking=True)
            ev['out'][sl].record(s_out)
        for st in (s_in, s_comp, s_out):
            stream.wait_stream(st)

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    s0 = torch.cuda.Event(enable_timing=True)
    s1 = torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(args.steps):
        step()
    s1.record(stream)
    torch.cuda.synchronize()
    ms = s0.elapsed_time(s1) / args.steps
    return {'value': round(total_bytes / (ms * 1e-3) / 1e9, 1), 'unit': 'GB/s',
            'h2d_bytes_per_step': h2d, 'd2h_bytes_per_step': d2h,
            'workload': 'same sweep at 1/8 of K per N (128 MiB real input per N) in 4 K-chunks, '
                        'pinned host buffers, copies on two copy streams overlapping the '
                        'transforms, all inside the timed region'}


def run_profile(args):
    """Launches for an ncu capture, no timing: `step` runs every plan of one benchmark step
    once (28 launches); `case` runs one plan per comma-separated spec
    KIND:N[:FORM[:M[:PREC]]] once (KIND c2c / r2c / c2r; FORM native, bf16, split3, split6
    or tf32 for the tensor-core forms of c2c; M default 1 for c2c, 8 otherwise; PREC 4 or
    8 bytes; K sized for --profile-bytes of input, default 1 GiB, or K = 2^20 for c2c
    with M = 1); `ragged` runs the ragged batch once in the class form (one kernel per tile
    function)."""
    import torch

    import bbfft_gb300 as bb

    stream = torch.cuda.current_stream().cuda_stream
    if args.profile == 'ragged':
        specs, nin, nout = ragged_specs(bb)
        x = torch.empty(nin, dtype=torch.float32, device='cuda').uniform_(-1, 1)
        y = torch.empty(nout, dtype=torch.float32, device='cuda')
        r = bb.Ragged([(bb.F32, bb.FORWARD, t, N, M, K, x.data_ptr() + 4 * io, y.data_ptr() + 4 * oo)
                       for (t, N, M, K, io, oo) in specs])
        r.set_launch_form(r.CLASSES)
        r.execute(stream)
        torch.cuda.synchronize()
        print('profiled ragged batch, units:', r.info().num_units)
        return
    forms = {'native': bb.COMPUTE_NATIVE, 'bf16': bb.COMPUTE_BF16,
             'split3': bb.COMPUTE_SPLIT_BF16_3TERM, 'split6': bb.COMPUTE_SPLIT_BF16,
             'tf32': bb.COMPUTE_SPLIT_TF32}
    if args.profile == 'step':
        cases = [('r2c' if i % 2 == 0 else 'c2r', N, 'native', M_BATCH, 4)
                 for N in SWEEP_N for i in range(2)]
    else:
        cases = []
        for spec in args.profile_case.split(','):
            f = spec.split(':')
            kind, N = f[0], int(f[1])
            form = f[2] if len(f) > 2 and f[2] else 'native'
            M = int(f[3]) if len(f) > 3 else (1 if kind == 'c2c' else M_BATCH)
            prec = int(f[4]) if len(f) > 4 else 4
            cases.append((kind, N, form, M, prec))
    cfgs = []
    for kind, N, form, M, prec in cases:
        words = prec // 4  # floats per real
        if kind == 'c2c':
            K = (1 << 20) if (M == 1 and args.profile_bytes is None) else \
                (args.profile_bytes or REAL_BYTES) // (M * N * 2 * prec)
            cfg = bb.configuration(1, [M, N, K], precision=prec, compute=forms[form])
            nin = nout = 2 * M * N * K * words
        elif kind in ('r2c', 'c2r'):
            K = (args.profile_bytes or REAL_BYTES) // (prec * M * N)
            if kind == 'r2c':
                cfg = bb.configuration(1, [M, N, K], precision=prec, type=bb.R2C)
                nin, nout = M * N * K * words, 2 * M * (N // 2 + 1) * K * words
            else:
                cfg = bb.configuration(1, [M, N, K], precision=prec, type=bb.C2R,
                                       direction=bb.BACKWARD)
                nin, nout = 2 * M * (N // 2 + 1) * K * words, M * N * K * words
        else:
            raise SystemExit('unknown profile case ' + kind)
        cfgs.append((cfg, nin, nout))
    # buffers sized from the largest input / output extent (in floats) of the cases
    x = torch.randn(max(c[1] for c in cfgs), device='cuda')
    y = torch.empty(max(c[2] for c in cfgs), device='cuda')
    assert x.numel() * 4 <= (6 << 30), 'profile cases hold a few GB at most'
    for cfg, nin, nout in cfgs:
        assert nin <= x.numel() and nout <= y.numel()
        plan = bb.Plan(cfg, stream=stream)
        plan.execute(x.data_ptr(), y.data_ptr())
        i = plan.info()
        print('plan', i.identifier.decode(), 'T', i.threads_per_transform, 'Mb', i.mb, 'Kb', i.kb,
              'V', i.vector_width, 'block', i.block_threads, 'smem', i.shared_bytes,
              'min_blocks', i.min_blocks)
    torch.cuda.synchronize()
    print('profiled launches:', len(cases))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--no-cpu', action='store_true')
    ap.add_argument('--cpu-sweeps', type=int, default=3, help='timed sweeps of the CPU sample')
    ap.add_argument('--no-legs', action='store_true', help='headline workload only')
    ap.add_argument('--legs', default='all',
                    help='comma-separated secondary legs to run (default: all): ' + ','.join(LEGS))
    ap.add_argument('--profile', choices=['step', 'case', 'ragged'], help='launches for an ncu capture')
    ap.add_argument('--profile-case', default='c2r:160')
    ap.add_argument('--profile-bytes', type=int, default=None,
                    help='input bytes of each --profile case plan (default 1 GiB)')
    args = ap.parse_args()
    if args.profile:
        run_profile(args)
        return
    if args.impl == 'reference':
        run_reference(args)
    else:
        run_ours(args)


if __name__ == '__main__':
    main()
