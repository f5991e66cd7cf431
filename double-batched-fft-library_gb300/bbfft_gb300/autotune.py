"""Autotuner for the double-batched FFT plans on GB300.

For a 1d configuration the tuner times candidate blockings of the plan -- transforms per
thread along M (V), the M- and K-extent of a CTA tile (Mb, Kb) -- with CUDA events on
device-resident data and records the fastest in a tuning table.  bbfft_plan_create
consults the table (one line per precision, kernel kind, N and M:
``<prec> <kind> <N> <M> <V> <Mb> <Kb> <CTAs per SM>``, the last being the resident-CTA
count the compile-time kernel's registers are sized for).  The radices and threads per transform stay
those of the library's heuristic, which the compile-time kernels are instantiated for.

Usage (on the GPU):  python -m bbfft_gb300.autotune [--out PATH] [--quick]
"""
import argparse
import os
import re
import sys

import bbfft_gb300 as bb

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_OUT = os.path.join(os.path.dirname(HERE), 'tuning', 'gb300.tune')

SWEEP_N = [16, 32, 64, 128, 256, 512, 48, 96, 160, 224, 384, 7, 11, 13]


def _tensor_elems(dim, shape, stride):
    return sum((shape[d] - 1) * stride[d] for d in range(dim + 2)) + 1


def tune_config(torch, prec, type, N, M, K, reps=4, verbose=False):
    """Time every candidate blocking of one 1d configuration; returns (entry, results)."""
    direction = bb.BACKWARD if type == bb.C2R else bb.FORWARD
    cfg = bb.configuration(1, [M, N, K], precision=prec, type=type, direction=direction)
    n_in = N // 2 + 1 if type == bb.C2R else N
    n_out = N // 2 + 1 if type == bb.R2C else N
    in_b = _tensor_elems(1, [M, n_in, K], list(cfg.istride)) * prec * (1 if type == bb.R2C else 2)
    out_b = _tensor_elems(1, [M, n_out, K], list(cfg.ostride)) * prec * (1 if type == bb.C2R else 2)
    x = torch.randn(in_b // 4 + 16, device='cuda')
    y = torch.empty(out_b // 4 + 16, device='cuda')
    stream = torch.cuda.current_stream()
    results = {}
    mbs = sorted({m for m in (M, 64, 32, 16, 8, 4, 2, 1) if m <= M and m <= 64}, reverse=True)
    occs = (2, 3) if prec == 4 else (2,)
    if prec == 4 and type == bb.C2R and N % 2 == 0:
        occs += (12, 13)  # paired c2r pre-process variants
    stages = [(None, 0)]
    if prec == 4 and type != bb.C2C and N % 2 == 0:
        stages += [(tuple(r), t) for r, t in alt_stages()[0].get(N // 2, [])]
    if prec == 4 and type == bb.C2C:
        stages += [(tuple(r), t) for r, t in alt_stages()[1].get(N, [])]
    for rad, T in stages:
     for V in (0, 1, 2, 4):
        for Mb in mbs:
            for Kb in (0, 1, 2, 4, 8, 16, 32, 64, 128, 256):
              for occ in occs:
                try:
                    plan = bb.Plan(cfg, stream=stream.cuda_stream,
                                   tuning=(list(rad) if rad else None, T, V, Mb, Kb, occ))
                except bb.BBFFTError:
                    continue
                info = plan.info()
                if rad and not info.specialized:
                    plan.destroy()
                    continue  # only the compile-time kernels of the alternatives are worth timing
                key = (info.vector_width, info.mb, info.kb, info.min_blocks or 2,
                       tuple(info.radix[:info.num_stages]) if rad else (), info.threads_per_transform if rad else 0)
                if key in results:
                    continue
                for _ in range(2):
                    plan.execute(x.data_ptr(), y.data_ptr())
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(reps):
                    plan.execute(x.data_ptr(), y.data_ptr())
                e1.record(stream)
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1) / reps
                results[key] = (ms, info.identifier.decode())
                plan.destroy()
    best_key = min(results, key=lambda k: results[k][0])
    ident = results[best_key][1]
    kind = re.match(r'gbfft_f\d+_([a-z0-9]+)_', ident).group(1)
    nbytes = (n_in * (prec if type == bb.R2C else 2 * prec) + n_out * (prec if type == bb.C2R else 2 * prec)) * M * K
    gbs = nbytes / (results[best_key][0] * 1e-3) / 1e9
    entry = (prec, kind, N, M) + best_key[:4] + (best_key[5], 'x'.join(map(str, best_key[4])))
    if verbose:
        worst = max(r[0] for r in results.values())
        print('prec %d type %d N %4d M %4d: best V=%d Mb=%d Kb=%d occ=%d T=%d rad=%s %.1f GB/s (%d '
              'candidates, worst %.2fx)' % (prec, type, N, M, best_key[0], best_key[1], best_key[2],
                                            best_key[3], best_key[5], best_key[4] or 'auto', gbs,
                                            len(results), worst / results[best_key][0]), flush=True)
    return entry, gbs


def default_configs(quick=False):
    """The configurations of the benchmark workloads."""
    cfgs = []
    for prec in (4, 8):
        for N in SWEEP_N:
            K = (1 << 30) // (prec * 8 * N)
            if quick:
                K = max(1, K // 8)
            cfgs.append((prec, bb.R2C, N, 8, K))
            cfgs.append((prec, bb.C2R, N, 8, K))
    # c2c, M=1: the N=64 K=16384 case and the N in {64, 256, 512} K=2^20 cases
    for N in (64, 256, 512):
        cfgs.append((4, bb.C2C, N, 1, (1 << 20) if not quick else (1 << 17)))
    # passes of the 2d 128x128 r2c (K=2048) and the 3d 64^3 c2c (K=64)
    cfgs.append((4, bb.R2C, 128, 1, 128 * 2048))
    cfgs.append((4, bb.C2C, 128, 65, 2048))
    cfgs.append((4, bb.C2R, 128, 1, 128 * 2048))
    cfgs.append((4, bb.C2C, 64, 1, 64 * 64 * 64))
    cfgs.append((4, bb.C2C, 64, 64, 64 * 64))
    cfgs.append((4, bb.C2C, 64, 4096, 64))
    return cfgs


def alt_stages():
    """Alternative (radices, threads per transform) with compile-time kernels: by real half
    length and by c2c length (csrc/gen_specializations.py ALT_STAGES, ALT_STAGES_C2C)."""
    csrc = os.path.join(os.path.dirname(HERE), 'csrc')
    if csrc not in sys.path:
        sys.path.insert(0, csrc)
    import gen_specializations

    return gen_specializations.ALT_STAGES, gen_specializations.ALT_STAGES_C2C


def read_table(path):
    """Entries of an existing table as (prec, kind, N, M, V, Mb, Kb, occ), GB/s."""
    out = []
    if not os.path.exists(path):
        return out
    for line in open(path):
        body, _, note = line.partition('#')
        f = body.split()
        if len(f) < 7:
            continue
        occ = int(f[7]) if len(f) > 7 else 2
        T = int(f[8]) if len(f) > 9 else 0
        rad = f[9] if len(f) > 9 else ''
        e = (int(f[0]), f[1], int(f[2]), int(f[3]), int(f[4]), int(f[5]), int(f[6]), occ, T, rad)
        try:
            gbs = float(note.strip())
        except ValueError:
            gbs = 0.0
        out.append((e, gbs))
    return out


def write_table(path, entries):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    lines = ['# bbfft GB300 tuning table: <prec bytes> <kind> <N> <M> <V> <Mb> <Kb> <CTAs per SM> '
             '[<threads per transform> <radices AxB>]  # GB/s',
             '# written by bbfft_gb300/autotune.py from CUDA-event timings on a GB300']
    for e, gbs in entries:
        head = '%d %s %d %d %d %d %d %d' % e[:8]
        if len(e) > 9 and e[9]:
            head += ' %d %s' % (e[8], e[9])
        lines.append('%s  # %.1f' % (head, gbs))
    with open(path, 'w') as f:
        f.write('\n'.join(lines) + '\n')


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument('--out', default=DEFAULT_OUT)
    ap.add_argument('--quick', action='store_true')
    ap.add_argument('--only-n', default='', help='comma-separated N: retune these, keep the rest')
    ap.add_argument('--prec', type=int, default=0, help='4 or 8: tune one precision only')
    args = ap.parse_args(argv)
    import torch

    os.environ['BBFFT_GB300_TUNING'] = 'off'  # candidates are set explicitly
    only = {int(n) for n in args.only_n.split(',') if n}
    kept = read_table(args.out) if only else []
    entries = []
    for prec, type, N, M, K in default_configs(args.quick):
        if (only and N not in only) or (args.prec and prec != args.prec):
            continue
        entries.append(tune_config(torch, prec, type, N, M, K, verbose=True))
    fresh = {e[:4] for e, _ in entries}
    entries = [(e, g) for e, g in kept if e[:4] not in fresh] + entries
    write_table(args.out, entries)
    print('wrote', args.out)


if __name__ == '__main__':
    sys.exit(main())
