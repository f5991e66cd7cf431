#!/usr/bin/env python3
"""Generate the compile-time-size kernel instantiations and their look-up table.

For every complex FFT length Nc in the lists below and every transform kind that uses
it, one kernel fft_kernel_ct<R, Kind, Nc, T, radices...> is instantiated with the radices
and threads-per-transform that the host heuristic (choose_radices in library.cpp,
restated here as choose_radices) picks.  The host looks a plan up in the generated
table and falls back to the runtime-size kernel when there is no entry.

Usage: gen_specializations.py OUTDIR   (writes kernels_ct_<prec>_<kind>.cu, ct_index.cpp)
"""
import os
import sys

# complex FFT lengths with compile-time kernels
EVEN_NC = [2, 4, 8, 16, 32, 64, 128, 256, 512, 24, 48, 80, 96, 112, 160, 192, 224, 384]
ODD_NC = [3, 5, 7, 9, 11, 13, 15, 25, 27]
KINDS = {0: 'c2c', 1: 'r2ch', 2: 'r2cf', 3: 'c2rh', 4: 'c2rf'}
UNROLLED = set(range(1, 14)) | {16}
UNIT_KERNELS = 48


def prime_factors(n):
    f, p = [], 2
    while n > 1:
        if n % p == 0:
            f.append(p)
            n //= p
        else:
            p += 1
    return f


def choose_radices(nc):
    """Same rule as choose_radices() in library.cpp."""
    if nc == 1:
        return [1]
    c2 = c3 = 0
    odd, big = [], []
    for p in prime_factors(nc):
        if p == 2:
            c2 += 1
        elif p == 3:
            c3 += 1
        elif p <= 13:
            odd.append(p)
        else:
            big.append(p)
    r = []
    while c3 >= 2:
        r.append(9)
        c3 -= 2
    if c3 == 1:
        if c2 >= 2 and c2 != 3 and c2 != 6:
            r.append(12)
            c2 -= 2
        elif c2 >= 1:
            r.append(6)
            c2 -= 1
        else:
            r.append(3)
    for p in odd:
        if p == 5 and c2 >= 1 and c2 % 3 == 1:
            r.append(10)
            c2 -= 1
        else:
            r.append(p)
    if c2 > 0:
        chunks = (c2 + 3) // 4
        for i in range(chunks):
            bits = c2 // chunks + (1 if i < c2 % chunks else 0)
            r.append(1 << bits)
    r.sort(reverse=True)
    return r + big


BIG_PRIMES = {17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61}


# A complex length k * P with a prime P = 17..47 and k <= REG_PRIME_KMAX runs its radix-P
# butterflies in registers, one per thread (dft<P> with literal coefficients), as the
# FIRST stage on k threads per transform, followed by the stages of k and no copy stages:
# the tensor-core form needs shared memory on both sides and several butterflies per warp,
# and leaves threads idle at so few butterflies per transform.  (A first try with the prime
# stage last on 6 threads per transform, most of them idle in that stage, was slower than
# the tensor-core form.)
REG_PRIME_MAX = 61
REG_PRIME_KMAX = 32


def reg_prime_of(nc):
    """The prime P of a register-prime length (smallest prime factor >= 17 of nc, with
    k = nc / P <= REG_PRIME_KMAX and no prime factor >= 17 in k), or 0; same rule as
    reg_prime_length() in library.cpp."""
    big = [q for q in sorted(BIG_PRIMES) if nc % q == 0]
    if not big or big[0] > REG_PRIME_MAX:
        return 0
    p, k = big[0], nc // big[0]
    if k > REG_PRIME_KMAX or any(k % q == 0 for q in BIG_PRIMES) or largest_prime_factor(k) > 16:
        return 0
    return p


def reg_prime_length(nc):
    return reg_prime_of(nc) > 0


def reg_prime_radices(nc):
    """[P] + the radices of k = nc / P (prime stage first)."""
    p = reg_prime_of(nc)
    return [p] + (choose_radices(nc // p) if nc > p else [])


def tile_threads(nc, rad, V=1, reg=False):
    """Threads per transform of a compile-time tile (same rule as tile_threads() in
    library.cpp): the count that leaves the fewest thread slots idle over the stages
    (a stage of nb butterflies runs ceil(nb / T) rounds on T threads), with at most 32
    complex values per thread (V transforms each) in any stage and at least 4 threads
    where a stage has 4 butterflies (consecutive threads load consecutive elements of a
    transform: 32-byte sectors when M = 1); ties go to more threads.  The tensor-core
    prime stages use every warp of the block and do not count, but with one of them T is
    at most 4 x its butterflies per transform where possible, so that a block of 256
    threads holds at least 64 of its butterflies (8 per warp).  `reg`: the prime stage runs
    in registers, one butterfly per thread: nc / P threads (reg_prime_length)."""
    if reg:
        return nc // rad[0]
    if len(rad) == 2 and rad[1] == 1:
        # one butterfly stage and the copy stage: every thread one butterfly in the first
        return nc // rad[0]
    tc = BIG_PRIMES
    nbmax = max([nc // r for r in rad if r not in tc] + [1])
    tcap = min([4 * (nc // r) for r in rad if r in tc] + [256])
    for hi in (min(nc, 256, tcap), min(nc, 256)):
        best_t, best_cost = None, None
        for t in range(min(4, nbmax), hi + 1):
            cost, ok = 0, True
            for r in rad:
                if r in tc:
                    continue
                rounds = -(-(nc // r) // t)
                if rounds * r * V > 32:
                    ok = False
                    break
                cost += rounds * t
            if ok and (best_cost is None or cost <= best_cost):
                best_t, best_cost = t, cost
        if best_t is not None:
            return best_t
    return 1


def stage_list(nc, kind, ragged=False, reg_ok=False):
    """Radices incl. the copy stages the host adds, and threads per transform (the rules
    of make_1d_pass in library.cpp; `ragged`: a compile-time tile, i.e. a pass of a ragged
    batch or a plan on a tile kernel; `reg_ok`: a cover tile, whose prime stage may run in
    registers)."""
    reg = ragged and reg_ok and reg_prime_length(nc)
    rad = reg_prime_radices(nc) if reg else choose_radices(nc)
    if rad[0] not in UNROLLED and not reg:
        rad = [1] + rad
    real = kind != 0
    post = kind == 1
    if not post and rad[-1] in BIG_PRIMES and not reg:
        rad = rad + [1]
    if real and not post and len(rad) == 1:
        rad = rad + [1]
    if ragged:
        return rad, tile_threads(nc, rad, reg=reg)
    pu = max([r for r in rad if r in UNROLLED] + [1])
    T = max(1, nc // pu) if pu > 1 else min(nc, 64)
    ptg = max([r for r in rad if r in BIG_PRIMES] + [0])
    if ptg:
        T = nc // ptg * (((ptg - 1) // 2 + 7) // 8)
    T = min(T, 512)
    return rad, T


def vector_width(prec, rad):
    """Transforms per thread along M (same rule as vector_width() in library.cpp): keep
    V * max radix complex values within 32 (float) / 16 (double) registers pairs."""
    pmax = max(rad)
    vmax = 4 if prec == 4 else 2
    budget = 32 if prec == 4 else 16
    v = vmax
    while v > 1 and v * pmax > budget:
        v //= 2
    return v


# Alternative radices / threads per transform for the float real half lengths whose default
# stages leave threads idle (the autotuner picks among them): a stage with nb butterflies
# over T threads runs ceil(nb / T) rounds.
ALT_STAGES = {
    80: [([10, 8], 10), ([8, 10], 8), ([8, 10], 10), ([16, 5], 5), ([5, 16], 5)],
    112: [([16, 7], 16), ([7, 16], 7), ([7, 16], 16), ([4, 4, 7], 28), ([7, 16], 32),
          ([4, 4, 7], 16), ([16, 7], 8)],
    192: [([8, 6, 4], 32), ([16, 12], 12), ([12, 16], 12), ([16, 12], 16), ([4, 6, 8], 48),
          ([16, 12], 24), ([12, 16], 24), ([8, 8, 3], 24), ([3, 8, 8], 24),
          ([12, 4, 4], 16), ([4, 4, 12], 16), ([16, 12], 8), ([12, 16], 8), ([8, 6, 4], 8)],
}


# the same for float c2c lengths
ALT_STAGES_C2C = {
    512: [([16, 8, 4], 32), ([8, 8, 8], 32), ([16, 16, 2], 32), ([4, 8, 16], 32), ([8, 8, 8], 16)],
}


def entries():
    out = []
    for prec in (4, 8):
        for kind in KINDS:
            ncs = EVEN_NC + ODD_NC if kind == 0 else (EVEN_NC if kind in (1, 3) else ODD_NC)
            for nc in ncs:
                rad, T = stage_list(nc, kind)
                if any(r not in UNROLLED for r in rad):
                    continue
                variants = [(rad, T)]
                if prec == 4 and kind in (1, 3):
                    variants += ALT_STAGES.get(nc, [])
                if prec == 4 and kind == 0:
                    variants += ALT_STAGES_C2C.get(nc, [])
                for rad, T in variants:
                    for V in sorted({1, vector_width(prec, rad)}):
                        # kernel variant: resident CTAs the register allocation is sized for,
                        # 2 (up to 128 registers) and for float also 3 (up to 80); plus 10 for
                        # the paired c2r pre-process (float c2r, even N).  The autotuner picks.
                        minbs = (2, 3) if prec == 4 else (2,)
                        if prec == 4 and kind == 3:
                            minbs += (12, 13)
                        for minb in minbs:
                            out.append((prec, kind, nc, T, rad, V, minb))
    return out


# Ragged batches: float c2c N = 16..512 step 8 and r2c N = 16..512 step 8 (half length
# 8..256 step 4), one thread per M (V = 1), as device functions of the persistent kernel.
RAGGED_FILES = 8


def ragged_entries():
    out = []
    for kind, ncs in ((0, range(16, 513, 8)), (1, range(8, 257, 4))):
        for nc in ncs:
            # the prime stage in registers up to P = 47 (the units compile for 128 registers)
            rad, T = stage_list(nc, kind, ragged=True, reg_ok=0 < reg_prime_of(nc) <= 47)
            if any(r not in UNROLLED and r not in BIG_PRIMES for r in rad):
                continue
            out.append((4, kind, nc, T, rad, 1))
            # vectorised over M (items with M a multiple of V and 16-byte aligned tensors);
            # the prime stages are scalar
            vw = vector_width(4, rad)
            if vw > 1 and not any(r in BIG_PRIMES for r in rad):
                out.append((4, kind, nc, tile_threads(nc, rad, vw), rad, vw))
    return out


def reg_prime_tile(nc, rad):
    """A cover tile whose prime stage runs in registers (stage_list with reg_ok): the
    prime is its first radix."""
    return reg_prime_length(nc) and rad[0] in BIG_PRIMES


def tile_min_blocks(rad, reg=False, cover=False):
    """Resident 256-thread CTAs the register budget of a tile kernel is sized for: 3 (80
    registers) with a tensor-core prime stage, whose tiles are otherwise limited by the
    latency of 2 CTAs per SM at 128 registers, and for the cover tiles without a prime
    stage (measured at 21 % achieved occupancy with 2; at 80 registers 7 of 354 spill, at
    most 16 bytes); 2 for the others and for a prime stage in registers up to P = 47
    (47 complex values per thread); 1 (255 registers) for P = 53..61."""
    if reg:
        return 1 if max(rad) > 47 else 2
    if cover:
        return 3
    return 3 if any(r in BIG_PRIMES for r in rad) else 2


def largest_prime_factor(n):
    return max(prime_factors(n)) if n > 1 else 1


def cover_entries():
    """Compile-time tiles (V = 1) for every other float length N <= 512 whose prime
    factors are at most 61, each kind: c2c N = 16..512, r2c / c2r even N (complex half
    length 8..256), r2c / c2r odd N = 17..511.  Lengths with a plan kernel or a ragged
    tile of their own are left out; longer prime factors stay on the runtime-size engine."""
    plan = set((k, nc) for (pr, k, nc, T, rad, V, minb) in entries() if pr == 4)
    rag = set((k, nc) for (pr, k, nc, T, rad, V) in ragged_entries())
    out = []
    for kind in KINDS:
        ncs = range(16, 513) if kind == 0 else (range(8, 257) if kind in (1, 3) else range(17, 512, 2))
        for nc in ncs:
            if largest_prime_factor(nc) > 61 or (kind, nc) in plan or (kind, nc) in rag:
                continue
            rad, T = stage_list(nc, kind, ragged=True, reg_ok=True)
            out.append((4, kind, nc, T, rad, 1))
    return out


COVER_UNIT_KERNELS = 40


def cover_units(outdir):
    """cover_ct_<g>.cu (one plan kernel per cover entry) and the host table lines."""
    ents = cover_entries()
    n_units = (len(ents) + COVER_UNIT_KERNELS - 1) // COVER_UNIT_KERNELS
    groups = [list(range(g, len(ents), n_units)) for g in range(n_units)]
    units = []
    for g, idx in enumerate(groups):
        src = ['// generated by gen_specializations.py: compile-time tiles of the other lengths',
               '#include "engine_ct.cuh"', '#include "kernels.hpp"', '', 'namespace gbfft {', '']
        for i in idx:
            prec, kind, nc, T, rad, V = ents[i]
            # odd real N (kinds 2, 4): tiles that run two real transforms per complex FFT
            # when the plan sets flag_pair
            two = 'true' if kind in (2, 4) else 'false'
            reg = reg_prime_tile(nc, rad)
            targs = 'float, %d, %d, %d, %d, %s, %s, %s' % (kind, nc, T, V, two, 'true' if reg else 'false',
                                                       ', '.join(map(str, rad)))
            src += ['__global__ void __launch_bounds__(256, %d) cover_ct_%d(const __grid_constant__ fft_params p) {' % (tile_min_blocks(rad, reg, cover=True), i),
                    '    fft_tile_ct_ragged_t<%s>(p, blockIdx.x);' % targs, '}', '']
        src += ['const void *cover_ct_kernel_%d(int i) {' % g, '    switch (i) {']
        for i in idx:
            src += ['    case %d:' % i, '        return reinterpret_cast<const void *>(&cover_ct_%d);' % i]
        src += ['    default:', '        return nullptr;', '    }', '}', '', '} // namespace gbfft', '']
        fn = os.path.join(outdir, 'cover_ct_%d.cu' % g)
        write(fn, '\n'.join(src))
        units.append(fn)
    host = ['const void *cover_ct_kernel_%d(int i);' % g for g in range(n_units)]
    host += ['', '// compile-time tile kernels of the other lengths (cover_entries), by table index',
             'const void *cover_ct_kernel(int i) {',
             '    switch (i %% %d) {' % n_units]
    for g in range(n_units):
        host += ['    case %d:' % g, '        return cover_ct_kernel_%d(i);' % g]
    host += ['    }', '    return nullptr;', '}', '', 'extern const ct_entry cover_ct_table[] = {']
    for prec, kind, nc, T, rad, V in ents:
        minb = tile_min_blocks(rad, reg_prime_tile(nc, rad), cover=True)
        host.append('    {%d, %d, %d, %d, %d, %d, {%s}, nullptr, %d},' % (prec, kind, nc, T, V, len(rad),
                                                                    ', '.join(map(str, rad)), minb))
    host += ['};', 'static const int kCoverSize = %d;' % len(ents), '',
             'int cover_ct_lookup(int prec, int kind, int nc, int T, const int *rad, int L) {',
             '    for (int i = 0; i < kCoverSize; ++i) {',
             '        const ct_entry &e = cover_ct_table[i];',
             '        if (e.prec != prec || e.kind != kind || e.nc != nc || e.T != T || e.L != L) {',
             '            continue;',
             '        }',
             '        bool same = true;',
             '        for (int s = 0; s < L; ++s) {',
             '            same = same && e.rad[s] == rad[s];',
             '        }',
             '        if (same) {',
             '            return i;',
             '        }',
             '    }',
             '    return -1;',
             '}', '']
    return units, host


def write(fn, text):
    if not os.path.exists(fn) or open(fn).read() != text:
        with open(fn, 'w') as f:
            f.write(text)


def ragged_units(outdir):
    """ragged_ct_<i>.cu (the variant functions, spread over RAGGED_FILES units),
    ragged_ct_dispatch.inc (declarations and the switch, included by ragged.cu) and the
    host table lines for ct_index.cpp."""
    ents = ragged_entries()
    cost = lambda e: e[2] * len(e[4]) + sum(r * r * 8 for r in e[4] if r in BIG_PRIMES)
    order = sorted(range(len(ents)), key=lambda i: -cost(ents[i]))
    groups = [[] for _ in range(RAGGED_FILES)]
    load = [0] * RAGGED_FILES
    for i in order:
        g = load.index(min(load))
        groups[g].append(i)
        load[g] += cost(ents[i])
    units = []
    for g, idx in enumerate(groups):
        src = ['// generated by gen_specializations.py: compile-time-size tiles of the ragged kernel',
               '#include "engine_ct.cuh"', '#include "kernels.hpp"', '', 'namespace gbfft {', '']
        for i in sorted(idx):
            prec, kind, nc, T, rad, V = ents[i]
            reg = reg_prime_tile(nc, rad)
            targs = 'float, %d, %d, %d, %d, false, %s, %s' % (kind, nc, T, V, 'true' if reg else 'false',
                                                          ', '.join(map(str, rad)))
            # V = 1 tiles without a prime stage: 3 resident CTAs (80 registers; 1 of 88 spills,
            # 12 bytes); the V = 2 / 4 variants hold more values per thread and keep 2
            minb = 3 if V == 1 and not reg and not any(r in BIG_PRIMES for r in rad) else \
                tile_min_blocks(rad, reg)
            src += ['__device__ __noinline__ void ragged_ct_%d(const fft_params &p, long long tile) {' % i,
                    '    fft_tile_ct_ragged_t<%s>(p, tile);' % targs,
                    '}', '',
                    '__global__ void __launch_bounds__(256, %d) ragged_class_ct_%d(const ragged_item_dev *__restrict__ items,' % (minb, i),
                    '                                                        const int2 *__restrict__ units) {',
                    '    __shared__ __align__(16) fft_params s_p;',
                    '    const int2 un = stage_unit_params(items, units, s_p);',
                    '    fft_tile_ct_ragged_t<%s>(s_p, un.y);' % targs,
                    '}', '',
                    '__global__ void __launch_bounds__(256, %d) plan_ct_%d(const __grid_constant__ fft_params p) {' % (minb, i),
                    '    fft_tile_ct_ragged_t<%s>(p, blockIdx.x);' % targs,
                    '}', '']
        for kname in ('ragged_class_ct', 'plan_ct'):
            src += ['const void *%s_kernel_%d(int vid) {' % (kname, g), '    switch (vid) {']
            for i in sorted(idx):
                src += ['    case %d:' % i, '        return reinterpret_cast<const void *>(&%s_%d);' % (kname, i)]
            src += ['    default:', '        return nullptr;', '    }', '}', '']
        src += ['} // namespace gbfft', '']
        fn = os.path.join(outdir, 'ragged_ct_%d.cu' % g)
        write(fn, '\n'.join(src))
        units.append(fn)
    inc = ['// generated by gen_specializations.py: compile-time-size ragged tiles', '']
    inc += ['__device__ void ragged_ct_%d(const fft_params &p, long long tile);' % i for i in range(len(ents))]
    inc += ['', '__device__ __forceinline__ void ragged_ct_call(int vid, const fft_params &p, long long tile) {',
            '    switch (vid) {']
    for i in range(len(ents)):
        inc += ['    case %d:' % i, '        ragged_ct_%d(p, tile);' % i, '        break;']
    inc += ['    }', '}', '']
    write(os.path.join(outdir, 'ragged_ct_dispatch.inc'), '\n'.join(inc))
    host = []
    for kname, what in (('ragged_class_ct', 'one class of a ragged batch (grid over the class\'s units)'),
                        ('plan_ct', 'a plan (grid over its tiles)')):
        host += ['const void *%s_kernel_%d(int vid);' % (kname, g) for g in range(RAGGED_FILES)]
        fn = 'ragged_class_kernel' if kname == 'ragged_class_ct' else 'ragged_plan_kernel'
        host += ['', '// compile-time tile kernel of %s, by table index' % what,
                 'const void *%s(int vid) {' % fn, '    const void *f = nullptr;']
        for g in range(RAGGED_FILES):
            host += ['    if (!f) {', '        f = %s_kernel_%d(vid);' % (kname, g), '    }']
        host += ['    return f;', '}', '']
    host += ['extern const ct_entry ragged_ct_table[] = {']
    for prec, kind, nc, T, rad, V in ents:
        minb = tile_min_blocks(rad, reg_prime_tile(nc, rad), cover=True)
        host.append('    {%d, %d, %d, %d, %d, %d, {%s}, nullptr, %d},' % (prec, kind, nc, T, V, len(rad),
                                                                    ', '.join(map(str, rad)), minb))
    host += ['};', 'static const int kRaggedSize = %d;' % len(ents), '',
             'int ragged_ct_lookup(int prec, int kind, int nc, int T, int V, const int *rad, int L) {',
             '    for (int i = 0; i < kRaggedSize; ++i) {',
             '        const ct_entry &e = ragged_ct_table[i];',
             '        if (e.prec != prec || e.kind != kind || e.nc != nc || e.T != T || e.V != V || e.L != L) {',
             '            continue;',
             '        }',
             '        bool same = true;',
             '        for (int s = 0; s < L; ++s) {',
             '            same = same && e.rad[s] == rad[s];',
             '        }',
             '        if (same) {',
             '            return i;',
             '        }',
             '    }',
             '    return -1;',
             '}', '']
    return units, host


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    ents = entries()
    files = {}
    for prec, kind, nc, T, rad, V, minb in ents:
        files.setdefault((prec, kind), []).append((nc, T, rad, V, minb))
    # units of at most UNIT_KERNELS kernels, compiled in parallel
    split = {}
    for (prec, kind), lst in files.items():
        n = (len(lst) + UNIT_KERNELS - 1) // UNIT_KERNELS
        for part in range(n):
            split[(prec, kind, part)] = lst[part::n]
    files = split
    index = ['// generated by gen_specializations.py', '#include "kernels.hpp"', '',
             'namespace gbfft {']
    tables = []
    for (prec, kind, part), lst in sorted(files.items()):
        R = 'float' if prec == 4 else 'double'
        name = 'ct_table_f%d_%s_%d' % (prec * 8, KINDS[kind], part)
        src = ['// generated by gen_specializations.py: compile-time-size FFT kernels',
               '#include "engine_ct.cuh"', '#include "kernels.hpp"', '', 'namespace gbfft {', '',
               'template <class R, int Kind, int NC, int TT, int V, int MINB, int... Ps>',
               '__global__ void __launch_bounds__(256, MINB % 10) fft_kernel_ct(const __grid_constant__ fft_params p) {',
               '    fft_tile_ct<R, Kind, NC, TT, V, (MINB >= 10), Ps...>(p);', '}', '',
               'extern const ct_entry %s[] = {' % name]
        for nc, T, rad, V, minb in lst:
            rs = ', '.join(map(str, rad))
            src.append('    {%d, %d, %d, %d, %d, %d, {%s}, reinterpret_cast<const void *>(&fft_kernel_ct<%s, %d, %d, %d, %d, %d, %s>), %d},'
                       % (prec, kind, nc, T, V, len(rad), rs, R, kind, nc, T, V, minb, rs, minb))
        src += ['};', 'extern const int %s_size = %d;' % (name, len(lst)), '', '} // namespace gbfft', '']
        fn = os.path.join(outdir, 'kernels_ct_f%d_%s_%d.cu' % (prec * 8, KINDS[kind], part))
        text = '\n'.join(src)
        if not os.path.exists(fn) or open(fn).read() != text:
            with open(fn, 'w') as f:
                f.write(text)
        index.append('extern const ct_entry %s[];' % name)
        index.append('extern const int %s_size;' % name)
        tables.append(name)
    index += ['', 'static const ct_entry *const kTables[] = {%s};' % ', '.join(tables),
              'static const int *const kSizes[] = {%s};' % ', '.join('&%s_size' % t for t in tables),
              '',
              'const ct_entry *ct_lookup(int prec, int kind, int nc, int T, int V, const int *rad, int L,',
              '                          int minb) {',
              '    for (unsigned t = 0; t < sizeof(kTables) / sizeof(kTables[0]); ++t) {',
              '        for (int i = 0; i < *kSizes[t]; ++i) {',
              '            const ct_entry &e = kTables[t][i];',
              '            if (e.prec != prec || e.kind != kind || e.nc != nc || e.T != T || e.V != V || e.L != L ||',
              '                e.minb != minb) {',
              '                continue;',
              '            }',
              '            bool same = true;',
              '            for (int s = 0; s < L; ++s) {',
              '                same = same && e.rad[s] == rad[s];',
              '            }',
              '            if (same) {',
              '                return &e;',
              '            }',
              '        }',
              '    }',
              '    return nullptr;',
              '}', '']
    rag_units, rag_host = ragged_units(outdir)
    cov_units, cov_host = cover_units(outdir)
    index += rag_host + cov_host + ['} // namespace gbfft', '']
    fn = os.path.join(outdir, 'ct_index.cpp')
    text = '\n'.join(index)
    if not os.path.exists(fn) or open(fn).read() != text:
        with open(fn, 'w') as f:
            f.write(text)
    return (sorted(os.path.join(outdir, 'kernels_ct_f%d_%s_%d.cu' % (p * 8, KINDS[k], n)) for p, k, n in files)
            + cov_units, rag_units)


if __name__ == '__main__':
    ct_units, rag_units = main(sys.argv[1])
    print('\n'.join(ct_units + rag_units))
