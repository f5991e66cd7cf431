#!/usr/bin/env python3
"""Generate prime_frag_table.cuh: the DFT coefficients of the odd prime radices 17..61 and
of the radices 16 and 32 as per-lane B fragments of mma.sync.m16n8k8 TF32, split into two
TF32 pieces each.

The tensor-core radix stage (prime_tc.cuh) forms, for a radix-P butterfly with pair sums
s_j = x_j + x_{P-j} and differences d_j = x_j - x_{P-j} (j = 1..H; H = (P-1)/2 for odd P,
P/2 - 1 for even P, whose element P/2 has no partner),
    U_k = sum_j cos(2 pi j k / P) s_j,    W_k = sum_j -sin(2 pi j k / P) d_j,
as two real matrix products whose K dimension is j and whose N dimension is k, both padded
to multiples of 8.  Lane l = 4 g + t of a warp holds, for k-step ks and n-tile nt, the
B-fragment entries (row t, col g) and (row t + 4, col g) of the 8 x 8 block, i.e. the
coefficients of j = 8 ks + t + 1 and j = 8 ks + t + 5 for k = 8 nt + g + 1.

Layout per radix: uint4 entries [ks][nt][lane][2]:
    [0] = {C_hi(j0), C_hi(j1), C_lo(j0), C_lo(j1)},  [1] = the same for S = -sin,
as TF32 bit patterns (float32 with the low 13 mantissa bits zero); hi is the coefficient
rounded to TF32 (nearest, ties away from zero, as cvt.rna.tf32.f32 rounds), lo the
rounded remainder, so hi + lo carries about 22 significant bits.  Entries with j > H or
k > H are zero.  The coefficients are evaluated in double precision (53 bits, far more
than the 22 kept).

Usage: gen_prime_frags.py OUTDIR
"""
import math
import os
import struct
import sys

PRIMES = [17, 19, 23, 29, 31, 37, 41, 43, 47, 53, 59, 61]
EVEN = [16, 32]
RADICES = PRIMES + EVEN


def pairs(P):
    return (P - 1) // 2 if P % 2 else P // 2 - 1


def f32_bits(x):
    return struct.unpack('<I', struct.pack('<f', x))[0]


def bits_f32(u):
    return struct.unpack('<f', struct.pack('<I', u))[0]


def tf32_rna(x):
    """Round a double to float32, then to TF32 (10 explicit mantissa bits), nearest with
    ties away from zero; returns the float32 bit pattern."""
    u = f32_bits(x)
    return ((u + 0x1000) & 0xFFFFE000) & 0xFFFFFFFF


def split(x):
    hi = tf32_rna(x)
    lo = tf32_rna(x - bits_f32(hi))
    return hi, lo


def frags(P):
    H = pairs(P)
    KS = (H + 7) // 8
    out = []
    for ks in range(KS):
        for nt in range(KS):
            for lane in range(32):
                g, t = lane >> 2, lane & 3
                k = 8 * nt + g + 1
                vals = []
                for fn in (math.cos, lambda a: -math.sin(a)):
                    pieces = []
                    for j in (8 * ks + t + 1, 8 * ks + t + 5):
                        if j <= H and k <= H:
                            pieces.append(split(fn(2.0 * math.pi * ((j * k) % P) / P)))
                        else:
                            pieces.append((0, 0))
                    vals.append((pieces[0][0], pieces[1][0], pieces[0][1], pieces[1][1]))
                out.extend(vals)
    return out


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    lines = ['// generated by gen_prime_frags.py: TF32 B fragments of the DFT coefficients of the',
             '// odd prime radices 17..61 and of 16 and 32 for the tensor-core radix stage',
             '// (prime_tc.cuh)',
             '#pragma once', '', 'namespace gbfft {', 'namespace ptc {', '']
    for P in RADICES:
        f = frags(P)
        lines.append('static __device__ const uint4 kFrag%d[%d] = {' % (P, len(f)))
        for e in f:
            lines.append('    {0x%08xu, 0x%08xu, 0x%08xu, 0x%08xu},' % e)
        lines.append('};')
        lines.append('')
    lines.append('template <int P> __device__ __forceinline__ const uint4 *frag_table() {')
    for i, P in enumerate(RADICES):
        lines.append('    %sif constexpr (P == %d) {' % ('' if i == 0 else '} else ', P))
        lines.append('        return kFrag%d;' % P)
    lines.append('    } else {')
    lines.append('        static_assert(P == 0, "no coefficient table for this radix");')
    lines.append('        return nullptr;')
    lines.append('    }')
    lines.append('}')
    lines += ['', '} // namespace ptc', '} // namespace gbfft', '']
    text = '\n'.join(lines)
    fn = os.path.join(outdir, 'prime_frag_table.cuh')
    if not os.path.exists(fn) or open(fn).read() != text:
        with open(fn, 'w') as fh:
            fh.write(text)
    return fn


if __name__ == '__main__':
    print(main(sys.argv[1]))
