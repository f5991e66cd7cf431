#!/usr/bin/env python3
"""Generate root_of_unity_table.cuh: exactly rounded cos/sin(2*pi*k/P) literals.

The in-register radix-P butterflies use the roots of unity w_P^k = exp(2*pi*i*k/P)
as compile-time constants.  Each constant is evaluated with 60 significant digits
(mpmath) and rounded ONCE to the target precision (double and float separately), so
the float constants are not double-rounded.  This mirrors the exactly-rounded
look-up tables of the reference (src/base/root_of_unity.hpp:16-1163, used through
power_of_w in src/base/root_of_unity.cpp:171-189), computed here by our own script.

Run: python gen_root_of_unity.py > root_of_unity_table.cuh
"""
import struct
import sys

import mpmath

PMAX = 64


def f32_literal(x):
    # round-to-nearest-even to binary32 from a 60-digit value
    d = float(x)  # nearest double
    f = struct.unpack('f', struct.pack('f', d))[0]
    # guard against double rounding: compare the two float neighbours directly
    import math
    cand = [f, math.nextafter(f, math.inf), math.nextafter(f, -math.inf)]
    cand = [struct.unpack('f', struct.pack('f', c))[0] for c in cand]
    best = min(cand, key=lambda c: (abs(mpmath.mpf(c) - x), struct.unpack('I', struct.pack('f', c))[0] & 1))
    return float(best).hex() + 'f'


def f64_literal(x):
    return float(x).hex()


def main(out):
    mpmath.mp.dps = 60
    offs = []
    cos_d, sin_d, cos_f, sin_f = [], [], [], []
    off = 0
    for p in range(PMAX + 1):
        offs.append(off)
        if p == 0:
            continue
        for k in range(p):
            a = 2 * mpmath.pi * k / p
            c, s = mpmath.cos(a), mpmath.sin(a)
            # exact zeros/ones at the symmetry points
            if abs(c) < mpmath.mpf(10) ** -50:
                c = mpmath.mpf(0)
            if abs(s) < mpmath.mpf(10) ** -50:
                s = mpmath.mpf(0)
            cos_d.append(f64_literal(c))
            sin_d.append(f64_literal(s))
            cos_f.append(f32_literal(c))
            sin_f.append(f32_literal(s))
        off += p
    w = out.write
    w('// Generated by gen_root_of_unity.py -- do not edit.\n')
    w('// cos/sin(2*pi*k/P) for 1 <= P <= %d, 0 <= k < P, each rounded once from 60 digits.\n' % PMAX)
    w('#pragma once\n\nnamespace gbfft {\nnamespace rou {\n\n')
    w('constexpr int kMaxP = %d;\n' % PMAX)
    w('constexpr int kOffset[%d] = {%s};\n\n' % (PMAX + 1, ', '.join(map(str, offs))))

    def arr(name, ty, vals):
        w('constexpr %s %s[%d] = {\n' % (ty, name, len(vals)))
        for i in range(0, len(vals), 4):
            w('    ' + ', '.join(vals[i:i + 4]) + ',\n')
        w('};\n\n')

    arr('kCosD', 'double', cos_d)
    arr('kSinD', 'double', sin_d)
    arr('kCosF', 'float', cos_f)
    arr('kSinF', 'float', sin_f)
    w('} // namespace rou\n} // namespace gbfft\n')


if __name__ == '__main__':
    main(sys.stdout)
