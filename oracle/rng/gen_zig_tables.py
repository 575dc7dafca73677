"""Generate the ziggurat tables used by the oracle's Gaussian sampler.

Test infrastructure (oracle): restates the table construction of the
Marsaglia & Tsang ziggurat (J. Stat. Softw. 5(8), 2000) in the 128-layer
variant whose base strip ends in the exponential wedge
exp(-R (x - R/2)) -- the variant behind gsl_ran_gaussian_ziggurat, which
genetIC calls at genetIC/src/simulation/field/randomfieldgenerator.hpp:149-150,191.

Construction (unnormalised density f(x) = exp(-x^2/2)):
  layer 127 (base strip) = rectangle [0,R] x [0,f(R)] plus the wedge, area
  v = R f(R) + f(R)/R; layers i = 126..0 each have area v:
  y_i = y_{i+1} + v / x_{i+1},  x_i = f^-1(y_i); R is the root of y_0 = 1.
Tables (index i = layer):
  ytab[i] = y_i, wtab[i] = x_{i+1} / 2^24 (i < 127), wtab[127] = (R + 1/R)/2^24,
  ktab[i] = floor(2^24 x_i / x_{i+1}) (i < 127), ktab[127] = floor(2^24 R/(R+1/R)).
The doubles are the exact values rounded to 12 significant digits, the
precision in which the published tables are distributed; R likewise.

Run:  python oracle/rng/gen_zig_tables.py > oracle/rng/zig_tables.h
"""
import mpmath as mp

mp.mp.dps = 50


def build(R):
    f = lambda t: mp.e ** (-t * t / 2)
    v = R * f(R) + f(R) / R
    x = [mp.mpf(0)] * 128
    y = [mp.mpf(0)] * 128
    x[127] = R
    y[127] = f(R)
    for i in range(126, -1, -1):
        y[i] = y[i + 1] + v / x[i + 1]
        x[i] = mp.sqrt(-2 * mp.log(y[i])) if y[i] < 1 else mp.mpf(0)
    return v, x, y


def main():
    R = mp.findroot(lambda r: build(r)[2][0] - 1, mp.mpf('3.44428647676'))
    v, x, y = build(R)
    two24 = mp.mpf(2) ** 24
    ytab = [y[i] for i in range(128)]
    ytab[0] = mp.mpf(1)
    wtab = [x[i + 1] / two24 for i in range(127)] + [(R + 1 / R) / two24]
    ktab = [0] + [int(mp.floor(two24 * x[i] / x[i + 1])) for i in range(1, 127)] \
        + [int(mp.floor(two24 * R / (R + 1 / R)))]
    g12 = lambda t: float('%.12g' % float(mp.nstr(t, 20)))
    print('/* Generated by gen_zig_tables.py -- do not edit. */')
    print('#pragma once')
    print('#define GIC_ZIG_R %r' % g12(R))
    print('static const double gic_zig_ytab[128] = {')
    print(',\n'.join('  %s' % float.hex(g12(t)) for t in ytab) + '};')
    print('static const double gic_zig_wtab[128] = {')
    print(',\n'.join('  %s' % float.hex(g12(t)) for t in wtab) + '};')
    print('static const unsigned int gic_zig_ktab[128] = {')
    print(',\n'.join('  %du' % k for k in ktab) + '};')


if __name__ == '__main__':
    main()
