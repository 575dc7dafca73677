"""Generate zig_tables.h, the ziggurat layer tables of the device Gaussian sampler.

genetIC samples its white noise with GSL's gsl_ran_gaussian_ziggurat
(genetIC/src/simulation/field/randomfieldgenerator.hpp:149-150,191), the
Marsaglia & Tsang ziggurat (J. Stat. Softw. 5(8), 2000) with 128 layers and an
exponential wedge exp(-R (x - R/2)) on the base strip.  The layer geometry
follows from R alone: layer 127 is [0,R] x [0,f(R)] plus the wedge, area
v = R f(R) + f(R)/R, each higher layer has area v, f(x) = exp(-x^2/2), and R is
fixed by y_0 = 1.  Values are rounded to 12 significant digits, the precision
in which the published tables are distributed.

Run:  python genetic_gb300/csrc/gen_zig_tables.py > genetic_gb300/csrc/zig_tables.h
"""
import mpmath as mp
import numpy as np

mp.mp.dps = 50


def layers(R):
    f = lambda t: mp.e ** (-t * t / 2)
    v = R * f(R) + f(R) / R
    xs, ys = [mp.mpf(0)] * 128, [mp.mpf(0)] * 128
    xs[127], ys[127] = R, f(R)
    for i in range(126, -1, -1):
        ys[i] = ys[i + 1] + v / xs[i + 1]
        xs[i] = mp.sqrt(-2 * mp.log(ys[i])) if ys[i] < 1 else mp.mpf(0)
    return xs, ys


def g12(t):
    return float('%.12g' % float(mp.nstr(t, 20)))


def f32(v):
    """The double v rounded to the nearest float (ties to even), as a C float literal."""
    return float.hex(float(np.float32(v))) + 'f'


if __name__ == '__main__':
    R = mp.findroot(lambda r: layers(r)[1][0] - 1, mp.mpf('3.4442864767'))
    xs, ys = layers(R)
    s = mp.mpf(2) ** 24
    y = [mp.mpf(1)] + ys[1:]
    w = [xs[i + 1] / s for i in range(127)] + [(R + 1 / R) / s]
    k = [0] + [int(mp.floor(s * xs[i] / xs[i + 1])) for i in range(1, 127)] + [int(mp.floor(s * R / (R + 1 / R)))]
    out = ['// Generated by gen_zig_tables.py; do not edit.', '#pragma once',
           '#define GIC_ZIG_PARAM_R %r' % g12(R),
           '#define GIC_ZIG_Y_INIT {' + ', '.join(float.hex(g12(t)) for t in y) + '}',
           '#define GIC_ZIG_W_INIT {' + ', '.join(float.hex(g12(t)) for t in w) + '}',
           '#define GIC_ZIG_K_INIT {' + ', '.join('%du' % v for v in k) + '}',
           # the same values rounded to float, for the single-precision slow-path decisions
           '#define GIC_ZIG_YF_INIT {' + ', '.join(f32(g12(t)) for t in y) + '}',
           '#define GIC_ZIG_WF_INIT {' + ', '.join(f32(g12(t)) for t in w) + '}']
    print('\n'.join(out))
