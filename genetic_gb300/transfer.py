"""Transfer tables in the CAMB text format genetIC reads (genetIC/src/cosmology/camb.hpp:224-268).

`bbks_table` tabulates the Bardeen, Bond, Kaiser & Szalay (1986) fit
T(q) = ln(1 + 2.34 q) / (2.34 q) [1 + 3.89 q + (16.1 q)^2 + (5.46 q)^3 + (6.71 q)^4]^(-1/4),
q = k / Gamma (k in h/Mpc), Gamma = Om h exp(-Ob (1 + sqrt(2 h) / Om)) (Sugiyama 1995),
as a 7-column pre-2015 CAMB file with every transfer column equal (column 6,
"total", is what genetIC uses without baryons; column 1 normalises).
"""
import numpy as np


def bbks(k, omega_m, omega_b, h):
    gamma = omega_m * h * np.exp(-omega_b * (1.0 + np.sqrt(2.0 * h) / omega_m))
    q = np.asarray(k, dtype=np.float64) / gamma
    return (np.log1p(2.34 * q) / (2.34 * q) *
            (1.0 + 3.89 * q + (16.1 * q) ** 2 + (5.46 * q) ** 3 + (6.71 * q) ** 4) ** -0.25)


def bbks_table(omega_m=0.31, omega_b=0.049, h=0.68, kmin=1e-5, kmax=1e3, rows=2000):
    k = np.logspace(np.log10(kmin), np.log10(kmax), rows)
    t = bbks(k, omega_m, omega_b, h)
    table = np.column_stack([k] + [t] * 6)
    # the values exactly as write_camb prints them, so a table in memory and
    # the same table read back from its file are identical
    return np.vectorize(lambda v: float('%.10e' % v))(table)


def write_camb(path, table):
    with open(path, 'w') as f:
        for row in table:
            f.write(' '.join('%.10e' % v for v in row) + '\n')


def read_camb(path):
    """Read a CAMB transfer file as genetIC does: numbers only, header lines skipped."""
    rows = []
    with open(path) as f:
        for line in f:
            parts = line.split()
            if not parts:
                continue
            try:
                rows.append([float(p) for p in parts])
            except ValueError:
                continue
    ncol = len(rows[0])
    return np.array([r for r in rows if len(r) == ncol], dtype=np.float64)
