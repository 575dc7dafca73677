"""Oracle (test infrastructure only): numpy reader for the tipsy files genetIC
writes (genetIC/src/io/tipsy.hpp:61-63, 109-145), standing in for pynbody in
the reference's comparator (tools/compare.py)."""
import numpy as np


def read_tipsy(path):
    """Return (time, gas[n,12], dark[n,9]) float32 arrays; endianness detected from the header."""
    raw = open(path, 'rb').read()
    for end in ('<', '>'):
        h = np.frombuffer(raw[8:32], end + 'i4')
        if h[0] == h[2] + h[3] + h[4] and h[1] == 3:
            break
    else:
        raise ValueError('not a tipsy file: %s' % path)
    t = float(np.frombuffer(raw[:8], end + 'f8')[0])
    nb, nd, ns, ndark, nstar, _ = h
    off = 32
    gas = np.frombuffer(raw, end + 'f4', count=ns * 12, offset=off).reshape(ns, 12)
    off += ns * 48
    dark = np.frombuffer(raw, end + 'f4', count=ndark * 9, offset=off).reshape(ndark, 9)
    return t, gas, dark
