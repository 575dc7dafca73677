"""Tipsy records packed on the device against the host packer (itself checked against
the oracle and the reference's tipsy file on the CPU), on the zoom2 geometry."""
import ctypes

import numpy as np
import pytest

import field_oracle as fo
from conftest import COSMO, make_generator
from test_writers import ORIGIN, ZOOM2, make_map, pack_host

pytestmark = pytest.mark.gpu

LEVELS = [('base', 50.0, 32), ('zoom', 8, 8, 8, 2, 32)]


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_device_tipsy_matches_host_packer(built, bbks, precision):
    from genetic_gb300 import _lib
    lib = _lib.load()
    gen = make_generator(precision, bbks, LEVELS, 8896131, 'random_seed')
    gen.done()
    parts = [gen.particles(l) for l in range(2)]
    replaced = fo.flag_cells(fo.Levels(ZOOM2), 0, (25., 25., 25.), 'cube', 10)
    lev, _ = fo.mapper_order(32, replaced, 32, 2, ORIGIN)
    m = make_map(ZOOM2, replaced, fo.tipsy_factors(ZOOM2, COSMO, lev))
    rc, want = pack_host(lib, m, [p for p, _ in parts], [v for _, v in parts])
    assert rc == 0
    n = len(want)
    got = np.zeros((n, 9), dtype=np.float32)
    gen._call('gic_tipsy_pack', ctypes.byref(m), 0, n, got.ctypes.data_as(ctypes.c_void_p))
    # the device reads the same doubles (float velocities widen exactly) and rounds alike
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # a window inside the fine particles, and one inside the coarse
    part = np.zeros((500, 9), dtype=np.float32)
    for first in (n - 600, 1000):
        gen._call('gic_tipsy_pack', ctypes.byref(m), first, 500, part.ctypes.data_as(ctypes.c_void_p))
        assert np.array_equal(part.view(np.uint32), want[first:first + 500].view(np.uint32))
    gen.close()
