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


@pytest.mark.parametrize('precision', ['mixed'])
def test_async_tipsy_pack_overlapping_realisations(built, bbks, precision):
    """gic_tipsy_pack_async after each of three realisations in a row, without waiting
    (two device record buffers alternate; the copies run on the copy stream): each
    pinned buffer holds its own realisation's records, the same bits as gic_tipsy_pack."""
    torch = pytest.importorskip('torch')
    replaced = fo.flag_cells(fo.Levels(ZOOM2), 0, (25., 25., 25.), 'cube', 10)
    lev, _ = fo.mapper_order(32, replaced, 32, 2, ORIGIN)
    m = make_map(ZOOM2, replaced, fo.tipsy_factors(ZOOM2, COSMO, lev))
    seeds = [21, 22, 23]
    want = []
    for seed in seeds:
        g = make_generator(precision, bbks, LEVELS, seed, 'random_seed')
        g.done()
        n = 32 ** 3 + 7 * len(replaced)  # coarse cells kept + 8 fine particles per replaced cell
        rec = np.zeros((n, 9), dtype=np.float32)
        g._call('gic_tipsy_pack', ctypes.byref(m), 0, n, rec.ctypes.data_as(ctypes.c_void_p))
        want.append(rec)
        g.close()
    gen = make_generator(precision, bbks, LEVELS, seeds[0], 'random_seed')
    bufs = [torch.zeros((n * 9,), dtype=torch.float32, pin_memory=True).numpy() for _ in seeds]
    for k, seed in enumerate(seeds):
        gen._call('gic_draw_noise', seed, 2)
        gen._call('gic_zeldovich', 1)
        gen._call('gic_tipsy_pack_async', ctypes.byref(m), 0, n, bufs[k].ctypes.data_as(ctypes.c_void_p))
    gen._call('gic_fetch_wait')
    gen.close()
    for k in range(len(seeds)):
        assert np.array_equal(bufs[k].view(np.uint32), want[k].reshape(-1).view(np.uint32)), k


def _gadget_host(lib, m, pos, vel, types, first, count):
    P = ctypes.POINTER(ctypes.c_double)
    pp = (P * len(pos))(*[np.ascontiguousarray(p).ctypes.data_as(P) for p in pos])
    vv = (P * len(vel))(*[np.ascontiguousarray(v).ctypes.data_as(P) for v in vel])
    t = (ctypes.c_int * len(types))(*types) if types else None
    out = (np.zeros((count, 3), np.float32), np.zeros((count, 3), np.float32), np.zeros(count, np.uint64),
           np.zeros(count, np.float32))
    rc = lib.gic_gadget_pack_host(ctypes.byref(m), pp, vv, t, first, count, *[o.ctypes.data_as(ctypes.c_void_p) for o in out],
                                  4)
    return rc, out


def _gadget_device(gen, m, types, first, count):
    t = (ctypes.c_int * len(types))(*types) if types else None
    out = (np.zeros((count, 3), np.float32), np.zeros((count, 3), np.float32), np.zeros(count, np.uint64),
           np.zeros(count, np.float32))
    gen._call('gic_gadget_pack', ctypes.byref(m), t, first, count, *[o.ctypes.data_as(ctypes.c_void_p) for o in out])
    return out


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
@pytest.mark.parametrize('types', [None, (3, 1), (1, 1)])
def test_device_gadget_matches_host_packer(built, bbks, precision, types):
    """gic_gadget_pack (the four blocks on the device) against gic_gadget_pack_host given the
    fetched particles, bit for bit: the whole file, and windows across the level boundary."""
    from genetic_gb300 import _lib
    lib = _lib.load()
    gen = make_generator(precision, bbks, LEVELS, 8896131, 'random_seed')
    gen.done()
    parts = [gen.particles(l) for l in range(2)]
    replaced = fo.flag_cells(fo.Levels(ZOOM2), 0, (25., 25., 25.), 'cube', 10)
    lev, _ = fo.mapper_order(32, replaced, 32, 2, ORIGIN)
    m = make_map(ZOOM2, replaced, fo.tipsy_factors(ZOOM2, COSMO, lev))
    n = len(lev)
    for first, count in ((0, n), (n - 5000, 4000), (27000, 3000)):
        rc, want = _gadget_host(lib, m, [p for p, _ in parts], [v for _, v in parts], types, first, count)
        assert rc == 0
        got = _gadget_device(gen, m, types, first, count)
        for a, b in zip(got, want):
            assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), (first, count)
    gen.close()


def test_device_gadget_one_level(built, bbks):
    from genetic_gb300 import _lib
    lib = _lib.load()
    gen = make_generator('mixed', bbks, [('base', 50.0, 32)], 8896131, 'random_seed')
    gen.done()
    pos, vel = gen.particles(0)
    one = [ZOOM2[0]]
    m = make_map(one, np.zeros(0, np.uint64), fo.tipsy_factors(one, COSMO, np.zeros(32 ** 3, int)))
    rc, want = _gadget_host(lib, m, [pos], [vel], None, 0, 32 ** 3)
    assert rc == 0
    got = _gadget_device(gen, m, None, 0, 32 ** 3)
    for a, b in zip(got, want):
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8))
    gen.close()
