"""The grafic writer's per-cell values packed on the device (gic_grafic_pack) against the
reference build's grafic files (tests/golden/grafic_zoom.npz, which the oracle's
restatement reproduces exactly): a 16^3 base of 50 Mpc/h with its subsampled grid, both
centred on (30, 20, 25) (whole-cell rolls), a factor-4 zoom of 16 cells and its
intermediate subsampled grid.  FP64: every float within one rounding step of the file's;
mixed: within 1e-5 of the largest value; ids exactly."""
import ctypes

import numpy as np
import pytest

from conftest import COSMO, make_generator
from test_oracle import GRAFIC_GRIDS, _load_golden

pytestmark = pytest.mark.gpu
NAMES = ('velcx', 'velcy', 'velcz', 'poscx', 'poscy', 'poscz', 'deltab')


def _pack(gen, eff, level, factor, roll, off):
    from genetic_gb300 import _lib
    n = {8: 8, 16: 16, 32: 8, 64: 16}[eff]
    g = _lib.GraficGrid(level, factor, (ctypes.c_int * 3)(*roll), float(np.sqrt(1.0 / (1.0 + COSMO['redshift']))), 1.0,
                        off)
    m = n ** 3
    vel = np.zeros(3 * m, np.float32)
    pos = np.zeros(3 * m, np.float32)
    dl = np.zeros(m, np.float32)
    ids = np.zeros(m, np.uint64)
    gen._call('gic_grafic_pack', ctypes.byref(g), 0, n, vel.ctypes.data_as(ctypes.c_void_p),
              pos.ctypes.data_as(ctypes.c_void_p), dl.ctypes.data_as(ctypes.c_void_p), ids.ctypes.data_as(ctypes.c_void_p))
    shape = (n, n, n)
    return ([vel[a * m:(a + 1) * m].reshape(shape) for a in range(3)] + [pos[a * m:(a + 1) * m].reshape(shape)
                                                                        for a in range(3)] + [dl.reshape(shape)],
            ids.reshape(shape))


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_grafic_pack_matches_reference_files(built, bbks, precision):
    g = _load_golden('grafic_zoom.npz')
    o = [int(v) for v in g['origin']]
    gen = make_generator(precision, bbks, [('base', 50.0, 16), ('zoom', o[0], o[1], o[2], 4, 16)], 8896131,
                         'random_seed')
    gen.done()
    for eff, level, factor, roll, off in GRAFIC_GRIDS:
        vals, ids = _pack(gen, eff, level, factor, roll, off)
        assert np.array_equal(ids, g['g%d_ic_particle_ids' % eff]), eff
        for name, got in zip(NAMES, vals):
            want = g['g%d_ic_%s' % (eff, name)]
            if precision == 'fp64':
                assert np.all(np.abs(got - want) <= np.spacing(np.abs(want))), (eff, name)
            else:
                assert np.abs(got - want).max() <= 1e-5 * np.abs(want).max(), (eff, name)
    # a window of slabs is the same bits as those slabs of the whole grid
    from genetic_gb300 import _lib
    eff, level, factor, roll, off = GRAFIC_GRIDS[1]
    whole, _ = _pack(gen, eff, level, factor, roll, off)
    gr = _lib.GraficGrid(level, factor, (ctypes.c_int * 3)(*roll), 0.1, 1.0, off)
    part = np.zeros(3 * 5 * 256, np.float32)
    gen._call('gic_grafic_pack', ctypes.byref(gr), 4, 5, part.ctypes.data_as(ctypes.c_void_p), None, None, None)
    assert np.array_equal(part[:5 * 256].reshape(5, 16, 16), whole[0][4:9])
    gen.close()


def test_grafic_pack_rejects_bad_grids(built, bbks):
    import genetic_gb300 as gg
    from genetic_gb300 import _lib
    gen = make_generator('mixed', bbks, [('base', 50.0, 16)], 8896131, 'random_seed')
    gen.done()
    buf = np.zeros(16 ** 3 * 3, np.float32)
    for level, factor, z0, nz in ((1, 1, 0, 16), (0, -3, 0, 5), (0, 0, 0, 16), (0, 1, 10, 7)):
        gr = _lib.GraficGrid(level, factor, (ctypes.c_int * 3)(0, 0, 0), 0.1, 1.0, 0)
        with pytest.raises(gg.GicError):
            gen._call('gic_grafic_pack', ctypes.byref(gr), z0, nz, buf.ctypes.data_as(ctypes.c_void_p), None, None,
                      None)
    gen.close()
