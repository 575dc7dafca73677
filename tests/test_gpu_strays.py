"""genetIC's stray particles on the GPU (gic_fetch_particles_matched): a zoom level's
particles on its resolution-matching grid, the zoom's own inside its window and the level
above's interpolated outside it, against the oracle (FP64 1e-10, mixed 1e-5) and, packed in
genetIC's mapper order, against the reference build's tipsy file of the same case."""
import os

import numpy as np
import pytest

import field_oracle as fo
from conftest import COSMO, make_generator
from test_writers import GOLDEN, make_map, pack_host, strays_oracle

pytestmark = pytest.mark.gpu
GPU_LEVELS = [('base', 50.0, 32), ('zoom', 15, 15, 12, 4, 32)]


def _gpu(precision, bbks, cells):
    gen = make_generator(precision, bbks, GPU_LEVELS, 8896131, 'random_seed')
    gen.done()
    p0 = gen.particles(0)
    p1 = gen.particles_matched(1, cells)
    gen.close()
    return p0, p1


@pytest.fixture(scope='module')
def oracle(bbks):
    fo.set_cr_log(True)
    r = strays_oracle(bbks)
    fo.set_cr_log(False)
    return r


def _needed_cells(r):
    """The matching grid's cells genetIC's mapper asks for: the r^3 cells under each flagged
    level-0 cell (including the ones outside the zoom window: the strays)."""
    nv, ratio = r['nv'], r['nv'] // 32
    rep = np.asarray(r['replaced'], dtype=np.int64)
    x, y, z = rep // (32 * 32), (rep // 32) % 32, rep % 32
    o = np.arange(ratio)
    fx = (x[:, None] * ratio + o[None, :])
    fy = (y[:, None] * ratio + o[None, :])
    fz = (z[:, None] * ratio + o[None, :])
    cells = (fx[:, :, None, None] * nv + fy[:, None, :, None]) * nv + fz[:, None, None, :]
    return np.unique(cells.ravel()).astype(np.uint64)


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-10), ('mixed', 1e-5)])
def test_stray_particles_match_oracle(built, bbks, oracle, precision, tol):
    cells = _needed_cells(oracle)
    (pos0, vel0), (pos1, vel1) = _gpu(precision, bbks, cells)
    scale = np.abs(oracle['vel'][1]).max() / fo.velocity_to_offset_ratio(COSMO)
    for pos, vel, want_p, want_v in ((pos0, vel0, oracle['pos'][0], oracle['vel'][0]),
                                     (pos1, vel1, oracle['pos'][1][cells], oracle['vel'][1][cells])):
        d = (pos - want_p + 25.0) % 50.0 - 25.0
        assert np.abs(d).max() <= tol * scale
        assert np.abs(vel - want_v).max() <= tol * np.abs(want_v).max()


def test_stray_tipsy_records_match_reference_file(built, bbks, oracle):
    from genetic_gb300 import _lib
    g = np.load(os.path.join(GOLDEN, 'strays_zoom4.npz'))
    cells = _needed_cells(oracle)
    (pos0, vel0), (pos1, vel1) = _gpu('fp64', bbks, cells)
    nv = oracle['nv']
    full_p = np.zeros((nv ** 3, 3))
    full_v = np.zeros((nv ** 3, 3))
    full_p[cells.astype(np.int64)] = pos1
    full_v[cells.astype(np.int64)] = vel1
    vlevels = [(50.0, 32, (0.0, 0.0, 0.0)), (50.0, nv, (0.0, 0.0, 0.0))]
    m = make_map(vlevels, np.asarray(oracle['replaced'], dtype=np.uint64), oracle['factors'], ratio=nv // 32,
                 origin=(0, 0, 0))
    rc, got = pack_host(_lib.load(), m, [pos0, full_p], [vel0, full_v])
    assert rc == 0 and len(got) == int(g['nrec'])
    stride = int(g['stride'])
    for mine, ref in ((got[::stride], g['every']), (got[-400:], g['tail'])):
        assert np.array_equal(mine[:, 0], ref[:, 0]) and np.array_equal(mine[:, 7:], ref[:, 7:])
        assert np.abs(mine[:, 1:4] - ref[:, 1:4]).max() <= 6e-8
        assert np.abs(mine[:, 4:7] - ref[:, 4:7]).max() <= 2e-7 * np.abs(ref[:, 4:7]).max()


def test_matched_argument_errors(built, bbks):
    import genetic_gb300 as g
    gen = make_generator('fp64', bbks, GPU_LEVELS, 8896131, 'random_seed')
    gen.done()
    with pytest.raises(g.GicError):
        gen.particles_matched(0, np.array([0], dtype=np.uint64))
    with pytest.raises(g.GicError):
        gen.particles_matched(1, np.array([128 ** 3], dtype=np.uint64))
    gen.close()
