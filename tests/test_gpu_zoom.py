"""Zoom realisations (two and three levels) on the GPU against the oracle and the reference grids."""
import os

import numpy as np
import pytest

import field_oracle as fo
from conftest import COSMO, make_generator

pytestmark = pytest.mark.gpu
FIELDS = ('delta', 'psi_x', 'psi_y', 'psi_z')
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')

ZOOM2 = [('base', 50.0, 32), ('zoom', 8, 8, 8, 2, 32)]
ZOOM3 = ZOOM2 + [('zoom', 8, 8, 8, 2, 32)]
GEOM = {2: [(50.0, 32, (0.0, 0.0, 0.0)), (25.0, 32, (12.5, 12.5, 12.5))]}
GEOM[3] = GEOM[2] + [(12.5, 32, (18.75, 18.75, 18.75))]


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def _gpu(precision, bbks, levels, cmd):
    gen = make_generator(precision, bbks, levels, 8896131, cmd)
    gen.done()
    out = [{f: gen.field(l, f) for f in FIELDS} for l in range(len(levels))]
    parts = [gen.particles(l) for l in range(len(levels))]
    gen.close()
    return out, parts


def _oracle(bbks, nlev, mode):
    fo.set_cr_log(True)
    geom = GEOM[nlev]
    w = fo.white_noise_levels([g[1] for g in geom], 8896131, mode)
    fo.set_cr_log(False)
    return fo.zoom_realisation(w, geom, fo.CambPower(bbks, COSMO))


@pytest.mark.parametrize('levels,nlev,cmd,mode', [(ZOOM2, 2, 'random_seed', 2), (ZOOM2, 2, 'random_seed_real_space', 0),
                                                  (ZOOM2, 2, 'random_seed_serial', 1), (ZOOM3, 3, 'random_seed', 2)])
def test_zoom_fp64_matches_oracle(built, bbks, levels, nlev, cmd, mode):
    got, parts = _gpu('fp64', bbks, levels, cmd)
    want = _oracle(bbks, nlev, mode)
    for l in range(nlev):
        for i, f in enumerate(FIELDS):
            assert _rel(got[l][f], want[l][i]) < 1e-10, (l, f)
    # particles of the finest level: centroid + combined displacement
    box, n, off = GEOM[nlev][-1]
    pos, vel = fo.particles(want[-1][1:], box, off, 50.0, fo.velocity_to_offset_ratio(COSMO))
    d = (parts[-1][0] - pos + 25.0) % 50.0 - 25.0
    assert np.abs(d).max() < 1e-10 * np.abs(want[-1][1]).max() + 1e-12
    assert _rel(parts[-1][1], vel) < 1e-10


def test_zoom_matches_reference_grids(built, bbks):
    g = np.load(os.path.join(GOLDEN, 'zoom2_parallel.npz'))
    got, _ = _gpu('fp64', bbks, ZOOM2, 'random_seed')
    for l in range(2):
        assert _rel(got[l]['delta'], g['delta%d' % l]) < 1e-10


def test_zoom_mixed_within_stated_error(built, bbks):
    got, _ = _gpu('mixed', bbks, ZOOM2, 'random_seed')
    want = _oracle(bbks, 2, 2)
    for l in range(2):
        for i, f in enumerate(FIELDS):
            assert _rel(got[l][f], want[l][i]) < 1e-5, (l, f)
