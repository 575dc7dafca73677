"""Single-level Zel'dovich realisations on the GPU against the oracle."""
import numpy as np
import pytest

import field_oracle as fo
from conftest import COSMO, make_generator

pytestmark = pytest.mark.gpu

FIELDS = ('delta', 'psi_x', 'psi_y', 'psi_z')


def _run(precision, bbks, n, box, cmd, seed=8896131):
    gen = make_generator(precision, bbks, [('base', box, n)], seed, cmd)
    gen.done()
    out = {f: gen.field(0, f) for f in FIELDS}
    out['pos'], out['vel'] = gen.particles(0)
    out['norm'] = gen.normalisation()
    gen.close()
    return out


def _oracle(bbks, n, box, mode, seed=8896131):
    fo.set_cr_log(True)
    w = fo.white_noise(n, seed, mode)
    fo.set_cr_log(False)
    power = fo.CambPower(bbks, COSMO)
    d = fo.zeldovich_fields(w, power, box)
    pos, vel = fo.particles(d[1:], box, (0, 0, 0), box, fo.velocity_to_offset_ratio(COSMO))
    return dict(zip(FIELDS, d), pos=pos, vel=vel, power=power)


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize('n,box,cmd,mode', [(64, 50.0, 'random_seed_serial', 1), (32, 50.0, 'random_seed', 2),
                                            (64, 100.0, 'random_seed_real_space', 0)])
def test_fp64_matches_oracle(built, bbks, n, box, cmd, mode):
    got = _run('fp64', bbks, n, box, cmd)
    want = _oracle(bbks, n, box, mode)
    amp, s8pre = got['norm']
    assert abs(amp / want['power'].amplitude - 1) < 1e-12
    assert abs(s8pre / want['power'].sigma8_pre - 1) < 1e-12
    for f in FIELDS:
        assert _rel(got[f], want[f]) < 1e-10, f
    disp = (got['pos'] - want['pos'] + box / 2) % box - box / 2
    assert np.abs(disp).max() < 1e-10 * np.abs(want['psi_x']).max() + 1e-12 * box
    assert _rel(got['vel'], want['vel']) < 1e-10


def test_mixed_matches_oracle_within_stated_error(built, bbks):
    n, box = 64, 50.0
    got = _run('mixed', bbks, n, box, 'random_seed_serial')
    want = _oracle(bbks, n, box, 1)
    for f in FIELDS:
        assert _rel(got[f], want[f]) < 1e-5, f
    disp_err = np.abs((got['pos'] - want['pos'] + box / 2) % box - box / 2).max()
    assert disp_err < 1e-5 * np.abs(want['psi_x']).max()


def test_grid_fixture_from_reference(built, bbks):
    """Golden delta written by the reference build (tests/golden/make_golden.py)."""
    import os
    g = np.load(os.path.join(os.path.dirname(__file__), 'golden', 'bbks32_serial.npz'))
    got = _run('fp64', bbks, 32, 50.0, 'random_seed_serial')
    assert _rel(got['delta'], g['delta']) < 1e-10
    disp = (got['pos'] - g['pos'].astype(np.float64) + 25.0) % 50.0 - 25.0
    assert np.abs(disp).max() < 5e-6


@pytest.mark.parametrize('precision', ['mixed', 'fp64'])
def test_native_fetch_matches_double_fetch(built, bbks, precision):
    """gic_fetch_particles_native: the same positions, and velocities in the context's own
    precision (float32 in the mixed form) that widen exactly to gic_fetch_particles' doubles."""
    from conftest import make_generator
    gen = make_generator(precision, bbks, [('base', 50.0, 32)], 8896131, 'random_seed')
    gen.done()
    pos, vel = gen.particles(0)
    pos_n, vel_n = gen.particles_native(0)
    gen.close()
    assert vel_n.dtype == (np.float32 if precision == 'mixed' else np.float64)
    assert np.array_equal(pos, pos_n)
    assert np.array_equal(vel, vel_n.astype(np.float64))


@pytest.mark.parametrize('precision', ['mixed', 'fp64'])
def test_async_fetch_overlapping_realisations(built, bbks, precision):
    """gic_fetch_particles_async: three realisations in a row, each fetched without waiting
    while the next one computes (the level alternates between two device buffer pairs; the
    third waits on the device for the first fetch), give the particles of each realisation,
    the same bits as a synchronous fetch of it."""
    import ctypes
    torch = pytest.importorskip('torch')
    from conftest import make_generator
    from genetic_gb300.generator import _ptr
    levels = [('base', 50.0, 32), ('zoom', 8, 8, 8, 2, 32)]
    seeds = [11, 12, 13]
    want = []
    for seed in seeds:
        g = make_generator(precision, bbks, levels, seed, 'random_seed')
        g.done()
        want.append([g.particles_native(l) for l in range(2)])
        g.close()
    gen = make_generator(precision, bbks, levels, seeds[0], 'random_seed')
    vdt = torch.float32 if precision == 'mixed' else torch.float64
    bufs = [[(torch.empty((32 ** 3, 3), dtype=torch.float64, pin_memory=True).numpy(),
              torch.empty((32 ** 3, 3), dtype=vdt, pin_memory=True).numpy()) for _ in range(2)] for _ in seeds]
    for k, seed in enumerate(seeds):
        gen._call('gic_draw_noise', seed, 2)
        gen._call('gic_zeldovich', 1)
        for l, (pos, vel) in enumerate(bufs[k]):
            gen._call('gic_fetch_particles_async', l, _ptr(pos), ctypes.c_void_p(vel.ctypes.data))
    gen._call('gic_fetch_wait')
    gen.close()
    for k in range(len(seeds)):
        for l in range(2):
            assert np.array_equal(bufs[k][l][0], want[k][l][0]), (k, l)
            assert np.array_equal(bufs[k][l][1], want[k][l][1]), (k, l)
