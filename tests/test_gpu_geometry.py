"""The headline's zoom geometry on the GPU, against the oracle and the reference build.

Zoom factor 4 (the ratio-4 block means, interpolation and deinterpolation the headline
runs), factor 3 over an integer number of coarse cells (the generic-ratio block means),
and factor 3 over a fractional number of them (genetIC's test_01c geometry), with the
headline's four modifications (mean overdensity +1.5 and mean velocities 0 in a 2 Mpc/h
sphere at the zoom centre) and the differentiation configuration's variance modification;
and the batch workload's zoom class (zoom factor 4 with half as many zoom cells: cell
ratio 2) with its two overdensity modifications.
The oracle reproduces the reference build's grids of these cases to 1e-11
(tests/golden/geom_*.npz, test_oracle.py).  FP64: 1e-10 relative; mixed: 1e-5.
"""
import os

import numpy as np
import pytest

import field_oracle as fo
from conftest import COSMO, make_generator
from test_oracle import (GEOM_LEVELS, MOD_CASES, RATIO2_LEVELS, RATIO2_MODS, VAR_CASES, oracle_modified,
                         oracle_ratio2, oracle_variance)

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
FIELDS = ('delta', 'psi_x', 'psi_y', 'psi_z')

ZOOM4 = [('base', 50.0, 32), ('zoom', 12, 12, 12, 4, 32)]
GPU_LEVELS = {
    'zoom4': ZOOM4,
    'zoom3f': [('base', 50.0, 32), ('zoom', 11, 11, 11, 3, 32)],
    'mod4': ZOOM4,
    'var4': ZOOM4,
    'mod3': [('base', 72.0, 48), ('zoom', 16, 16, 16, 3, 48)],
}


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _realise(gen, nlev):
    gen.done(apply_modifications=False)
    fields = [{f: gen.field(l, f) for f in FIELDS} for l in range(nlev)]
    parts = [gen.particles(l) for l in range(nlev)]
    return fields, parts


def _check_fields(got, parts, want, levels, tol):
    periodic = levels[0][0]
    ratio = fo.velocity_to_offset_ratio(COSMO)
    for l, (box, n, off) in enumerate(levels):
        for i, f in enumerate(FIELDS):
            assert _rel(got[l][f], want[l][i]) < tol, (l, f, _rel(got[l][f], want[l][i]))
        pos, vel = fo.particles(want[l][1:], box, off, periodic, ratio)
        d = (parts[l][0] - pos + periodic / 2) % periodic - periodic / 2
        assert np.abs(d).max() < tol * np.abs(want[l][1]).max() + 1e-12, l
        assert _rel(parts[l][1], vel) < tol, l


@pytest.fixture(scope='module')
def realisations(bbks):
    out = {}
    for name, levels in GEOM_LEVELS.items():
        fo.set_cr_log(True)
        w = fo.white_noise_levels([l[1] for l in levels], 8896131, 2)
        fo.set_cr_log(False)
        out[name] = fo.zoom_realisation(w, levels, fo.CambPower(bbks, COSMO))
    return out


@pytest.mark.parametrize('name', ['zoom4', 'zoom3f'])
def test_zoom_geometry_fp64(built, bbks, realisations, name):
    gen = make_generator('fp64', bbks, GPU_LEVELS[name], 8896131, 'random_seed')
    got, parts = _realise(gen, 2)
    gen.close()
    _check_fields(got, parts, realisations[name], GEOM_LEVELS[name], 1e-10)
    g = np.load(os.path.join(GOLDEN, 'geom_%s.npz' % name))
    for l in range(2):
        assert _rel(got[l]['delta'], g['delta%d' % l]) < 1e-10, l


@pytest.mark.parametrize('name', ['zoom4', 'zoom3f'])
def test_zoom_geometry_mixed(built, bbks, realisations, name):
    gen = make_generator('mixed', bbks, GPU_LEVELS[name], 8896131, 'random_seed')
    got, parts = _realise(gen, 2)
    gen.close()
    _check_fields(got, parts, realisations[name], GEOM_LEVELS[name], 1e-5)


@pytest.fixture(scope='module')
def modified(bbks):
    return {case: oracle_modified(bbks, case, cr_log=True) for case in ('mod4', 'mod3')}


def _gpu_modified(precision, bbks, case):
    c = MOD_CASES[case]
    gen = make_generator(precision, bbks, GPU_LEVELS[case], 8896131, 'random_seed')
    gen.centre(*c.get('centre', (25., 25., 25.)))
    gen.select_sphere(c['radius'])
    values = {name: gen.calculate(name) for name, _, _ in c['mods']}
    for name, _, t in c['mods']:
        gen.modify(name, 'absolute', t)
    chi2 = gen.apply_modifications()
    noise = [gen.noise(l) for l in range(2)]
    fields, parts = _realise(gen, 2)
    flagged = gen.flagged.copy()
    gen.close()
    return dict(values=values, chi2=chi2, noise=noise, fields=fields, parts=parts, flagged=flagged)


@pytest.mark.parametrize('case', ['mod4', 'mod3'])
def test_geometry_modifications_fp64(built, bbks, modified, case):
    got = _gpu_modified('fp64', bbks, case)
    want = modified[case]
    assert np.array_equal(np.sort(got['flagged']), np.sort(want['flagged']))
    for k, v in want['values'].items():
        assert abs(got['values'][k] - v) <= 1e-10 * max(abs(v), 1e-3), k
    assert abs(got['chi2'][0] / want['chi2'][0] - 1) < 1e-11
    d_got, d_want = got['chi2'][1] - got['chi2'][0], want['chi2'][1] - want['chi2'][0]
    assert abs(d_got - d_want) < 1e-9 * abs(d_want)
    for l, w2 in enumerate(want['modified']):
        assert np.abs(got['noise'][l] - w2).max() < 1e-10 * np.abs(w2).max(), l
    levels = MOD_CASES[case]['levels']
    fields = fo.zoom_realisation(want['modified'], levels, fo.CambPower(bbks, COSMO))
    _check_fields(got['fields'], got['parts'], fields, levels, 1e-10)
    g = np.load(os.path.join(GOLDEN, 'geom_%s.npz' % case))
    for name in ('overdensity', 'vx', 'vy', 'vz'):
        assert '%.6g' % got['values'][name] == '%.6g' % float(g[name]), name
    assert '%.6g' % d_got == '%.6g' % float(g['delta_chi2'])
    for l in range(2):
        assert _rel(got['fields'][l]['delta'], g['delta%d' % l]) < 1e-10, l


@pytest.mark.parametrize('case', ['mod4', 'mod3'])
def test_geometry_modifications_mixed(built, bbks, modified, case):
    got = _gpu_modified('mixed', bbks, case)
    want = modified[case]
    for k, v in want['values'].items():
        assert abs(got['values'][k] - v) <= 1e-5 * max(abs(v), 1e-3), k
    assert abs(got['chi2'][1] / want['chi2'][1] - 1) < 1e-5
    for l, w2 in enumerate(want['modified']):
        assert np.abs(got['noise'][l] - w2).max() < 1e-5 * np.abs(w2).max(), l
    levels = MOD_CASES[case]['levels']
    fields = fo.zoom_realisation(want['modified'], levels, fo.CambPower(bbks, COSMO))
    _check_fields(got['fields'], got['parts'], fields, levels, 1e-5)


def _gpu_variance(precision, bbks):
    c = VAR_CASES['var4']
    gen = make_generator(precision, bbks, GPU_LEVELS['var4'], 8896131, 'random_seed')
    gen.centre(25, 25, 25)
    gen.select_sphere(c['select'][1])
    gen.filtering_scale(c['scale'])
    var = gen.calculate('variance')
    od = gen.calculate('overdensity')
    gen.modify('overdensity', 'relative', 1)
    gen.modify('variance', 'relative', c['rel'])
    chi2 = gen.apply_modifications()
    final = gen.calculate('variance')
    noise = [gen.noise(l) for l in range(2)]
    gen.done(apply_modifications=False)
    delta = [gen.field(l, 'delta') for l in range(2)]
    gen.close()
    return dict(variance=var, overdensity=od, chi2=chi2, final=final, noise=noise, delta=delta)


@pytest.fixture(scope='module')
def variance4(bbks):
    return oracle_variance(bbks, 'var4', cr_log=True)


def test_geometry_variance_fp64(built, bbks, variance4):
    got = _gpu_variance('fp64', bbks)
    want = variance4
    assert abs(got['variance'] / want['variance'] - 1) < 1e-10
    assert abs(got['overdensity'] - want['overdensity']) < 1e-10 * abs(want['overdensity'])
    d_got, d_want = got['chi2'][1] - got['chi2'][0], want['chi2'][1] - want['chi2'][0]
    assert abs(d_got - d_want) < 1e-7 * abs(d_want)
    assert abs(got['final'] / want['final'] - 1) < 1e-9
    for l, w2 in enumerate(want['modified']):
        assert np.abs(got['noise'][l] - w2).max() < 1e-9 * np.abs(w2).max(), l
    g = np.load(os.path.join(GOLDEN, 'geom_var4.npz'))
    assert '%.6g' % got['variance'] == '%.6g' % float(g['variance'])
    assert '%.6g' % d_got == '%.6g' % float(g['delta_chi2'])
    for l in range(2):
        assert _rel(got['delta'][l], g['delta%d' % l]) < 1e-9, l


def test_geometry_variance_mixed(built, bbks, variance4):
    got = _gpu_variance('mixed', bbks)
    want = variance4
    assert abs(got['variance'] / want['variance'] - 1) < 1e-5
    for l, w2 in enumerate(want['modified']):
        assert np.abs(got['noise'][l] - w2).max() < 1e-5 * np.abs(w2).max(), l
    assert abs(got['final'] / want['final'] - 1) < 1e-5


RATIO2_GPU = [('base', 100.0, 64), ('zoom', 24, 24, 24, 4, 32)]


@pytest.mark.parametrize('precision,tol', [('fp64', 1e-10), ('mixed', 1e-5)])
def test_ratio2_zoom_with_modifications(built, bbks, precision, tol):
    want = oracle_ratio2(bbks, cr_log=True)
    gen = make_generator(precision, bbks, RATIO2_GPU, 8896131, 'random_seed')
    values = []
    for centre, radius, target in RATIO2_MODS:
        gen.centre(*centre)
        gen.select_sphere(radius)
        values.append(gen.calculate('overdensity'))
        gen.modify('overdensity', 'absolute', target)
    chi2 = gen.apply_modifications()
    fields, parts = _realise(gen, 2)
    gen.close()
    for v, w in zip(values, want['values']):
        assert abs(v - w) <= tol * max(abs(w), 1e-3)
    d_got, d_want = chi2[1] - chi2[0], want['chi2'][1] - want['chi2'][0]
    assert abs(d_got - d_want) < 10 * tol * abs(d_want)
    ref = fo.zoom_realisation(want['modified'], RATIO2_LEVELS, fo.CambPower(bbks, COSMO))
    _check_fields(fields, parts, ref, RATIO2_LEVELS, tol)
    g = np.load(os.path.join(GOLDEN, 'geom_ratio2.npz'))
    for l in range(2):
        assert _rel(fields[l]['delta'], g['delta%d' % l]) < tol, l
