"""The path at the configurations' own sizes, on the GPU against the oracle.

* White noise of a 256^3 grid (100 Mpc/h) in every seeding mode, and of a 512^3 grid in
  the parallel Fourier mode: bit for bit (the real-space mode: its gaussian stream bit for
  bit, its half spectrum to the transform's rounding).
* A 256^3 base (100 Mpc/h) plus a 256^3 zoom of side 25 Mpc/h (factor 4) centred at
  (50, 50, 50), with the four modifications in a 2 Mpc/h sphere at the centre (mean
  overdensity +1.5, mean velocities 0): per field (delta, psi, velocities, displacements of
  both levels) the max and RMS relative error |a - b| / max|b| against the FP64 oracle.
  FP64 within 1e-10; the mixed form within 1e-5.
"""
import json

import numpy as np
import pytest

import field_oracle as fo
from conftest import COSMO, make_generator

pytestmark = pytest.mark.gpu
SEED = 8896131
FIELDS = ('delta', 'psi_x', 'psi_y', 'psi_z')


@pytest.mark.parametrize('n,cmd,mode', [(256, 'random_seed_serial', 1), (256, 'random_seed', 2),
                                        (256, 'seedfourier_reverse', 3), (512, 'random_seed', 2)])
def test_white_noise_bit_exact_at_config_size(built, bbks, n, cmd, mode):
    gen = make_generator('fp64', bbks, [('base', 100.0, n)], SEED, cmd)
    gen.draw()
    got = gen.noise(0)
    gen.close()
    fo.set_cr_log(True)
    want = fo.white_noise(n, SEED, mode)
    fo.set_cr_log(False)
    assert np.array_equal(got.real, want.real) and np.array_equal(got.imag, want.imag)


def test_real_space_white_noise_at_config_size(built, bbks):
    n = 256
    gen = make_generator('fp64', bbks, [('base', 100.0, n)], SEED, 'random_seed_real_space')
    stream = gen.gaussian_stream(SEED, n ** 3)
    gen.draw()
    got = gen.noise(0)
    gen.close()
    fo.set_cr_log(True)
    assert np.array_equal(stream, fo.gaussian_stream(SEED, n ** 3)[0])
    want = fo.white_noise(n, SEED, 0)
    fo.set_cr_log(False)
    assert np.abs(got - want).max() < 1e-12 * np.abs(want).max()


C3_GPU = [('base', 100.0, 256), ('zoom', 96, 96, 96, 4, 256)]
C3_LEVELS = [(100.0, 256, (0.0, 0.0, 0.0)), (25.0, 256, (37.5, 37.5, 37.5))]
C3_MODS = [('overdensity', 0, 1.5), ('vx', 0, 0.0), ('vy', 1, 0.0), ('vz', 2, 0.0)]


@pytest.fixture(scope='module')
def c3_oracle(bbks):
    """The FP64 oracle on the two-level 256^3 configuration with the four modifications."""
    import os
    fo.set_fft_workers(os.cpu_count())
    L = fo.Levels(C3_LEVELS)
    fo.set_cr_log(True)
    w = fo.white_noise_levels([256, 256], SEED, 2)
    fo.set_cr_log(False)
    p_dm = fo.CambPower(bbks, COSMO, column=1)
    ratio = fo.velocity_to_offset_ratio(COSMO)
    flagged = fo.flag_cells(L, 1, (50., 50., 50.), 'sphere', 2.0)
    covs, values = [], {}
    for name, d, t in C3_MODS:
        loc = fo.localisation_covector(L, flagged, 'overdensity' if name == 'overdensity' else 'velocity', d)
        cv = fo.multilevel_covector(L, loc, p_dm, None if name == 'overdensity' else ratio)
        values[name] = fo.inner(cv, w)
        covs.append(cv)
    before = fo.chi2_levels(L, w)
    w2 = fo.apply_linear_modifications(L, w, covs, [float(np.float32(t)) for _, _, t in C3_MODS])
    after = fo.chi2_levels(L, w2)
    fields = fo.zoom_realisation(w2, C3_LEVELS, fo.CambPower(bbks, COSMO))
    parts = [fo.particles(f[1:], box, off, 100.0, ratio) for (box, _, off), f in zip(C3_LEVELS, fields)]
    fo.set_fft_workers(None)
    return dict(values=values, chi2=(before, after), noise=w2, fields=fields, parts=parts)


def _c3_errors(precision, bbks, want):
    gen = make_generator(precision, bbks, C3_GPU, SEED, 'random_seed')
    gen.centre(50, 50, 50)
    gen.select_sphere(2.0)
    values = {name: gen.calculate(name) for name, _, _ in C3_MODS}
    for name, _, t in C3_MODS:
        gen.modify(name, 'absolute', t)
    chi2 = gen.apply_modifications()
    gen.done(apply_modifications=False)
    err = {}

    def record(key, a, b, periodic=None):
        d = a - b
        if periodic:
            d = (d + periodic / 2) % periodic - periodic / 2
        scale = float(np.abs(b).max()) if periodic is None else float(np.abs(want['fields'][lev][1]).max())
        err[key] = {'max': float(np.abs(d).max() / scale), 'rms': float(np.sqrt(np.mean(d * d)) / scale)}

    for lev in range(2):
        for i, f in enumerate(FIELDS):
            record('L%d.%s' % (lev, f), gen.field(lev, f), want['fields'][lev][i])
        pos, vel = gen.particles(lev)
        record('L%d.velocity' % lev, vel, want['parts'][lev][1])
        record('L%d.displacement' % lev, pos, want['parts'][lev][0], periodic=100.0)
    gen.close()
    return values, chi2, err


def test_c3_fp64_matches_oracle(built, bbks, c3_oracle):
    values, chi2, err = _c3_errors('fp64', bbks, c3_oracle)
    print('C3 fp64 vs FP64 oracle:', json.dumps(err))
    for k, v in c3_oracle['values'].items():
        assert abs(values[k] - v) <= 1e-10 * max(abs(v), 1e-3), k
    d_got, d_want = chi2[1] - chi2[0], c3_oracle['chi2'][1] - c3_oracle['chi2'][0]
    assert abs(d_got - d_want) < 1e-9 * abs(d_want)
    for key, e in err.items():
        assert e['max'] < 1e-10, (key, e)


def test_c3_mixed_within_stated_error(built, bbks, c3_oracle):
    values, chi2, err = _c3_errors('mixed', bbks, c3_oracle)
    print('C3 mixed vs FP64 oracle:', json.dumps(err))
    for k, v in c3_oracle['values'].items():
        assert abs(values[k] - v) <= 1e-5 * max(abs(v), 1e-3), k
    assert abs(chi2[1] / c3_oracle['chi2'][1] - 1) < 1e-5
    for key, e in err.items():
        assert e['max'] < 1e-5, (key, e)
