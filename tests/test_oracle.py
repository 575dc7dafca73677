"""The oracle against the reference's own known answers (CPU)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import field_oracle as fo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_TESTS = os.path.join(subprocess.run(['make', '-s', '-C', os.path.join(ROOT, 'oracle'), 'print-ref'],
                                        capture_output=True, text=True).stdout.strip(), 'tests')
REF_BIN = os.path.join(ROOT, 'oracle', '_ref', 'genetIC')
GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def test_chi2_real_space_seed_matches_reference_fixture():
    # genetIC/tests/test_02k_chisquare_onelevel/reference.txt: random_seed_real_space 13842314, 64^3
    fo.set_cr_log(False)
    w = fo.white_noise(64, 13842314, 0)
    assert '%.10g' % fo.chi2(w) == '261733.3011'


def test_cr_log_mode_changes_nothing_at_this_size():
    fo.set_cr_log(True)
    a, _ = fo.gaussian_stream(13842314, 200000)
    fo.set_cr_log(False)
    b, _ = fo.gaussian_stream(13842314, 200000)
    assert np.max(np.abs(a - b)) <= 2e-16 * np.max(np.abs(a))


def test_ranlux_stream_first_values_stable():
    s = fo.ranlux_stream(1, 48)
    assert s.dtype == np.uint32 and s.max() < 2 ** 24
    # stream is a pure function of the seed
    assert np.array_equal(s, fo.ranlux_stream(1, 48))
    assert not np.array_equal(s, fo.ranlux_stream(2, 48))


def _load_golden(name):
    return np.load(os.path.join(GOLDEN, name))


@pytest.mark.parametrize('mode', ['serial', 'parallel', 'real'])
def test_field_oracle_matches_reference_delta(mode, bbks):
    """Golden delta grids written by the reference build (tests/golden/make_golden.py)."""
    from conftest import COSMO
    g = _load_golden('bbks32_%s.npz' % mode)
    fo.set_cr_log(False)
    w = fo.white_noise(32, 8896131, {'serial': 1, 'parallel': 2, 'real': 0}[mode])
    power = fo.CambPower(bbks, COSMO)
    d, px, py, pz = fo.zeldovich_fields(w, power, 50.0)
    ref = g['delta']
    assert np.abs(d - ref).max() <= 1e-12 * np.abs(ref).max()
    if 'pos' not in g:
        return
    pos, vel = fo.particles([px, py, pz], 50.0, (0, 0, 0), 50.0, fo.velocity_to_offset_ratio(COSMO))
    # tipsy stores float32 positions in box units: compare to float32 resolution
    dp = pos - g['pos'].astype(np.float64)
    dp = (dp + 25.0) % 50.0 - 25.0
    assert np.abs(dp).max() < 5e-6


def _run_reference(tmp_path, name):
    src = os.path.join(REF_TESTS, name)
    dst = tmp_path / name
    shutil.copytree(src, dst)
    for dat in ('camb_transfer_kmax40_z0.dat', 'camb_transfer_kmax40_z0_post2015.dat'):
        shutil.copy(os.path.join(REF_TESTS, dat), tmp_path / dat)
    r = subprocess.run([REF_BIN, 'paramfile.txt'], cwd=dst, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return dst, r.stdout + r.stderr


needs_reference = pytest.mark.skipif(not (os.path.isdir(REF_TESTS) and os.path.exists(REF_BIN)),
                                     reason='reference sources / build not present')


@needs_reference
@pytest.mark.parametrize('name', ['test_02k_chisquare_onelevel', 'test_02m_chisquare_twolevels',
                                  'test_02l_chisquare_modification', 'test_02f_onelevelvariance',
                                  'test_02g_multilevelvariance'])
def test_reference_build_log_fixtures(tmp_path, name):
    import re
    d, out = _run_reference(tmp_path, name)
    lines = [re.sub(r'^ [0-9]{4}-[0-9]{2}-[0-9]{2} [0-9]{2}:[0-9]{2}:[0-9]{2}   ', '', l) for l in out.splitlines()]
    for want in open(d / 'reference.txt').read().splitlines():
        if want.strip():
            assert want in lines, want


@needs_reference
@pytest.mark.parametrize('name', ['test_13_parallel_seed', 'test_05a_seed_old'])
def test_reference_build_tipsy_fixtures(tmp_path, name):
    from tipsy_reader import read_tipsy
    d, _ = _run_reference(tmp_path, name)
    out = [f for f in os.listdir(d) if f.endswith('.tipsy')][0]
    _, _, a = read_tipsy(d / out)
    _, _, b = read_tipsy(d / 'reference_output')
    assert np.array_equal(a, b)


@needs_reference
def test_reference_build_grid_fixture(tmp_path):
    d, _ = _run_reference(tmp_path, 'test_01c_zoom_grid')
    for g in ('grid-0.npy', 'grid-1.npy'):
        np.testing.assert_almost_equal(np.load(d / g), np.load(d / 'reference_grid' / g), decimal=4)


ZOOM_LEVELS = {
    'zoom2': [(50.0, 32, (0.0, 0.0, 0.0)), (25.0, 32, (12.5, 12.5, 12.5))],
    'zoom3': [(50.0, 32, (0.0, 0.0, 0.0)), (25.0, 32, (12.5, 12.5, 12.5)), (12.5, 32, (18.75, 18.75, 18.75))],
}


@pytest.mark.parametrize('name,mode,tol', [('zoom2', 'parallel', 1e-12), ('zoom2', 'real', 1e-12),
                                           ('zoom3', 'parallel', 2e-7)])
def test_zoom_oracle_matches_reference_grids(bbks, name, mode, tol):
    from conftest import COSMO
    g = _load_golden('%s_%s.npz' % (name, mode))
    levels = ZOOM_LEVELS[name]
    fo.set_cr_log(False)
    w = fo.white_noise_levels([l[1] for l in levels], 8896131, {'parallel': 2, 'real': 0}[mode])
    out = fo.zoom_realisation(w, levels, fo.CambPower(bbks, COSMO))
    for l in range(len(levels)):
        ref = g['delta%d' % l]
        assert np.abs(out[l][0] - ref).max() <= tol * np.abs(ref).max(), l


MOD_CASES = {
    'mod1': dict(levels=[(50.0, 32, (0.0, 0.0, 0.0))], radius=5,
                 mods=[('overdensity', 0, 0.05), ('vx', 0, 0.0)]),
    'mod2': dict(levels=[(50.0, 32, (0.0, 0.0, 0.0)), (25.0, 32, (12.5, 12.5, 12.5))], radius=3,
                 mods=[('overdensity', 0, 0.05), ('vx', 0, 0.0), ('vy', 1, 0.0), ('vz', 2, 0.0)]),
    # the headline's zoom factor 4 and its four modifications (mean overdensity +1.5 and the
    # three mean velocities 0 in a 2 Mpc/h sphere at the zoom centre), at 32^3 + 32^3
    'mod4': dict(levels=[(50.0, 32, (0.0, 0.0, 0.0)), (12.5, 32, (18.75, 18.75, 18.75))], radius=2,
                 mods=[('overdensity', 0, 1.5), ('vx', 0, 0.0), ('vy', 1, 0.0), ('vz', 2, 0.0)]),
    # zoom factor 3 (generic-ratio block means) on a 72 Mpc/h, 48^3 base
    'mod3': dict(levels=[(72.0, 48, (0.0, 0.0, 0.0)), (24.0, 48, (24.0, 24.0, 24.0))], radius=2,
                 centre=(36., 36., 36.),
                 mods=[('overdensity', 0, 1.5), ('vx', 0, 0.0), ('vy', 1, 0.0), ('vz', 2, 0.0)]),
}


def oracle_modified(bbks, case, cr_log=False):
    """Modified noise, covector values and chi^2 of a MOD_CASES entry, from the oracle."""
    from conftest import COSMO
    c = MOD_CASES[case]
    L = fo.Levels(c['levels'])
    fo.set_cr_log(cr_log)
    w = fo.white_noise_levels([l[1] for l in c['levels']], 8896131, 2)
    fo.set_cr_log(False)
    p_dm = fo.CambPower(bbks, COSMO, column=1)
    vs = fo.velocity_to_offset_ratio(COSMO)
    flagged = fo.flag_cells(L, len(c['levels']) - 1, c.get('centre', (25., 25., 25.)), 'sphere', c['radius'])
    covs, targets, values = [], [], {}
    for name, d, t in c['mods']:
        loc = fo.localisation_covector(L, flagged, 'overdensity' if name == 'overdensity' else 'velocity', d)
        cv = fo.multilevel_covector(L, loc, p_dm, None if name == 'overdensity' else vs)
        values[name] = fo.inner(cv, w)
        covs.append(cv)
        targets.append(float(np.float32(t)))
    before = fo.chi2_levels(L, w)
    w2 = fo.apply_linear_modifications(L, w, covs, targets)
    after = fo.chi2_levels(L, w2)
    return dict(levels=L, noise=w, modified=w2, values=values, chi2=(before, after), flagged=flagged)


@pytest.mark.parametrize('case', ['mod1', 'mod2'])
def test_modification_oracle_matches_reference(bbks, case):
    from conftest import COSMO
    g = _load_golden('%s.npz' % case)
    r = oracle_modified(bbks, case)
    # log lines carry 6 significant digits
    assert '%.6g' % r['values']['overdensity'] == '%.6g' % float(g['overdensity'])
    assert '%.6g' % r['values']['vx'] == '%.6g' % float(g['vx'])
    assert '%.6g' % (r['chi2'][1] - r['chi2'][0]) == '%.6g' % float(g['delta_chi2'])
    levels = MOD_CASES[case]['levels']
    out = fo.zoom_realisation(r['modified'], levels, fo.CambPower(bbks, COSMO))
    for l in range(len(levels)):
        ref = g['delta%d' % l].astype(np.float64)
        assert np.abs(out[l][0] - ref).max() <= 2e-7 * np.abs(ref).max()


# --- quadratic (variance) modification ----------------------------------------------

REF_COSMO = dict(omega_m=0.279, omega_lambda=0.721, omega_b=0.0, hubble=0.701, sigma8=0.817, ns=0.96, redshift=99.0)
needs_reference_tests = pytest.mark.skipif(not os.path.isdir(REF_TESTS), reason='reference test fixtures not present')


def _ref_camb():
    from genetic_gb300.transfer import read_camb
    return read_camb(os.path.join(REF_TESTS, 'camb_transfer_kmax40_z0.dat'))


@needs_reference_tests
@pytest.mark.parametrize('name,levels,centre,size,want', [
    # test_02f_onelevelvariance: select_cube 20 at (8, 8, 8), filtering_scale 10000
    ('02f', [(64.0, 64, (0, 0, 0))], (8., 8., 8.), 20, '0.00182096'),
    # test_02g_multilevelvariance: zoom 4x at the origin, select_cube 16 at (8, 8, 8)
    ('02g', [(64.0, 64, (0, 0, 0)), (16.0, 64, (0., 0., 0.))], (8., 8., 8.), 16, '0.00396257'),
])
def test_variance_oracle_matches_reference_values(name, levels, centre, size, want):
    np.seterr(over='ignore')
    L = fo.Levels(levels)
    fo.set_cr_log(False)
    w = fo.white_noise_levels([l[1] for l in levels], 8896131, 0)
    fl = [fo.flag_cells(L, l, centre, 'cube', size) for l in range(len(levels))]
    p_dm = fo.CambPower(_ref_camb(), REF_COSMO, column=1)
    assert '%.6g' % fo.variance_value(L, w, fl, 10000., p_dm) == want


@needs_reference_tests
def test_quadratic_oracle_matches_reference_grids():
    """test_02i_multilevel_algorithm: overdensity held, variance doubled, two levels."""
    np.seterr(over='ignore')
    levels = [(64.0, 64, (0, 0, 0)), (16.0, 64, (24., 24., 24.))]
    L = fo.Levels(levels)
    fo.set_cr_log(False)
    w = fo.white_noise_levels([64, 64], 8896131, 0)
    fl = [fo.flag_cells(L, l, (32.5, 32.5, 32.5), 'cube', 6.0) for l in range(2)]
    p_dm = fo.CambPower(_ref_camb(), REF_COSMO, column=1)
    cv = fo.multilevel_covector(L, fo.localisation_covector(L, fl[-1], 'overdensity'), p_dm, None)
    od, var = fo.inner(cv, w), fo.variance_value(L, w, fl, 2.0, p_dm)
    assert ('%.6g' % od, '%.6g' % var) == ('0.00298075', '0.00232681')
    before = fo.chi2_levels(L, w)
    w1, vecs = fo.apply_linear_modifications(L, w, [cv], [od], return_vectors=True)
    w2, steps = fo.apply_quadratic_modification(L, w1, vecs, fl, 2.0, p_dm, 2.0 * var)
    assert steps == 10
    assert '%.6g' % (fo.chi2_levels(L, w2) - before) == '3893.93'
    out = fo.zoom_realisation(w2, levels, fo.CambPower(_ref_camb(), REF_COSMO))
    for l in range(2):
        ref = np.load(os.path.join(REF_TESTS, 'test_02i_multilevel_algorithm', 'reference_grid', 'grid-%d.npy' % l))
        # the reference fixture was written with FFTW; the oracle's exact DFTs differ by ~3e-9 after the iterations
        assert np.abs(out[l][0] - ref).max() <= 1e-8 * np.abs(ref).max()


VAR_CASES = {
    'var1': dict(levels=[(50.0, 32, (0.0, 0.0, 0.0))], select=('sphere', 8), scale=4.0, rel=3.0),
    'var2': dict(levels=[(50.0, 32, (0.0, 0.0, 0.0)), (25.0, 32, (12.5, 12.5, 12.5))], select=('sphere', 4),
                 scale=3.0, rel=1.5),
    # the differentiation configuration's variance modification (3 Mpc/h filter, 5 Mpc/h sphere,
    # variance x 1.3, overdensity held) on the factor-4 zoom, at 32^3 + 32^3
    'var4': dict(levels=[(50.0, 32, (0.0, 0.0, 0.0)), (12.5, 32, (18.75, 18.75, 18.75))], select=('sphere', 5),
                 scale=3.0, rel=1.3),
}


def oracle_variance(bbks, case, cr_log=False):
    """Values, step count, chi^2 and modified noise of a VAR_CASES entry (overdensity
    held at its value, variance scaled by `rel`), from the oracle."""
    from conftest import COSMO
    np.seterr(over='ignore')
    c = VAR_CASES[case]
    L = fo.Levels(c['levels'])
    fo.set_cr_log(cr_log)
    w = fo.white_noise_levels([l[1] for l in c['levels']], 8896131, 2)
    fo.set_cr_log(False)
    p_dm = fo.CambPower(bbks, COSMO, column=1)
    fl = [fo.flag_cells(L, l, (25., 25., 25.), *c['select']) for l in range(len(c['levels']))]
    cv = fo.multilevel_covector(L, fo.localisation_covector(L, fl[-1], 'overdensity'), p_dm, None)
    od, var = fo.inner(cv, w), fo.variance_value(L, w, fl, c['scale'], p_dm)
    before = fo.chi2_levels(L, w)
    w1, vecs = fo.apply_linear_modifications(L, w, [cv], [od], return_vectors=True)
    target = float(np.float32(c['rel'])) * var
    w2, steps = fo.apply_quadratic_modification(L, w1, vecs, fl, c['scale'], p_dm, target)
    after = fo.chi2_levels(L, w2)
    return dict(levels=L, noise=w, modified=w2, overdensity=od, variance=var, steps=steps, chi2=(before, after),
                flagged=fl, target=target, final=fo.variance_value(L, w2, fl, c['scale'], p_dm))


@pytest.mark.parametrize('case', ['var1', 'var2'])
def test_variance_oracle_matches_goldens(bbks, case):
    from conftest import COSMO
    g = _load_golden('%s.npz' % case)
    r = oracle_variance(bbks, case)
    assert '%.6g' % r['variance'] == '%.6g' % float(g['variance'])
    assert '%.6g' % r['overdensity'] == '%.6g' % float(g['overdensity'])
    assert r['steps'] == int(g['steps'])
    assert '%.6g' % (r['chi2'][1] - r['chi2'][0]) == '%.6g' % float(g['delta_chi2'])
    assert abs(r['final'] / r['target'] - 1) < 1e-3
    out = fo.zoom_realisation(r['modified'], VAR_CASES[case]['levels'], fo.CambPower(bbks, COSMO))
    for l in range(len(VAR_CASES[case]['levels'])):
        ref = g['delta%d' % l]
        assert np.abs(out[l][0] - ref).max() <= 1e-11 * np.abs(ref).max(), l


# --- second-order LPT (no reference counterpart: checked against the analytic solution) ---

def test_lpt2_oracle_two_plane_waves():
    """delta = A cos(k1 x) + B cos(k2 y): S = A B cos(k1 x) cos(k2 y) and
    psi2 = (3/7) grad S / (k1^2 + k2^2); a single plane wave has psi2 = 0."""
    n, box = 32, 50.0
    k1, k2, A, B = 2 * np.pi * 3 / box, 2 * np.pi * 2 / box, 0.05, 0.03
    g = np.arange(n) * box / n
    X, Y, _ = np.meshgrid(g, g, g, indexing='ij')
    for a, b in ((A, B), (A, 0.0)):
        dk = fo.fft_r2c(a * np.cos(k1 * X) + b * np.cos(k2 * Y))
        phi = [fo.fft_c2r(s) for s in fo.potential_hessian_spectra(dk, box)]
        assert np.abs(fo.lpt2_source(phi) - a * b * np.cos(k1 * X) * np.cos(k2 * Y)).max() < 1e-15
        psi2 = [fo.fft_c2r(s) for s in fo.displacement_spectra(fo.fft_r2c(fo.lpt2_source(phi)) * fo.LPT2_FACTOR, box)]
        K2 = k1 * k1 + k2 * k2
        want = [(3 / 7) * a * b * -k1 * np.sin(k1 * X) * np.cos(k2 * Y) / K2,
                (3 / 7) * a * b * -k2 * np.cos(k1 * X) * np.sin(k2 * Y) / K2, 0 * X]
        for p, w in zip(psi2, want):
            assert np.abs(p - w).max() < 1e-15


# --- operations on the white noise ----------------------------------------------------

OPS_CASES = {
    'ops_reverse': ('reverse', None, 1), 'ops_reverse_small_k': ('reverse_small_k', 0.5, 1),
    'ops_fix_power': ('fix_power', None, 1), 'ops_reverse_small_k_zoom': ('reverse_small_k', 0.7, 2),
    'ops_fix_power_zoom': ('fix_power', None, 2),
}
OPS_LEVELS = {1: [(50.0, 32, (0.0, 0.0, 0.0))], 2: [(50.0, 32, (0.0, 0.0, 0.0)), (25.0, 32, (12.5, 12.5, 12.5))]}


def oracle_noise_op(case, cr_log=False):
    op, param, nlev = OPS_CASES[case]
    levels = OPS_LEVELS[nlev]
    fo.set_cr_log(cr_log)
    w = fo.white_noise_levels([l[1] for l in levels], 8896131, 2)
    fo.set_cr_log(False)
    if op == 'reverse':
        w = [-x for x in w]
    elif op == 'reverse_small_k':
        w = [fo.noise_reverse_small_k(x, l[0], param) for x, l in zip(w, levels)]
    else:
        w = [fo.noise_unit_modulus(x) for x in w]
    return levels, w


@pytest.mark.parametrize('case', sorted(OPS_CASES))
def test_noise_op_oracle_matches_reference(bbks, case):
    from conftest import COSMO
    g = _load_golden('%s.npz' % case)
    levels, w = oracle_noise_op(case)
    out = fo.zoom_realisation(w, levels, fo.CambPower(bbks, COSMO))
    for l in range(len(levels)):
        ref = g['delta%d' % l]
        assert np.abs(out[l][0] - ref).max() <= 1e-12 * np.abs(ref).max(), l


# --- potential and angular-momentum modifications ----------------------------------------

MOD_MORE_CASES = {
    'mod_pot1': dict(levels=[(50.0, 32, (0.0, 0.0, 0.0))], centre=(25., 25., 25.), select=('sphere', 5),
                     calc=['potential'], mods=[('potential', 'relative', 2.0)]),
    'mod_am1': dict(levels=[(50.0, 32, (0.0, 0.0, 0.0))], centre=(25., 25., 25.), select=('ellipse', (10, 7.5, 5)),
                    calc=['Ly', 'Lz'], mods=[('Ly', 'absolute', 100.0), ('Lz', 'relative', 0.5)]),
    'mod_am2': dict(levels=[(50.0, 32, (0.0, 0.0, 0.0)), (25.0, 32, (12.5, 12.5, 12.5))], centre=(25.3, 24.8, 25.),
                    select=('sphere', 4), calc=['Lx', 'potential'],
                    mods=[('Lx', 'absolute', 50.0), ('potential', 'absolute', 0.0)]),
}


def oracle_mod_more(bbks, case, cr_log=False):
    from conftest import COSMO
    c = MOD_MORE_CASES[case]
    L = fo.Levels(c['levels'])
    fo.set_cr_log(cr_log)
    w = fo.white_noise_levels([l[1] for l in c['levels']], 8896131, 2)
    fo.set_cr_log(False)
    p_dm = fo.CambPower(bbks, COSMO, column=1)
    vs = fo.velocity_to_offset_ratio(COSMO)
    flagged = fo.flag_cells(L, len(c['levels']) - 1, c['centre'], *c['select'])

    def covector(name):
        if name == 'potential':
            loc = fo.localisation_covector(L, flagged, 'overdensity')
            return fo.multilevel_covector(L, loc, p_dm, None, potential_cosmo=COSMO)
        d = {'Lx': 0, 'Ly': 1, 'Lz': 2}[name]
        return fo.multilevel_covector(L, fo.localisation_covector_am(L, flagged, d), p_dm, vs)

    values = {name: fo.inner(covector(name), w) for name in c['calc']}
    covs, targets = [], []
    for name, kind, t in c['mods']:
        cv = covector(name)
        t32 = float(np.float32(t))
        targets.append(t32 * fo.inner(cv, w) if kind == 'relative' else t32)
        covs.append(cv)
    before = fo.chi2_levels(L, w)
    w2 = fo.apply_linear_modifications(L, w, covs, targets)
    after = fo.chi2_levels(L, w2)
    return dict(levels=L, noise=w, modified=w2, values=values, chi2=(before, after), flagged=flagged)


@pytest.mark.parametrize('case', sorted(MOD_MORE_CASES))
def test_potential_and_angular_momentum_oracle(bbks, case):
    from conftest import COSMO
    g = _load_golden('%s.npz' % case)
    r = oracle_mod_more(bbks, case)
    for name, v in r['values'].items():
        assert '%.6g' % v == '%.6g' % float(g[name]), name
    assert '%.6g' % (r['chi2'][1] - r['chi2'][0]) == '%.6g' % float(g['delta_chi2'])
    levels = MOD_MORE_CASES[case]['levels']
    out = fo.zoom_realisation(r['modified'], levels, fo.CambPower(bbks, COSMO))
    for l in range(len(levels)):
        ref = g['delta%d' % l]
        assert np.abs(out[l][0] - ref).max() <= 1e-11 * np.abs(ref).max(), l


# --- splicing -----------------------------------------------------------------------------

SPLICE_CASES = {
    'splice1': dict(levels=[(50.0, 32, (0.0, 0.0, 0.0))], select=('sphere', 8)),
    'splice2': dict(levels=[(50.0, 32, (0.0, 0.0, 0.0)), (25.0, 32, (12.5, 12.5, 12.5))], select=('sphere', 5)),
}


def oracle_splice(bbks, case, cr_log=False):
    from conftest import COSMO
    c = SPLICE_CASES[case]
    L = fo.Levels(c['levels'])
    fo.set_cr_log(cr_log)
    w = fo.white_noise_levels([l[1] for l in c['levels']], 8896131, 2)
    wn = fo.white_noise_levels([l[1] for l in c['levels']], 8896132, 0)
    fo.set_cr_log(False)
    fl = [fo.flag_cells(L, l, (25., 25., 25.), *c['select']) for l in range(len(c['levels']))]
    out, its = fo.splice_levels(L.levels, w, wn, fo.CambPower(bbks, COSMO), fl)
    return out, its


@needs_reference_tests
def test_splice_oracle_matches_reference_fixture():
    """test_24_splicing: real-space seed, 16^3, select_sphere 10, splice 8896132."""
    power = fo.CambPower(_ref_camb(), REF_COSMO)
    L = fo.Levels([(50.0, 16, (0, 0, 0))])
    fo.set_cr_log(False)
    w = fo.white_noise_levels([16], 8896131, 0)
    wn = fo.white_noise_levels([16], 8896132, 0)
    fl = [fo.flag_cells(L, 0, (25., 25., 25.), 'sphere', 10)]
    s, its = fo.splice_levels(L.levels, w, wn, power, fl)
    assert its == [16]
    out = fo.zoom_realisation(s, L.levels, power)
    ref = np.load(os.path.join(REF_TESTS, 'test_24_splicing', 'reference_grid', 'grid-0.npy'))
    assert np.abs(out[0][0] - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize('case', sorted(SPLICE_CASES))
def test_splice_oracle_matches_goldens(bbks, case):
    from conftest import COSMO
    g = _load_golden('%s.npz' % case)
    out, its = oracle_splice(bbks, case)
    assert its == list(g['iterations'])
    levels = SPLICE_CASES[case]['levels']
    fields = fo.zoom_realisation(out, levels, fo.CambPower(bbks, COSMO))
    for l in range(len(levels)):
        ref = g['delta%d' % l]
        assert np.abs(fields[l][0] - ref).max() <= 1e-12 * np.abs(ref).max(), l


# --- the headline's geometry: zoom factors 4 and 3 (tests/golden/geom_*.npz) ---------------

GEOM_LEVELS = {
    'zoom4': [(50.0, 32, (0.0, 0.0, 0.0)), (12.5, 32, (18.75, 18.75, 18.75))],
    # factor 3 over 10 2/3 coarse cells (genetIC's test_01c geometry at 32^3)
    'zoom3f': [(50.0, 32, (0.0, 0.0, 0.0)), (50.0 / 3, 32, (17.1875, 17.1875, 17.1875))],
}


@pytest.mark.parametrize('name', ['zoom4', 'zoom3f'])
def test_geometry_oracle_matches_reference_grids(bbks, name):
    from conftest import COSMO
    g = _load_golden('geom_%s.npz' % name)
    levels = GEOM_LEVELS[name]
    fo.set_cr_log(False)
    w = fo.white_noise_levels([l[1] for l in levels], 8896131, 2)
    out = fo.zoom_realisation(w, levels, fo.CambPower(bbks, COSMO))
    for l in range(len(levels)):
        ref = g['delta%d' % l]
        assert np.abs(out[l][0] - ref).max() <= 1e-12 * np.abs(ref).max(), l


@pytest.mark.parametrize('case', ['mod4', 'mod3'])
def test_geometry_modification_oracle_matches_reference(bbks, case):
    from conftest import COSMO
    g = _load_golden('geom_%s.npz' % case)
    r = oracle_modified(bbks, case)
    for name in ('overdensity', 'vx', 'vy', 'vz'):
        assert '%.6g' % r['values'][name] == '%.6g' % float(g[name]), name
    assert '%.6g' % (r['chi2'][1] - r['chi2'][0]) == '%.6g' % float(g['delta_chi2'])
    levels = MOD_CASES[case]['levels']
    out = fo.zoom_realisation(r['modified'], levels, fo.CambPower(bbks, COSMO))
    for l in range(len(levels)):
        ref = g['delta%d' % l]
        assert np.abs(out[l][0] - ref).max() <= 1e-11 * np.abs(ref).max(), l


# The batch workload's zoom class at 64^3 (tests/golden/geom_ratio2.npz): a zoom of a quarter of
# a 100 Mpc/h base's side (zoom factor 4) with 32 cells, half the base's cell size, and two
# overdensity modifications on different spheres
RATIO2_LEVELS = [(100.0, 64, (0.0, 0.0, 0.0)), (25.0, 32, (37.5, 37.5, 37.5))]
RATIO2_MODS = [((50.0, 50.0, 50.0), 1.5, 1.0), ((55.0, 50.0, 50.0), 3.0, -0.5)]


def oracle_ratio2(bbks, cr_log=False):
    from conftest import COSMO
    L = fo.Levels(RATIO2_LEVELS)
    fo.set_cr_log(cr_log)
    w = fo.white_noise_levels([64, 32], 8896131, 2)
    fo.set_cr_log(False)
    p_dm = fo.CambPower(bbks, COSMO, column=1)
    covs, values = [], []
    for centre, radius, _ in RATIO2_MODS:
        flagged = fo.flag_cells(L, 1, centre, 'sphere', radius)
        cv = fo.multilevel_covector(L, fo.localisation_covector(L, flagged, 'overdensity', 0), p_dm, None)
        values.append(fo.inner(cv, w))
        covs.append(cv)
    before = fo.chi2_levels(L, w)
    w2 = fo.apply_linear_modifications(L, w, covs, [t for _, _, t in RATIO2_MODS])
    return dict(values=values, chi2=(before, fo.chi2_levels(L, w2)), modified=w2)


def test_ratio2_zoom_oracle_matches_reference(bbks):
    from conftest import COSMO
    g = _load_golden('geom_ratio2.npz')
    r = oracle_ratio2(bbks)
    assert ['%.6g' % v for v in r['values']] == ['%.6g' % v for v in g['overdensity']]
    assert '%.6g' % (r['chi2'][1] - r['chi2'][0]) == '%.6g' % float(g['delta_chi2'])
    out = fo.zoom_realisation(r['modified'], RATIO2_LEVELS, fo.CambPower(bbks, COSMO))
    for l in range(2):
        ref = g['delta%d' % l]
        assert np.abs(out[l][0] - ref).max() <= 1e-11 * np.abs(ref).max(), l


def test_geometry_variance_oracle_matches_reference(bbks):
    from conftest import COSMO
    g = _load_golden('geom_var4.npz')
    r = oracle_variance(bbks, 'var4')
    assert '%.6g' % r['variance'] == '%.6g' % float(g['variance'])
    assert '%.6g' % r['overdensity'] == '%.6g' % float(g['overdensity'])
    assert r['steps'] == int(g['steps'])
    assert '%.6g' % (r['chi2'][1] - r['chi2'][0]) == '%.6g' % float(g['delta_chi2'])
    out = fo.zoom_realisation(r['modified'], VAR_CASES['var4']['levels'], fo.CambPower(bbks, COSMO))
    for l in range(2):
        ref = g['delta%d' % l]
        assert np.abs(out[l][0] - ref).max() <= 1e-11 * np.abs(ref).max(), l


# --- grafic output (io/grafic.hpp) -----------------------------------------------------

@needs_reference
def test_reference_build_reproduces_test_12_grafic(tmp_path):
    """genetIC's own grafic fixture (test_12_grafic: subsampled base, intermediate and zoom
    grids): the reference build here writes every file byte for byte."""
    dst, _ = _run_reference(tmp_path, 'test_12_grafic')
    ref = os.path.join(REF_TESTS, 'test_12_grafic', 'reference_grafic')
    for d in sorted(os.listdir(ref)):
        for f in sorted(os.listdir(os.path.join(ref, d))):
            assert open(os.path.join(dst, d, f), 'rb').read() == open(os.path.join(ref, d, f), 'rb').read(), (d, f)


# the grafic stack of tests/golden/grafic_zoom.npz (make_golden.py GRAFIC): effective resolution,
# level, factor, CenteredGrid roll, first id
GRAFIC_GRIDS = [(8, 0, -2, (0, 0, 0), 0), (16, 0, 1, (-1, 1, 0), 512), (32, 1, -2, (0, 0, 0), 4608),
                (64, 1, 1, (0, 0, 0), 5120)]


def grafic_oracle(bbks, cr_log=False):
    from conftest import COSMO
    g = _load_golden('grafic_zoom.npz')
    o = [int(v) for v in g['origin']]
    levels = [(50.0, 16, (0., 0., 0.)), (12.5, 16, tuple(o[a] * 50.0 / 16 for a in range(3)))]
    fo.set_cr_log(cr_log)
    w = fo.white_noise_levels([16, 16], 8896131, 2)
    fo.set_cr_log(False)
    fields = fo.zoom_realisation(w, levels, fo.CambPower(bbks, COSMO))
    ratio = fo.velocity_to_offset_ratio(COSMO)
    vf = np.sqrt(1.0 / (1.0 + COSMO['redshift']))
    out = {}
    for eff, l, fac, roll, off in GRAFIC_GRIDS:
        box, n, offs = levels[l]
        out[eff] = fo.grafic_slabs(fields[l], box, n, offs, 50.0, fac, roll, ratio, vf, 1.0, off)
    return g, out


def test_grafic_oracle_matches_reference_files(bbks):
    """The writer's restatement (grafic_slabs) against the reference build's grafic files: the
    centred and subsampled base grids, the intermediate and the zoom grid, every velocity,
    displacement and overdensity record and every id, exactly."""
    g, out = grafic_oracle(bbks)
    for eff, (vel, pos, dl, ids) in out.items():
        for k, arr in zip(('velcx', 'velcy', 'velcz', 'poscx', 'poscy', 'poscz', 'deltab'), vel + pos + [dl]):
            assert np.array_equal(arr, g['g%d_ic_%s' % (eff, k)]), (eff, k)
        assert np.array_equal(ids, g['g%d_ic_particle_ids' % eff]), eff
