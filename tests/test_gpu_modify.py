"""Linear modifications on the GPU against the oracle and the reference's logged values."""
import os

import numpy as np
import pytest

import field_oracle as fo
from conftest import COSMO, make_generator
from test_oracle import MOD_CASES, oracle_modified

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')

LEVELS = {'mod1': [('base', 50.0, 32)], 'mod2': [('base', 50.0, 32), ('zoom', 8, 8, 8, 2, 32)]}


def _gpu(precision, bbks, case):
    c = MOD_CASES[case]
    gen = make_generator(precision, bbks, LEVELS[case], 8896131, 'random_seed')
    gen.centre(25, 25, 25)
    gen.select_sphere(c['radius'])
    values = {name: gen.calculate(name) for name, _, _ in c['mods']}
    for name, _, t in c['mods']:
        gen.modify(name, 'absolute', t)
    chi2 = gen.apply_modifications()
    noise = [gen.noise(l) for l in range(len(c['levels']))]
    gen.done(apply_modifications=False)
    delta = [gen.field(l, 'delta') for l in range(len(c['levels']))]
    flagged = gen.flagged.copy()
    gen.close()
    return dict(values=values, chi2=chi2, noise=noise, delta=delta, flagged=flagged)


@pytest.mark.parametrize('case', ['mod1', 'mod2'])
def test_modifications_fp64_match_oracle(built, bbks, case):
    got = _gpu('fp64', bbks, case)
    want = oracle_modified(bbks, case, cr_log=True)
    assert np.array_equal(np.sort(got['flagged']), np.sort(want['flagged']))
    for k, v in want['values'].items():
        assert abs(got['values'][k] - v) <= 1e-10 * max(abs(v), 1e-3), k
    assert abs(got['chi2'][0] / want['chi2'][0] - 1) < 1e-11
    assert abs((got['chi2'][1] - got['chi2'][0]) - (want['chi2'][1] - want['chi2'][0])) < 1e-7 * abs(
        want['chi2'][1] - want['chi2'][0]) + 1e-9
    for l, w2 in enumerate(want['modified']):
        assert np.abs(got['noise'][l] - w2).max() < 1e-10 * np.abs(w2).max()
    g = np.load(os.path.join(GOLDEN, '%s.npz' % case))
    assert '%.6g' % got['values']['overdensity'] == '%.6g' % float(g['overdensity'])
    assert '%.6g' % (got['chi2'][1] - got['chi2'][0]) == '%.6g' % float(g['delta_chi2'])
    for l in range(len(MOD_CASES[case]['levels'])):
        ref = g['delta%d' % l].astype(np.float64)
        assert np.abs(got['delta'][l] - ref).max() <= 2e-7 * np.abs(ref).max()


def test_modifications_mixed_within_stated_error(built, bbks):
    got = _gpu('mixed', bbks, 'mod2')
    want = oracle_modified(bbks, 'mod2', cr_log=True)
    for l, w2 in enumerate(want['modified']):
        assert np.abs(got['noise'][l] - w2).max() < 1e-5 * np.abs(w2).max()
    assert abs(got['chi2'][1] / want['chi2'][1] - 1) < 1e-5
