"""Quadratic (variance) modification on the GPU against the oracle and the
reference build's goldens (tests/golden/var*.npz)."""
import os

import numpy as np
import pytest

from conftest import make_generator
from test_oracle import VAR_CASES, oracle_variance

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')

LEVELS = {'var1': [('base', 50.0, 32)], 'var2': [('base', 50.0, 32), ('zoom', 8, 8, 8, 2, 32)]}


def _gpu(precision, bbks, case):
    c = VAR_CASES[case]
    gen = make_generator(precision, bbks, LEVELS[case], 8896131, 'random_seed')
    gen.centre(25, 25, 25)
    getattr(gen, 'select_' + c['select'][0])(c['select'][1])
    gen.filtering_scale(c['scale'])
    var = gen.calculate('variance')
    od = gen.calculate('overdensity')
    gen.modify('overdensity', 'relative', 1)
    gen.modify('variance', 'relative', c['rel'])
    chi2 = gen.apply_modifications()
    final = gen.calculate('variance')
    noise = [gen.noise(l) for l in range(len(c['levels']))]
    gen.done(apply_modifications=False)
    delta = [gen.field(l, 'delta') for l in range(len(c['levels']))]
    flagged = [f.copy() for f in gen.flagged_levels]
    gen.close()
    return dict(variance=var, overdensity=od, chi2=chi2, final=final, noise=noise, delta=delta, flagged=flagged)


@pytest.fixture(scope='module')
def oracle_cases(bbks):
    return {case: oracle_variance(bbks, case, cr_log=True) for case in VAR_CASES}


@pytest.mark.parametrize('case', ['var1', 'var2'])
def test_variance_fp64_matches_oracle_and_golden(built, bbks, oracle_cases, case):
    got = _gpu('fp64', bbks, case)
    want = oracle_cases[case]
    for a, b in zip(got['flagged'], want['flagged']):
        assert np.array_equal(a, b)
    assert abs(got['variance'] / want['variance'] - 1) < 1e-10
    assert abs(got['overdensity'] - want['overdensity']) < 1e-10 * abs(want['overdensity'])
    d_got, d_want = got['chi2'][1] - got['chi2'][0], want['chi2'][1] - want['chi2'][0]
    assert abs(d_got - d_want) < 1e-7 * abs(d_want)
    assert abs(got['final'] / want['final'] - 1) < 1e-9
    for l, w2 in enumerate(want['modified']):
        assert np.abs(got['noise'][l] - w2).max() < 1e-9 * np.abs(w2).max(), l
    g = np.load(os.path.join(GOLDEN, '%s.npz' % case))
    assert '%.6g' % got['variance'] == '%.6g' % float(g['variance'])
    assert '%.6g' % d_got == '%.6g' % float(g['delta_chi2'])
    for l in range(len(VAR_CASES[case]['levels'])):
        ref = g['delta%d' % l]
        assert np.abs(got['delta'][l] - ref).max() <= 1e-9 * np.abs(ref).max(), l


@pytest.mark.parametrize('case', ['var1', 'var2'])
def test_variance_mixed_within_stated_error(built, bbks, oracle_cases, case):
    """Mixed precision (FP32 fields, FP64 scalars): the iterated solve stays within
    1e-5 of the FP64 oracle's modified noise and reaches the same target."""
    got = _gpu('mixed', bbks, case)
    want = oracle_cases[case]
    assert abs(got['variance'] / want['variance'] - 1) < 1e-5
    errs = [float(np.abs(got['noise'][l] - w2).max() / np.abs(w2).max()) for l, w2 in enumerate(want['modified'])]
    print('mixed %s: modified-noise max rel err %s, final variance %.8g vs %.8g' % (case, errs, got['final'],
                                                                                 want['final']))
    assert max(errs) < 1e-5
    assert abs(got["final"] / want["final"] - 1) < 1e-5


def test_variance_argument_errors(built, bbks):
    import genetic_gb300 as g
    gen = make_generator('fp64', bbks, LEVELS['var1'], 8896131, 'random_seed')
    gen.centre(25, 25, 25)
    gen.select_sphere(5)
    with pytest.raises(g.GicError, match='filtering_scale'):
        gen.calculate('variance')
    gen.filtering_scale(0.5)  # below the 50/32 Mpc/h cell
    with pytest.raises(g.GicError, match='smallest pixel size'):
        gen.calculate('variance')
    gen.close()
