"""Potential and angular-momentum modifications on the GPU against the oracle and the
reference build's goldens (tests/golden/mod_pot1, mod_am1, mod_am2)."""
import os

import numpy as np
import pytest

from conftest import make_generator
from test_oracle import MOD_MORE_CASES, oracle_mod_more

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
GEN_LEVELS = {1: [('base', 50.0, 32)], 2: [('base', 50.0, 32), ('zoom', 8, 8, 8, 2, 32)]}


def _gpu(precision, bbks, case):
    c = MOD_MORE_CASES[case]
    gen = make_generator(precision, bbks, GEN_LEVELS[len(c['levels'])], 8896131, 'random_seed')
    gen.centre(*c['centre'])
    kind, size = c['select']
    if kind == 'ellipse':
        gen.select_ellipse(*size)
    else:
        getattr(gen, 'select_' + kind)(size)
    values = {name: gen.calculate(name) for name in c['calc']}
    for name, how, t in c['mods']:
        gen.modify(name, how, t)
    chi2 = gen.apply_modifications()
    noise = [gen.noise(l) for l in range(len(c['levels']))]
    gen.done(apply_modifications=False)
    delta = [gen.field(l, 'delta') for l in range(len(c['levels']))]
    gen.close()
    return dict(values=values, chi2=chi2, noise=noise, delta=delta)


@pytest.mark.parametrize('case', sorted(MOD_MORE_CASES))
def test_potential_and_angular_momentum_fp64(built, bbks, case):
    got = _gpu('fp64', bbks, case)
    want = oracle_mod_more(bbks, case, cr_log=True)
    for k, v in want['values'].items():
        assert abs(got['values'][k] - v) <= 1e-10 * abs(v), k
    d_got, d_want = got['chi2'][1] - got['chi2'][0], want['chi2'][1] - want['chi2'][0]
    assert abs(d_got - d_want) <= 1e-7 * abs(d_want) + 1e-9
    for l, w2 in enumerate(want['modified']):
        assert np.abs(got['noise'][l] - w2).max() < 1e-10 * np.abs(w2).max(), l
    g = np.load(os.path.join(GOLDEN, '%s.npz' % case))
    for name in want['values']:
        assert '%.6g' % got['values'][name] == '%.6g' % float(g[name]), name
    for l in range(len(got['delta'])):
        ref = g['delta%d' % l]
        assert np.abs(got['delta'][l] - ref).max() <= 1e-10 * np.abs(ref).max(), l


def test_angular_momentum_mixed(built, bbks):
    got = _gpu('mixed', bbks, 'mod_am2')
    want = oracle_mod_more(bbks, 'mod_am2', cr_log=True)
    for l, w2 in enumerate(want['modified']):
        assert np.abs(got['noise'][l] - w2).max() < 1e-5 * np.abs(w2).max(), l
