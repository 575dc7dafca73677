"""reverse, reverse_small_k and fix_power on the GPU against the oracle and the
reference build's grids (tests/golden/ops_*.npz)."""
import os

import numpy as np
import pytest

from conftest import make_generator
from test_oracle import OPS_CASES, oracle_noise_op

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
GEN_LEVELS = {1: [('base', 50.0, 32)], 2: [('base', 50.0, 32), ('zoom', 8, 8, 8, 2, 32)]}


def _gpu(precision, bbks, case):
    op, param, nlev = OPS_CASES[case]
    gen = make_generator(precision, bbks, GEN_LEVELS[nlev], 8896131, 'random_seed')
    if op == 'fix_power':
        gen.fix_power()
    elif op == 'reverse':
        gen.reverse()
    else:
        gen.reverse_small_k(param)
    gen.done()
    out = dict(noise=[gen.noise(l) for l in range(nlev)], delta=[gen.field(l, 'delta') for l in range(nlev)])
    gen.close()
    return out


@pytest.mark.parametrize('case', sorted(OPS_CASES))
def test_noise_ops_fp64(built, bbks, case):
    got = _gpu('fp64', bbks, case)
    _, w = oracle_noise_op(case, cr_log=True)
    g = np.load(os.path.join(GOLDEN, '%s.npz' % case))
    for l in range(len(w)):
        assert np.abs(got['noise'][l] - w[l]).max() <= 1e-15 * max(1.0, np.abs(w[l]).max()), l
        ref = g['delta%d' % l]
        assert np.abs(got['delta'][l] - ref).max() <= 1e-12 * np.abs(ref).max(), l


def test_noise_ops_mixed(built, bbks):
    got = _gpu('mixed', bbks, 'ops_fix_power_zoom')
    g = np.load(os.path.join(GOLDEN, 'ops_fix_power_zoom.npz'))
    for l in range(2):
        ref = g['delta%d' % l]
        assert np.abs(got['delta'][l] - ref).max() <= 1e-5 * np.abs(ref).max(), l
