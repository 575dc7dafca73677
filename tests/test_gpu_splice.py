"""Splicing on the GPU against the oracle and the reference build's goldens
(tests/golden/splice*.npz), including the CG iteration counts."""
import os

import numpy as np
import pytest

from conftest import make_generator
from test_oracle import SPLICE_CASES, oracle_splice

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), 'golden')
GEN_LEVELS = {1: [('base', 50.0, 32)], 2: [('base', 50.0, 32), ('zoom', 8, 8, 8, 2, 32)]}


def _gpu(precision, bbks, case):
    c = SPLICE_CASES[case]
    nl = len(c['levels'])
    gen = make_generator(precision, bbks, GEN_LEVELS[nl], 8896131, 'random_seed')
    gen.centre(25, 25, 25)
    getattr(gen, 'select_' + c['select'][0])(c['select'][1])
    its = gen.splice(8896132)
    noise = [gen.noise(l) for l in range(nl)]
    gen.done()
    delta = [gen.field(l, 'delta') for l in range(nl)]
    gen.close()
    return its, noise, delta


@pytest.mark.parametrize('case', sorted(SPLICE_CASES))
def test_splice_fp64(built, bbks, case):
    its, noise, delta = _gpu('fp64', bbks, case)
    want, want_its = oracle_splice(bbks, case, cr_log=True)
    g = np.load(os.path.join(GOLDEN, '%s.npz' % case))
    assert its == want_its == list(g['iterations'])
    for l, w in enumerate(want):
        assert np.abs(noise[l] - w).max() <= 1e-10 * np.abs(w).max(), l
        ref = g['delta%d' % l]
        assert np.abs(delta[l] - ref).max() <= 1e-10 * np.abs(ref).max(), l


def test_splice_mixed_within_stated_error(built, bbks):
    """FP32 fields: the CG stops at the reference's tolerance (1e-6 of the right-hand
    side) or when it stops improving; the spliced noise stays within 1e-5."""
    its, noise, _ = _gpu('mixed', bbks, 'splice2')
    want, _ = oracle_splice(bbks, 'splice2', cr_log=True)
    errs = [float(np.abs(noise[l] - w).max() / np.abs(w).max()) for l, w in enumerate(want)]
    print('mixed splice: iterations %s, max rel err %s' % (its, errs))
    assert max(errs) < 1e-5
