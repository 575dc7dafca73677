"""Second-order LPT on the GPU against the oracle's restatement (no genetIC
counterpart; the oracle is checked against the analytic two-plane-wave solution)."""
import numpy as np
import pytest

import field_oracle as fo
from conftest import COSMO, make_generator

pytestmark = pytest.mark.gpu

CASES = {
    'single32': [(50.0, 32, (0.0, 0.0, 0.0))],
    'zoom2': [(50.0, 32, (0.0, 0.0, 0.0)), (25.0, 32, (12.5, 12.5, 12.5))],
}
GEN_LEVELS = {'single32': [('base', 50.0, 32)], 'zoom2': [('base', 50.0, 32), ('zoom', 8, 8, 8, 2, 32)]}


def _gpu(precision, bbks, case):
    gen = make_generator(precision, bbks, GEN_LEVELS[case], 8896131, 'random_seed')
    gen.done(order=2)
    nl = len(CASES[case])
    out = dict(psi2=[[gen.field(l, 'psi2_' + a) for a in 'xyz'] for l in range(nl)],
               psi=[[gen.field(l, 'psi_' + a) for a in 'xyz'] for l in range(nl)],
               particles=[gen.particles(l) for l in range(nl)])
    gen.close()
    return out


def _oracle(bbks, case):
    levels = CASES[case]
    fo.set_cr_log(True)
    w = fo.white_noise_levels([l[1] for l in levels], 8896131, 2)
    fo.set_cr_log(False)
    psi1 = [f[1:] for f in fo.zoom_realisation(w, levels, fo.CambPower(bbks, COSMO))]
    psi2 = fo.lpt2_realisation(w, levels, fo.CambPower(bbks, COSMO))
    return psi1, psi2


@pytest.mark.parametrize('case', ['single32', 'zoom2'])
def test_lpt2_fp64_matches_oracle(built, bbks, case):
    got = _gpu('fp64', bbks, case)
    psi1, psi2 = _oracle(bbks, case)
    levels = CASES[case]
    ratio = fo.velocity_to_offset_ratio(COSMO)
    for l, (box, n, off) in enumerate(levels):
        for a in range(3):
            ref = psi2[l][a]
            assert np.abs(got['psi2'][l][a] - ref).max() <= 1e-10 * np.abs(ref).max(), (l, a)
            assert np.abs(got['psi'][l][a] - psi1[l][a]).max() <= 1e-10 * np.abs(psi1[l][a]).max(), (l, a)
        pos, vel = fo.particles_lpt2(psi1[l], psi2[l], box, off, levels[0][0], ratio)
        gpos, gvel = got['particles'][l]
        d = (gpos - pos + levels[0][0] / 2) % levels[0][0] - levels[0][0] / 2
        assert np.abs(d).max() < 1e-10 * box
        assert np.abs(gvel - vel).max() <= 1e-10 * np.abs(vel).max()
    # the second-order term is a small correction to the first
    s1 = max(np.abs(p).max() for p in psi1[-1])
    s2 = max(np.abs(p).max() for p in psi2[-1])
    assert 0 < s2 < 0.2 * s1


def test_lpt2_mixed_within_stated_error(built, bbks):
    """FP32 fields: psi2 within 1e-5 of the FP64 oracle (relative to its maximum)."""
    got = _gpu('mixed', bbks, 'zoom2')
    _, psi2 = _oracle(bbks, 'zoom2')
    errs = [float(np.abs(got['psi2'][l][a] - psi2[l][a]).max() / np.abs(psi2[l][a]).max())
            for l in range(2) for a in range(3)]
    print('mixed 2LPT max rel err per field', errs)
    assert max(errs) < 1e-5
