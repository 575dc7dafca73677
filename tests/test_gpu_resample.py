"""genetIC's supersample / subsample on the GPU (gic_fetch_particles_resampled): the
particles of a level on a virtual grid over its region, against the oracle (FP64 1e-10,
mixed 1e-5), and packed in genetIC's mapper order against the reference build's own
tipsy files (tests/golden/resample_*.npz, to one float rounding step)."""
import os

import numpy as np
import pytest

import field_oracle as fo
from conftest import COSMO, make_generator
from test_writers import GOLDEN, ORIGIN, RESAMPLE, make_map, pack_host, resampled_oracle

pytestmark = pytest.mark.gpu

GPU_LEVELS = {
    'super1': [('base', 50.0, 16)],
    'sub1': [('base', 50.0, 32)],
    'superzoom': [('base', 50.0, 32), ('zoom', 8, 8, 8, 2, 32)],
}


def _gpu(precision, bbks, name):
    levels, lev, factor, _ = RESAMPLE[name]
    gen = make_generator(precision, bbks, GPU_LEVELS[name], 8896131, 'random_seed')
    gen.done()
    out = [gen.particles_resampled(l, factor) if l == lev else gen.particles(l) for l in range(len(levels))]
    gen.close()
    return [p for p, _ in out], [v for _, v in out]


@pytest.mark.parametrize('name', sorted(RESAMPLE))
@pytest.mark.parametrize('precision,tol', [('fp64', 1e-10), ('mixed', 1e-5)])
def test_resampled_particles_match_oracle(built, bbks, name, precision, tol):
    fo.set_cr_log(True)
    want = resampled_oracle(bbks, name)
    fo.set_cr_log(False)
    pos, vel = _gpu(precision, bbks, name)
    periodic = RESAMPLE[name][0][0][0]
    for l in range(len(pos)):
        d = (pos[l] - want['pos'][l] + periodic / 2) % periodic - periodic / 2
        scale = np.abs(want['vel'][l]).max() / fo.velocity_to_offset_ratio(COSMO)
        assert np.abs(d).max() <= tol * scale, (l, np.abs(d).max() / scale)
        assert np.abs(vel[l] - want['vel'][l]).max() <= tol * np.abs(want['vel'][l]).max(), l


@pytest.mark.parametrize('name', sorted(RESAMPLE))
def test_resampled_tipsy_records_match_reference_file(built, bbks, name):
    """The device's resampled particles, packed by the host packer in genetIC's mapper
    order with the virtual grids' masses and softenings, against genetIC's own file."""
    from genetic_gb300 import _lib
    g = np.load(os.path.join(GOLDEN, 'resample_%s.npz' % name))
    levels, lev, factor, sel = RESAMPLE[name]
    r = resampled_oracle(bbks, name)
    pos, vel = _gpu('fp64', bbks, name)
    nv = [int(round(len(p) ** (1 / 3))) for p in pos]
    vlevels = [(b, nv[l], off) for l, (b, _, off) in enumerate(levels)]
    replaced = (fo.flag_cells(fo.Levels(levels), 0, (25., 25., 25.), *sel) if sel else np.zeros(0, dtype=np.uint64))
    m = make_map(vlevels, replaced.astype(np.uint64), r['factors'], ratio=nv[-1] // (nv[0] // 2) if sel else 1,
                 origin=ORIGIN)
    rc, got = pack_host(_lib.load(), m, pos, vel)
    assert rc == 0 and len(got) == int(g['nrec'])
    stride = int(g['stride'])
    for mine, ref in ((got[::stride], g['every']), (got[-400:], g['tail'])):
        assert np.array_equal(mine[:, 0], ref[:, 0]) and np.array_equal(mine[:, 7:], ref[:, 7:])
        assert np.abs(mine[:, 1:4] - ref[:, 1:4]).max() <= 6e-8
        assert np.abs(mine[:, 4:7] - ref[:, 4:7]).max() <= 2e-7 * np.abs(ref[:, 4:7]).max()


def test_resample_argument_errors(built, bbks):
    import genetic_gb300 as g
    gen = make_generator('fp64', bbks, [('base', 50.0, 32)], 8896131, 'random_seed')
    gen.done()
    for factor in (1, 0, -1, -3, 128):
        with pytest.raises(g.GicError):
            gen.particles_resampled(0, factor)
    gen.close()
