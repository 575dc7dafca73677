"""Batches of realisations (gic_batch_*): the worker threads, the per-context
streams and the captured graph give the same bits as realising each context on
its own through the plain entry points."""
import numpy as np
import pytest

from conftest import make_generator

pytestmark = pytest.mark.gpu

SPECS = [
    ([('base', 50.0, 32)], None),
    ([('base', 75.0, 48)], None),
    ([('base', 50.0, 32)], None),
    ([('base', 50.0, 32), ('zoom', 8, 8, 8, 2, 32)], [((25.0, 25.0, 25.0), 3.0, 0.05)]),
    ([('base', 100.0, 64), ('zoom', 24, 24, 24, 4, 32)], [((50.0, 50.0, 50.0), 1.5, 1.0), ((52.0, 50.0, 50.0), 2.0, -0.5)]),
]


def _make(bbks, spec, precision):
    levels, mods = spec
    g = make_generator(precision, bbks, levels, 1, 'random_seed')
    for centre, radius, target in (mods or []):
        g.centre(*centre)
        g.select_sphere(radius)
        g.modify('overdensity', 'absolute', target)
    return g


def _individual(bbks, spec, precision, seed, order):
    g = _make(bbks, spec, precision)
    g._call('gic_draw_noise', seed, 2)
    if spec[1]:
        g.apply_modifications()
    g._call('gic_zeldovich', order)
    out = [(g.field(l, 'delta'), g.particles(l)) for l in range(len(spec[0]))]
    g.close()
    return out


def _collect(g, nl):
    return [(g.field(l, 'delta'), g.particles(l)) for l in range(nl)]


@pytest.mark.parametrize('precision,order', [('mixed', 1), ('fp64', 1), ('mixed', 2)])
def test_batch_matches_individual_realisations(built, bbks, precision, order):
    from genetic_gb300.batch import Batch
    gens = [_make(bbks, s, precision) for s in SPECS]
    with Batch(gens) as b:
        for seeds in ([11, 12, 13, 14, 15], [21, 22, 23, 24, 25]):  # capture, then replay with new noise
            b.realise(seeds, order=order, threads=3)
            for g, spec, seed in zip(gens, SPECS, seeds):
                got = _collect(g, len(spec[0]))
                want = _individual(bbks, spec, precision, seed, order)
                for (d, (p, v)), (d2, (p2, v2)) in zip(got, want):
                    assert np.array_equal(d, d2), (seed, 'delta')
                    assert np.array_equal(p, p2), (seed, 'pos')
                    assert np.array_equal(v, v2), (seed, 'vel')
    for g in gens:
        g.close()


def test_batch_rejects_duplicate_contexts(built, bbks):
    import genetic_gb300 as gg
    from genetic_gb300.batch import Batch
    g = _make(bbks, SPECS[0], 'mixed')
    with pytest.raises(gg.GicError):
        Batch([g, g])
    g.close()
