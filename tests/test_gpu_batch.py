"""Batches of realisations (gic_batch_*): the captured graph (noise, modifications,
fields and particles of every context), the per-context streams and the worker
threads give the same bits as realising each context on its own through the plain
entry points; one zoom of the 64-realisation batch workload, realised by the graph,
against the FP64 oracle."""
import json

import numpy as np
import pytest

import field_oracle as fo
from conftest import COSMO, make_generator

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


def _check_same(gens, specs, bbks, precision, seeds, order):
    for g, spec, seed in zip(gens, specs, seeds):
        got = _collect(g, len(spec[0]))
        want = _individual(bbks, spec, precision, seed, order)
        for (d, (p, v)), (d2, (p2, v2)) in zip(got, want):
            assert np.array_equal(d, d2), (seed, 'delta')
            assert np.array_equal(p, p2), (seed, 'pos')
            assert np.array_equal(v, v2), (seed, 'vel')


@pytest.mark.parametrize('precision,order', [('mixed', 1), ('fp64', 1), ('mixed', 2)])
def test_batch_matches_individual_realisations(built, bbks, precision, order):
    from genetic_gb300.batch import Batch
    gens = [_make(bbks, s, precision) for s in SPECS]
    with Batch(gens) as b:
        # capture, then replay twice with new noise
        for k, seeds in enumerate(([11, 12, 13, 14, 15], [21, 22, 23, 24, 25], [31, 32, 33, 34, 35])):
            b.realise(seeds, order=order, threads=3)
            contexts, kernels, replays, off = b.graph_info()
            assert off == '' and contexts == len(SPECS) and kernels > 0 and replays == k, b.graph_info()
            _check_same(gens, SPECS, bbks, precision, seeds, order)
    for g in gens:
        g.close()


def test_batch_recaptures_when_a_target_changes(built, bbks):
    """The graph holds the modification targets: changing one captures again."""
    from genetic_gb300.batch import Batch
    gens = [_make(bbks, s, 'mixed') for s in SPECS]
    with Batch(gens) as b:
        b.realise([1, 2, 3, 4, 5])
        b.realise([6, 7, 8, 9, 10])
        assert b.graph_info()[2] == 1
        specs = list(SPECS)
        specs[3] = (SPECS[3][0], [((25.0, 25.0, 25.0), 3.0, 0.2)])
        gens[3].clear_modifications()
        gens[3].centre(25.0, 25.0, 25.0)
        gens[3].select_sphere(3.0)
        gens[3].modify('overdensity', 'absolute', 0.2)
        b.realise([11, 12, 13, 14, 15])
        assert b.graph_info()[2] == 0  # captured again
        b.realise([16, 17, 18, 19, 20])
        assert b.graph_info()[2] == 1
        _check_same(gens, specs, bbks, 'mixed', [16, 17, 18, 19, 20], 1)
    for g in gens:
        g.close()


def test_batch_realises_variance_modifications_beside_the_graph(built, bbks):
    """A context with a quadratic modification (its iteration count is a host
    decision) is realised eagerly beside the graph, with the same bits."""
    from genetic_gb300.batch import Batch
    gens = [_make(bbks, s, 'mixed') for s in SPECS[:3]]
    q = make_generator('mixed', bbks, [('base', 50.0, 32)], 1, 'random_seed')
    q.centre(25.0, 25.0, 25.0)
    q.select_sphere(8.0)
    q.filtering_scale(3.0)
    q.modify('variance', 'relative', 1.3)
    with Batch(gens + [q]) as b:
        for seeds in ([1, 2, 3, 4], [5, 6, 7, 8]):
            b.realise(seeds)
            assert b.graph_info()[0] == 3
            _check_same(gens, SPECS[:3], bbks, 'mixed', seeds[:3], 1)
            ref = make_generator('mixed', bbks, [('base', 50.0, 32)], 1, 'random_seed')
            ref.centre(25.0, 25.0, 25.0)
            ref.select_sphere(8.0)
            ref.filtering_scale(3.0)
            ref.modify('variance', 'relative', 1.3)
            ref._call('gic_draw_noise', seeds[3], 2)
            ref.apply_modifications()
            ref._call('gic_zeldovich', 1)
            assert np.array_equal(q.field(0, 'delta'), ref.field(0, 'delta'))
            assert np.array_equal(q.particles(0)[0], ref.particles(0)[0])
            ref.close()
    for g in gens + [q]:
        g.close()


# one two-level zoom of the 64-realisation batch workload: a 256^3 base (100 Mpc/h) plus a
# 128^3 zoom of side 25 Mpc/h centred at (50, 50, 50) (genetIC zoom factor 4: a quarter of the
# base side, cells half the base cells), overdensity +1.0 in a
# 1.5 Mpc/h sphere at the centre and -0.5 in a 3 Mpc/h sphere 5 Mpc/h along x
ZOOM64 = ([('base', 100.0, 256), ('zoom', 96, 96, 96, 4, 128)],
          [((50.0, 50.0, 50.0), 1.5, 1.0), ((55.0, 50.0, 50.0), 3.0, -0.5)])
ZOOM64_LEVELS = [(100.0, 256, (0.0, 0.0, 0.0)), (25.0, 128, (37.5, 37.5, 37.5))]
ZOOM64_SEED = 8896131


def _zoom64_oracle(bbks):
    import os
    fo.set_fft_workers(os.cpu_count())
    L = fo.Levels(ZOOM64_LEVELS)
    fo.set_cr_log(True)
    w = fo.white_noise_levels([256, 128], ZOOM64_SEED, 2)
    fo.set_cr_log(False)
    p_dm = fo.CambPower(bbks, COSMO, column=1)
    covs = []
    for centre, radius, _ in ZOOM64[1]:
        flagged = fo.flag_cells(L, 1, centre, 'sphere', radius)
        covs.append(fo.multilevel_covector(L, fo.localisation_covector(L, flagged, 'overdensity', 0), p_dm, None))
    w2 = fo.apply_linear_modifications(L, w, covs, [float(np.float32(t)) for _, _, t in ZOOM64[1]])
    fields = fo.zoom_realisation(w2, ZOOM64_LEVELS, fo.CambPower(bbks, COSMO))
    ratio = fo.velocity_to_offset_ratio(COSMO)
    parts = [fo.particles(f[1:], box, off, 100.0, ratio) for (box, _, off), f in zip(ZOOM64_LEVELS, fields)]
    fo.set_fft_workers(None)
    return fields, parts


def test_batch_zoom_of_the_64_realisation_workload_matches_oracle(built, bbks):
    """The zoom, realised by a replay of the batch graph beside two single-level boxes,
    against the FP64 oracle: per field the max relative error |a - b| / max|b| within
    1e-5 (the mixed form's bound)."""
    from genetic_gb300.batch import Batch
    fields, parts = _zoom64_oracle(bbks)
    gens = [_make(bbks, SPECS[0], 'mixed'), _make(bbks, ZOOM64, 'mixed'), _make(bbks, SPECS[1], 'mixed')]
    with Batch(gens) as b:
        b.realise([1, 2, 3])
        b.realise([4, ZOOM64_SEED, 5])
        assert b.graph_info()[:3:2] == (3, 1), b.graph_info()
    g = gens[1]
    err = {}
    for lev in range(2):
        for i, f in enumerate(('delta', 'psi_x', 'psi_y', 'psi_z')):
            a, want = g.field(lev, f), fields[lev][i]
            err['L%d.%s' % (lev, f)] = float(np.abs(a - want).max() / np.abs(want).max())
        pos, vel = g.particles(lev)
        err['L%d.velocity' % lev] = float(np.abs(vel - parts[lev][1]).max() / np.abs(parts[lev][1]).max())
        d = (pos - parts[lev][0] + 50.0) % 100.0 - 50.0
        err['L%d.displacement' % lev] = float(np.abs(d).max() / np.abs(fields[lev][1]).max())
    print('batch zoom (256^3 + 128^3, 2 modifications) vs FP64 oracle:', json.dumps(err))
    for key, e in err.items():
        assert e < 1e-5, (key, e)
    for g in gens:
        g.close()


def test_batch_rejects_duplicate_contexts(built, bbks):
    import genetic_gb300 as gg
    from genetic_gb300.batch import Batch
    g = _make(bbks, SPECS[0], 'mixed')
    with pytest.raises(gg.GicError):
        Batch([g, g])
    g.close()
