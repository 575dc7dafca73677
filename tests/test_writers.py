"""Tipsy records in genetIC's particle-mapper order (CPU): the oracle against the
reference's own tipsy file, and the C ABI's host packer against the oracle."""
import ctypes
import os

import numpy as np
import pytest

import field_oracle as fo

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, 'tests', 'golden')

# the reference run of tests/golden/make_golden.py:tipsy_goldens (the zoom2 case)
ZOOM2 = [(50.0, 32, (0.0, 0.0, 0.0)), (25.0, 32, (12.5, 12.5, 12.5))]
ORIGIN = (8, 8, 8)


def make_map(levels, replaced, factors, ratio=2, origin=ORIGIN):
    """A map of one level, or of two with `replaced` level-0 cells."""
    from genetic_gb300._lib import GicParticleMap
    lv = [(n, ratio if l else 1, origin if l else (0, 0, 0)) for l, (_, n, _) in enumerate(levels)]
    return GicParticleMap.of(lv, [replaced], *factors)


def pack_host(lib, m, pos, vel, first=0, count=None, threads=4):
    total = ctypes.c_ulonglong()
    assert lib.gic_tipsy_count(ctypes.byref(m), ctypes.byref(total)) == 0
    if count is None:
        count = total.value - first
    out = np.zeros((count, 9), dtype=np.float32)
    P = ctypes.POINTER(ctypes.c_double)
    pp = (P * len(pos))(*[np.ascontiguousarray(p).ctypes.data_as(P) for p in pos])
    vv = (P * len(vel))(*[np.ascontiguousarray(v).ctypes.data_as(P) for v in vel])
    rc = lib.gic_tipsy_pack_host(ctypes.byref(m), pp, vv, first, count, out.ctypes.data_as(ctypes.c_void_p), threads)
    return rc, out


@pytest.fixture(scope='module')
def zoom2_particles(bbks):
    from conftest import COSMO
    w = fo.white_noise_levels([l[1] for l in ZOOM2], 8896131, 2)
    out = fo.zoom_realisation(w, ZOOM2, fo.CambPower(bbks, COSMO))
    ratio = fo.velocity_to_offset_ratio(COSMO)
    pv = [fo.particles(out[l][1:4], b, off, ZOOM2[0][0], ratio) for l, (b, n, off) in enumerate(ZOOM2)]
    replaced = fo.flag_cells(fo.Levels(ZOOM2), 0, (25., 25., 25.), 'cube', 10)
    order = fo.mapper_order(32, replaced, 32, 2, ORIGIN)
    factors = fo.tipsy_factors(ZOOM2, COSMO, order[0])
    return dict(pos=[p for p, _ in pv], vel=[v for _, v in pv], replaced=replaced, order=order, factors=factors)


def test_oracle_tipsy_matches_reference_file(zoom2_particles):
    g = np.load(os.path.join(GOLDEN, 'tipsy_zoom2.npz'))
    z = zoom2_particles
    ref = g['dark']
    assert int(g['header'][0]) == len(z['order'][1]) == len(ref)
    got = fo.tipsy_records(z['order'], z['pos'], z['vel'], *z['factors'])
    # mass and softening follow from the geometry and the summed masses: exact
    assert np.array_equal(got[:, 0], ref[:, 0]) and np.array_equal(got[:, 7:], ref[:, 7:])
    # positions (box units, |x| <= 0.5) and velocities: the oracle's doubles agree with the
    # reference build's to ~1e-12, so the floats agree to one rounding step
    assert np.abs(got[:, 1:4] - ref[:, 1:4]).max() <= 6e-8
    assert np.abs(got[:, 4:7] - ref[:, 4:7]).max() <= 2e-7 * np.abs(ref[:, 4:7]).max()


def test_host_packer_matches_oracle_bit_for_bit(built, zoom2_particles):
    from genetic_gb300 import _lib
    lib = _lib.load()
    z = zoom2_particles
    m = make_map(ZOOM2, z['replaced'], z['factors'])
    want = fo.tipsy_records(z['order'], z['pos'], z['vel'], *z['factors'])
    rc, got = pack_host(lib, m, z['pos'], z['vel'])
    assert rc == 0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # a window straddling the two levels, and a single thread
    n_kept = 32 ** 3 - len(z['replaced'])
    rc, part = pack_host(lib, m, z['pos'], z['vel'], first=n_kept - 100, count=900, threads=1)
    assert rc == 0 and np.array_equal(part.view(np.uint32), want[n_kept - 100:n_kept + 800].view(np.uint32))


def test_mapper_order_one_level_and_wrapped_origin(built):
    """Cell ids carried through the positions: the packer's order is the oracle's."""
    from genetic_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(5)
    # one level: every cell in order
    n = 8
    pos = [np.repeat(np.arange(n ** 3, dtype=np.float64)[:, None], 3, 1)]
    vel = [np.zeros((n ** 3, 3))]
    m = make_map([(1.0, n, (0, 0, 0))], [], ([1.0], [0.0], 1.0, 1.0, 1.0))
    rc, got = pack_host(lib, m, pos, vel)
    assert rc == 0 and np.array_equal(got[:, 1], np.arange(n ** 3, dtype=np.float32) - 0.5)
    # two levels, ratio 4, zoom origin near the top corner so blocks wrap around the box
    n0, r, n1, org = 8, 4, 16, (6, 6, 7)
    coords = [(x, y, z) for x in (6, 7, 0, 1) for y in (6, 7, 0, 1) for z in (7, 0, 1, 2)]
    cells = np.array(sorted(rng.choice([(x * n0 + y) * n0 + z for x, y, z in coords], 20, replace=False)))
    pos = [np.repeat(np.arange(n0 ** 3, dtype=np.float64)[:, None], 3, 1),
           np.repeat(1000. + np.arange(n1 ** 3, dtype=np.float64)[:, None], 3, 1)]
    vel = [np.zeros((n0 ** 3, 3)), np.zeros((n1 ** 3, 3))]
    m = make_map([(1.0, n0, (0, 0, 0)), (1.0, n1, (0, 0, 0))], cells, ([1.0, 1.0], [0.0, 0.0], 1.0, 1.0, 1.0),
                 ratio=r, origin=org)
    rc, got = pack_host(lib, m, pos, vel)
    lev, want = fo.mapper_order(n0, cells, n1, r, org)
    assert rc == 0
    assert np.array_equal(got[:, 1].astype(np.float64) + 0.5, want + 1000. * lev)


def test_tipsy_map_errors(built):
    from genetic_gb300 import _lib
    lib = _lib.load()
    f = ([1.0, 1.0], [0.0, 0.0], 1.0, 1.0, 1.0)
    cnt = ctypes.c_ulonglong()
    # a replaced cell outside the level-1 grid (the reference throws out_of_range)
    m = make_map([(1.0, 8, (0, 0, 0)), (1.0, 8, (0, 0, 0))], [0, 4 * 8 * 8], f, ratio=2, origin=(0, 0, 0))
    assert lib.gic_tipsy_count(ctypes.byref(m), ctypes.byref(cnt)) == _lib.GIC_ERR_INVALID_ARG
    assert b'outside high resolution grid' in lib.gic_last_error(None)
    # not ascending
    m = make_map([(1.0, 8, (0, 0, 0)), (1.0, 8, (0, 0, 0))], [5, 3], f, ratio=2, origin=(0, 0, 0))
    assert lib.gic_tipsy_count(ctypes.byref(m), ctypes.byref(cnt)) == _lib.GIC_ERR_INVALID_ARG
    # a window past the end
    m = make_map([(1.0, 4, (0, 0, 0))], [], f)
    pos = [np.zeros((64, 3))]
    rc, _ = pack_host(lib, m, pos, pos, first=60, count=5)
    assert rc == _lib.GIC_ERR_INVALID_ARG
    assert lib.gic_tipsy_count(ctypes.byref(m), ctypes.byref(cnt)) == 0 and cnt.value == 64


def test_gadget_blocks_match_reference_file_and_oracle(built, zoom2_particles):
    from genetic_gb300 import _lib
    lib = _lib.load()
    g = np.load(os.path.join(GOLDEN, 'gadget_zoom2.npz'))
    z = zoom2_particles
    n = len(z['order'][1])
    assert int(g['npart'][1]) == n
    want_pos, want_vel, want_mass = fo.gadget_blocks(z['order'], z['pos'], z['vel'], z['factors'][0])
    # the oracle against the reference's file: masses exact, positions (Mpc/h, < 50) and
    # velocities to one float rounding step
    assert np.array_equal(want_mass, g['mass'])
    assert np.abs(want_pos - g['pos']).max() <= 4e-6
    assert np.abs(want_vel - g['vel']).max() <= 1e-6 * np.abs(g['vel']).max()
    # the C ABI's host packer against the oracle, bit for bit
    m = make_map(ZOOM2, z['replaced'], z['factors'])
    pos = np.zeros((n, 3), np.float32)
    vel = np.zeros((n, 3), np.float32)
    ids = np.zeros(n, np.uint64)
    mass = np.zeros(n, np.float32)
    P = ctypes.POINTER(ctypes.c_double)
    pp = (P * 2)(*[np.ascontiguousarray(p).ctypes.data_as(P) for p in z['pos']])
    vv = (P * 2)(*[np.ascontiguousarray(v).ctypes.data_as(P) for v in z['vel']])
    ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
    assert lib.gic_gadget_pack_host(ctypes.byref(m), pp, vv, None, 0, n, ptr(pos), ptr(vel), ptr(ids), ptr(mass), 3) == 0
    assert np.array_equal(pos.view(np.uint32), want_pos.view(np.uint32))
    assert np.array_equal(vel.view(np.uint32), want_vel.view(np.uint32))
    assert np.array_equal(mass, want_mass) and np.array_equal(ids, np.arange(n, dtype=np.uint64))
    # ids alone, for a window
    ids2 = np.zeros(10, np.uint64)
    assert lib.gic_gadget_pack_host(ctypes.byref(m), None, None, None, 500, 10, None, None, ptr(ids2), None, 1) == 0
    assert np.array_equal(ids2, np.arange(500, 510, dtype=np.uint64))


ZOOM3 = ZOOM2 + [(12.5, 32, (18.75, 18.75, 18.75))]


def test_three_level_tipsy_matches_reference_and_oracle(built, bbks):
    """Nested mappers: the finest level's blocks follow the level-1 cell ids of their parents."""
    from conftest import COSMO
    from genetic_gb300 import _lib
    from genetic_gb300._lib import GicParticleMap
    lib = _lib.load()
    g = np.load(os.path.join(GOLDEN, 'tipsy_zoom3.npz'))
    w = fo.white_noise_levels([l[1] for l in ZOOM3], 8896131, 2)
    out = fo.zoom_realisation(w, ZOOM3, fo.CambPower(bbks, COSMO))
    ratio = fo.velocity_to_offset_ratio(COSMO)
    pv = [fo.particles(out[l][1:4], b, off, ZOOM3[0][0], ratio) for l, (b, n, off) in enumerate(ZOOM3)]
    levels = [(32, 1, (0, 0, 0)), (32, 2, (8, 8, 8)), (32, 2, (8, 8, 8))]
    # level 0's flagged cube, and its cells' blocks on level 1 (genetIC carries the flags down)
    rep0 = fo.flag_cells(fo.Levels(ZOOM3), 0, (25., 25., 25.), 'cube', 10)
    rep1 = np.sort(fo.block_cells(rep0, 32, 32, 2, (8, 8, 8)))
    order = fo.mapper_order_levels(levels, [rep0, rep1])
    factors = fo.tipsy_factors(ZOOM3, COSMO, order[0])
    want = fo.tipsy_records(order, [p for p, _ in pv], [v for _, v in pv], *factors)
    assert len(want) == int(g['header'][0])
    first = int(g['first'])
    ref = np.concatenate([g['head'], g['tail']])
    mine = np.concatenate([want[:len(g['head'])], want[first:]])
    assert np.array_equal(mine[:, 0], ref[:, 0]) and np.array_equal(mine[:, 7:], ref[:, 7:])
    assert np.abs(mine[:, 1:4] - ref[:, 1:4]).max() <= 6e-8
    assert np.abs(mine[:, 4:7] - ref[:, 4:7]).max() <= 2e-7 * np.abs(ref[:, 4:7]).max()
    # the host packer against the oracle, bit for bit
    m = GicParticleMap.of(levels, [rep0, rep1, []], *factors)
    cnt = ctypes.c_ulonglong()
    assert lib.gic_tipsy_count(ctypes.byref(m), ctypes.byref(cnt)) == 0 and cnt.value == len(want)
    rc, got = pack_host(lib, m, [p for p, _ in pv], [v for _, v in pv])
    assert rc == 0 and np.array_equal(got.view(np.uint32), want.view(np.uint32))
    rc, part = pack_host(lib, m, [p for p, _ in pv], [v for _, v in pv], first=first - 7, count=1000, threads=3)
    assert rc == 0 and np.array_equal(part.view(np.uint32), want[first - 7:first + 993].view(np.uint32))
    # a level-1 cell that is not under a replaced level-0 cell is refused
    bad = GicParticleMap.of(levels, [rep0, np.array([0])], *factors)
    assert lib.gic_tipsy_count(ctypes.byref(bad), ctypes.byref(cnt)) == _lib.GIC_ERR_INVALID_ARG


def test_tipsy_factors_match_oracle(built, zoom2_particles):
    """TipsyOutput's factors, the masses summed one by one in mapper order: exactly the oracle's."""
    from conftest import COSMO
    from genetic_gb300 import _lib
    lib = _lib.load()
    z = zoom2_particles
    mass, eps, pf, vf, mf = z['factors']
    m = make_map(ZOOM2, z['replaced'], (mass, eps, 0.0, 0.0, 0.0))
    got = [ctypes.c_double() for _ in range(3)]
    a = 1.0 / (1.0 + COSMO['redshift'])
    assert lib.gic_tipsy_factors(ctypes.byref(m), COSMO['omega_m'], COSMO['hubble'], a, ZOOM2[0][0],
                                 *[ctypes.byref(g) for g in got]) == 0
    assert (got[0].value, got[1].value, got[2].value) == (pf, vf, mf)


def test_file_headers_match_reference_bytes():
    """The tipsy and gadget2 headers of the zoom2 files, byte for byte (the tipsy header's
    trailing padding excepted: the reference leaves it unset)."""
    from conftest import COSMO
    from genetic_gb300 import writers
    a = 1.0 / (1.0 + COSMO['redshift'])
    t = np.load(os.path.join(GOLDEN, 'tipsy_zoom2.npz'))
    n = int(t['header'][0])
    assert writers.tipsy_header(a, n)[:28] == bytes(t['header_bytes'])
    g = np.load(os.path.join(GOLDEN, 'gadget_zoom2.npz'))
    h = writers.gadget_header(2, [0, n, 0, 0, 0, 0], [0.0] * 6, a, COSMO['redshift'], ZOOM2[0][0], COSMO['omega_m'],
                              COSMO['omega_lambda'], COSMO['hubble'])
    assert h == bytes(g['header_bytes'])
    h3 = writers.gadget_header(3, [0, n, 0, 0, 0, 0], [0.0] * 6, a, COSMO['redshift'], ZOOM2[0][0], COSMO['omega_m'],
                               COSMO['omega_lambda'], COSMO['hubble'])
    assert h3 == bytes(g['header3_bytes'])


def test_gadget_file_round_trip(tmp_path):
    from genetic_gb300 import writers
    rng = np.random.default_rng(3)
    pos, vel = rng.random((10, 3)).astype(np.float32), rng.random((10, 3)).astype(np.float32)
    ids, mass = np.arange(10, dtype=np.uint64), np.full(10, 2.5, np.float32)
    h = writers.gadget_header(3, [0, 10, 0, 0, 0, 0], [0.0] * 6, 0.01, 99.0, 50.0, 0.31, 0.69, 0.68)
    writers.write_gadget(tmp_path / 'g', h, pos, vel, ids, mass)
    rec = writers.read_fortran_records(tmp_path / 'g')
    assert rec[0] == h and len(rec) == 5
    assert np.array_equal(np.frombuffer(rec[1], np.float32).reshape(-1, 3), pos)
    assert np.array_equal(np.frombuffer(rec[3], np.uint64), ids)
    assert np.frombuffer(h[196:208], '<i4', 2).tolist() == [0, 1]


def test_zoom_masks_and_map_follow_genetic(built):
    """The generator's zoom bookkeeping: the flagged cube becomes the zoom mask, its cells'
    blocks the new level's flags and the next zoom's mask; the map's count and factors are
    the oracle's for the zoom2 and zoom3 cases."""
    from conftest import COSMO
    from genetic_gb300 import _lib, writers
    lib = _lib.load()
    flags0 = fo.flag_cells(fo.Levels(ZOOM3), 0, (25., 25., 25.), 'cube', 10)
    mask0, r0, flags1 = writers.zoom_mask(flags0, 32, (8, 8, 8), 2, 32)
    assert r0 == 2 and np.array_equal(mask0, np.sort(flags0))
    assert np.array_equal(flags1, np.sort(fo.block_cells(flags0, 32, 32, 2, (8, 8, 8))))
    mask1, r1, _ = writers.zoom_mask(flags1, 32, (8, 8, 8), 2, 32)
    assert r1 == 2 and np.array_equal(mask1, flags1)
    cnt = ctypes.c_ulonglong()
    for levels, masks, n in ((ZOOM2, [(mask0, 2, (8, 8, 8))], 34280),
                             (ZOOM3, [(mask0, 2, (8, 8, 8)), (mask1, 2, (8, 8, 8))], 46376)):
        m = writers.particle_map(levels, masks, COSMO)
        assert lib.gic_tipsy_count(ctypes.byref(m), ctypes.byref(cnt)) == 0 and cnt.value == n
        geo = [(32, 1, (0, 0, 0))] + [(32, 2, (8, 8, 8))] * (len(levels) - 1)
        order = fo.mapper_order_levels(geo, [mask0, mask1][:len(levels) - 1])
        mass, eps, pf, vf, mf = fo.tipsy_factors(levels, COSMO, order[0])
        assert (m.pos_factor, m.vel_factor, m.mass_factor) == (pf, vf, mf)
        assert [m.mass[l] for l in range(len(levels))] == mass and [m.eps[l] for l in range(len(levels))] == eps
    # cells outside the zoom window are dropped from the mask, as genetIC trims them
    mask, _, _ = writers.zoom_mask(np.array([0, 8 * 32 * 32 + 8 * 32 + 8]), 32, (8, 8, 8), 2, 32)
    assert mask.tolist() == [8 * 32 * 32 + 8 * 32 + 8]


def test_generator_writes_reference_files(built, zoom2_particles, tmp_path):
    """ICGenerator.write_tipsy / write_gadget on the zoom2 case, with the oracle's particles
    standing in for the device's (and the host packer for the device packer, which the GPU
    tests show to be bit-identical): the files match the reference's."""
    from conftest import COSMO
    from genetic_gb300 import _lib, writers
    from genetic_gb300.generator import ICGenerator
    lib = _lib.load()
    z = zoom2_particles
    gen = ICGenerator.__new__(ICGenerator)
    gen._lib, gen._ctx = lib, None
    gen.levels = ZOOM2
    gen.cosmo = dict(COSMO)
    mask, ratio, _ = writers.zoom_mask(z['replaced'], 32, ORIGIN, 2, 32)
    gen.zoom_masks = [(mask, ratio, ORIGIN)]
    gen.gadget_types = [1, 1]
    gen.particles = lambda l: (z['pos'][l], z['vel'][l])

    def fake_call(name, m, first, count, out):
        assert name == 'gic_tipsy_pack'
        P = ctypes.POINTER(ctypes.c_double)
        pp = (P * 2)(*[p.ctypes.data_as(P) for p in z['pos']])
        vv = (P * 2)(*[v.ctypes.data_as(P) for v in z['vel']])
        assert lib.gic_tipsy_pack_host(m, pp, vv, first, count, out, 2) == 0
    gen._call = fake_call
    gen.write_tipsy(tmp_path / 'out.tipsy')
    gen.write_gadget(tmp_path / 'out.gadget2')
    t = np.load(os.path.join(GOLDEN, 'tipsy_zoom2.npz'))
    raw = open(tmp_path / 'out.tipsy', 'rb').read()
    assert raw[:28] == bytes(t['header_bytes'])
    dark = np.frombuffer(raw[32:], np.float32).reshape(-1, 9)
    assert np.array_equal(dark[:, 0], t['dark'][:, 0]) and np.abs(dark[:, 1:4] - t['dark'][:, 1:4]).max() <= 6e-8
    g = np.load(os.path.join(GOLDEN, 'gadget_zoom2.npz'))
    rec = writers.read_fortran_records(tmp_path / 'out.gadget2')
    assert rec[0] == bytes(g['header_bytes']) and len(rec) == 5
    assert np.abs(np.frombuffer(rec[1], np.float32).reshape(-1, 3) - g['pos']).max() <= 4e-6
    assert np.array_equal(np.frombuffer(rec[4], np.float32), g['mass'])
    assert np.array_equal(np.frombuffer(rec[3], np.uint64), np.arange(len(g['mass']), dtype=np.uint64))


def test_outformat_commands_name_files_like_genetic(built, tmp_path):
    from genetic_gb300.generator import ICGenerator
    gen = ICGenerator.__new__(ICGenerator)
    gen._ctx = None
    gen.base_dir, gen.output_dir, gen.output_name, gen.output_format = str(tmp_path), './', '', None
    gen.precision, gen.cosmo, gen.levels = 'fp64', {'redshift': 99.0}, [(50.0, 32, (0, 0, 0))]
    written = []
    gen.write_tipsy = lambda p: written.append(p)
    gen.write_gadget = lambda p, v=2: written.append((p, v))
    gen.outformat('tipsy')
    gen.write()
    assert written[-1] == os.path.join(str(tmp_path), './', 'IC_doub_z99_32') + '.tipsy'
    gen.outdir('sub')
    gen.outname('out')
    gen.outformat('3')
    gen.write()
    assert written[-1] == (os.path.join(str(tmp_path), 'sub', 'out') + '.gadget3', 3)
    gen.outformat('grafic')
    with pytest.raises(NotImplementedError):
        gen.write()
    with pytest.raises(ValueError):
        gen.outformat('fits')


def test_gadget_particle_types_match_reference_file(built, zoom2_particles, tmp_path):
    """gadget_particle_type 3 on the base level and 1 on the zoom: the file holds type 1 (the
    zoom's particles) first, ids keep the mapper index, and one mass per type goes to the
    header with no mass block, as in the reference's file."""
    from conftest import COSMO
    from genetic_gb300 import writers
    from genetic_gb300.generator import ICGenerator
    z = zoom2_particles
    g = np.load(os.path.join(GOLDEN, 'gadget_types_zoom2.npz'))
    gen = ICGenerator.__new__(ICGenerator)
    from genetic_gb300 import _lib
    gen._lib, gen._ctx = _lib.load(), None
    gen.levels, gen.cosmo = ZOOM2, dict(COSMO)
    mask, ratio, _ = writers.zoom_mask(z['replaced'], 32, ORIGIN, 2, 32)
    gen.zoom_masks = [(mask, ratio, ORIGIN)]
    gen.gadget_types, gen._mru_gadget_type, gen._used_gadget_types = [1], 1, set()
    gen.gadget_particle_type(3)
    gen.gadget_types.append(gen._mru_gadget_type)  # the zoom level, as _add_level records it
    gen._used_gadget_types.add(gen._mru_gadget_type)
    gen.gadget_particle_type(1)
    assert gen.gadget_types == [3, 1]
    with pytest.raises(ValueError, match='reuse'):
        gen.gadget_particle_type(3)
    gen.particles = lambda l: (z['pos'][l], z['vel'][l])
    gen.write_gadget(tmp_path / 'out.gadget2')
    rec = writers.read_fortran_records(tmp_path / 'out.gadget2')
    assert len(rec) == 4 and rec[0] == bytes(g['header_bytes'])
    assert np.array_equal(np.frombuffer(rec[3], np.uint64), g['ids'])
    assert np.abs(np.frombuffer(rec[1], np.float32).reshape(-1, 3)[::97] - g['pos97']).max() <= 4e-6


def test_flagged_particle_type_matches_reference_files(built, zoom2_particles, tmp_path):
    """gadget_flagged_particle_type 4 after flagging a 3 Mpc/h sphere on the zoom level: the
    flagged particles move to the end, in the gadget file (as type 4) and in the tipsy file."""
    from conftest import COSMO
    from genetic_gb300 import _lib, writers
    from genetic_gb300.generator import ICGenerator
    z = zoom2_particles
    g = np.load(os.path.join(GOLDEN, 'flagged_type_zoom2.npz'))
    gen = ICGenerator.__new__(ICGenerator)
    gen._lib, gen._ctx = _lib.load(), None
    gen.levels, gen.cosmo = ZOOM2, dict(COSMO)
    mask, ratio, _ = writers.zoom_mask(z['replaced'], 32, ORIGIN, 2, 32)
    gen.zoom_masks = [(mask, ratio, ORIGIN)]
    gen.gadget_types, gen._mru_gadget_type, gen._used_gadget_types = [1, 1], 1, {1}
    gen.flagged_levels = [fo.flag_cells(fo.Levels(ZOOM2), l, (25., 25., 25.), 'sphere', 3) for l in range(2)]
    gen._flagged_type = None
    gen.gadget_flagged_particle_type(4)
    assert len(gen._flagged_snapshot) == 208
    gen.particles = lambda l: (z['pos'][l], z['vel'][l])
    gen.write_gadget(tmp_path / 'out.gadget2')
    rec = writers.read_fortran_records(tmp_path / 'out.gadget2')
    assert len(rec) == int(g['gadget_nrec']) and rec[0] == bytes(g['gadget_header'])
    assert np.array_equal(np.frombuffer(rec[3], np.uint64), g['gadget_ids'])
    assert np.array_equal(np.frombuffer(rec[4], np.float32), g['gadget_mass'])
    assert np.abs(np.frombuffer(rec[1], np.float32).reshape(-1, 3)[::97] - g['gadget_pos97']).max() <= 4e-6
    gen.write_tipsy(tmp_path / 'out.tipsy')
    raw = open(tmp_path / 'out.tipsy', 'rb').read()
    assert raw[:28] == bytes(g['tipsy_header'])
    dark = np.frombuffer(raw[32:], np.float32).reshape(-1, 9)
    for mine, ref in ((dark[::37], g['tipsy37']), (dark[-400:], g['tipsy_tail'])):
        assert np.array_equal(mine[:, 0], ref[:, 0]) and np.array_equal(mine[:, 7:], ref[:, 7:])
        assert np.abs(mine[:, 1:4] - ref[:, 1:4]).max() <= 6e-8


def _host_only_generator():
    """An ICGenerator whose level bookkeeping runs without a device (gic_level_add skipped)."""
    from genetic_gb300 import _lib
    from genetic_gb300.generator import ICGenerator
    gen = ICGenerator.__new__(ICGenerator)
    gen._lib, gen._ctx = _lib.load(), None
    gen._init_state('fp64', 0)
    gen._call = lambda name, *args: None
    return gen


@pytest.mark.parametrize('case', ['centre', 'wrap', 'nested'])
def test_zoom_grid_places_zooms_like_genetic(built, case):
    """zoom_grid's lower corners against those genetIC logs for the same commands
    (tests/golden/make_golden.py: ZOOM_GRID_CASES)."""
    import sys
    sys.path.insert(0, GOLDEN)
    from make_golden import ZOOM_GRID_CASES
    want = np.load(os.path.join(GOLDEN, 'zoom_grid_corners.npz'))[case].tolist()
    gen = _host_only_generator()
    gen.base_grid(50.0, 32)
    got = []
    for line in ZOOM_GRID_CASES[case].split('\n'):
        cmd, *args = line.split()
        getattr(gen, cmd)(*args)
        if cmd == 'zoom_grid':
            (box_a, n_a, off_a), (_, _, off) = gen.levels[-2], gen.levels[-1]
            got.append([int(round((o - oa) / (box_a / n_a))) for o, oa in zip(off, off_a)])
    assert got == want


def test_select_nearest_flags_the_finest_cell_at_the_centre(built):
    gen = _host_only_generator()
    gen.base_grid(50.0, 32)
    gen.centre(25.0, 25.0, 25.0)
    gen.select_cube(10)
    gen.zoom_grid_with_origin_at(8, 8, 8, 2, 32)
    gen.centre(49.9, 20.1, 12.6)  # outside the zoom in x: refused
    with pytest.raises(ValueError):
        gen.select_nearest()
    gen.centre(20.1, 12.6, 36.0)
    gen.select_nearest()
    dx = 25.0 / 32
    want = ((int((20.1 - 12.5) // dx)) * 32 + int((12.6 - 12.5) // dx)) * 32 + int((36.0 - 12.5) // dx)
    assert gen.flagged.tolist() == [want] and len(gen.flagged_levels[0]) == 0


def _zoom2_host_generator(tmp_path):
    gen = _host_only_generator()
    gen.base_dir = str(tmp_path)
    gen.base_grid(50.0, 32)
    gen.centre(25, 25, 25)
    gen.select_cube(10)
    gen.zoom_grid_with_origin_at(8, 8, 8, 2, 32)
    return gen


def test_id_files_match_genetic(built, tmp_path):
    """dump_IDfile after flagging a sphere, and IDfile + dump_IDfile of a list mixing coarse
    and zoom particles, against genetIC's files and logged centre (zoom2 case)."""
    import sys
    sys.path.insert(0, GOLDEN)
    from make_golden import ID_FILE_IN
    g = np.load(os.path.join(GOLDEN, 'id_files_zoom2.npz'))
    gen = _zoom2_host_generator(tmp_path)
    gen.centre(25, 25, 25)
    gen.select_sphere(3)
    gen.dump_id_file('a.txt')
    assert np.loadtxt(tmp_path / 'a.txt', dtype=np.int64).tolist() == g['dump_ids'].tolist()
    gen = _zoom2_host_generator(tmp_path)
    (tmp_path / 'in.txt').write_text(''.join('%d\n' % i for i in ID_FILE_IN))
    gen.id_file('in.txt')
    gen.dump_id_file('b.txt')
    assert np.loadtxt(tmp_path / 'b.txt', dtype=np.int64).tolist() == g['load_ids'].tolist()
    # the centre genetIC logs to 12 significant digits
    assert np.allclose(gen.centre_point, g['load_centre'], rtol=0, atol=1e-9)


def test_dump_tipsy_matches_genetic_file(built, bbks, tmp_path):
    """dump_tipsy after done: the combined overdensity at every particle in mapper order,
    byte for byte the reference's file (the oracle's delta standing in for the device's)."""
    from conftest import COSMO
    g = np.load(os.path.join(GOLDEN, 'dump_tipsy_zoom2.npz'))
    w = fo.white_noise_levels([32, 32], 8896131, 2)
    out = fo.zoom_realisation(w, ZOOM2, fo.CambPower(bbks, COSMO))
    gen = _zoom2_host_generator(tmp_path)
    gen.field = lambda l, name: out[l][0]
    gen.dump_tipsy('field.tipsy')
    assert open(tmp_path / 'field.tipsy', 'rb').read() == bytes(g['raw'])


def test_gadget_num_files_matches_genetic(built, zoom2_particles, tmp_path):
    """gadget_num_files 3: each file's header and ids as genetIC splits them."""
    from genetic_gb300 import writers
    z = zoom2_particles
    g = np.load(os.path.join(GOLDEN, 'gadget_files_zoom2.npz'))
    gen = _zoom2_host_generator(tmp_path)
    gen.particles = lambda l: (z['pos'][l], z['vel'][l])
    gen.gadget_num_files(3)
    gen.cosmo.update(dict(omega_m=0.31, omega_lambda=0.69, hubble=0.68, redshift=99.0))
    gen.write_gadget(str(tmp_path / 'out.gadget2'))
    for i in range(3):
        rec = writers.read_fortran_records(tmp_path / ('out.gadget2.%d' % i))
        assert len(rec) == int(g['nrec%d' % i]) and rec[0] == bytes(g['header%d' % i])
        assert np.array_equal(np.frombuffer(rec[3], np.uint64), g['ids%d' % i])


# --- genetIC's supersample / subsample (tests/golden/resample_*.npz) -------------------------

RESAMPLE = {
    # name: (levels, resampled level, factor, replaced-cell selection)
    'super1': ([(50.0, 16, (0.0, 0.0, 0.0))], 0, 2, None),
    'sub1': ([(50.0, 32, (0.0, 0.0, 0.0))], 0, -2, None),
    'superzoom': (ZOOM2, 1, 2, ('cube', 10)),
}


def resampled_oracle(bbks, name):
    """The oracle's particles of RESAMPLE[name] with the resampled level on its virtual grid:
    positions and velocities per level, the mapper order and the tipsy factors."""
    from conftest import COSMO
    levels, lev, factor, sel = RESAMPLE[name]
    fo.set_cr_log(False)
    w = fo.white_noise_levels([l[1] for l in levels], 8896131, 2)
    fields = fo.zoom_realisation(w, levels, fo.CambPower(bbks, COSMO))
    ratio = fo.velocity_to_offset_ratio(COSMO)
    periodic = levels[0][0]
    pos, vel, vlevels, soft = [], [], [], []
    for l, (b, n, off) in enumerate(levels):
        psi = fields[l][1:4]
        nv, sc = n, 1.0
        if l == lev:
            psi, nv = fo.resample_displacements(psi, b, n, off, periodic, factor)
            sc = float(factor) if factor > 1 else 1.0
        p, v = fo.particles(psi, b, off, periodic, ratio)
        pos.append(p)
        vel.append(v)
        vlevels.append((b, nv, off))
        soft.append(sc)
    if sel is None:
        order = (np.zeros(vlevels[0][1] ** 3, dtype=int), np.arange(vlevels[0][1] ** 3))
    else:
        replaced = fo.flag_cells(fo.Levels(levels), 0, (25., 25., 25.), *sel)
        n0, n1 = vlevels[0][1], vlevels[1][1]
        order = fo.mapper_order(n0, replaced, n1, n1 // (n0 // 2), ORIGIN)
    factors = fo.tipsy_factors(vlevels, COSMO, order[0], soft)
    return dict(pos=pos, vel=vel, order=order, factors=factors)


@pytest.mark.parametrize('name', sorted(RESAMPLE))
def test_resampled_oracle_matches_reference_file(bbks, name):
    g = np.load(os.path.join(GOLDEN, 'resample_%s.npz' % name))
    r = resampled_oracle(bbks, name)
    assert len(r['order'][1]) == int(g['nrec'])
    got = fo.tipsy_records(r['order'], r['pos'], r['vel'], *r['factors'])
    stride = int(g['stride'])
    for mine, ref in ((got[::stride], g['every']), (got[-400:], g['tail'])):
        assert np.array_equal(mine[:, 0], ref[:, 0]) and np.array_equal(mine[:, 7:], ref[:, 7:])
        assert np.abs(mine[:, 1:4] - ref[:, 1:4]).max() <= 6e-8
        assert np.abs(mine[:, 4:7] - ref[:, 4:7]).max() <= 2e-7 * np.abs(ref[:, 4:7]).max()


# --- stray particles (genetIC's strays_on; tests/golden/strays_zoom4.npz) ----------------------

STRAYS = [(50.0, 32, (0.0, 0.0, 0.0)), (12.5, 32, (23.4375, 23.4375, 18.75))]  # zoom at cell (15, 15, 12)
STRAYS_ORIGIN = (15, 15, 12)


def strays_oracle(bbks):
    """The oracle's particles of the strays case: level 0 as usual, the zoom level on its
    resolution-matching grid (128^3 over the whole box), mapper order and tipsy factors."""
    from conftest import COSMO
    fo.set_cr_log(False)
    w = fo.white_noise_levels([32, 32], 8896131, 2)
    fields = fo.zoom_realisation(w, STRAYS, fo.CambPower(bbks, COSMO))
    ratio = fo.velocity_to_offset_ratio(COSMO)
    psi, nv, vgeom = fo.matched_displacements(fields[1][1:4], STRAYS[1], fields[0][1:4], STRAYS[0], 50.0)
    pv0 = fo.particles(fields[0][1:4], 50.0, (0.0, 0.0, 0.0), 50.0, ratio)
    pv1 = fo.particles(psi, vgeom[0], vgeom[2], 50.0, ratio)
    replaced = fo.flag_cells(fo.Levels(STRAYS), 0, (25., 25., 25.), 'sphere', 3.0)
    order = fo.mapper_order(32, replaced, nv, nv // 32, (0, 0, 0))
    factors = fo.tipsy_factors([STRAYS[0], vgeom], COSMO, order[0])
    return dict(pos=[pv0[0], pv1[0]], vel=[pv0[1], pv1[1]], order=order, factors=factors, replaced=replaced, nv=nv)


def test_strays_oracle_matches_reference_file(bbks):
    g = np.load(os.path.join(GOLDEN, 'strays_zoom4.npz'))
    r = strays_oracle(bbks)
    assert len(r['order'][1]) == int(g['nrec'])
    got = fo.tipsy_records(r['order'], r['pos'], r['vel'], *r['factors'])
    stride = int(g['stride'])
    for mine, ref in ((got[::stride], g['every']), (got[-400:], g['tail'])):
        assert np.array_equal(mine[:, 0], ref[:, 0]) and np.array_equal(mine[:, 7:], ref[:, 7:])
        assert np.abs(mine[:, 1:4] - ref[:, 1:4]).max() <= 6e-8
        assert np.abs(mine[:, 4:7] - ref[:, 4:7]).max() <= 2e-7 * np.abs(ref[:, 4:7]).max()
