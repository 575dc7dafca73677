"""Particle files as genetIC writes them: tipsy (io/tipsy.hpp) and gadget 2/3 (io/gadget.hpp).

The particle data come from the C ABI's packers (gic_tipsy_pack, gic_tipsy_pack_host,
gic_gadget_pack_host) in genetIC's particle-mapper order; this module adds the headers
and the framing.  Byte order is the host's, as genetIC's memory-mapped writers use it
(both x86-64 and aarch64 are little-endian).
"""
import struct

import numpy as np

GADGET_HEADER_BYTES = 256


def tipsy_header(scalefactor, n_dark, n_gas=0, n_star=0):
    """io_header_tipsy (tipsy.hpp:21-28, 241-247): scale factor, particle counts and ndim = 3;
    the structure's 4 trailing padding bytes are written as zeros."""
    n = n_dark + n_gas + n_star
    return struct.pack('<d5i4x', scalefactor, n, 3, n_gas, n_dark, n_star)


def write_tipsy(path, scalefactor, dark):
    """A tipsy file of dark-matter records only: the header, then `dark` (n x 9 float32,
    TipsyParticle::dark), as TipsyOutput::operator() lays it out (tipsy.hpp:200-262)."""
    dark = np.ascontiguousarray(dark, dtype=np.float32).reshape(-1, 9)
    with open(path, 'wb') as f:
        f.write(tipsy_header(scalefactor, len(dark)))
        f.write(dark.tobytes())


def gadget_header(version, npart, masses, scalefactor, redshift, box, omega_m, omega_lambda, hubble, num_files=1,
                  double_precision=False):
    """io_header_2 / io_header_3 (gadget.hpp:25-110) as createGadget2Header and
    createGadget3Header fill it (gadget.hpp:116-229): zeroed, then the six-type counts
    and masses, time and redshift, totals with their high words, the box and the
    cosmology; gadget 3 adds flag_doubleprecision and flag_ic_info = 1.  Baryons (type 0)
    switch on the sfr, feedback and cooling flags."""
    if version not in (2, 3):
        raise ValueError('Unknown gadget format')
    npart = [int(v) for v in npart]
    gas = 1 if npart[0] > 0 else 0
    h = bytearray(GADGET_HEADER_BYTES)
    struct.pack_into('<6I', h, 0, *[v & 0xffffffff for v in npart])
    struct.pack_into('<6d', h, 24, *[float(m) for m in masses])
    struct.pack_into('<2d2i', h, 72, scalefactor, redshift, gas, gas)
    struct.pack_into('<6I', h, 96, *[v & 0xffffffff for v in npart])
    struct.pack_into('<2i4d2i', h, 120, gas, num_files, box, omega_m, omega_lambda, hubble, 0, 0)
    struct.pack_into('<6I', h, 168, *[v >> 32 for v in npart])
    struct.pack_into('<i', h, 192, 0)
    if version == 3:
        struct.pack_into('<2if', h, 196, 1 if double_precision else 0, 1, 0.0)
    return bytes(h)


def fortran_record(data):
    """A record framed by its length in bytes before and after (MemMapFileWriter::getMemMapFortran)."""
    n = struct.pack('<i', len(data))
    return n + data + n


def write_gadget(path, header, pos, vel, ids, mass=None):
    """A single-file gadget snapshot: header, positions, velocities, ids and, for variable
    masses, the mass block, each as one Fortran record (GadgetOutput::operator(), gadget.hpp:481-520)."""
    with open(path, 'wb') as f:
        f.write(fortran_record(header))
        f.write(fortran_record(np.ascontiguousarray(pos).tobytes()))
        f.write(fortran_record(np.ascontiguousarray(vel).tobytes()))
        f.write(fortran_record(np.ascontiguousarray(ids).tobytes()))
        if mass is not None:
            f.write(fortran_record(np.ascontiguousarray(mass).tobytes()))


def read_fortran_records(path):
    """The records of a Fortran-framed file."""
    raw = open(path, 'rb').read()
    out, off = [], 0
    while off < len(raw):
        n = struct.unpack_from('<i', raw, off)[0]
        out.append(raw[off + 4:off + 4 + n])
        if struct.unpack_from('<i', raw, off + 4 + n)[0] != n:
            raise ValueError('bad record framing at byte %d' % off)
        off += n + 8
    return out


def block_cells(parents, n_parent, n_child, ratio, origin):
    """The ratio^3 cells (x, y, z ascending) that each parent cell covers on a child grid
    whose corner is parent cell `origin` (Grid::insertCubeIdsIntoVector, grid.hpp:704-729)."""
    p = np.asarray(parents, dtype=np.int64)
    px, py, pz = p // (n_parent * n_parent), (p // n_parent) % n_parent, p % n_parent
    px, py, pz = (px - origin[0]) % n_parent, (py - origin[1]) % n_parent, (pz - origin[2]) % n_parent
    s = np.arange(ratio ** 3)
    sx, sy, sz = s // (ratio * ratio), (s // ratio) % ratio, s % ratio
    fx = px[:, None] * ratio + sx[None, :]
    fy = py[:, None] * ratio + sy[None, :]
    fz = pz[:, None] * ratio + sz[None, :]
    return ((fx * n_child + fy) * n_child + fz).ravel()


def zoom_mask(flags_above, n_above, origin, zoomfac, n_new):
    """What ICGenerator::initZoomGridWithLowLeftCornerAt keeps of the cells flagged on the
    level above when a zoom level is added (ic.hpp:480-596): the zoom mask (the flagged
    cells inside the zoom window, ascending), the cell-size ratio, and the cells of the new
    level that become flagged (those under the mask's cells).  ratio is None when the
    cell sizes are not in an integer ratio (genetIC's mapper then refuses the zoom)."""
    c = np.asarray(flags_above, dtype=np.int64)
    span = n_above // int(zoomfac)
    coords = (c // (n_above * n_above), (c // n_above) % n_above, c % n_above)
    inside = np.ones(len(c), dtype=bool)
    for a in range(3):
        inside &= (coords[a] - int(origin[a])) % n_above < span
    mask = np.sort(c[inside]).astype(np.uint64)
    num = int(zoomfac) * int(n_new)
    ratio = num // n_above if num % n_above == 0 else None
    if ratio is None:
        return mask, None, np.zeros(0, dtype=np.uint64)
    new_flags = np.sort(block_cells(mask, n_above, int(n_new), ratio, origin)).astype(np.uint64)
    return mask, ratio, new_flags


def particle_map(levels, zoom_masks, cosmo, flagged=None):
    """The gic_particle_map of a context: levels [(box, n, offset)]; zoom_masks[l - 1] =
    (mask, ratio, origin) of zoom level l; each level's particle mass and softening as
    ZeldovichParticleEvaluator gives them (27.744948 Om L^3 (dx/L)^3 and 0.01075 dx,
    zeldovich.hpp:55-62, 112-121); TipsyOutput's factors from gic_tipsy_factors.
    flagged: cells of the finest level given their own gadget type, which genetIC moves
    to the end of the order with one more TwoLevelParticleMapper on the finest grid
    (ic.hpp:1176-1185); the map then has one more level, of ratio 1, over the finest."""
    import ctypes

    from . import _lib
    L = levels[0][0]
    lv = [(levels[0][1], 1, (0, 0, 0))]
    replaced = []
    for (box, n, _), (mask, ratio, origin) in zip(levels[1:], zoom_masks):
        if ratio is None or len(mask) == 0:
            raise ValueError('a zoom level needs flagged cells on the level above and an integer cell-size ratio')
        lv.append((n, ratio, tuple(int(o) for o in origin)))
        replaced.append(mask)
    dx = [box / n for box, n, _ in levels]
    if flagged is not None:
        if len(flagged) == 0:
            raise ValueError('no cells are flagged on the finest level for their own gadget type')
        replaced.append(np.sort(np.asarray(flagged, dtype=np.uint64)))
        lv.append((levels[-1][1], 1, (0, 0, 0)))
        dx.append(dx[-1])
    replaced.append([])
    om = cosmo['omega_m']
    mass = [27.744948 * om * pow(L, 3.0) * pow(d / L, 3.0) for d in dx]
    eps = [d * 1.0 * 0.01075 for d in dx]
    m = _lib.GicParticleMap.of(lv, replaced, mass, eps, 0.0, 0.0, 0.0)
    f = [ctypes.c_double() for _ in range(3)]
    a = 1.0 / (1.0 + cosmo['redshift'])
    lib = _lib.load()
    _lib.check(None, lib.gic_tipsy_factors(ctypes.byref(m), om, cosmo['hubble'], a, L, *[ctypes.byref(v) for v in f]))
    m.pos_factor, m.vel_factor, m.mass_factor = f[0].value, f[1].value, f[2].value
    return m


def gadget_type_counts(m, level_types):
    """Particles per gadget type and the header's per-type masses, as
    GadgetOutput::preScanForMassesAndParticleNumbers finds them (gadget.hpp:325-372): a
    type's mass is its particles' mass when they all share one; if any type mixes
    masses, the file stores every mass (None is returned for the masses)."""
    runs = []
    for l in range(m.nlevels):
        have = m.n[0] ** 3 if l == 0 else m.n_replaced[l - 1] * m.ratio[l] ** 3
        runs.append(have - m.n_replaced[l])
    npart, per_type = [0] * 6, [set() for _ in range(6)]
    for l, t in enumerate(level_types[:m.nlevels]):
        npart[t] += runs[l]
        if runs[l]:
            per_type[t].add(m.mass[l])
    if any(len(s) > 1 for s in per_type):
        return npart, None
    return npart, [min(s) if s else 0.0 for s in per_type]


def mapper_order(levels, zoom_masks, flagged=None):
    """(level, cell) of every particle in genetIC's mapper order (one TwoLevelParticleMapper
    per zoom level, ic.hpp:1150-1185; twolevelmapper.hpp:262-320, 869-893): each zoom drops
    its mask's cells from the order so far and appends their blocks in ascending cell id.
    levels: [(box, n, offset)]; zoom_masks[l - 1] = (mask, ratio, origin); flagged: the
    finest level's cells moved to the end as their own gadget type (map level len(levels))."""
    n0 = levels[0][1]
    lev = np.zeros(n0 ** 3, dtype=np.int64)
    cells = np.arange(n0 ** 3, dtype=np.int64)
    steps = [(l, mask, ratio, origin) for l, (mask, ratio, origin) in enumerate(zoom_masks, 1)]
    if flagged is not None:
        steps.append((len(levels), flagged, 1, (0, 0, 0)))
    for l, mask, ratio, origin in steps:
        n_parent = levels[l - 1][1]
        n_child = levels[min(l, len(levels) - 1)][1]
        rep = np.sort(np.asarray(mask, dtype=np.int64))
        drop = (lev == l - 1) & np.isin(cells, rep)
        lev, cells = lev[~drop], cells[~drop]
        fine = block_cells(rep, n_parent, n_child, ratio, origin)
        lev = np.concatenate([lev, np.full(len(fine), l, dtype=np.int64)])
        cells = np.concatenate([cells, fine])
    return lev, cells


def gadget_file_split(npart, nfiles):
    """How GadgetOutput spreads the particles over `nfiles` files (gadget.hpp:355-420):
    nTotal / nFiles particles per file, the last file taking the rest, and each file's
    particles taken from the types in order.  Returns (particles per file, per-file counts
    per type)."""
    total = sum(npart)
    per_file = [total // nfiles] * (nfiles - 1) + [total - (total // nfiles) * (nfiles - 1)]
    left = list(npart)
    per_type = []
    for nf in per_file:
        room, this = nf, [0] * 6
        for t in range(6):
            this[t] = min(left[t], room)
            room -= this[t]
            left[t] -= this[t]
        per_type.append(this)
    return per_file, per_type
