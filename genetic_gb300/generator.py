"""Host-side driver of the GPU realisation path, mirroring genetIC's ICGenerator.

Method names are genetIC's paramfile commands (genetIC/src/main.cpp:22-172) and
their arguments mean the same; `run_paramfile` dispatches a paramfile line by
line like genetIC's parser (genetIC/src/tools/parser.hpp:193-211).  Geometry
and bookkeeping stay on the host; every field operation goes through the C ABI
of libgicgpu.so.
"""
import ctypes
import os

import numpy as np

from . import _lib, geometry, writers
from ._lib import check
from .transfer import read_camb

_DP = ctypes.POINTER(ctypes.c_double)


def _ptr(a):
    return a.ctypes.data_as(_DP)


class ICGenerator:
    """The realisation state of one set of initial conditions on one GPU."""

    def __init__(self, precision='fp64', device=0, mem_limit=0):
        """mem_limit: bytes of device memory the context may hold (0: no limit); a call
        that would allocate past it fails with GIC_ERR_OOM and the context stays usable."""
        lib = _lib.load()
        self._lib = lib
        opts = _lib.GicDeviceOpts(_lib.GIC_FP64 if precision == 'fp64' else _lib.GIC_MIXED, device, int(mem_limit))
        ctx = ctypes.c_void_p()
        st = lib.gic_create(ctypes.byref(ctx), ctypes.byref(opts))
        if st != _lib.GIC_OK:
            raise _lib.GicError(st, lib.gic_last_error(None).decode())
        self._ctx = ctx
        self._init_state(precision, device)

    def _init_state(self, precision, device):
        """The host-side state of a new context (no device call)."""
        self.precision = precision
        self.device = device
        # genetIC's defaults for Om, Ob, h, ns (genetIC/src/ic.hpp:200-210); Ol, s8
        # and zin have no default there and are always set by a paramfile
        self.cosmo = dict(omega_m=0.3, omega_lambda=0.7, omega_b=0.0, hubble=0.701, sigma8=0.8, ns=0.96,
                          redshift=0.0)
        self.levels = []  # (box, n, offset)
        self.seed = None
        self.seed_mode = None
        self.base_dir = '.'
        self._drawn = False
        self._done = False
        self.centre_point = (0.0, 0.0, 0.0)
        self.flagged = None  # flagged cells of the finest level (linear indices)
        self.zoom_masks = []  # per zoom level: (replaced cells of the level above, ratio, origin)
        self.output_dir, self.output_name, self.output_format = './', '', None
        # gadget particle type per level (ic.hpp:80, 606-614, 680-700)
        self.gadget_types, self._mru_gadget_type, self._used_gadget_types = [], 1, set()
        # gadget_flagged_particle_type: the type and the finest level's flags at genetIC's
        # last particle-mapper rebuild (ic.hpp:705-714, 1176-1185)
        self._flagged_type, self._flagged_snapshot = None, None
        self.gadget_files = 1

    # -- lifetime --------------------------------------------------------------
    def close(self):
        if self._ctx:
            self._lib.gic_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _call(self, name, *args):
        check(self._ctx, getattr(self._lib, name)(self._ctx, *args))

    def memory_use(self):
        """(bytes of device memory the context holds, its mem_limit)."""
        used, limit = ctypes.c_size_t(), ctypes.c_size_t()
        self._call('gic_memory_use', ctypes.byref(used), ctypes.byref(limit))
        return used.value, limit.value

    # -- cosmology (main.cpp:31-37) ------------------------------------------------
    def Om(self, v):
        self.cosmo['omega_m'] = float(v)

    def Ol(self, v):
        self.cosmo['omega_lambda'] = float(v)

    def Ob(self, v):
        self.cosmo['omega_b'] = float(v)

    def hubble(self, v):
        self.cosmo['hubble'] = float(v)

    def s8(self, v):
        self.cosmo['sigma8'] = float(v)

    def ns(self, v):
        self.cosmo['ns'] = float(v)

    def zin(self, v):
        self.cosmo['redshift'] = float(v)

    def _push_cosmology(self):
        c = _lib.GicCosmo(**self.cosmo)
        self._call('gic_set_cosmology', ctypes.byref(c))

    def camb(self, path_or_table):
        """Load a CAMB transfer table (path, or an (nrows, ncols) array) with the current cosmology."""
        if isinstance(path_or_table, str):
            path = path_or_table if os.path.isabs(path_or_table) else os.path.join(self.base_dir, path_or_table)
            table = read_camb(path)
        else:
            table = np.asarray(path_or_table, dtype=np.float64)
        table = np.ascontiguousarray(table, dtype=np.float64)
        self._push_cosmology()
        self._call('gic_set_transfer', _ptr(table), table.shape[0], table.shape[1])

    def normalisation(self):
        a, s = ctypes.c_double(), ctypes.c_double()
        self._call('gic_get_normalisation', ctypes.byref(a), ctypes.byref(s))
        return a.value, s.value

    # -- grids (main.cpp:92-94, ic.hpp:365-598) ------------------------------------
    def base_grid(self, box, n):
        self._add_level(float(box), int(n), (0.0, 0.0, 0.0))

    basegrid = base_grid

    def zoom_grid_with_origin_at(self, x0, y0, z0, zoomfac, n):
        box0, n0, off0 = self.levels[-1]
        dx0 = box0 / n0
        if int(x0) < 0 or int(y0) < 0 or int(z0) < 0:
            raise ValueError('The newly initialised zoom level is not fully contained within the previous level')
        offset = tuple(off0[i] + int(c) * dx0 for i, c in enumerate((x0, y0, z0)))
        # the zoom mask and the flags carried to the new level (ic.hpp:480-596)
        flags = getattr(self, 'flagged_levels', [])
        above = flags[-1] if len(flags) == len(self.levels) else np.zeros(0, dtype=np.uint64)
        origin = (int(x0), int(y0), int(z0))
        mask, ratio, new_flags = writers.zoom_mask(above, n0, origin, int(zoomfac), int(n))
        self._add_level(box0 / int(zoomfac), int(n), offset)
        self.zoom_masks.append((mask, ratio, origin))
        if len(flags) == len(self.levels) - 1:
            self.flagged_levels = list(flags) + [new_flags]
            self.flagged = new_flags
        self._update_mapper()

    def _update_mapper(self):
        """ICGenerator::updateParticleMapper's part that reads state: the finest level's
        flagged cells, kept for the flagged particles' own gadget type."""
        if getattr(self, '_flagged_type', None) is None:
            return
        flags = getattr(self, 'flagged_levels', [])
        cells = flags[-1] if len(flags) == len(self.levels) and len(flags) else np.zeros(0, dtype=np.uint64)
        self._flagged_snapshot = np.sort(np.asarray(cells, dtype=np.uint64))

    def gadget_num_files(self, n):
        """ICGenerator::setGadgetNumFiles (ic.hpp:674-676): gadget output over n files."""
        n = int(n)
        if n < 1:
            raise ValueError('the number of gadget files must be positive')
        self.gadget_files = n

    def gadget_flagged_particle_type(self, t):
        """ICGenerator::setFlaggedGadgetParticleType (ic.hpp:705-714): the finest level's
        flagged cells become particles of type t, at the end of the particle order."""
        t = int(t)
        if not 0 <= t < 6:
            raise ValueError('Gadget particle type must be between 0 and 5')
        if t in self._used_gadget_types:
            raise ValueError('Cannot reuse a gadget particle type; this type was already used in a different '
                             'section of the ICs')
        self._flagged_type = t
        self._used_gadget_types.add(t)
        self._update_mapper()

    zoomgrid_with_origin_at = zoom_grid_with_origin_at

    def zoom_grid(self, zoomfac, n):
        """ICGenerator::initZoomGrid (ic.hpp:398-476): a zoom level of n cells per side and
        1/zoomfac of the finest level's size, placed around that level's flagged cells."""
        if not self.levels:
            raise RuntimeError('Cannot initialise a zoom grid before initialising the base grid')
        flags = getattr(self, 'flagged_levels', [])
        above = flags[-1] if len(flags) == len(self.levels) else np.zeros(0, dtype=np.uint64)
        box, na, off = self.levels[-1]
        x0, y0, z0 = geometry.zoom_corner(above, na, box, off, self.levels[0][0], int(zoomfac))
        self.zoom_grid_with_origin_at(x0, y0, z0, zoomfac, n)

    zoomgrid = zoom_grid

    def _add_level(self, box, n, offset):
        lid = ctypes.c_int()
        self._call('gic_level_add', box, n, offset[0], offset[1], offset[2], ctypes.byref(lid))
        self.levels.append((box, n, offset))
        self.gadget_types.append(self._mru_gadget_type)
        if len(self.gadget_types) > 1:  # the type selected before is now in use (ic.hpp:611-613)
            self._used_gadget_types.add(self._mru_gadget_type)

    def gadget_particle_type(self, t):
        """ICGenerator::setGadgetParticleType (ic.hpp:690-701): the gadget type of the deepest level."""
        t = int(t)
        if not 0 <= t < 6:
            raise ValueError('Gadget particle type must be between 0 and 5')
        if t != self._mru_gadget_type:
            if t in self._used_gadget_types:
                raise ValueError('Cannot reuse a gadget particle type; this type was already used in a different '
                                 'section of the ICs')
            self._mru_gadget_type = t
        if not self.levels:
            raise RuntimeError("Can't set a gadget particle type until a level has been initialised to set it for")
        self.gadget_types[-1] = t
        self._update_mapper()

    # -- seeding (main.cpp:44-52) ----------------------------------------------------
    def _seed(self, seed, mode):
        if self.seed is not None:
            raise RuntimeError('The random number generator has already been seeded')
        self.seed, self.seed_mode = int(seed), mode

    def random_seed(self, seed):
        self._seed(seed, _lib.GIC_SEED_FOURIER_PARALLEL)

    seedfourier_parallel = random_seed

    def random_seed_serial(self, seed):
        self._seed(seed, _lib.GIC_SEED_FOURIER_SERIAL)

    seedfourier = random_seed_serial

    def random_seed_real_space(self, seed):
        self._seed(seed, _lib.GIC_SEED_REAL_SPACE)

    seed_ = random_seed_real_space

    def seedfourier_reverse(self, seed):
        self._seed(seed, _lib.GIC_SEED_FOURIER_REVERSE)

    # -- cell selection (ic.hpp:1458-1583) ------------------------------------------
    def centre(self, x, y, z):
        self.centre_point = (float(x), float(y), float(z))

    def _select(self, inside):
        """Flag, on every level, the cells whose wrapped offset from the centre passes
        `inside` (ic.hpp:1458-1485)."""
        period = self.levels[0][0]
        self.flagged_levels = []
        for box, n, off in self.levels:
            dx = box / n
            d = []
            for a in range(3):
                x = np.arange(n) * dx + off[a] + dx / 2 - self.centre_point[a]
                x = np.where(x > period / 2, x - period, x)
                x = np.where(x < -period / 2, x + period, x)
                d.append(x)
            # sphere and cube tests grow with each |offset|: a slab whose x offset fails
            # with y = z = 0 has no flagged cell
            zero = np.zeros(1)
            Y, Z = d[1][:, None], d[2][None, :]
            cells = []
            for i in np.flatnonzero(inside(d[0], zero, zero)):
                cells.append(np.flatnonzero(inside(d[0][i], Y, Z).ravel()) + i * n * n)
            flat = np.concatenate(cells) if cells else np.zeros(0, dtype=np.int64)
            self.flagged_levels.append(np.ascontiguousarray(flat, dtype=np.uint64))
        self.flagged = self.flagged_levels[-1]

    def select_nearest(self):
        """ICGenerator::selectNearest (ic.hpp:1447-1455): every flag is cleared, then the finest
        level's cell holding the centre is flagged (Grid::getIndexFromPoint, grid.hpp:672-677:
        floor of the wrapped offset from the level's corner over the cell size)."""
        period = self.levels[0][0]
        box, n, off = self.levels[-1]
        dx = box / n
        idx = []
        for a in range(3):
            d = (self.centre_point[a] - off[a]) % period
            idx.append(int(np.floor(d / dx)))
        if any(i < 0 or i >= n for i in idx):
            raise ValueError('the centre is not on the finest level')
        cell = (idx[0] * n + idx[1]) * n + idx[2]
        self.flagged_levels = [np.zeros(0, dtype=np.uint64) for _ in self.levels[:-1]]
        self.flagged_levels.append(np.array([cell], dtype=np.uint64))
        self.flagged = self.flagged_levels[-1]

    # -- particle ID files (ic.hpp:1374-1439; io/input.hpp:33-39, 99-106) ---------------
    def _order(self):
        flagged = self._flagged_snapshot if getattr(self, '_flagged_type', None) is not None else None
        return writers.mapper_order(self.levels, self.zoom_masks, flagged)

    def _flags(self):
        flags = getattr(self, 'flagged_levels', [])
        if len(flags) != len(self.levels):
            return [np.zeros(0, dtype=np.uint64) for _ in self.levels]
        return [np.asarray(f, dtype=np.uint64) for f in flags]

    def dump_id_file(self, fname):
        """ICGenerator::dumpID: the map indices of the flagged cells that are particles,
        ascending, one per line (ParticleMapper::getFlaggedParticles)."""
        lev, cells = self._order()
        flags = self._flags()
        keep = np.zeros(len(cells), dtype=bool)
        for l in range(int(lev.max()) + 1):
            sel = lev == l
            keep[sel] = np.isin(cells[sel], flags[min(l, len(flags) - 1)].astype(np.int64))
        with open(os.path.join(self.base_dir, fname), 'w') as f:
            f.writelines('%d\n' % i for i in np.flatnonzero(keep))

    def merge_id_file(self, fname):
        """ICGenerator::appendID: flags the cells of the particles listed in the file, and the
        replaced cells above them (TwoLevelParticleMapper::flagParticles flags a zoom
        particle's parent on the level above), then centres on the deepest flagged level."""
        with open(os.path.join(self.base_dir, fname)) as f:
            ids = np.unique(np.array(f.read().split(), dtype=np.int64))
        lev, cells = self._order()
        if len(ids) and (ids[0] < 0 or ids[-1] >= len(cells)):
            raise ValueError('Particle ID out of range')
        nl = len(self.levels)
        add = [[] for _ in range(nl)]
        for l, c in zip(lev[ids], cells[ids]):
            l = min(int(l), nl - 1)  # the flagged-type level lies on the finest grid
            c = int(c)
            while True:
                add[l].append(c)
                if l == 0:
                    break
                mask, ratio, origin = self.zoom_masks[l - 1]
                n, na = self.levels[l][1], self.levels[l - 1][1]
                p = [c // (n * n), (c // n) % n, c % n]
                q = [(p[a] // ratio + origin[a]) % na for a in range(3)]
                c, l = (q[0] * na + q[1]) * na + q[2], l - 1
        flags = self._flags()
        self.flagged_levels = [np.union1d(flags[l].astype(np.int64), np.array(add[l], dtype=np.int64)).astype(np.uint64)
                               for l in range(nl)]
        self.flagged = self.flagged_levels[-1]
        self._centre_on_flags()

    def id_file(self, fname):
        """ICGenerator::loadID: every flag cleared, then merge_id_file."""
        self.flagged_levels = [np.zeros(0, dtype=np.uint64) for _ in self.levels]
        self.merge_id_file(fname)

    IDfile = id_file
    append_IDfile = merge_id_file
    dump_IDfile = dump_id_file

    def dump_tipsy(self, fname):
        """ICGenerator::saveTipsyArray (ic.hpp:891-899, io/tipsy.hpp:39-52): the overdensity at
        every particle in mapper order, as floats after a 4-byte count."""
        lev, cells = self._order()
        nl = len(self.levels)
        deltas = [self.field(l, 'delta').ravel() for l in range(nl)]
        vals = np.empty(len(cells), dtype=np.float32)
        for l in np.unique(lev):
            sel = lev == l
            vals[sel] = deltas[min(int(l), nl - 1)][cells[sel]]
        with open(os.path.join(self.base_dir, fname), 'wb') as f:
            f.write(np.array([len(cells) & 0xffffffff], dtype='<u4').tobytes())
            f.write(vals.astype('<f4').tobytes())

    def _centre_on_flags(self):
        """ICGenerator::getCentre (ic.hpp:1374-1385) with Grid::getCentreWrapped (grid.hpp:466-494):
        on the deepest level with flags, the mean of the wrapped offsets from its first flagged
        cell's centroid, added back and wrapped into the box."""
        period = self.levels[0][0]
        deep = [l for l, f in enumerate(self.flagged_levels) if len(f)]
        if not deep:
            return
        l = deep[-1]
        box, n, off = self.levels[l]
        dx = box / n
        c = np.asarray(self.flagged_levels[l], dtype=np.int64)
        idx = (c // (n * n), (c // n) % n, c % n)
        centre = []
        for a in range(3):
            x = idx[a] * dx + off[a] + dx / 2
            run = 0.0
            for v in x[1:] - x[0]:
                if v > period / 2:
                    v -= period
                if v < -period / 2:
                    v += period
                run += v
            v = run / len(x) + x[0]
            v = float(np.fmod(v, period))
            centre.append(v + period if v < 0 else v)
        self.centre_point = tuple(centre)

    def select_sphere(self, radius):
        r2 = float(np.float32(radius) * np.float32(radius))
        self._select(lambda X, Y, Z: X * X + Y * Y + Z * Z < r2)

    def select_ellipse(self, a, b, c):
        """ICGenerator::selectEllipse (ic.hpp:1503-1513): semi-axes parsed as floats."""
        a2, b2, c2 = (float(np.float32(v) * np.float32(v)) for v in (a, b, c))
        self._select(lambda X, Y, Z: X * X / a2 + Y * Y / b2 + Z * Z / c2 < 1.)

    def select_cube(self, side):
        h = float(np.float32(side) / np.float32(2))
        self._select(lambda X, Y, Z: (np.abs(X) < h) & (np.abs(Y) < h) & (np.abs(Z) < h))

    # -- modifications (modificationmanager.hpp) ---------------------------------------
    # names as ModificationManager matches them, case-insensitively (modificationmanager.hpp:160-192)
    _KINDS = {'overdensity': _lib.GIC_MOD_OVERDENSITY, 'vx': _lib.GIC_MOD_VX, 'vy': _lib.GIC_MOD_VY,
              'vz': _lib.GIC_MOD_VZ, 'potential': _lib.GIC_MOD_POTENTIAL, 'lx': _lib.GIC_MOD_LX, 'ly': _lib.GIC_MOD_LY,
              'lz': _lib.GIC_MOD_LZ}

    def _kind(self, name):
        try:
            return self._KINDS[name.lower()]
        except KeyError:
            raise ValueError('%s is an unknown modification name' % name) from None

    def _cells(self):
        if self.flagged is None or len(self.flagged) == 0:
            raise RuntimeError('Linear modifications use exclusively information from the highest resolution grid '
                               'but no cells have been flagged on this grid.')
        return self.flagged.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)), len(self.flagged)

    # quadratic modifications: ic.hpp:150-161 (filtering scale, 10 initial steps, 0.001 precision)
    variance_filterscale = -1.0
    initial_number_steps = 10
    precision_target = 0.001

    def filtering_scale(self, scale):
        """setVarianceFilteringScale (ic.hpp:355-358), parsed as a double."""
        self.variance_filterscale = float(scale)

    def _level_cells(self):
        flagged = getattr(self, 'flagged_levels', None)
        if flagged is None or len(flagged) != len(self.levels):
            flagged = [np.zeros(0, dtype=np.uint64) for _ in self.levels]
        self._keep = flagged
        ptrs = (ctypes.c_void_p * len(flagged))(*[f.ctypes.data if len(f) else None for f in flagged])
        counts = (ctypes.c_size_t * len(flagged))(*[len(f) for f in flagged])
        return ptrs, counts

    def calculate(self, name):
        self.draw()
        v = ctypes.c_double()
        if name.lower() == 'variance':
            ptrs, counts = self._level_cells()
            self._call('gic_calculate_variance', ptrs, counts, self.variance_filterscale, ctypes.byref(v))
            return v.value
        cells, n = self._cells()
        self._call('gic_calculate', self._kind(name), cells, n, ctypes.byref(v))
        return v.value

    def modify(self, name, kind, target):
        """`modify name absolute|relative target`; genetIC parses the target as a float (ic.hpp:1613)."""
        self.draw()
        rel = {'relative': 1, 'absolute': 0}[kind.lower()]
        if name.lower() == 'variance':
            ptrs, counts = self._level_cells()
            self._call('gic_add_variance_modification', ptrs, counts, self.variance_filterscale,
                       float(np.float32(target)), rel, self.initial_number_steps, self.precision_target)
        else:
            cells, n = self._cells()
            self._call('gic_add_modification', self._kind(name), cells, n, float(np.float32(target)), rel)
        self._nmods = getattr(self, '_nmods', 0) + 1

    def clear_modifications(self):
        self._call('gic_clear_modifications')
        self._nmods = 0

    def apply_modifications(self):
        before, after = ctypes.c_double(), ctypes.c_double()
        self._call('gic_apply_modifications', ctypes.byref(before), ctypes.byref(after))
        self.last_chi2 = (before.value, after.value)
        return before.value, after.value

    # -- realisation -------------------------------------------------------------
    def draw(self):
        """initialiseAllRandomComponents (ic.hpp:1334-1352): draw, then the exact power
        spectrum if `fix_power` was given."""
        if self._drawn:
            return
        if self.seed is None:
            raise RuntimeError('The random number generator has not been seeded')
        self._call('gic_draw_noise', self.seed, self.seed_mode)
        if getattr(self, '_fix_power', False):
            self._call('gic_noise_op', _lib.GIC_NOISE_UNIT_MODULUS, 0.0)
        self._drawn = True

    def fix_power(self):
        """setExactPowerSpectrumEnforcement (ic.hpp:669-671)."""
        self._fix_power = True

    exact_power_spectrum_enforcement = fix_power

    def splice(self, new_seed):
        """ICGenerator::splice (ic.hpp:1658-1688): the flagged cells of every level take a
        new real-space white-noise draw; returns the CG iterations per level."""
        self.draw()
        ptrs, counts = self._level_cells()
        its = (ctypes.c_int * len(self.levels))()
        self._call('gic_splice', int(new_seed), ptrs, counts, its)
        return list(its)

    def zerolevel(self, level):
        """ICGenerator::zeroLevel (ic.hpp:787-802, a testing command): the drawn white noise of
        one level set to zero."""
        self.draw()
        level = int(level)
        if not 0 <= level < len(self.levels):
            raise ValueError('level %d does not exist' % level)
        n = self.levels[level][1]
        zeros = np.zeros(n * n * (n // 2 + 1) * 2, dtype=np.float64)
        self._call('gic_set_noise', level, _ptr(zeros))

    zero_level = zerolevel

    def reverse(self):
        """ICGenerator::reverse (ic.hpp:1652-1655): the white noise changes sign."""
        self.draw()
        self._call('gic_noise_op', _lib.GIC_NOISE_REVERSE, 0.0)

    def reverse_small_k(self, kmax):
        """ICGenerator::reverseSmallK (ic.hpp:1690-1705), kmax in h/Mpc."""
        self.draw()
        self._call('gic_noise_op', _lib.GIC_NOISE_REVERSE_SMALL_K, float(kmax))

    def done(self, apply_modifications=True, order=1):
        """Draw the noise if needed, apply the queued modifications, then P(k), the
        Zel'dovich fields and particles (ic.hpp:1633-1648); order=2 adds the
        second-order (2LPT) displacements, an extension genetIC does not have.  With an
        output format set (outformat), the particle file is written, as genetIC's done does."""
        self.draw()
        self._modified = False
        if apply_modifications and self._has_modifications():
            self.apply_modifications()
        self._call('gic_zeldovich', int(order))
        self._done = True
        if self.output_format is not None:
            self.write()

    # -- output (ic.hpp:735-760, 1275-1331; io.hpp:35-90) ----------------------------------
    _FORMATS = {'gadget2': 2, 'gadget3': 3, 'tipsy': 4, 'grafic': 5, 'gadgethdf': 6, 'swift': 7}

    def outdir(self, path):
        self.output_dir = str(path)

    def outname(self, name):
        self.output_name = str(name)

    def outformat(self, fmt):
        """A format by number (2-7) or name, as genetIC's OutputFormat reads it (io.hpp:66-90)."""
        s = str(fmt).strip().lower()
        v = int(s) if s.isdigit() else self._FORMATS.get(s)
        if v not in self._FORMATS.values():
            raise ValueError('Unknown output format %r' % fmt)
        self.output_format = v
        self._update_mapper()

    def output_path(self):
        """ICGenerator::getOutputPath (ic.hpp:753-760), relative to the paramfile's directory."""
        folder = os.path.join(self.base_dir, self.output_dir)
        if self.output_name:
            return os.path.join(folder, self.output_name)
        return os.path.join(folder, 'IC_%s_z%g_%d' % ('float' if self.precision == 'mixed' else 'doub',
                                                      self.cosmo['redshift'], self.levels[0][1]))

    def write(self):
        """The particle file in the chosen format (ICGenerator::write, ic.hpp:1275-1331): tipsy and
        gadget 2/3 are written here; the other formats are genetIC's own writers."""
        path = self.output_path()
        if self.output_format == 4:
            self.write_tipsy(path + '.tipsy')
        elif self.output_format in (2, 3):
            self.write_gadget(path + '.gadget%d' % self.output_format, self.output_format)
        else:
            name = {v: k for k, v in self._FORMATS.items()}[self.output_format]
            raise NotImplementedError('outformat %s is written by genetIC\'s own writer' % name)

    def _has_modifications(self):
        return getattr(self, '_nmods', 0) > 0

    def chi2(self):
        self.draw()
        v = ctypes.c_double()
        self._call('gic_chi2', ctypes.byref(v))
        return v.value

    # -- results -----------------------------------------------------------------
    def noise(self, level=0):
        n = self.levels[level][1]
        out = np.empty((n, n, n // 2 + 1, 2), dtype=np.float64)
        self._call('gic_fetch_level', level, _lib.GIC_FIELD_NOISE, _ptr(out))
        return out[..., 0] + 1j * out[..., 1]

    def field(self, level=0, name='delta'):
        what = {'delta': _lib.GIC_FIELD_DELTA, 'psi_x': _lib.GIC_FIELD_PSI_X, 'psi_y': _lib.GIC_FIELD_PSI_Y,
                'psi_z': _lib.GIC_FIELD_PSI_Z, 'psi2_x': _lib.GIC_FIELD_PSI2_X, 'psi2_y': _lib.GIC_FIELD_PSI2_Y,
                'psi2_z': _lib.GIC_FIELD_PSI2_Z}[name]
        n = self.levels[level][1]
        out = np.empty((n, n, n), dtype=np.float64)
        self._call('gic_fetch_level', level, what, _ptr(out))
        return out

    def particles(self, level=0):
        n = self.levels[level][1]
        pos = np.empty((n ** 3, 3), dtype=np.float64)
        vel = np.empty((n ** 3, 3), dtype=np.float64)
        self._call('gic_fetch_particles', level, _ptr(pos), _ptr(vel))
        return pos, vel

    def particles_native(self, level=0):
        """Positions (doubles) and velocities in the context's precision (float32 in the
        mixed form), as the device holds them."""
        n = self.levels[level][1]
        pos = np.empty((n ** 3, 3), dtype=np.float64)
        vel = np.empty((n ** 3, 3), dtype=np.float64 if self.precision == 'fp64' else np.float32)
        self._call('gic_fetch_particles_native', level, _ptr(pos), ctypes.c_void_p(vel.ctypes.data))
        return pos, vel

    def particles_resampled(self, level, factor):
        """Particles of `level` on genetIC's supersampled (factor >= 2) or subsampled
        (factor <= -2) virtual grid of the same region: (positions, velocities)."""
        n = self.levels[level][1]
        # sizes the library refuses get a one-particle buffer: the call reports the error
        nv = n * factor if factor > 1 else (n // -factor if factor < -1 else 1)
        nv = nv if nv <= 2048 else 1
        pos = np.empty((nv ** 3, 3), dtype=np.float64)
        vel = np.empty((nv ** 3, 3), dtype=np.float64)
        self._call('gic_fetch_particles_resampled', level, int(factor), _ptr(pos), _ptr(vel))
        return pos, vel

    def particles_matched(self, level, cells):
        """Particles of the listed cells of `level`'s resolution-matching grid (genetIC's
        output grid of a zoom level with strays on): (positions, velocities)."""
        cells = np.ascontiguousarray(cells, dtype=np.uint64)
        pos = np.empty((len(cells), 3), dtype=np.float64)
        vel = np.empty((len(cells), 3), dtype=np.float64)
        self._call('gic_fetch_particles_matched', level, cells.ctypes.data_as(ctypes.POINTER(ctypes.c_ulonglong)),
                   len(cells), _ptr(pos), _ptr(vel))
        return pos, vel

    # -- particle files (io/tipsy.hpp, io/gadget.hpp) ------------------------------------
    def particle_map(self):
        """The gic_particle_map of this context: genetIC's particle-mapper order over the zoom
        masks, with the flagged particles' own gadget type as one more level when it is set."""
        flagged = self._flagged_snapshot if getattr(self, '_flagged_type', None) is not None else None
        return writers.particle_map(self.levels, self.zoom_masks, self.cosmo, flagged)

    def _host_particles(self, nlevels):
        # a map level past the context's levels is the flagged particles of the finest level
        parts = [self.particles(min(l, len(self.levels) - 1)) for l in range(nlevels)]
        P = ctypes.POINTER(ctypes.c_double)
        pos = (P * nlevels)(*[p.ctypes.data_as(P) for p, _ in parts])
        vel = (P * nlevels)(*[v.ctypes.data_as(P) for _, v in parts])
        return parts, pos, vel

    def tipsy_records(self):
        """The tipsy dark-matter records (n x 9 float32) in mapper order, packed on the device
        for one or two levels and by host threads for more."""
        m = self.particle_map()
        n = ctypes.c_ulonglong()
        check(None, self._lib.gic_tipsy_count(ctypes.byref(m), ctypes.byref(n)))
        out = np.empty((n.value, 9), dtype=np.float32)
        if m.nlevels <= 2:
            self._call('gic_tipsy_pack', ctypes.byref(m), 0, n.value, out.ctypes.data_as(ctypes.c_void_p))
        else:
            keep, pos, vel = self._host_particles(m.nlevels)
            check(None, self._lib.gic_tipsy_pack_host(ctypes.byref(m), pos, vel, 0, n.value,
                                                      out.ctypes.data_as(ctypes.c_void_p), 0))
        return out

    def write_tipsy(self, path):
        """The particles as genetIC's tipsy file (TipsyOutput, tipsy.hpp:200-262)."""
        writers.write_tipsy(path, 1.0 / (1.0 + self.cosmo['redshift']), self.tipsy_records())

    def write_gadget(self, path, version=2):
        """The particles as genetIC's single-file gadget snapshot, every level of particle
        type 1 (GadgetOutput, gadget.hpp:481-520): float positions and velocities, ids, and
        the mass block when the levels' masses differ."""
        m = self.particle_map()
        n = ctypes.c_ulonglong()
        check(None, self._lib.gic_tipsy_count(ctypes.byref(m), ctypes.byref(n)))
        keep, pos, vel = self._host_particles(m.nlevels)
        pos3 = np.empty((n.value, 3), dtype=np.float32)
        vel3 = np.empty((n.value, 3), dtype=np.float32)
        ids = np.empty(n.value, dtype=np.uint64)
        mass = np.empty(n.value, dtype=np.float32)
        ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)  # noqa: E731
        types = list(getattr(self, 'gadget_types', [])) or [1] * len(self.levels)
        if getattr(self, '_flagged_type', None) is not None:
            types.append(self._flagged_type)
        tarr = (ctypes.c_int * m.nlevels)(*types)
        check(None, self._lib.gic_gadget_pack_host(ctypes.byref(m), pos, vel, tarr, 0, n.value, ptr(pos3), ptr(vel3),
                                                   ptr(ids), ptr(mass), 0))
        npart, masses = writers.gadget_type_counts(m, types)
        variable = masses is None
        c = self.cosmo
        nfiles = getattr(self, 'gadget_files', 1)
        per_file, per_type = writers.gadget_file_split(npart, nfiles)
        at = 0
        for i, (nf, counts) in enumerate(zip(per_file, per_type)):
            # the header's counts are this file's; the totals and the file count are the run's
            h = bytearray(writers.gadget_header(version, npart, [0.0] * 6 if variable else masses,
                                                1.0 / (1.0 + c['redshift']), c['redshift'], self.levels[0][0],
                                                c['omega_m'], c['omega_lambda'], c['hubble'], num_files=nfiles))
            h[0:24] = np.array(counts, dtype='<u4').tobytes()
            s = slice(at, at + nf)
            writers.write_gadget(path if nfiles == 1 else '%s.%d' % (path, i), bytes(h), pos3[s], vel3[s], ids[s],
                                 mass[s] if variable else None)
            at += nf

    def gaussian_stream(self, seed, count):
        out = np.empty(int(count), dtype=np.float64)
        self._call('gic_gaussian_stream', int(seed), int(count), _ptr(out))
        return out


_COMMANDS = {
    'Om': 'Om', 'Ol': 'Ol', 'Ob': 'Ob', 'hubble': 'hubble', 's8': 's8', 'ns': 'ns', 'zin': 'zin',
    'camb': 'camb', 'basegrid': 'base_grid', 'base_grid': 'base_grid',
    'zoomgrid_with_origin_at': 'zoom_grid_with_origin_at', 'zoom_grid_with_origin_at': 'zoom_grid_with_origin_at',
    'zoomgrid': 'zoom_grid', 'zoom_grid': 'zoom_grid',
    'random_seed': 'random_seed', 'seedfourier_parallel': 'random_seed',
    'random_seed_serial': 'random_seed_serial', 'seedfourier': 'random_seed_serial',
    'random_seed_real_space': 'random_seed_real_space', 'seed': 'random_seed_real_space',
    'seedfourier_reverse': 'seedfourier_reverse', 'done': 'done', 'chi2': 'chi2',
    'centre': 'centre', 'center': 'centre', 'select_sphere': 'select_sphere', 'select_cube': 'select_cube',
    'select_ellipse': 'select_ellipse', 'select_nearest': 'select_nearest',
    'zerolevel': 'zerolevel', 'zero_level': 'zerolevel',
    'IDfile': 'id_file', 'id_file': 'id_file', 'append_IDfile': 'merge_id_file', 'merge_id_file': 'merge_id_file',
    'dump_IDfile': 'dump_id_file', 'dump_id_file': 'dump_id_file', 'dump_tipsy': 'dump_tipsy',
    'calculate': 'calculate', 'modify': 'modify', 'clear_modifications': 'clear_modifications',
    'filtering_scale': 'filtering_scale', 'fix_power': 'fix_power',
    'exact_power_spectrum_enforcement': 'fix_power', 'reverse': 'reverse', 'reverse_small_k': 'reverse_small_k',
    'splice': 'splice',
    'apply_modifications': 'apply_modifications',
    'outname': 'outname', 'outdir': 'outdir', 'outformat': 'outformat',
    'gadget_particle_type': 'gadget_particle_type', 'gadget_num_files': 'gadget_num_files', 'gadget_flagged_particle_type': 'gadget_flagged_particle_type',
}
# output-side commands handled by genetIC's own writers; accepted and ignored here
_IGNORED = {'dump_grid', 'dump_ps'}


_COMMANDS_LOWER = {k.lower(): v for k, v in _COMMANDS.items()}
_IGNORED_LOWER = {k.lower() for k in _IGNORED}


def parse_paramfile(path):
    """(line number, method, args) for each realisation command of a paramfile."""
    out = []
    with open(path) as f:
        for lineno, line in enumerate(f, 1):
            line = line.split('#')[0].strip()
            if not line:
                continue
            parts = line.split()
            # genetIC matches command names case-insensitively (tools/parser.hpp:171, 243)
            cmd, args = parts[0].lower(), parts[1:]
            if cmd in _IGNORED_LOWER:
                continue
            if cmd not in _COMMANDS_LOWER:
                raise ValueError('%s:%d: command %r is not on the GPU realisation path' % (path, lineno, parts[0]))
            out.append((lineno, _COMMANDS_LOWER[cmd], args))
    return out


def run_paramfile(path, precision='fp64', device=0):
    """Run a genetIC paramfile's realisation commands on the GPU; returns the ICGenerator."""
    commands = parse_paramfile(path)
    gen = ICGenerator(precision=precision, device=device)
    gen.base_dir = os.path.dirname(os.path.abspath(path))
    for lineno, method, args in commands:
        getattr(gen, method)(*args)
    return gen
