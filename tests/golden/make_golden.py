"""Regenerate the golden fixtures in this directory from the reference build.

Runs oracle/_ref/genetIC (genetIC's own sources built by oracle/Makefile) on
32^3 BBKS realisations in a 50 Mpc/h box at z = 99 (seed 8896131) in the three
seeding modes and stores the reference's real-space delta grid (dump_grid) and
its tipsy particle positions converted to Mpc/h.

Run:  python tests/golden/make_golden.py   (needs the reference sources)
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'oracle'))
from genetic_gb300.transfer import bbks_table, write_camb  # noqa: E402
from tipsy_reader import read_tipsy  # noqa: E402

REF_BIN = os.path.join(ROOT, 'oracle', '_ref', 'genetIC')
PARAMS = """Om 0.31
Ol 0.69
Ob 0
hubble 0.68
s8 0.81
ns 0.965
zin 99
{seedcmd} 8896131
camb bbks.dat
outname out
outdir ./
outformat tipsy
basegrid 50.0 32
done
dump_grid 0
"""


ZOOM_PARAMS = """Om 0.31
Ol 0.69
Ob 0
hubble 0.68
s8 0.81
ns 0.965
zin 99
{seedcmd} 8896131
camb bbks.dat
outname out
outdir ./
outformat tipsy
basegrid 50.0 32
centre 25 25 25
select_cube 10
{zooms}
done
{dumps}
"""
ZOOMS = {
    # two levels: a 25 Mpc/h zoom (factor 2) at coarse cell (8, 8, 8) around the
    # flagged 10 Mpc/h cube at the box centre
    'zoom2': ['zoom_grid_with_origin_at 8 8 8 2 32'],
    # three levels: a further factor-2 zoom inside the first
    'zoom3': ['zoom_grid_with_origin_at 8 8 8 2 32', 'zoom_grid_with_origin_at 8 8 8 2 32'],
}


def zoom_goldens():
    for name, zooms in ZOOMS.items():
        for mode, cmd in (('parallel', 'random_seed'), ('real', 'random_seed_real_space')):
            if name == 'zoom3' and mode == 'real':
                continue
            with tempfile.TemporaryDirectory() as d:
                write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
                dumps = '\n'.join('dump_grid %d' % l for l in range(len(zooms) + 1))
                open(os.path.join(d, 'paramfile.txt'), 'w').write(
                    ZOOM_PARAMS.format(seedcmd=cmd, zooms='\n'.join(zooms), dumps=dumps))
                subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
                grids = {'delta%d' % l: np.load(os.path.join(d, 'grid-%d.npy' % l)) for l in range(len(zooms) + 1)}
                if name == 'zoom3':
                    grids = {k: v.astype(np.float32) for k, v in grids.items()}
                np.savez_compressed(os.path.join(HERE, '%s_%s.npz' % (name, mode)), **grids)


MOD_BASE = """Om 0.31
Ol 0.69
Ob 0
hubble 0.68
s8 0.81
ns 0.965
zin 99
random_seed 8896131
camb bbks.dat
outname out
outdir ./
outformat tipsy
basegrid 50.0 32
"""
MODS = {
    # one level: 5 Mpc/h sphere at the centre, mean overdensity 0.05 and vx = 0
    'mod1': """centre 25 25 25
select_sphere 5
calculate overdensity
calculate vx
modify overdensity absolute 0.05
modify vx absolute 0
chi2
done
dump_grid 0
""",
    # two levels: zoom factor 2 around the centre, 3 Mpc/h sphere, overdensity 0.05 and vx = vy = vz = 0
    'mod2': """centre 25 25 25
select_cube 10
zoom_grid_with_origin_at 8 8 8 2 32
centre 25 25 25
select_sphere 3
calculate overdensity
calculate vx
modify overdensity absolute 0.05
modify vx absolute 0
modify vy absolute 0
modify vz absolute 0
done
dump_grid 0
dump_grid 1
""",
}


def mod_goldens():
    import re
    for name, tail in MODS.items():
        with tempfile.TemporaryDirectory() as d:
            write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
            open(os.path.join(d, 'paramfile.txt'), 'w').write(MOD_BASE + tail)
            r = subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True, text=True)
            log = r.stdout + r.stderr
            vals = {}
            for key, pat in (('overdensity', r'overdensity: calculated value = (\S+)'),
                             ('vx', r'vx: calculated value = (\S+)'),
                             ('chi2_post', r'Post-modification chi\^2 = (\S+)'),
                             ('delta_chi2', r'Modification Delta chi\^2 = (\S+)')):
                m = re.search(pat, log)
                vals[key] = float(m.group(1))
            nlev = 2 if name == 'mod2' else 1
            grids = {'delta%d' % l: np.load(os.path.join(d, 'grid-%d.npy' % l)).astype(np.float32) for l in range(nlev)}
            np.savez_compressed(os.path.join(HERE, '%s.npz' % name), **grids,
                                **{k: np.array(v) for k, v in vals.items()})


VARS = {
    # one level: variance of the 4 Mpc/h high-passed overdensity in an 8 Mpc/h sphere,
    # with the mean overdensity held and the variance tripled (20 steps after the trial)
    'var1': """centre 25 25 25
select_sphere 8
filtering_scale 4
calculate variance
calculate overdensity
modify overdensity relative 1
modify variance relative 3
done
dump_grid 0
""",
    # two levels: zoom factor 2 around the centre; 4 Mpc/h sphere flagged on both levels
    'var2': """centre 25 25 25
select_cube 10
zoom_grid_with_origin_at 8 8 8 2 32
centre 25 25 25
select_sphere 4
filtering_scale 3
calculate variance
calculate overdensity
modify overdensity relative 1
modify variance relative 1.5
done
dump_grid 0
dump_grid 1
""",
}


def var_goldens():
    import re
    for name, tail in VARS.items():
        with tempfile.TemporaryDirectory() as d:
            write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
            open(os.path.join(d, 'paramfile.txt'), 'w').write(MOD_BASE + tail)
            r = subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True, text=True)
            log = r.stdout + r.stderr
            vals = {}
            for key, pat in (('variance', r'variance: calculated value = (\S+)'),
                             ('overdensity', r'overdensity: calculated value = (\S+)'),
                             ('chi2_post', r'Post-modification chi\^2 = (\S+)'),
                             ('delta_chi2', r'Modification Delta chi\^2 = (\S+)')):
                vals[key] = float(re.search(pat, log).group(1))
            m = re.search(r'(\d+) steps are required for the quadratic algorithm', log)
            vals['steps'] = int(m.group(1)) if m else 10
            nlev = 2 if name == 'var2' else 1
            grids = {'delta%d' % l: np.load(os.path.join(d, 'grid-%d.npy' % l)) for l in range(nlev)}
            np.savez_compressed(os.path.join(HERE, '%s.npz' % name), **grids,
                                **{k: np.array(v) for k, v in vals.items()})


OPS = {
    # noise operations on one level and on two (the zoom2 geometry)
    'ops_reverse': (['reverse'], 1),
    'ops_reverse_small_k': (['reverse_small_k 0.5'], 1),
    'ops_fix_power': (['fix_power'], 1),
    'ops_reverse_small_k_zoom': (['reverse_small_k 0.7'], 2),
    'ops_fix_power_zoom': (['fix_power'], 2),
}


def ops_goldens():
    for name, (cmds, nlev) in OPS.items():
        with tempfile.TemporaryDirectory() as d:
            write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
            zoom = 'centre 25 25 25\nselect_cube 10\nzoom_grid_with_origin_at 8 8 8 2 32\n' if nlev == 2 else ''
            body = (MOD_BASE + zoom + '\n'.join(cmds) + '\ndone\n' +
                    ''.join('dump_grid %d\n' % l for l in range(nlev)))
            # fix_power must precede the first draw: put it before the grid commands' draw
            open(os.path.join(d, 'paramfile.txt'), 'w').write(body)
            subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
            grids = {'delta%d' % l: np.load(os.path.join(d, 'grid-%d.npy' % l)) for l in range(nlev)}
            np.savez_compressed(os.path.join(HERE, '%s.npz' % name), **grids)


MODS_MORE = {
    # potential and angular momentum, one level and a factor-2 zoom
    'mod_pot1': ("""centre 25 25 25
select_sphere 5
calculate potential
modify potential relative 2
done
dump_grid 0
""", 1),
    'mod_am1': ("""centre 25 25 25
select_ellipse 10 7.5 5
calculate Ly
calculate Lz
modify Ly absolute 100
modify Lz relative 0.5
done
dump_grid 0
""", 1),
    'mod_am2': ("""centre 25 25 25
select_cube 10
zoom_grid_with_origin_at 8 8 8 2 32
center 25.3 24.8 25
select_sphere 4
calculate Lx
calculate potential
modify Lx absolute 50
modify potential absolute 0
done
dump_grid 0
dump_grid 1
""", 2),
}


def mod_more_goldens():
    import re
    for name, (tail, nlev) in MODS_MORE.items():
        with tempfile.TemporaryDirectory() as d:
            write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
            open(os.path.join(d, 'paramfile.txt'), 'w').write(MOD_BASE + tail)
            r = subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True, text=True)
            log = r.stdout + r.stderr
            vals = {}
            for key in ('potential', 'Lx', 'Ly', 'Lz'):
                m = re.search(r'%s: calculated value = (\S+)' % key, log)
                if m:
                    vals[key] = float(m.group(1))
            vals['delta_chi2'] = float(re.search(r'Modification Delta chi\^2 = (\S+)', log).group(1))
            grids = {'delta%d' % l: np.load(os.path.join(d, 'grid-%d.npy' % l)) for l in range(nlev)}
            np.savez_compressed(os.path.join(HERE, '%s.npz' % name), **grids, **{k: np.array(v) for k, v in vals.items()})


SPLICES = {
    'splice1': ("""centre 25 25 25
select_sphere 8
splice 8896132
done
dump_grid 0
""", 1),
    'splice2': ("""centre 25 25 25
select_cube 10
zoom_grid_with_origin_at 8 8 8 2 32
centre 25 25 25
select_sphere 5
splice 8896132
done
dump_grid 0
dump_grid 1
""", 2),
}


def splice_goldens():
    import re
    for name, (tail, nlev) in SPLICES.items():
        with tempfile.TemporaryDirectory() as d:
            write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
            open(os.path.join(d, 'paramfile.txt'), 'w').write(MOD_BASE + tail)
            r = subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True, text=True)
            its = [int(v) for v in re.findall(r'Conjugate gradient ended after (\d+) iterations', r.stdout + r.stderr)]
            grids = {'delta%d' % l: np.load(os.path.join(d, 'grid-%d.npy' % l)) for l in range(nlev)}
            np.savez_compressed(os.path.join(HERE, '%s.npz' % name), **grids, iterations=np.array(its))


def tipsy_goldens():
    """The reference's tipsy file of the two-level zoom2 case (random_seed): header and dark records."""
    with tempfile.TemporaryDirectory() as d:
        write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
        open(os.path.join(d, 'paramfile.txt'), 'w').write(
            ZOOM_PARAMS.format(seedcmd='random_seed', zooms='\n'.join(ZOOMS['zoom2']), dumps=''))
        subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
        raw = open(os.path.join(d, 'out.tipsy'), 'rb').read()
        header = np.frombuffer(raw[8:28], '<i4').copy()
        t, _, dark = read_tipsy(os.path.join(d, 'out.tipsy'))
        np.savez_compressed(os.path.join(HERE, 'tipsy_zoom2.npz'), scalefactor=np.float64(t), header=header, dark=dark,
                            header_bytes=np.frombuffer(raw[:28], np.uint8).copy())


def gadget_types_goldens():
    """The reference's gadget2 file of the zoom2 case with gadget particle types: level 0 of
    type 3, the zoom level of type 1, so the file holds the zoom's particles first: header
    bytes, ids and every 97th position."""
    with tempfile.TemporaryDirectory() as d:
        write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
        params = ZOOM_PARAMS.format(seedcmd='random_seed', zooms='gadget_particle_type 3\n' + '\n'.join(ZOOMS['zoom2'])
                                    + '\ngadget_particle_type 1', dumps='')
        open(os.path.join(d, 'paramfile.txt'), 'w').write(params.replace('outformat tipsy', 'outformat gadget2'))
        subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
        # one mass per type: the masses are in the header and there is no mass block
        header, pos, vel, ids = read_fortran_records(os.path.join(d, 'out.gadget2'))
        np.savez_compressed(os.path.join(HERE, 'gadget_types_zoom2.npz'), header_bytes=np.frombuffer(header, np.uint8).copy(),
                            ids=np.frombuffer(ids, '<u8').copy(), pos97=np.frombuffer(pos, '<f4').reshape(-1, 3)[::97].copy())


def flagged_type_goldens():
    """The zoom2 case with the finest level's cells in a 3 Mpc/h sphere given gadget type 4:
    genetIC moves them to the end of the particle order.  The gadget2 file (header bytes,
    ids, every 97th position) and the tipsy file (header bytes, every 37th record, the last
    400 records)."""
    out = {}
    for fmt in ('gadget2', 'tipsy'):
        with tempfile.TemporaryDirectory() as d:
            write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
            zooms = '\n'.join(ZOOMS['zoom2']) + '\ncentre 25 25 25\nselect_sphere 3\ngadget_flagged_particle_type 4'
            params = ZOOM_PARAMS.format(seedcmd='random_seed', zooms=zooms, dumps='')
            open(os.path.join(d, 'paramfile.txt'), 'w').write(params.replace('outformat tipsy', 'outformat ' + fmt))
            subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
            if fmt == 'tipsy':
                raw = open(os.path.join(d, 'out.tipsy'), 'rb').read()
                _, _, dark = read_tipsy(os.path.join(d, 'out.tipsy'))
                out.update(tipsy_header=np.frombuffer(raw[:28], np.uint8).copy(), tipsy37=dark[::37].copy(),
                           tipsy_tail=dark[-400:].copy())
            else:
                rec = read_fortran_records(os.path.join(d, 'out.gadget2'))
                out.update(gadget_header=np.frombuffer(rec[0], np.uint8).copy(), gadget_ids=np.frombuffer(rec[3], '<u8').copy(),
                           gadget_pos97=np.frombuffer(rec[1], '<f4').reshape(-1, 3)[::97].copy(), gadget_nrec=np.int64(len(rec)))
                if len(rec) > 4:
                    out['gadget_mass'] = np.frombuffer(rec[4], '<f4').copy()
    np.savez_compressed(os.path.join(HERE, 'flagged_type_zoom2.npz'), **out)


ZOOM_GRID_CASES = {
    # flagged cube at the centre, one zoom
    'centre': 'centre 25 25 25\nselect_cube 10\nzoom_grid 2 32',
    # a sphere across the periodic corner: the window wraps
    'wrap': 'centre 2 2 48\nselect_sphere 5\nzoom_grid 4 32',
    # two nested zooms; the second is moved inside the first
    'nested': 'centre 30 28 25\nselect_sphere 6\nzoom_grid 2 32\ncentre 32 27 25\nselect_sphere 2\nzoom_grid 2 32',
}


def zoom_grid_goldens():
    """The lower corners genetIC's zoom_grid chooses (its log's "Low-left corner in parent
    grid"), for ZOOM_GRID_CASES on a 32^3, 50 Mpc/h base."""
    import re
    out = {}
    for name, cmds in ZOOM_GRID_CASES.items():
        with tempfile.TemporaryDirectory() as d:
            write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
            params = PARAMS.format(seedcmd='random_seed').replace('done\ndump_grid 0\n', cmds + '\n')
            open(os.path.join(d, 'paramfile.txt'), 'w').write(params)
            r = subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True, text=True)
            corners = re.findall(r'Low-left corner in parent grid = \((-?\d+), (-?\d+), (-?\d+)\)', r.stdout + r.stderr)
            out[name] = np.array([[int(v) for v in c] for c in corners])
    np.savez_compressed(os.path.join(HERE, 'zoom_grid_corners.npz'), **out)


ID_FILE_IN = [0, 5, 100, 32552 + 3, 32552 + 1000, 34000]


def id_file_goldens():
    """genetIC's particle ID files on the zoom2 case: the ids it dumps for a 3 Mpc/h sphere,
    and, after loading ID_FILE_IN, the ids it dumps back and the centre it logs."""
    import re
    out = {}
    cases = {'dump': 'centre 25 25 25\nselect_sphere 3\ndump_IDfile ids.txt',
             'load': 'IDfile in.txt\ndump_IDfile ids.txt'}
    for name, cmds in cases.items():
        with tempfile.TemporaryDirectory() as d:
            write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
            open(os.path.join(d, 'in.txt'), 'w').write(''.join('%d\n' % i for i in ID_FILE_IN))
            params = ZOOM_PARAMS.format(seedcmd='random_seed', zooms='\n'.join(ZOOMS['zoom2']) + '\n' + cmds, dumps='')
            open(os.path.join(d, 'paramfile.txt'), 'w').write(params)
            r = subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True, text=True)
            out[name + '_ids'] = np.loadtxt(os.path.join(d, 'ids.txt'), dtype=np.int64, ndmin=1)
            centres = re.findall(r'Centre of region is (\S+) (\S+) (\S+)', r.stdout + r.stderr)
            if centres:
                out[name + '_centre'] = np.array([float(v) for v in centres[-1]])
    np.savez_compressed(os.path.join(HERE, 'id_files_zoom2.npz'), **out)


def dump_tipsy_goldens():
    """genetIC's dump_tipsy of the zoom2 case after done: the overdensity of every particle in
    mapper order (a 4-byte count, then floats)."""
    with tempfile.TemporaryDirectory() as d:
        write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
        params = ZOOM_PARAMS.format(seedcmd='random_seed', zooms='\n'.join(ZOOMS['zoom2']), dumps='dump_tipsy field.tipsy')
        open(os.path.join(d, 'paramfile.txt'), 'w').write(params)
        subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
        raw = open(os.path.join(d, 'field.tipsy'), 'rb').read()
        np.savez_compressed(os.path.join(HERE, 'dump_tipsy_zoom2.npz'), raw=np.frombuffer(raw, np.uint8).copy())


def gadget_files_goldens():
    """The zoom2 case written over 3 gadget2 files: each file's header bytes and ids."""
    out = {}
    with tempfile.TemporaryDirectory() as d:
        write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
        params = ZOOM_PARAMS.format(seedcmd='random_seed', zooms='\n'.join(ZOOMS['zoom2']) + '\ngadget_num_files 3', dumps='')
        open(os.path.join(d, 'paramfile.txt'), 'w').write(params.replace('outformat tipsy', 'outformat gadget2'))
        subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
        for i in range(3):
            rec = read_fortran_records(os.path.join(d, 'out.gadget2.%d' % i))
            out['header%d' % i] = np.frombuffer(rec[0], np.uint8).copy()
            out['ids%d' % i] = np.frombuffer(rec[3], '<u8').copy()
            out['nrec%d' % i] = np.int64(len(rec))
    np.savez_compressed(os.path.join(HERE, 'gadget_files_zoom2.npz'), **out)


def tipsy3_goldens():
    """The reference's tipsy file of the three-level zoom3 case: its header and the records
    of the finest level (the level-1 particles are all replaced), which follow the level-1
    cell ids of their parents."""
    with tempfile.TemporaryDirectory() as d:
        write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
        open(os.path.join(d, 'paramfile.txt'), 'w').write(
            ZOOM_PARAMS.format(seedcmd='random_seed', zooms='\n'.join(ZOOMS['zoom3']), dumps=''))
        subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
        raw = open(os.path.join(d, 'out.tipsy'), 'rb').read()
        header = np.frombuffer(raw[8:28], '<i4').copy()
        _, _, dark = read_tipsy(os.path.join(d, 'out.tipsy'))
        first = 32 ** 3 - 216
        np.savez_compressed(os.path.join(HERE, 'tipsy_zoom3.npz'), header=header, first=np.int64(first),
                            head=dark[:64].copy(), tail=dark[first:].copy())


def read_fortran_records(path):
    """The records of a Fortran-framed binary file (int32 length before and after each)."""
    raw = open(path, 'rb').read()
    recs, off = [], 0
    while off < len(raw):
        n = int(np.frombuffer(raw[off:off + 4], '<i4')[0])
        recs.append(raw[off + 4:off + 4 + n])
        assert int(np.frombuffer(raw[off + 4 + n:off + 8 + n], '<i4')[0]) == n
        off += n + 8
    return recs


def gadget_goldens():
    """The reference's gadget2 file of the zoom2 case: positions, velocities and masses
    (every level is gadget type 1; the id block is checked to hold 0..n-1)."""
    with tempfile.TemporaryDirectory() as d:
        write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
        params = ZOOM_PARAMS.format(seedcmd='random_seed', zooms='\n'.join(ZOOMS['zoom2']), dumps='')
        open(os.path.join(d, 'paramfile.txt'), 'w').write(params.replace('outformat tipsy', 'outformat gadget2'))
        subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
        header, pos, vel, ids, mass = read_fortran_records(os.path.join(d, 'out.gadget2'))
        # the same run written as gadget3: its header
        open(os.path.join(d, 'paramfile.txt'), 'w').write(params.replace('outformat tipsy', 'outformat gadget3'))
        subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
        header3 = read_fortran_records(os.path.join(d, 'out.gadget3'))[0]
        npart = np.frombuffer(header[:24], '<i4')
        ids = np.frombuffer(ids, '<u8')
        assert np.array_equal(ids, np.arange(len(ids)))
        np.savez_compressed(os.path.join(HERE, 'gadget_zoom2.npz'), npart=npart.copy(),
                            header_bytes=np.frombuffer(header, np.uint8).copy(),
                            header3_bytes=np.frombuffer(header3, np.uint8).copy(),
                            header_mass=np.frombuffer(header[24:72], '<f8').copy(),
                            pos=np.frombuffer(pos, '<f4').reshape(-1, 3), vel=np.frombuffer(vel, '<f4').reshape(-1, 3),
                            mass=np.frombuffer(mass, '<f4'))


# The headline's geometry at sizes the reference build finishes in seconds: zoom factor 4
# (the compiled ratio-4 block means and interpolation), factor 3 with an integer number of
# coarse cells under the zoom (the generic-ratio block means; a 72 Mpc/h, 48^3 base) and factor 3 over a fractional
# number of them (genetIC's test_01c geometry: 32 fine cells over 10 2/3 coarse ones), with
# the headline's four modifications in a 2 Mpc/h sphere and the variance modification of the
# differentiation configuration (3 Mpc/h filter, 5 Mpc/h sphere, variance x 1.3).
GEOMETRY = {
    'zoom4': ('basegrid 50.0 32', 'centre 25 25 25\nselect_cube 10\nzoom_grid_with_origin_at 12 12 12 4 32', 2, ''),
    'zoom3f': ('basegrid 50.0 32', 'centre 25 25 25\nselect_cube 10\nzoom_grid_with_origin_at 11 11 11 3 32', 2, ''),
    'mod4': ('basegrid 50.0 32', 'centre 25 25 25\nselect_cube 10\nzoom_grid_with_origin_at 12 12 12 4 32', 2,
             """centre 25 25 25
select_sphere 2
calculate overdensity
calculate vx
calculate vy
calculate vz
modify overdensity absolute 1.5
modify vx absolute 0
modify vy absolute 0
modify vz absolute 0
"""),
    # dx = 1.5 and 0.5 Mpc/h, exact in binary: with thirds of a cell (50 Mpc/h over 48 cells)
    # the reference build's own grid containment assertion fails
    'mod3': ('basegrid 72.0 48', 'centre 36 36 36\nselect_cube 10\nzoom_grid_with_origin_at 16 16 16 3 48', 2,
             """centre 36 36 36
select_sphere 2
calculate overdensity
calculate vx
calculate vy
calculate vz
modify overdensity absolute 1.5
modify vx absolute 0
modify vy absolute 0
modify vz absolute 0
"""),
    'var4': ('basegrid 50.0 32', 'centre 25 25 25\nselect_cube 10\nzoom_grid_with_origin_at 12 12 12 4 32', 2,
             """centre 25 25 25
select_sphere 5
filtering_scale 3
calculate variance
calculate overdensity
modify overdensity relative 1
modify variance relative 1.3
"""),
}


def geometry_goldens():
    """Reference-build grids (float64), logged calculated values, chi^2 change and quadratic
    step counts of the GEOMETRY cases (random_seed 8896131)."""
    import re
    for name, (base, zoom, nlev, mods) in GEOMETRY.items():
        with tempfile.TemporaryDirectory() as d:
            write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
            body = MOD_BASE.replace('basegrid 50.0 32', base) + zoom + '\n' + mods + 'done\n' + ''.join(
                'dump_grid %d\n' % l for l in range(nlev))
            open(os.path.join(d, 'paramfile.txt'), 'w').write(body)
            r = subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True, text=True)
            log = r.stdout + r.stderr
            vals = {}
            for key in ('overdensity', 'vx', 'vy', 'vz', 'variance'):
                m = re.search(r'%s: calculated value = (\S+)' % key, log)
                if m:
                    vals[key] = float(m.group(1))
            m = re.search(r'Modification Delta chi\^2 = (\S+)', log)
            if m:
                vals['delta_chi2'] = float(m.group(1))
            m = re.search(r'(\d+) steps are required for the quadratic algorithm', log)
            if 'variance' in mods:
                vals['steps'] = int(m.group(1)) if m else 10
            grids = {'delta%d' % l: np.load(os.path.join(d, 'grid-%d.npy' % l)) for l in range(nlev)}
            np.savez_compressed(os.path.join(HERE, 'geom_%s.npz' % name), **grids,
                                **{k: np.array(v) for k, v in vals.items()})


# genetIC's supersample / subsample: particles of virtual grids (tipsy records).  A 16^3 base
# supersampled x2, a 32^3 base subsampled x2, and the zoom2 geometry with its zoom level
# supersampled x2 (the finest level is the one genetIC supersamples).
RESAMPLE = {
    'super1': ('basegrid 50.0 16', 'supersample 2', 3),
    'sub1': ('basegrid 50.0 32', 'subsample 2', 1),
    'superzoom': ('basegrid 50.0 32\ncentre 25 25 25\nselect_cube 10\nzoom_grid_with_origin_at 8 8 8 2 32', 'supersample 2',
                  37),
}


def resample_goldens():
    """Header bytes and dark records (every `stride`-th, plus the last 400) of the reference's
    tipsy files with supersampling or subsampling."""
    for name, (grids, cmd, stride) in RESAMPLE.items():
        with tempfile.TemporaryDirectory() as d:
            write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
            body = MOD_BASE.replace('basegrid 50.0 32', grids) + cmd + '\ndone\n'
            open(os.path.join(d, 'paramfile.txt'), 'w').write(body)
            subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
            raw = open(os.path.join(d, 'out.tipsy'), 'rb').read()
            _, _, dark = read_tipsy(os.path.join(d, 'out.tipsy'))
            np.savez_compressed(os.path.join(HERE, 'resample_%s.npz' % name), header_bytes=np.frombuffer(raw[:28], np.uint8).copy(),
                                nrec=np.int64(len(dark)), stride=np.int64(stride), every=dark[::stride].copy(),
                                tail=dark[-400:].copy())


def strays_goldens():
    """genetIC with stray particles on: a factor-4 zoom at cell (15, 15, 12) of a 32^3 base
    whose flagged 3 Mpc/h sphere reaches outside the zoom window (genetIC's test_06a
    geometry, Fourier seeding).  Header bytes and dark records (every 7th and the last 400)."""
    with tempfile.TemporaryDirectory() as d:
        write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
        body = 'strays_on\n' + MOD_BASE + 'centre 25 25 25\nselect_sphere 3.0\nzoom_grid_with_origin_at 15 15 12 4 32\ndone\n'
        open(os.path.join(d, 'paramfile.txt'), 'w').write(body)
        subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
        raw = open(os.path.join(d, 'out.tipsy'), 'rb').read()
        _, _, dark = read_tipsy(os.path.join(d, 'out.tipsy'))
        np.savez_compressed(os.path.join(HERE, 'strays_zoom4.npz'), header_bytes=np.frombuffer(raw[:28], np.uint8).copy(),
                            nrec=np.int64(len(dark)), stride=np.int64(7), every=dark[::7].copy(), tail=dark[-400:].copy())


# The batch workload's zoom class at 64^3: a 100 Mpc/h base of 64 cells and a zoom of a quarter
# of its side (zoom factor 4) with 32 cells, so the zoom cells are half the base cells (ratio 2,
# fewer zoom cells than the window's base cells x 4), centred at (50, 50, 50); overdensity +1.0
# in a 1.5 Mpc/h sphere at the centre and -0.5 in a 3 Mpc/h sphere 5 Mpc/h along x.
RATIO2 = """centre 50 50 50
select_cube 10
zoom_grid_with_origin_at 24 24 24 4 32
centre 50 50 50
select_sphere 1.5
calculate overdensity
modify overdensity absolute 1.0
centre 55 50 50
select_sphere 3
calculate overdensity
modify overdensity absolute -0.5
done
dump_grid 0
dump_grid 1
"""


def ratio2_golden():
    """Reference-build grids, the two logged overdensities and the chi^2 change of RATIO2."""
    import re
    with tempfile.TemporaryDirectory() as d:
        write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
        open(os.path.join(d, 'paramfile.txt'), 'w').write(MOD_BASE.replace('basegrid 50.0 32', 'basegrid 100.0 64') +
                                                           RATIO2)
        r = subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True, text=True)
        log = r.stdout + r.stderr
        values = [float(v) for v in re.findall(r'overdensity: calculated value = (\S+)', log)]
        dchi2 = float(re.search(r'Modification Delta chi\^2 = (\S+)', log).group(1))
        grids = {'delta%d' % l: np.load(os.path.join(d, 'grid-%d.npy' % l)) for l in range(2)}
        np.savez_compressed(os.path.join(HERE, 'geom_ratio2.npz'), **grids, overdensity=np.array(values),
                            delta_chi2=np.array(dchi2))


# genetIC's grafic writer: a 16^3 base of 50 Mpc/h written with one subsampled level below it
# (`subsample 2`), a factor-4 zoom of 16 cells around a 5 Mpc/h sphere at the centre with its
# intermediate factor-2 subsampled grid,
# and the output centred on (30, 20, 25) (`center_output`: the coarse grids are rolled by whole
# cells, the finer ones keep their cells); the geometry of genetIC's test_12_grafic at 16^3.
GRAFIC = """subsample 2
centre 25 25 25
select_sphere 5
zoomgrid 4 16
centre 30 20 25
center_output
done
"""
GRAFIC_FILES = ('ic_velcx', 'ic_velcy', 'ic_velcz', 'ic_poscx', 'ic_poscy', 'ic_poscz', 'ic_deltab', 'ic_refmap',
                'ic_particle_ids')


def read_grafic(path, n, ids=False):
    """A grafic file: the 44-byte header record, then n slabs of n^2 values (Fortran records)."""
    raw = open(path, 'rb').read()
    header = np.frombuffer(raw[4:48], np.uint8).copy()
    item = 8 if ids else 4
    rec = 8 + n * n * item
    out = np.empty((n, n * n), dtype=np.uint64 if ids else np.float32)
    for z in range(n):
        o = 52 + z * rec
        out[z] = np.frombuffer(raw[o + 4:o + 4 + n * n * item], np.uint64 if ids else np.float32)
    return header, out.reshape(n, n, n)


def grafic_goldens():
    """The reference build's grafic files of the GRAFIC case (Fourier seeding): per grid of the
    stack, its header and every record of each field, and the zoom's origin from the log."""
    import re
    with tempfile.TemporaryDirectory() as d:
        write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
        body = MOD_BASE.replace('basegrid 50.0 32', 'basegrid 50.0 16').replace('outformat tipsy', 'outformat grafic')
        open(os.path.join(d, 'paramfile.txt'), 'w').write(body + GRAFIC)
        r = subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True, text=True)
        log = r.stdout + r.stderr
        origin = [int(v) for v in re.search(r'Low-left corner in parent grid = \((\d+), (\d+), (\d+)\)', log).groups()]
        out = {'origin': np.array(origin)}
        for eff in sorted(int(x.split('_')[-1]) for x in os.listdir(d) if x.startswith('out.grafic_')):
            gd = os.path.join(d, 'out.grafic_%d' % eff)
            n = int(np.frombuffer(open(os.path.join(gd, 'ic_velcx'), 'rb').read()[4:8], np.int32)[0])
            for f in GRAFIC_FILES:
                header, arr = read_grafic(os.path.join(gd, f), n, ids=f == 'ic_particle_ids')
                out['g%d_%s' % (eff, f)] = arr
            out['g%d_header' % eff] = header
        np.savez_compressed(os.path.join(HERE, 'grafic_zoom.npz'), **out)


def main():
    for mode, cmd in (('serial', 'random_seed_serial'), ('parallel', 'random_seed'), ('real', 'random_seed_real_space')):
        with tempfile.TemporaryDirectory() as d:
            write_camb(os.path.join(d, 'bbks.dat'), bbks_table())
            open(os.path.join(d, 'paramfile.txt'), 'w').write(PARAMS.format(seedcmd=cmd))
            subprocess.run([REF_BIN, 'paramfile.txt'], cwd=d, check=True, capture_output=True)
            delta = np.load(os.path.join(d, 'grid-0.npy'))
            _, _, dark = read_tipsy(os.path.join(d, 'out.tipsy'))
            pos = (dark[:, 1:4].astype(np.float64) + 0.5) * 50.0
            if mode == 'serial':
                np.savez_compressed(os.path.join(HERE, 'bbks32_%s.npz' % mode), delta=delta, pos=pos.astype(np.float32))
            else:
                np.savez_compressed(os.path.join(HERE, 'bbks32_%s.npz' % mode), delta=delta)


if __name__ == '__main__':
    if len(sys.argv) > 1:  # named generators only, e.g. geometry_goldens
        for fn in sys.argv[1:]:
            globals()[fn]()
        sys.exit(0)
    main()
    geometry_goldens()
    ratio2_golden()
    grafic_goldens()
    resample_goldens()
    strays_goldens()
    zoom_goldens()
    mod_goldens()
    var_goldens()
    ops_goldens()
    mod_more_goldens()
    splice_goldens()
    tipsy_goldens()
    gadget_goldens()
    tipsy3_goldens()
    gadget_types_goldens()
    flagged_type_goldens()
    zoom_grid_goldens()
    id_file_goldens()
    dump_tipsy_goldens()
    gadget_files_goldens()
