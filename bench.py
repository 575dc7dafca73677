"""Throughput of the GB300 field-realisation path (Mparticles/s).

One step = one complete Zel'dovich (or 2LPT) realisation of the workload: white
noise drawn from the seed, the workload's modifications applied, multiplied by
sqrt(P(k)), displacement spectra, inverse FFTs, zoom combination where the
workload has zoom levels, and particle positions/velocities -- with the transfer
table already on the device
(`value`), or end to end through the C ABI from host memory (`e2e`: the
transfer table uploaded and the sigma8 normalisation recomputed every step,
particles copied back to pinned host memory every step: positions as doubles, velocities
in the context's precision).

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]
Under torchrun each rank runs an independent replica on its own GPU
(realisations do not share data): value = all particles / max-over-ranks time.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MODS4 = dict(centre=(50.0, 50.0, 50.0), radius=2.0,
             list=[('overdensity', 1.5), ('vx', 0.0), ('vy', 0.0), ('vz', 0.0)])
WORKLOADS = {
    # 512^3 base grid in a 100 Mpc/h box plus a 512^3 zoom of side 25 Mpc/h (factor 4)
    # centred at (50, 50, 50) Mpc/h: the headline two-level configuration
    # with 4 linear modifications in a 2 Mpc/h sphere at the zoom centre: mean
    # overdensity +1.5 and the three mean velocity components 0
    'zoom512': dict(levels=[('base', 100.0, 512), ('zoom', 192, 192, 192, 4, 512)], seed_cmd='random_seed',
                    precision='mixed', replaced=128 ** 3, mods=MODS4),
    'zoom512_fp64': dict(levels=[('base', 100.0, 512), ('zoom', 192, 192, 192, 4, 512)], seed_cmd='random_seed',
                         precision='fp64', replaced=128 ** 3, mods=MODS4),
    'zoom512_nomod': dict(levels=[('base', 100.0, 512), ('zoom', 192, 192, 192, 4, 512)], seed_cmd='random_seed',
                          precision='mixed', replaced=128 ** 3),
    # the same with second-order (2LPT) displacements and velocities
    'zoom512_lpt2': dict(levels=[('base', 100.0, 512), ('zoom', 192, 192, 192, 4, 512)], seed_cmd='random_seed',
                         precision='mixed', replaced=128 ** 3, mods=MODS4, order=2),
    'zoom512_lpt2_fp64': dict(levels=[('base', 100.0, 512), ('zoom', 192, 192, 192, 4, 512)],
                              seed_cmd='random_seed', precision='fp64', replaced=128 ** 3, mods=MODS4, order=2),
    'zoom256': dict(levels=[('base', 100.0, 256), ('zoom', 96, 96, 96, 4, 256)], seed_cmd='random_seed',
                    precision='mixed', replaced=64 ** 3),
    # the headline layout at 384^3 (fields of 0.23 GB, above L2; a few GB on the device):
    # the case kernel profiles of the modification algebra are captured on
    'zoom384': dict(levels=[('base', 100.0, 384), ('zoom', 144, 144, 144, 4, 384)], seed_cmd='random_seed',
                    precision='mixed', replaced=96 ** 3, mods=MODS4),
    # 512^3 single level, 100 Mpc/h box (the single-level configuration at 512^3)
    'za512': dict(levels=[('base', 100.0, 512)], seed_cmd='random_seed', precision='mixed'),
    'za512_fp64': dict(levels=[('base', 100.0, 512)], seed_cmd='random_seed', precision='fp64'),
    'za256': dict(levels=[('base', 100.0, 256)], seed_cmd='random_seed', precision='mixed'),
}
# 64 independent realisations in one batch (mixed precision, seeds 1..64): 32 single-level
# 128^3 boxes (50 Mpc/h), 24 single-level 192^3 boxes (75 Mpc/h) and 8 two-level zooms of a
# 256^3 base (100 Mpc/h) plus a 128^3 zoom of side 25 Mpc/h centred at (50, 50, 50) (genetIC zoom
# factor 4, cells half the base cells), each zoom
# with 2 modifications: overdensity +1.0 in a 1.5 Mpc/h sphere at the centre and -0.5 in a
# 3 Mpc/h sphere 5 Mpc/h along x
BATCH64 = ([dict(levels=[('base', 50.0, 128)], mods=[])] * 32 +
           [dict(levels=[('base', 75.0, 192)], mods=[])] * 24 +
           [dict(levels=[('base', 100.0, 256), ('zoom', 96, 96, 96, 4, 128)], replaced=64 ** 3,
                 mods=[((50.0, 50.0, 50.0), 1.5, 1.0), ((55.0, 50.0, 50.0), 3.0, -0.5)])] * 8)
WORKLOADS['batch64'] = dict(batch=BATCH64, precision='mixed', seed_cmd='random_seed', levels=[])
DEFAULT_WORKLOAD = 'zoom512'
COSMO = dict(omega_m=0.31, omega_lambda=0.69, omega_b=0.0, hubble=0.68, sigma8=0.81, ns=0.965, redshift=99.0)
SEED = 8896131
METRIC = "Mparticles/s, 512³ 2-level Zel'dovich IC: FP32+FP64 vs plain FP64 at ≤1e-5 err"


def dist_env():
    rank = int(os.environ.get('RANK', 0))
    world = int(os.environ.get('WORLD_SIZE', 1))
    local = int(os.environ.get('LOCAL_RANK', 0))
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_gen(wl, table, device):
    import genetic_gb300 as g
    gen = g.ICGenerator(precision=wl['precision'], device=device)
    for k, v in (('Om', COSMO['omega_m']), ('Ol', COSMO['omega_lambda']), ('Ob', 0.0), ('hubble', COSMO['hubble']),
                 ('s8', COSMO['sigma8']), ('ns', COSMO['ns']), ('zin', COSMO['redshift'])):
        getattr(gen, k)(v)
    gen.camb(table)
    for lev in wl['levels']:
        if lev[0] == 'base':
            gen.base_grid(lev[1], lev[2])
        else:
            gen.zoom_grid_with_origin_at(*lev[1:])
    getattr(gen, wl['seed_cmd'])(SEED)
    if wl.get('mods'):
        gen.centre(*wl['mods']['centre'])
        gen.select_sphere(wl['mods']['radius'])
        for name, target in wl['mods']['list']:
            gen.modify(name, 'absolute', target)
    return gen


def n_particles(wl):
    """Particles written out: every cell of every level, less the base cells the zoom replaces
    (genetIC's two-level particle mapper, genetIC/src/simulation/particles/mapper/twolevelmapper.hpp)."""
    return sum(lev[2] ** 3 if lev[0] == 'base' else lev[5] ** 3 for lev in wl['levels']) - wl.get('replaced', 0)


def tipsy_map(wl):
    """The gic_particle_map of a one- or two-level workload: the zoom replaces the base cells it
    covers; masses, softenings and TipsyOutput's factors as genetIC forms them
    (genetic_gb300.writers.particle_map).  None for other workloads."""
    from genetic_gb300 import writers
    levels = wl['levels']
    _, L, n0 = levels[0]
    if len(levels) > 2 or n0 > 1024:
        return None, None
    geo = [(L, n0, (0.0, 0.0, 0.0))]
    masks = []
    total = n0 ** 3
    if len(levels) == 2:
        _, ox, oy, oz, factor, n1 = levels[1]
        span = n0 // factor
        ratio = factor * n1 // n0
        dx0 = L / n0
        geo.append((L / factor, n1, (ox * dx0, oy * dx0, oz * dx0)))
        ax = [(o + np.arange(span)) % n0 for o in (ox, oy, oz)]
        rep = np.sort(((ax[0][:, None, None] * n0 + ax[1][None, :, None]) * n0 + ax[2][None, None, :]).ravel())
        masks.append((rep.astype(np.uint64), ratio, (ox, oy, oz)))
        total += len(rep) * (ratio ** 3 - 1)
    return writers.particle_map(geo, masks, COSMO), total


class Clocks:
    """nvidia-smi samples while the timed region runs."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), 'gic_bench_clocks_%d.csv' % os.getpid())

    def __enter__(self):
        try:
            self.f = open(self.path, 'w')
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index),
                 '--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
                 'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
                 'clocks_event_reasons.sw_power_cap', '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc:
            return None
        sm, mx, reasons = [], [], set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for line in open(self.path):
            parts = [p.strip() for p in line.split(',')]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[3:7]):
                if v.lower() == 'active':
                    reasons.add(name)
        if not sm:
            return None
        return {'sm_mhz': float(np.median(sm)), 'sm_max_mhz': max(mx), 'reasons': sorted(reasons), 'samples': len(sm)}


def measured_peak_hbm():
    try:
        peaks = json.load(open(os.path.join(ROOT, 'MEASURED_PEAKS.json')))
        return float(peaks['hbm_gbs']), 'measured'
    except (OSError, KeyError, ValueError):
        return 6800.0, 'fallback'


def profiled_traffic(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summaries (profiles/*.md), or None."""
    import glob
    import re
    for path in sorted(glob.glob(os.path.join(ROOT, 'profiles', '*.md'))):
        for line in open(path):
            m = re.match(r'traffic_bytes (.+): (\d+)\s*$', line)
            if m and m.group(1) == kernel:
                return int(m.group(2))
    return None


def fft_roofline(gen, wl, stream, reps=20, field=None):
    """Average device time of one inverse 3-D FFT of the finest level's x displacement field
    (or of `field`)."""
    import torch
    from genetic_gb300 import _lib
    level = len(wl['levels']) - 1
    n = gen.levels[level][1]
    s = 4 if wl['precision'] == 'mixed' else 8
    nc = n * n * (n // 2 + 1)
    what = _lib.GIC_FIELD_PSI_X if field is None else field
    # the field is in real space after a realisation: forward then inverse keeps it meaningful
    for _ in range(3):
        gen._call('gic_fft', level, what, -1)
        gen._call('gic_fft', level, what, +1)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * reps + 1)]
    times = []
    for r in range(reps):
        gen._call('gic_fft', level, what, -1)
        ev[2 * r].record(stream)
        gen._call('gic_fft', level, what, +1)
        ev[2 * r + 1].record(stream)
    torch.cuda.synchronize()
    for r in range(reps):
        times.append(ev[2 * r].elapsed_time(ev[2 * r + 1]) * 1e-3)
    t = float(np.mean(times))
    algorithmic = 6.0 * (2 * s) * nc  # 3 passes, read + write of the half spectrum
    peak, kind = measured_peak_hbm()
    achieved = algorithmic / t / 1e9
    kernel = 'fft_c2r_3d (%d^3, %s)' % (n, 'fp32' if s == 4 else 'fp64')
    return {'bound': 'hbm', 'achieved': round(achieved, 1), 'peak': peak, 'unit': 'GB/s',
            'frac': round(achieved / peak, 4), 'traffic': profiled_traffic(kernel), 'kernel': kernel,
            'ms_per_launch': round(t * 1e3, 4), 'peak_source': kind}


def fft_choice(gen):
    """The FFT passes the tuner chose per transform size: {n: "<cols>,<rows>,<planes>"}
    (the GIC_FFT_TILE value that pins them, e.g. for a profiler run)."""
    out = {}
    for _, n, _ in gen.levels:
        c, r, p = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        if gen._lib.gic_fft_choice(gen._ctx, n, ctypes.byref(c), ctypes.byref(r), ctypes.byref(p)) == 0:
            out[str(n)] = '%d,%d,%d' % (c.value, r.value, p.value)
    return out


def fft_only(n, precision, table, device):
    """One single-level n^3 context whose white noise is set from the host (a seeded
    Gaussian half spectrum), then the FFT roofline of its field: the transform passes
    alone, on a small device footprint."""
    import torch
    from genetic_gb300 import _lib
    from genetic_gb300.generator import _ptr
    wl = dict(levels=[('base', 100.0, n)], seed_cmd='random_seed', precision=precision)
    gen = make_gen(wl, table, device)
    rng = np.random.default_rng(SEED)
    gen._call('gic_set_noise', 0, _ptr(np.ascontiguousarray(rng.standard_normal((n, n, n // 2 + 1, 2)))))
    sptr = ctypes.c_void_p()
    _lib.check(gen._ctx, gen._lib.gic_get_stream(gen._ctx, ctypes.byref(sptr)))
    stream = torch.cuda.ExternalStream(sptr.value, device=torch.device('cuda', device))
    roof = fft_roofline(gen, wl, stream, field=_lib.GIC_FIELD_NOISE)
    passes = fft_choice(gen)
    gen.close()
    print(json.dumps({'fft_only': n, 'precision': precision, 'roofline': roof, 'fft_passes': passes}))


def cpu_baseline_port(n=192, box=75.0, threads=None):
    """The oracle's restatement of the path on the host: one single-level realisation."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import field_oracle as fo
    from genetic_gb300.transfer import bbks_table
    table = bbks_table()
    t0 = time.perf_counter()
    w = fo.white_noise(n, SEED, 2)
    power = fo.CambPower(table, COSMO)
    d = fo.zeldovich_fields(w, power, box)
    fo.particles(d[1:], box, (0, 0, 0), box, fo.velocity_to_offset_ratio(COSMO))
    dt = time.perf_counter() - t0
    return n ** 3 / dt / 1e6, dt


def cpu_zoom_sample(n=96, workers=None):
    """The headline pipeline at a bounded size, by the oracle on the host: base n^3 in
    100 Mpc/h plus an n^3 zoom of side 25 Mpc/h (factor 4) at the centre, the four linear
    modifications in a 2 Mpc/h sphere (chi^2 before and after), Zel'dovich particles
    of both levels.  FFTs on `workers` threads; noise and placement single-threaded."""
    sys.path.insert(0, os.path.join(ROOT, 'oracle'))
    import field_oracle as fo
    from genetic_gb300.transfer import bbks_table
    fo.set_fft_workers(workers)
    table = bbks_table()
    off = (n - n // 4) // 2 * 100.0 / n
    levels = [(100.0, n, (0.0, 0.0, 0.0)), (25.0, n, (off, off, off))]
    t0 = time.perf_counter()
    L = fo.Levels(levels)
    w = fo.white_noise_levels([n, n], SEED, 2)
    p_dm = fo.CambPower(table, COSMO, column=1)
    power = fo.CambPower(table, COSMO)
    ratio = fo.velocity_to_offset_ratio(COSMO)
    flagged = fo.flag_cells(L, 1, (50.0, 50.0, 50.0), 'sphere', 2.0)
    covs = []
    for kind, d in (('overdensity', 0), ('velocity', 0), ('velocity', 1), ('velocity', 2)):
        loc = fo.localisation_covector(L, flagged, kind, d)
        covs.append(fo.multilevel_covector(L, loc, p_dm, None if kind == 'overdensity' else ratio))
    fo.chi2_levels(L, w)
    w2 = fo.apply_linear_modifications(L, w, covs, [1.5, 0.0, 0.0, 0.0])
    fo.chi2_levels(L, w2)
    fields = fo.zoom_realisation(w2, levels, power)
    for (box, nn, o), f in zip(levels, fields):
        fo.particles(f[1:], box, o, 100.0, ratio)
    dt = time.perf_counter() - t0
    fo.set_fft_workers(None)
    npart = 2 * n ** 3 - (n // 4) ** 3
    return npart / dt / 1e6, dt, npart


def run_reference(args, wl, rank, world):
    """The reference arm: the oracle's restatement of the path on the host cores, on a
    bounded sample of the headline workload (genetIC itself is a C++ program that is
    not installable as a package and whose sources are not on the GPU host)."""
    if rank != 0:
        return
    workers = os.cpu_count() or 1
    vals = []
    for _ in range(args.warmup):
        cpu_zoom_sample(workers=workers)
    for _ in range(args.steps):
        v, dt, npart = cpu_zoom_sample(workers=workers)
        vals.append(dt)
    t = float(np.mean(vals))
    value = npart / t / 1e6
    sample = ('oracle restatement (C RANLUX+ziggurat, numpy/scipy pocketfft FFTs on %d threads) of the headline '
              'pipeline at 96^3 + 96^3 zoom with the 4 modifications, %d particles per step' % (workers, npart))
    line = {'impl': 'reference', 'metric': METRIC, 'value': round(value, 4), 'unit': 'Mparticles/s',
            'n_gpus': args.gpus, 'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(t * 1e3, 2),
            'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64', 'data': 'synthetic',
            'config': {'workload': args.workload, 'sample': sample},
            'cpu_baseline': {'value': round(value, 4), 'unit': 'Mparticles/s', 'cores': workers, 'kind': 'port',
                             'sample': sample},
            'e2e': {'value': round(value, 4), 'unit': 'Mparticles/s', 'h2d_bytes_per_step': 0,
                    'd2h_bytes_per_step': 0}}
    print(json.dumps(line))


def run_batch(args, wl, table, local, rank, world):
    """The batch workload through gic_batch_realise: one step = one realisation of
    every member.  Also times the same realisations one after another through the
    plain entry points, for comparison."""
    import torch
    from genetic_gb300.batch import Batch
    from genetic_gb300.generator import _ptr
    gens = []
    for m in wl['batch']:
        w = dict(levels=m['levels'], precision=wl['precision'], seed_cmd=wl['seed_cmd'])
        gen = make_gen(w, table, local)
        for centre, radius, target in m['mods']:
            gen.centre(*centre)
            gen.select_sphere(radius)
            gen.modify('overdensity', 'absolute', target)
        gens.append(gen)
    npart = sum(n_particles(dict(levels=m['levels'], replaced=m.get('replaced', 0))) for m in wl['batch'])
    batch = Batch(gens)
    stream = torch.cuda.ExternalStream(batch.stream(), device=torch.device('cuda', local))
    nthreads = min(16, os.cpu_count() or 1)

    def step(i):
        batch.realise([1 + k + 64 * i for k in range(len(gens))], threads=nthreads)

    for i in range(args.warmup):
        step(i)
    launches0 = ctypes.c_ulonglong()
    gens[0]._lib.gic_launch_count(ctypes.byref(launches0))
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    if args.profile_range:
        torch.cuda.profiler.start()
    with Clocks(local) as clk:
        start.record(stream)
        for i in range(args.steps):
            step(args.warmup + i)
        end.record(stream)
        torch.cuda.synchronize()
    if args.profile_range:
        torch.cuda.profiler.stop()
    barrier(world)
    launches1 = ctypes.c_ulonglong()
    gens[0]._lib.gic_launch_count(ctypes.byref(launches1))
    t = max_over_ranks(start.elapsed_time(end) * 1e-3 / args.steps, world)
    # the same realisations one at a time through the plain entry points
    t0 = time.perf_counter()
    for k, gen in enumerate(gens):
        gen._call('gic_draw_noise', 1 + k, 2)
        if wl['batch'][k]['mods']:
            gen._call('gic_apply_modifications', None, None)
        gen._call('gic_zeldovich', 1)
    torch.cuda.synchronize()
    t_seq = time.perf_counter() - t0
    # end to end: every member's particles copied back to pinned host memory each step
    # (positions as doubles, velocities in float32, the mixed form's own precision)
    pinned = []
    for gen in gens:
        for lev in range(len(gen.levels)):
            n = gen.levels[lev][1]
            pinned.append((gen, lev, torch.empty((n ** 3, 3), dtype=torch.float64, pin_memory=True).numpy(),
                           torch.empty((n ** 3, 3), dtype=torch.float32, pin_memory=True).numpy()))
    t0 = time.perf_counter()
    for i in range(args.steps):
        step(i)
        for gen, lev, pos, vel in pinned:
            gen._call('gic_fetch_particles_native', lev, _ptr(pos), ctypes.c_void_p(vel.ctypes.data))
    t_e2e = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
    d2h = sum(p.nbytes + v.nbytes for _, _, p, v in pinned)
    batch.close()
    for gen in gens:
        gen.close()
    if rank != 0:
        return
    line = {
        'metric': METRIC, 'value': round(npart * world / t / 1e6, 3), 'unit': 'Mparticles/s', 'n_gpus': world,
        'steps': args.steps, 'warmup': args.warmup, 'ms_per_step': round(t * 1e3, 3), 'higher_is_better': True,
        'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32+f64', 'data': 'synthetic',
        'config': {'workload': args.workload, 'members': '32 x 128^3 (50 Mpc/h), 24 x 192^3 (75 Mpc/h), '
                   '8 x (256^3 base 100 Mpc/h + 128^3 zoom of 25 Mpc/h, 2 overdensity modifications)',
                   'realisations_per_step': len(gens), 'particles_per_step': npart, 'host_threads': nthreads,
                   'sequential_ms_per_step': round(t_seq * 1e3, 3), 'precision': wl['precision'],
                   'parallelism': 'replicas' if world > 1 else 'single GPU',
                   'l2': 'inputs larger than L2 (the batch holds tens of GB)'},
        'e2e': {'value': round(npart * world / t_e2e / 1e6, 3), 'unit': 'Mparticles/s', 'h2d_bytes_per_step': 0,
                'd2h_bytes_per_step': int(d2h)},
        'gpu_launches': int(launches1.value - launches0.value),
        'clocks': clk.summary(),
    }
    print(json.dumps(line))


def accuracy(wl_name, wl, table, device):
    """Per-field max and RMS relative error (|a - b| / max|b|) of the workload's mixed
    form against its plain FP64 form, both on the GPU, same seed and modifications."""
    import genetic_gb300 as g  # noqa: F401
    mixed = dict(wl, precision='mixed')
    fp64 = dict(wl, precision='fp64')
    order = wl.get('order', 1)
    gens = []
    for w in (mixed, fp64):
        gen = make_gen(w, table, device)
        gen._call('gic_draw_noise', SEED, 2)
        if w.get('mods'):
            c = ctypes.c_double(), ctypes.c_double()
            gen._call('gic_apply_modifications', ctypes.byref(c[0]), ctypes.byref(c[1]))
        gen._call('gic_zeldovich', order)
        gens.append(gen)
    names = ['delta', 'psi_x', 'psi_y', 'psi_z'] + (['psi2_x', 'psi2_y', 'psi2_z'] if order == 2 else [])
    out = {}
    for lev in range(len(wl['levels'])):
        for name in names:
            a = gens[0].field(lev, name)
            b = gens[1].field(lev, name)
            scale = float(np.abs(b).max())
            d = np.abs(a - b)
            out['L%d.%s' % (lev, name)] = {'max': float(d.max() / scale), 'rms': float(np.sqrt(np.mean(d * d)) / scale)}
            del a, b, d
    for gen in gens:
        gen.close()
    worst_disp = max(v['max'] for k, v in out.items() if '.psi' in k)
    print(json.dumps({'accuracy': wl_name, 'reference': 'plain FP64 GPU path', 'fields': out,
                      'max_rel_displacement_err': worst_disp}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--workload', default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--profile-range', action='store_true',
                    help='bracket the timed steps with cudaProfilerStart/Stop (for ncu --profile-from-start off)')
    ap.add_argument('--accuracy', action='store_true',
                    help='print the per-field error of the mixed form against FP64 instead of timing')
    ap.add_argument('--fft-only', type=int, default=0, metavar='N',
                    help='time the inverse + forward 3-D FFT of one N^3 field (set from the host, no realisation; '
                         'about 2 N^3 x 8 bytes on the device in the mixed form) and print its roofline: a small case '
                         'for profiling the transform passes')
    args = ap.parse_args()
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group('gloo')
    wl = WORKLOADS[args.workload]
    if args.impl == 'reference':
        run_reference(args, wl, rank, world)
        return

    import torch
    from genetic_gb300 import _lib
    from genetic_gb300.transfer import bbks_table
    torch.cuda.set_device(local)
    table = np.ascontiguousarray(bbks_table())
    if args.accuracy:
        accuracy(args.workload, wl, table, local)
        return
    if args.fft_only:
        fft_only(args.fft_only, wl['precision'], table, local)
        return
    if wl.get('batch'):
        run_batch(args, wl, table, local, rank, world)
        return
    gen = make_gen(wl, table, local)
    sptr = ctypes.c_void_p()
    _lib.check(gen._ctx, gen._lib.gic_get_stream(gen._ctx, ctypes.byref(sptr)))
    stream = torch.cuda.ExternalStream(sptr.value, device=torch.device('cuda', local))
    mode = {'random_seed': _lib.GIC_SEED_FOURIER_PARALLEL, 'random_seed_serial': _lib.GIC_SEED_FOURIER_SERIAL,
            'random_seed_real_space': _lib.GIC_SEED_REAL_SPACE}[wl['seed_cmd']]
    npart = n_particles(wl)

    has_mods = bool(wl.get('mods'))
    chi2 = ctypes.c_double(), ctypes.c_double()

    def step(i):
        gen._call('gic_draw_noise', SEED + i, mode)
        if has_mods:
            gen._call('gic_apply_modifications', ctypes.byref(chi2[0]), ctypes.byref(chi2[1]))
        gen._call('gic_zeldovich', wl.get('order', 1))

    for i in range(args.warmup):
        step(i)
    launches0 = ctypes.c_ulonglong()
    gen._lib.gic_launch_count(ctypes.byref(launches0))
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    if args.profile_range:
        torch.cuda.profiler.start()
    with Clocks(local) as clk:
        start.record(stream)
        for i in range(args.steps):
            step(args.warmup + i)
        end.record(stream)
        torch.cuda.synchronize()
    if args.profile_range:
        torch.cuda.profiler.stop()
    barrier(world)
    launches1 = ctypes.c_ulonglong()
    gen._lib.gic_launch_count(ctypes.byref(launches1))
    t = max_over_ranks(start.elapsed_time(end) * 1e-3 / args.steps, world)
    value = npart * world / t / 1e6

    # end to end through the C ABI, host buffers (pinned), copies inside the timed region:
    # positions as doubles, velocities in the precision the context computes them
    # (gic_fetch_particles_async: float32 in the mixed form).  Each step's particles are fetched
    # without waiting, into one of two host buffer sets, while the next step computes (the
    # library alternates two device buffer pairs); the clock stops after the last fetch lands.
    vel_dtype = torch.float64 if wl['precision'] == 'fp64' else torch.float32
    pinned = []
    for _ in range(2):
        sets = []
        for lev in range(len(wl['levels'])):
            n = gen.levels[lev][1]
            pos = torch.empty((n ** 3, 3), dtype=torch.float64, pin_memory=True).numpy()
            vel = torch.empty((n ** 3, 3), dtype=vel_dtype, pin_memory=True).numpy()
            sets.append((pos, vel))
        pinned.append(sets)
    table_pinned = torch.empty(table.shape, dtype=torch.float64, pin_memory=True).numpy()
    table_pinned[...] = table
    from genetic_gb300.generator import _ptr

    def e2e_step(i):
        gen._call('gic_set_transfer', _ptr(table_pinned), table.shape[0], table.shape[1])
        step(i)
        for lev, (pos, vel) in enumerate(pinned[i % 2]):
            gen._call('gic_fetch_particles_async', lev, _ptr(pos), ctypes.c_void_p(vel.ctypes.data))

    # both host buffer sets once before the clock (the first transfer into fresh pinned pages is slow)
    e2e_step(0)
    e2e_step(1)
    gen._call('gic_fetch_wait')
    barrier(world)
    t0 = time.perf_counter()
    for i in range(args.steps):
        e2e_step(i)
    gen._call('gic_fetch_wait')
    t_e2e = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
    d2h = sum(p.nbytes + v.nbytes for p, v in pinned[0])
    del pinned

    # end to end to genetIC's tipsy records: the step, then the records of every particle
    # in mapper order packed on the device and copied to pinned host memory without waiting
    # (gic_tipsy_pack_async, two host buffers), overlapping the next step
    e2e_tipsy = None
    try:
        tmap, ntot = tipsy_map(wl)
        if tmap is not None:
            recs = [torch.empty((ntot * 9,), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]

            def tipsy_step(i):
                step(i)
                gen._call('gic_tipsy_pack_async', ctypes.byref(tmap), 0, ntot,
                          recs[i % 2].ctypes.data_as(ctypes.c_void_p))

            tipsy_step(0)
            tipsy_step(1)
            gen._call('gic_fetch_wait')
            barrier(world)
            t0 = time.perf_counter()
            for i in range(args.steps):
                tipsy_step(i)
            gen._call('gic_fetch_wait')
            t_tipsy = max_over_ranks((time.perf_counter() - t0) / args.steps, world)
            n0 = wl['levels'][0][2]
            e2e_tipsy = {'value': round(ntot * world / t_tipsy / 1e6, 3), 'unit': 'Mparticles/s',
                         'h2d_bytes_per_step': int(8 * tmap.n_replaced[0] + 16 * n0 * n0 + 8),
                         'd2h_bytes_per_step': int(recs[0].nbytes)}
            del recs
    except Exception as e:  # reported, never fatal to the benchmark line
        e2e_tipsy = {'error': str(e)[:200]}
    roof = fft_roofline(gen, wl, stream)
    fft_passes = fft_choice(gen)
    gen.close()

    if rank != 0:
        return
    line = {
        'metric': METRIC, 'value': round(value, 3), 'unit': 'Mparticles/s', 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': round(t * 1e3, 3), 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': 'f32+f64' if wl['precision'] == 'mixed' else 'f64', 'data': 'synthetic',
        'config': {'workload': args.workload, 'levels': [list(l) for l in wl['levels']],
                   'modifications': ([m[0] + '=' + str(m[1]) for m in wl['mods']['list']] +
                                     ['sphere r=%g at %s' % (wl['mods']['radius'], wl['mods']['centre'])])
                   if wl.get('mods') else [],
                   'precision': wl['precision'], 'seeding': wl['seed_cmd'], 'transfer': 'BBKS table, 2000 rows',
                   'lpt_order': wl.get('order', 1),
                   'particles_per_step': npart, 'l2': 'inputs larger than L2 (fields >= 0.5 GB)',
                   'parallelism': 'replicas' if world > 1 else 'single GPU', 'fft_passes': fft_passes},
        'e2e': {'value': round(npart * world / t_e2e / 1e6, 3), 'unit': 'Mparticles/s',
                'h2d_bytes_per_step': int(table.nbytes), 'd2h_bytes_per_step': int(d2h)},
        'e2e_tipsy': e2e_tipsy,
        'gpu_launches': int(launches1.value - launches0.value),
        'roofline': roof,
        'clocks': clk.summary(),
    }
    if not args.no_cpu_baseline:
        workers = os.cpu_count() or 1
        v, dt, npart_cpu = cpu_zoom_sample(workers=workers)
        line['cpu_baseline'] = {'value': round(v, 4), 'unit': 'Mparticles/s', 'cores': workers, 'kind': 'port',
                                'sample': 'oracle restatement of the headline pipeline at 96^3 + 96^3 zoom with '
                                          'the 4 modifications, %d particles (%.1f s; FFTs on %d threads)'
                                          % (npart_cpu, dt, workers)}
    print(json.dumps(line))


if __name__ == '__main__':
    main()
