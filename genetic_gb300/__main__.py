"""Run Zel'dovich realisations from the command line.

python -m genetic_gb300 paramfile.txt [--precision mixed|fp64]
    runs a genetIC paramfile as `genetIC paramfile.txt` does: its realisation commands on
    the GPU, and `done` writes the tipsy or gadget file its outformat/outname/outdir name.
python -m genetic_gb300 --base 512 [--box 100] [--zoom 512 --factor 4] [--precision mixed|fp64]
                         [--seed 8896131] [--mode random_seed|random_seed_serial|random_seed_real_space]
                         [--repeat 1]
The zoom (if any) is centred in the box.  BBKS transfer function, Om 0.31,
Ol 0.69, h 0.68, s8 0.81, ns 0.965, z 99.  Prints the wall time per realisation.
"""
import argparse
import time

from .generator import ICGenerator
from .transfer import bbks_table


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('paramfile', nargs='?', help="a genetIC paramfile to run")
    ap.add_argument('--base', type=int, default=128)
    ap.add_argument('--box', type=float, default=100.0)
    ap.add_argument('--zoom', type=int, default=0)
    ap.add_argument('--factor', type=int, default=4)
    ap.add_argument('--precision', default='mixed', choices=['mixed', 'fp64'])
    ap.add_argument('--seed', type=int, default=8896131)
    ap.add_argument('--mode', default='random_seed',
                    choices=['random_seed', 'random_seed_serial', 'random_seed_real_space'])
    ap.add_argument('--repeat', type=int, default=1)
    args = ap.parse_args()
    if args.paramfile:
        from .generator import run_paramfile
        t0 = time.perf_counter()
        gen = run_paramfile(args.paramfile, precision=args.precision)
        print('paramfile %s: %.1f ms' % (args.paramfile, (time.perf_counter() - t0) * 1e3))
        gen.close()
        return
    with ICGenerator(precision=args.precision) as gen:
        for cmd, v in (('Om', 0.31), ('Ol', 0.69), ('Ob', 0.0), ('hubble', 0.68), ('s8', 0.81), ('ns', 0.965),
                       ('zin', 99)):
            getattr(gen, cmd)(v)
        gen.camb(bbks_table())
        gen.base_grid(args.box, args.base)
        if args.zoom:
            span = args.base // args.factor
            corner = (args.base - span) // 2
            gen.zoom_grid_with_origin_at(corner, corner, corner, args.factor, args.zoom)
        getattr(gen, args.mode)(args.seed)
        for r in range(args.repeat):
            t0 = time.perf_counter()
            gen.draw() if r == 0 else gen._call('gic_draw_noise', args.seed, gen.seed_mode)
            gen._call('gic_zeldovich', 1)
            print('realisation %d: %.1f ms' % (r, (time.perf_counter() - t0) * 1e3))


if __name__ == '__main__':
    main()
