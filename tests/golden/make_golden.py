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
    main()
