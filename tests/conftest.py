import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, 'oracle'))


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300)')


@pytest.fixture(scope='session')
def built():
    """libgicgpu.so and liboracle.so, built if missing."""
    from genetic_gb300 import build as b
    if not os.path.exists(b.LIB):
        b.build()
    import field_oracle
    field_oracle.lib()
    return b.LIB


COSMO = dict(omega_m=0.31, omega_lambda=0.69, omega_b=0.0, hubble=0.68, sigma8=0.81, ns=0.965, redshift=99.0)


@pytest.fixture(scope='session')
def bbks():
    from genetic_gb300.transfer import bbks_table
    return bbks_table()


def make_generator(precision, table, levels, seed, mode_cmd, cosmo=COSMO):
    import genetic_gb300 as g
    gen = g.ICGenerator(precision=precision)
    gen.Om(cosmo['omega_m'])
    gen.Ol(cosmo['omega_lambda'])
    gen.Ob(cosmo['omega_b'])
    gen.hubble(cosmo['hubble'])
    gen.s8(cosmo['sigma8'])
    gen.ns(cosmo['ns'])
    gen.zin(cosmo['redshift'])
    gen.camb(table)
    for lev in levels:
        if lev[0] == 'base':
            gen.base_grid(lev[1], lev[2])
        else:
            gen.zoom_grid_with_origin_at(*lev[1:])
    getattr(gen, mode_cmd)(seed)
    return gen
