"""A plain C program over the C ABI (tests/capi/realise32.c), compiled with the system C
compiler and linked against libgicgpu.so: its 32^3 FP64 realisation against the oracle."""
import os
import subprocess

import numpy as np
import pytest

import field_oracle as fo
from conftest import COSMO

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_c_program(tmp_path):
    from genetic_gb300 import build as b
    exe = str(tmp_path / 'realise32')
    subprocess.run([os.environ.get('CC', 'gcc'), '-O2', '-std=c99', '-I', os.path.join(ROOT, 'include'),
                    os.path.join(ROOT, 'tests', 'capi', 'realise32.c'), '-o', exe, '-L', os.path.dirname(b.LIB),
                    '-lgicgpu', '-Wl,-rpath,' + os.path.dirname(b.LIB)], check=True)
    return exe


def test_c_program_realisation_matches_oracle(built, bbks, tmp_path):
    exe = build_c_program(tmp_path)
    table = np.ascontiguousarray(bbks, dtype=np.float64)
    table.tofile(str(tmp_path / 'table.bin'))
    out = tmp_path / 'out.bin'
    r = subprocess.run([exe, str(tmp_path / 'table.bin'), str(table.shape[0]), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    m = 32 ** 3
    raw = np.fromfile(str(out), dtype=np.float64)
    delta, pos, vel = raw[:m].reshape(32, 32, 32), raw[m:4 * m].reshape(m, 3), raw[4 * m:].reshape(m, 3)
    fo.set_cr_log(True)
    w = fo.white_noise(32, 8896131, 1)
    fo.set_cr_log(False)
    d = fo.zeldovich_fields(w, fo.CambPower(bbks, COSMO), 50.0)
    assert np.abs(delta - d[0]).max() < 1e-10 * np.abs(d[0]).max()
    p, v = fo.particles(d[1:], 50.0, (0, 0, 0), 50.0, fo.velocity_to_offset_ratio(COSMO))
    dd = (pos - p + 25.0) % 50.0 - 25.0
    assert np.abs(dd).max() < 1e-10 * np.abs(d[1]).max() + 1e-12
    assert np.abs(vel - v).max() < 1e-10 * np.abs(v).max()
