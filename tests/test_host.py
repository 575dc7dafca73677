"""Host-side logic and the C ABI, without a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, 'genetic_gb300', 'csrc')


def _declared_symbols():
    text = open(os.path.join(ROOT, 'include', 'gicgpu.h')).read()
    return sorted(set(re.findall(r'GIC_API\s+(?:const\s+)?\w+\s*\*?\s*(gic_\w+)\s*\(', text)))


def test_library_exports_every_declared_symbol(built):
    from genetic_gb300 import _lib
    lib = ctypes.CDLL(built)
    declared = _declared_symbols()
    assert len(declared) >= 14
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(_lib.SIGNATURES), 'binding and header disagree'


def test_create_without_gpu_fails_cleanly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    from genetic_gb300 import _lib
    lib = _lib.load()
    ctx = ctypes.c_void_p()
    st = lib.gic_create(ctypes.byref(ctx), None)
    assert st == _lib.GIC_ERR_CUDA
    assert b'CUDA' in lib.gic_last_error(None) or b'device' in lib.gic_last_error(None)
    assert lib.gic_destroy(None) == 0
    assert lib.gic_level_add(None, 1.0, 8, 0.0, 0.0, 0.0, None) == _lib.GIC_ERR_INVALID_ARG


def test_ziggurat_tables_agree_with_oracle():
    a = open(os.path.join(ROOT, 'oracle', 'rng', 'zig_tables.h')).read()
    b = open(os.path.join(CSRC, 'zig_tables.h')).read()
    hx = lambda s: re.findall(r'0x[0-9a-f.]+p[+-]\d+(?!f)\b', s)
    line = lambda s, name: re.search(r'#define %s \{([^}]*)\}' % name, s).group(1)
    oracle_doubles = hx(a)
    doubles = hx(line(b, 'GIC_ZIG_Y_INIT')) + hx(line(b, 'GIC_ZIG_W_INIT'))
    assert oracle_doubles == doubles and len(doubles) == 256
    assert re.findall(r'(\d+)u', a) == re.findall(r'(\d+)u', b)
    # the device's single-precision decision tables are those doubles rounded to nearest
    for dname, fname in (('GIC_ZIG_Y_INIT', 'GIC_ZIG_YF_INIT'), ('GIC_ZIG_W_INIT', 'GIC_ZIG_WF_INIT')):
        d = [float.fromhex(v) for v in hx(line(b, dname))]
        f = [float.fromhex(v[:-1]) for v in re.findall(r'0x[0-9a-f.]+p[+-]\d+f', line(b, fname))]
        assert len(f) == len(d) and all(float(np.float32(x)) == y for x, y in zip(d, f))


HOST_TEST = r'''
#include "bigint576.h"
#include "ddlog.h"
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <cmath>
extern "C" void oracle_ranlux_stream(unsigned long seed, uint32_t *out, uint64_t n);
static void step24(uint32_t *y, uint32_t &c, int n) {
  for (int s = 0; s < n; ++s) {
    int32_t d = (int32_t)y[14] - (int32_t)y[0] - (int32_t)c;
    c = (uint32_t)d >> 31;
    uint32_t w = (uint32_t)d & 0xFFFFFF;
    for (int k = 0; k < 23; ++k) y[k] = y[k + 1];
    y[23] = w;
  }
}
int main() {
  int bad = 0;
  unsigned long seeds[3] = {1, 8896131, 13842314};
  for (unsigned long seed : seeds) {
    const int nb = 300;
    std::vector<uint32_t> ref(24 * nb);
    oracle_ranlux_stream(seed, ref.data(), ref.size());
    uint32_t y0[24];
    ranlux_seed_state(y0, seed);
    U576 a, Y0;
    u576_ranlux_multiplier(a);
    u576_from_state(Y0, y0, 0);
    for (int j0 : {0, 1, 7, 131, 299}) {
      U576 A, Y;
      u576_powmod(A, a, 794ull * j0);
      u576_mulmod(Y, A, Y0);
      uint32_t y[24], c = 0;
      u576_to_state(y, Y);
      for (int b = j0; b < nb; ++b) {
        step24(y, c, 794);
        for (int k = 0; k < 24; ++k) bad += y[k] != ref[b * 24 + k];
      }
    }
  }
  int badlog = 0;
  for (uint32_t k = 1; k <= 16777216u; k += 97) {
    long double u = (long double)k / 16777216.0L;
#if defined(__aarch64__)
    double q = (double)logl(u);
#else
    double q = (double)logq((__float128)u);
#endif
    badlog += q != gic_log_k24(k);
  }
  printf("%d %d\n", bad, badlog);
  return 0;
}
'''


def test_jump_ahead_and_tail_log_on_host(tmp_path, built):
    src = tmp_path / 't.cpp'
    quad = '' if os.uname().machine == 'aarch64' else '#include <quadmath.h>\n'
    src.write_text(quad + HOST_TEST)
    exe = tmp_path / 't'
    libs = [] if os.uname().machine == 'aarch64' else ['-lquadmath']
    subprocess.run(['g++', '-O2', '-ffp-contract=off', '-I', CSRC, str(src),
                    os.path.join(ROOT, 'oracle', 'rng', 'oracle_rng.c'), '-o', str(exe), '-lm'] + libs, check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out == ['0', '0'], out


def test_bbks_table_format(tmp_path):
    from genetic_gb300.transfer import bbks_table, write_camb, read_camb, bbks
    t = bbks_table()
    assert t.shape == (2000, 7)
    assert np.all(t[:, 1:] == t[:, [1]])
    assert abs(t[0, 1] - 1.0) < 1e-3
    p = tmp_path / 'tf.dat'
    write_camb(str(p), t)
    assert np.array_equal(read_camb(str(p)), t)
    # large-scale limit and monotone decline
    assert np.all(np.diff(bbks(np.logspace(-3, 2, 50), 0.31, 0.049, 0.68)) < 0)


def test_paramfile_parser(tmp_path):
    from genetic_gb300 import generator
    p = tmp_path / 'p.txt'
    p.write_text('Om 0.3\n# comment\nbasegrid 50 32 # trailing\noutformat tipsy\nrandom_seed 5\ndone\n')
    cmds = generator.parse_paramfile(str(p))
    assert [c[1] for c in cmds] == ['Om', 'base_grid', 'outformat', 'random_seed', 'done']
    assert cmds[1][2] == ['50', '32']
    p.write_text('supersample 2\n')
    with pytest.raises(ValueError, match='not on the GPU realisation path'):
        generator.parse_paramfile(str(p))


def test_c_program_compiles_and_links_against_the_library(built, tmp_path):
    """tests/capi/realise32.c, a plain C caller, builds against include/gicgpu.h and links libgicgpu.so."""
    from test_gpu_capi import build_c_program
    assert os.path.exists(build_c_program(tmp_path))


def test_genetic_side_hook_compiles_against_genetic_headers():
    """include/gicgpu_genetic.hpp (DeviceRealisation, DeviceBackedParticleEvaluator) compiled
    against genetIC's own headers by oracle/Makefile's `hook` target, where they are present."""
    import subprocess
    oracle = os.path.join(ROOT, 'oracle')
    ref = subprocess.run(['make', '-s', '-C', oracle, 'print-ref'], capture_output=True, text=True).stdout.strip()
    if not os.path.isdir(os.path.join(ref, 'src')):
        pytest.skip('genetIC sources not present')
    r = subprocess.run(['make', '-s', '-C', oracle, '-B', '_ref/hook_check.o'], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
