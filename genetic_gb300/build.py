"""Build libgicgpu.so (the CUDA kernels and the C ABI) in the package directory.

nvcc compiles each translation unit for sm_103a in parallel, then links one
shared library.  Nothing is installed: the library sits next to this file.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libgicgpu.so')
SOURCES = ['capi.cu', 'rng.cu', 'fft.cu', 'kspace.cu', 'particles.cu', 'zoom.cu', 'modify.cu', 'batch.cu', 'writers.cu']
# the host packer rounds every product and difference separately, as genetIC's host build does;
# the transfer spline's host solve gives the same bits on every host architecture
SOURCE_FLAGS = {'writers.cu': ['-Xcompiler', '-ffp-contract=off'], 'kspace.cu': ['-Xcompiler', '-ffp-contract=off']}
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-fvisibility=hidden',
         '--expt-relaxed-constexpr']


def nvcc():
    for cand in (os.environ.get('NVCC'), '/usr/local/cuda/bin/nvcc', 'nvcc'):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    raise RuntimeError('nvcc not found')


def _compile(src, extra):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + '.o')
    cmd = [nvcc(), *ARCH, *FLAGS, *SOURCE_FLAGS.get(src, []), *extra, '-I', os.path.join(HERE, '..', 'include'), '-c',
           os.path.join(CSRC, src), '-o', obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s%s' % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False, extra_flags=()):
    os.makedirs(BUILD, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, list(extra_flags)), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err.strip():
                print(err, file=sys.stderr)
    cmd = [nvcc(), *ARCH, '-shared', '-o', LIB, *objs, '-lcudart']
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('link failed:\n%s%s' % (r.stdout, r.stderr))
    return LIB


if __name__ == '__main__':
    print(build(verbose=True, extra_flags=sys.argv[1:]))
