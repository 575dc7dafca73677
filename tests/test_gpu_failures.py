"""Failure paths of the C ABI, made on the host or with bounded device waits (no GPU fault).

* mem_limit: a call that would allocate past the context's limit fails with
  GIC_ERR_OOM; the context stays usable and later calls that fit give the same
  results as an unlimited context.
* Transfer tables genetIC cannot use (too few valid rows, species columns with
  invalid entries in different rows, a wrong column count) are refused with
  GIC_ERR_INVALID_ARG (camb.hpp:224-268, interpolation.hpp:81-110).
* The FFT plane pass's bounded waits: with every wait given a target no task can
  reach, each gives up after a few polls, the kernel ends, and the call returns
  GIC_ERR_TIMEOUT; cleared again, the same context transforms correctly.
"""
import ctypes
import os

import numpy as np
import pytest

from conftest import make_generator

pytestmark = pytest.mark.gpu
SEED = 8896131


def _za(gen):
    gen.done()
    return [gen.field(l, 'psi_x') for l in range(len(gen.levels))]


def test_mem_limit_refuses_and_context_stays_usable(built, bbks):
    import genetic_gb300 as g
    from genetic_gb300 import _lib
    levels = [('base', 50.0, 64)]
    free = make_generator('fp64', bbks, levels, SEED, 'random_seed')
    want = _za(free)
    used_za, limit = free.memory_use()
    assert limit == 0 and used_za > 0
    free.centre(25, 25, 25)
    free.select_sphere(5)
    free.modify('overdensity', 'absolute', 0.5)
    free.apply_modifications()
    assert free.memory_use()[0] > used_za + (1 << 20)
    free.close()

    limit = used_za + (1 << 20)
    gen = g.ICGenerator(precision='fp64', mem_limit=limit)
    for k, v in (('Om', 0.31), ('Ol', 0.69), ('Ob', 0.0), ('hubble', 0.68), ('s8', 0.81), ('ns', 0.965), ('zin', 99)):
        getattr(gen, k)(v)
    gen.camb(bbks)
    gen.base_grid(50.0, 64)
    gen.random_seed(SEED)
    got = _za(gen)
    assert np.array_equal(got[0], want[0])
    used, got_limit = gen.memory_use()
    assert got_limit == limit and used <= limit
    gen.centre(25, 25, 25)
    gen.select_sphere(5)
    gen.modify('overdensity', 'absolute', 0.5)
    with pytest.raises(g.GicError) as e:
        gen.apply_modifications()
    assert e.value.code == _lib.GIC_ERR_OOM
    assert 'mem_limit' in str(e.value)
    assert gen.memory_use()[0] <= limit
    # usable afterwards: the refused call left the noise as it was
    gen._call('gic_clear_modifications')
    gen._call('gic_zeldovich', 1)
    assert np.array_equal(gen.field(0, 'psi_x'), want[0])
    gen.close()


def _transfer_status(table):
    import genetic_gb300 as g
    from genetic_gb300 import _lib
    from genetic_gb300.generator import _ptr
    gen = g.ICGenerator(precision='fp64')
    for k, v in (('Om', 0.31), ('Ol', 0.69), ('Ob', 0.0), ('hubble', 0.68), ('s8', 0.81), ('ns', 0.965), ('zin', 99)):
        getattr(gen, k)(v)
    gen._push_cosmology()
    t = np.ascontiguousarray(table, dtype=np.float64)
    st = gen._lib.gic_set_transfer(gen._ctx, _ptr(t), t.shape[0], t.shape[1])
    msg = gen._lib.gic_last_error(gen._ctx).decode()
    gen.close()
    return st, msg


def test_unusable_transfer_tables_are_refused(built, bbks):
    from genetic_gb300 import _lib
    nan = bbks.copy()
    nan[:, 1:] = np.nan
    st, msg = _transfer_status(nan)
    assert st == _lib.GIC_ERR_INVALID_ARG and 'valid values' in msg
    neg = bbks.copy()
    neg[:, 6] = -neg[:, 6]
    st, msg = _transfer_status(neg)
    assert st == _lib.GIC_ERR_INVALID_ARG
    holes = bbks.copy()
    holes[10:20, 6] = np.nan  # the total column loses rows the dark-matter column keeps
    st, msg = _transfer_status(holes)
    assert st == _lib.GIC_ERR_INVALID_ARG
    st, msg = _transfer_status(bbks[:, :5])
    assert st == _lib.GIC_ERR_INVALID_ARG and 'columns' in msg
    st, msg = _transfer_status(bbks)
    assert st == _lib.GIC_OK, msg


def test_plane_pass_wait_gives_up_with_timeout(built, bbks, monkeypatch):
    import genetic_gb300 as g
    from genetic_gb300 import _lib
    # the x pass and then the plane pass (variant 0) for every whole transform
    monkeypatch.setenv('GIC_FFT_TILE', '0,0,0')
    gen = make_generator('mixed', bbks, [('base', 100.0, 256)], SEED, 'random_seed')
    monkeypatch.delenv('GIC_FFT_TILE')
    gen.done()
    want = gen.field(0, 'psi_x')
    gen._call('gic_fft', 0, _lib.GIC_FIELD_PSI_X, -1)
    assert gen._lib.gic_set_fft_wait(gen._ctx, 16, 1) == _lib.GIC_OK
    with pytest.raises(g.GicError) as e:
        gen._call('gic_fft', 0, _lib.GIC_FIELD_PSI_X, +1)
    assert e.value.code == _lib.GIC_ERR_TIMEOUT
    assert 'gave up' in str(e.value)
    # cleared: the next transforms wait normally and round trip
    assert gen._lib.gic_set_fft_wait(gen._ctx, 0, 0) == _lib.GIC_OK
    gen.close()
    gen = make_generator('mixed', bbks, [('base', 100.0, 256)], SEED, 'random_seed')
    gen.done()
    assert gen._lib.gic_set_fft_wait(gen._ctx, 0, 0) == _lib.GIC_OK
    gen._call('gic_fft', 0, _lib.GIC_FIELD_PSI_X, -1)
    gen._call('gic_fft', 0, _lib.GIC_FIELD_PSI_X, +1)
    got = gen.field(0, 'psi_x')
    gen.close()
    assert np.abs(got - want).max() < 1e-5 * np.abs(want).max()
