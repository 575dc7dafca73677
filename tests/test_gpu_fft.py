"""Device FFTs against numpy on the half-spectrum layout."""
import numpy as np
import pytest

import field_oracle as fo
from conftest import make_generator

pytestmark = pytest.mark.gpu


def _noise_roundtrip(precision, n, bbks):
    gen = make_generator(precision, bbks, [('base', 50.0, n)], 7, 'random_seed')
    rng = np.random.default_rng(n)
    c = rng.standard_normal((n, n, n // 2 + 1)) + 1j * rng.standard_normal((n, n, n // 2 + 1))
    c = fo.fft_r2c(fo.fft_c2r(c))  # a consistent (Hermitian) half spectrum
    buf = np.ascontiguousarray(np.stack([c.real, c.imag], -1))
    import ctypes
    from genetic_gb300.generator import _ptr
    gen._call('gic_set_noise', 0, _ptr(buf))
    gen._call('gic_fft', 0, 0, +1)  # inverse in place: noise buffer now real
    # read back via the field path: copy raw buffer as complex then interpret padded reals
    raw = gen.noise(0)
    gen._call('gic_fft', 0, 0, -1)
    back = gen.noise(0)
    gen.close()
    reals = np.stack([raw.real, raw.imag], -1).reshape(n, n, -1)[:, :, :n]
    return c, reals, back


@pytest.mark.parametrize('n', [8, 16, 32, 64, 128, 192])
def test_fft_fp64(built, bbks, n):
    c, reals, back = _noise_roundtrip('fp64', n, bbks)
    want = fo.fft_c2r(c)
    assert np.abs(reals - want).max() < 1e-12 * np.abs(want).max()
    assert np.abs(back - c).max() < 1e-12 * np.abs(c).max()


@pytest.mark.parametrize('n', [16, 64, 256])
def test_fft_fp32(built, bbks, n):
    c, reals, back = _noise_roundtrip('mixed', n, bbks)
    want = fo.fft_c2r(c)
    assert np.abs(reals - want).max() < 2e-5 * np.abs(want).max()
    assert np.abs(back - c).max() < 2e-5 * np.abs(c).max()


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
@pytest.mark.parametrize('n', [32, 128, 256])
def test_fft_passes_bit_identical_across_tiles(built, bbks, precision, n, monkeypatch):
    """Every pass variant the tuner may pick (tile widths, fused first/last stages)
    and the runtime-length passes give bit-identical results: they share the radix
    schedule, the twiddles and the rounding of every operation (complex products
    are explicit fused multiply-adds)."""
    out = {}
    for tile in ('generic', '0,0', '1,1', '2,2', '3,3', '0,2', '2,0', '1,3', '3,3,0', '1,2,1', '0,1,2', '4,1', '5,3',
                 '6,3', '6,0', '6,2,1', '7,1'):
        monkeypatch.setenv('GIC_FFT_TILE', tile)
        _, reals, back = _noise_roundtrip(precision, n, bbks)
        out[tile] = (reals, back)
    ref = out['generic']
    for tile, (reals, back) in out.items():
        assert np.array_equal(reals, ref[0]), tile
        assert np.array_equal(back, ref[1]), tile


def test_fft_fp64_256(built, bbks):
    c, reals, back = _noise_roundtrip('fp64', 256, bbks)
    want = fo.fft_c2r(c)
    assert np.abs(reals - want).max() < 1e-12 * np.abs(want).max()
    assert np.abs(back - c).max() < 1e-12 * np.abs(c).max()


def _roundtrip_raw(precision, n, bbks, seed):
    """Inverse then forward transform of a seeded random half spectrum; the real field
    and the recovered coefficients (no oracle: for comparing pass variants)."""
    gen = make_generator(precision, bbks, [('base', 50.0, n)], 7, 'random_seed')
    rng = np.random.default_rng(seed)
    buf = rng.standard_normal((n, n, n // 2 + 1, 2))
    from genetic_gb300.generator import _ptr
    gen._call('gic_set_noise', 0, _ptr(buf))
    gen._call('gic_fft', 0, 0, +1)
    raw = gen.noise(0)
    gen._call('gic_fft', 0, 0, -1)
    back = gen.noise(0)
    gen.close()
    return raw, back


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_plane_pass_bit_identical_512(built, bbks, precision, monkeypatch):
    """The plane pass (y transforms and z rows of each x plane in one persistent
    kernel, ordered through L2) gives the same bits as the separate y and z passes,
    in every lag variant, for 512^3 in both precisions."""
    monkeypatch.setenv('GIC_FFT_TILE', '3,3')
    ref = _roundtrip_raw(precision, 512, bbks, 11)
    for tile in ('1,0', '3,3,0', '3,3,1', '3,3,2', '4,1', '5,1', '6,1', '6,3', '6,3,0', '7,1', '7,3', '7,3,1'):
        monkeypatch.setenv('GIC_FFT_TILE', tile)
        raw, back = _roundtrip_raw(precision, 512, bbks, 11)
        assert np.array_equal(raw, ref[0]), tile
        assert np.array_equal(back, ref[1]), tile


BOXES = [((3, 5, 0), (9, 17, 1)), ((60, 50, 7), (10, 20, 3)), ((0, 0, 0), (64, 12, 5)), ((17, 0, 2), (5, 64, 64)),
         ((1, 2, 3), (64, 64, 64))]


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
@pytest.mark.parametrize('n,tile', [(64, None), (256, None), (256, '6,3')])
def test_box_transforms_match_whole(built, bbks, precision, n, tile, monkeypatch):
    """Transforms restricted to a box of cells (the rows and planes outside skipped)
    give the whole transform's bits: forward transforms of fields zero outside the
    box (padding words of every row left non-zero, which the transform must not
    read), inverse transforms inside the box; boxes wrap around the grid.  With the
    tuner's passes, and with the TMA-staged strided pass pinned."""
    from genetic_gb300.generator import _ptr
    if tile:
        monkeypatch.setenv('GIC_FFT_TILE', tile)
    gen = make_generator(precision, bbks, [('base', 50.0, n)], 7, 'random_seed')
    rng = np.random.default_rng(5)
    sx = n // 64
    for start, length in BOXES:
        start = np.array([s * sx for s in start], dtype=np.int32)
        length = np.array([min(n, l * sx) for l in length], dtype=np.int32)
        inside = [((np.arange(n) - start[a]) % n) < length[a] for a in range(3)]
        mask = inside[0][:, None, None] & inside[1][None, :, None] & inside[2][None, None, :]
        # forward: padded real layout, zero outside the box, padding words non-zero
        real = np.zeros((n, n, 2 * (n // 2 + 1)))
        real[:, :, :n] = np.where(mask, rng.standard_normal((n, n, n)), 0.0)
        real[:, :, n:] = 7.0
        out = {}
        for kind in ('whole', 'box'):
            gen._call('gic_set_noise', 0, _ptr(np.ascontiguousarray(real)))
            if kind == 'whole':
                gen._call('gic_fft', 0, 0, -1)
            else:
                gen._call('gic_fft_box', 0, 0, -1, _ptr(start), _ptr(length))
            out[kind] = gen.noise(0)
        assert np.array_equal(out['whole'], out['box']), (start, length)
        # inverse: the reals inside the box
        spec = np.ascontiguousarray(rng.standard_normal((n, n, n // 2 + 1, 2)))
        for kind in ('whole', 'box'):
            gen._call('gic_set_noise', 0, _ptr(spec))
            if kind == 'whole':
                gen._call('gic_fft', 0, 0, +1)
            else:
                gen._call('gic_fft_box', 0, 0, +1, _ptr(start), _ptr(length))
            raw = gen.noise(0)
            out[kind] = np.stack([raw.real, raw.imag], -1).reshape(n, n, -1)[:, :, :n]
        assert np.array_equal(out['whole'][mask], out['box'][mask]), (start, length)
    gen.close()


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_tma_pass_bit_identical_in_the_modification_algebra(built, bbks, precision, monkeypatch):
    """The TMA-staged strided pass (its plain and store-windowed passes; the others fall
    back to the fused pass) against the fused pass everywhere, through the whole
    two-level realisation at 256^3 + 256^3 (zoom factor 4) with the four modifications:
    every field and particle is the same bits (in FP64 too: the path is deterministic)."""
    levels = [('base', 100.0, 256), ('zoom', 96, 96, 96, 4, 256)]
    out = {}
    for tile in ('3,3', '6,3'):
        monkeypatch.setenv('GIC_FFT_TILE', tile)
        gen = make_generator(precision, bbks, levels, 8896131, 'random_seed')
        gen.centre(50, 50, 50)
        gen.select_sphere(2.0)
        for name, t in (('overdensity', 1.5), ('vx', 0.0), ('vy', 0.0), ('vz', 0.0)):
            gen.modify(name, 'absolute', t)
        chi2 = gen.apply_modifications()
        gen.done(apply_modifications=False)
        out[tile] = (chi2, [gen.field(l, f) for l in range(2) for f in ('delta', 'psi_x', 'psi_y', 'psi_z')],
                     [gen.particles(l) for l in range(2)])
        gen.close()
    a, b = out['3,3'], out['6,3']
    assert a[0] == b[0]
    for x, y in zip(a[1], b[1]):
        assert np.array_equal(x, y)
    for (p, v), (p2, v2) in zip(a[2], b[2]):
        assert np.array_equal(p, p2) and np.array_equal(v, v2)


@pytest.mark.parametrize('precision', ['mixed'])
def test_shuffle_pass_box_inverse_512(built, bbks, precision, monkeypatch):
    """The TMA-staged pass with warp-shuffle stages (candidate 7, 512^3 FP32) on a box-restricted
    inverse transform (store windows on x and y) gives the fused pass's bits inside the box."""
    from genetic_gb300.generator import _ptr
    n = 512
    rng = np.random.default_rng(3)
    spec = np.ascontiguousarray(rng.standard_normal((n, n, n // 2 + 1, 2)))
    start = np.array([500, 37, 5], dtype=np.int32)
    length = np.array([40, 100, 512], dtype=np.int32)
    out = {}
    for tile in ('3,3', '7,3'):
        monkeypatch.setenv('GIC_FFT_TILE', tile)
        gen = make_generator(precision, bbks, [('base', 100.0, n)], 7, 'random_seed')
        gen._call('gic_set_noise', 0, _ptr(spec))
        gen._call('gic_fft_box', 0, 0, +1, _ptr(start), _ptr(length))
        raw = gen.noise(0)
        gen.close()
        real = np.stack([raw.real, raw.imag], -1).reshape(n, n, -1)[:, :, :n]
        ix = [(start[a] + np.arange(length[a])) % n for a in range(3)]
        out[tile] = real[np.ix_(ix[0], ix[1], ix[2])]
    assert np.array_equal(out['3,3'], out['7,3'])


@pytest.mark.parametrize('precision', ['fp64', 'mixed'])
def test_column_tables_bit_identical_in_the_modification_algebra(built, bbks, precision, monkeypatch):
    """The x passes' per-|k|^2 multipliers read from the per-coefficient layouts (the
    default from 256^3 up) against the gathers from the tables by |k|^2 (GIC_FFT_COLTAB=0),
    through the two-level realisation at 256^3 + 256^3 with the four modifications: the
    zoom combination's low-pass, the modification algebra's filters and the metric's
    epilogue all see the same values, so every field and particle is the same bits."""
    levels = [('base', 100.0, 256), ('zoom', 96, 96, 96, 4, 256)]
    out = {}
    for flag in ('0', '1'):
        monkeypatch.setenv('GIC_FFT_COLTAB', flag)
        gen = make_generator(precision, bbks, levels, 8896131, 'random_seed')
        gen.centre(50, 50, 50)
        gen.select_sphere(2.0)
        for name, t in (('overdensity', 1.5), ('vx', 0.0), ('vy', 0.0), ('vz', 0.0)):
            gen.modify(name, 'absolute', t)
        chi2 = gen.apply_modifications()
        gen.done(apply_modifications=False)
        out[flag] = (chi2, [gen.field(l, f) for l in range(2) for f in ('delta', 'psi_x', 'psi_y', 'psi_z')],
                     [gen.particles(l) for l in range(2)])
        gen.close()
    monkeypatch.delenv('GIC_FFT_COLTAB')
    a, b = out['0'], out['1']
    assert a[0] == b[0]
    for x, y in zip(a[1], b[1]):
        assert np.array_equal(x, y)
    for (p, v), (p2, v2) in zip(a[2], b[2]):
        assert np.array_equal(p, p2) and np.array_equal(v, v2)
