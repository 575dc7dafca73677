"""Oracle (test infrastructure only): numpy restatement of genetIC's
single-level field-realisation path, used to check the GPU library.

Every function cites the genetIC code it restates.  Nothing in the shipped
library imports this module; only tests/, the smoke check and the benchmark's
CPU-baseline leg do.  White noise comes from the C restatement of the RANLUX +
ziggurat stream in rng/oracle_rng.c (liboracle.so), whose outputs are pinned to
the reference's golden chi^2 values and tipsy files.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBORACLE = os.path.join(HERE, '_ref', 'liboracle.so')

_lib = None


def build():
    """Build liboracle.so (no reference sources needed)."""
    subprocess.run(['make', '-s', '-C', HERE, '_ref/liboracle.so'], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIBORACLE):
            build()
        L = ctypes.CDLL(LIBORACLE)
        L.oracle_draw_white_noise.argtypes = [ctypes.c_int, ctypes.c_ulong, ctypes.c_int,
                                              ctypes.POINTER(ctypes.c_double)]
        L.oracle_gaussian_stream.argtypes = [ctypes.c_ulong, ctypes.POINTER(ctypes.c_double), ctypes.c_uint64]
        L.oracle_gaussian_stream.restype = ctypes.c_uint64
        L.oracle_ranlux_stream.argtypes = [ctypes.c_ulong, ctypes.POINTER(ctypes.c_uint32), ctypes.c_uint64]
        L.oracle_rng_set_cr_log.argtypes = [ctypes.c_int]
        L.oracle_draw_white_noise_levels.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_ulong,
                                                     ctypes.c_int, ctypes.POINTER(ctypes.POINTER(ctypes.c_double))]
        _lib = L
    return _lib


def set_cr_log(on):
    """Ziggurat tail log: C library (as GSL on glibc) or correctly rounded."""
    lib().oracle_rng_set_cr_log(1 if on else 0)


def gaussian_stream(seed, n):
    out = np.empty(int(n), dtype=np.float64)
    used = lib().oracle_gaussian_stream(int(seed), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(n))
    return out, int(used)


def ranlux_stream(seed, n):
    out = np.empty(int(n), dtype=np.uint32)
    lib().oracle_ranlux_stream(int(seed), out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), int(n))
    return out


# --- white noise (randomfieldgenerator.hpp:122-260) ---------------------------

_FFT_WORKERS = None


def set_fft_workers(workers):
    """Host threads for the transforms (scipy.fft's pocketfft); None: numpy, one thread."""
    global _FFT_WORKERS
    _FFT_WORKERS = workers


def fft_r2c(real):
    """Unitary forward transform, N^-1.5 (fourier.hpp:479-518)."""
    n = real.shape[0]
    if _FFT_WORKERS:
        import scipy.fft
        return scipy.fft.rfftn(real, workers=_FFT_WORKERS) / n ** 1.5
    return np.fft.rfftn(real) / n ** 1.5


def mirror(c):
    """Hermitian mirroring of the kz = 0 and N/2 planes before c2r (fourier.hpp:331-357)."""
    c = c.copy()
    n = c.shape[0]
    h = n // 2
    for kz in (0, h):
        p = c[:, :, kz]
        src = p.copy()
        for kx in range(h + 1, n):
            p[kx, :] = np.conj(src[n - kx, (-np.arange(n)) % n])
        for kx in (0, h):
            ky = np.arange(h + 1, n)
            p[kx, ky] = np.conj(src[kx, n - ky])
    return c


def fft_c2r(c):
    """Unitary inverse transform of a half spectrum, N^-1.5, after mirroring."""
    n = c.shape[0]
    if _FFT_WORKERS:
        import scipy.fft
        return scipy.fft.irfftn(mirror(c), s=(n, n, n), axes=(0, 1, 2), workers=_FFT_WORKERS) * n ** 1.5
    return np.fft.irfftn(mirror(c), s=(n, n, n), axes=(0, 1, 2)) * n ** 1.5


def white_noise(n, seed, mode):
    """Half spectrum (n, n, n/2+1) of the white noise genetIC draws (modes as in gicgpu.h)."""
    if mode == 0:
        real = np.empty(n ** 3, dtype=np.float64)
        lib().oracle_draw_white_noise(n, int(seed), 0, real.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        c = fft_r2c(real.reshape(n, n, n))
        c[0, 0, 0] = 0.0 + 1j * c[0, 0, 0].imag
        return c
    out = np.empty(n * n * (n // 2 + 1) * 2, dtype=np.float64)
    rc = lib().oracle_draw_white_noise(n, int(seed), int(mode), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    assert rc == 0
    out = out.reshape(n, n, n // 2 + 1, 2)
    return out[..., 0] + 1j * out[..., 1]


def white_noise_levels(ns, seed, mode):
    """Half spectra of every level, drawn in genetIC's level order."""
    bufs = []
    for n in ns:
        size = n ** 3 if mode == 0 else n * n * (n // 2 + 1) * 2
        bufs.append(np.empty(size, dtype=np.float64))
    arr = (ctypes.POINTER(ctypes.c_double) * len(ns))(*[b.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for b in bufs])
    nn = (ctypes.c_int * len(ns))(*ns)
    assert lib().oracle_draw_white_noise_levels(len(ns), nn, int(seed), int(mode), arr) == 0
    out = []
    for n, b in zip(ns, bufs):
        if mode == 0:
            c = fft_r2c(b.reshape(n, n, n))
            c[0, 0, 0] = 0.0 + 1j * c[0, 0, 0].imag
        else:
            b = b.reshape(n, n, n // 2 + 1, 2)
            c = b[..., 0] + 1j * b[..., 1]
        out.append(c)
    return out


def chi2(noise):
    """Hermitian-weighted sum of |w_k|^2 (multilevelfield.hpp:461-487, fourier.hpp:110-151)."""
    n = noise.shape[0]
    w = np.full(noise.shape[2], 2.0)
    w[0] = 1.0
    w[n // 2] = 1.0
    return float(np.sum(np.abs(noise) ** 2 * w[None, None, :]))


# --- power spectrum (camb.hpp, interpolation.hpp, parameters.hpp) -------------

class NaturalSpline:
    """Natural cubic spline in GSL's second-derivative form (interpolation.hpp:46-76)."""

    def __init__(self, x, y):
        x = np.asarray(x, float)
        y = np.asarray(y, float)
        n = len(x)
        c = np.zeros(n)
        if n >= 3:
            m = n - 2
            h0 = x[1:-1] - x[:-2]
            h1 = x[2:] - x[1:-1]
            diag = 2.0 * (h0 + h1)
            off = h1.copy()
            rhs = 3.0 * ((y[2:] - y[1:-1]) / h1 - (y[1:-1] - y[:-2]) / h0)
            for i in range(1, m):
                w = off[i - 1] / diag[i - 1]
                diag[i] -= w * off[i - 1]
                rhs[i] -= w * rhs[i - 1]
            c[m] = rhs[m - 1] / diag[m - 1]
            for i in range(m - 2, -1, -1):
                c[i + 1] = (rhs[i] - off[i] * c[i + 2]) / diag[i]
        self.x, self.y, self.c = x, y, c

    def __call__(self, v):
        v = np.asarray(v, float)
        x, y, c = self.x, self.y, self.c
        lo = np.clip(np.searchsorted(x, v, side='right') - 1, 0, len(x) - 2)
        h = x[lo + 1] - x[lo]
        dx = v - x[lo]
        dy = y[lo + 1] - y[lo]
        b = dy / h - h * (c[lo + 1] + 2.0 * c[lo]) / 3.0
        d = (c[lo + 1] - c[lo]) / (3.0 * h)
        out = y[lo] + dx * (b + dx * (c[lo] + dx * d))
        return np.where((v < x[0]) | (v > x[-1]), 0.0, out)


def growth_factor(a, om, ol):
    """Carroll, Press & Turner fit (parameters.hpp:55-70), including its single-precision a^3."""
    a3f = float(np.power(np.float32(a), np.float32(3.0)))
    hsq = om / a3f + (1. - om - ol) / a / a + ol
    return 2.5 * a * om / a ** 3.0 / hsq / (
        (om / hsq / a / a / a) ** float(np.float32(4.0) / np.float32(7.0)) - ol / hsq
        + (1. + 0.5 * om / a ** 3.0 / hsq) * (1. + 1. / 70. * ol / hsq))


class CambPower:
    """P(k) = A k^ns T(k)^2 from a CAMB table (camb.hpp:173-328)."""

    def __init__(self, table, cosmo, column=6):
        table = np.asarray(table, float)
        ncols = table.shape[1]
        assert ncols in (7, 13)
        tnorm = table[0, 1]
        keep = table[:, 0] > 0
        k = table[keep, 0]
        t = table[keep, column] / tnorm
        with np.errstate(divide='ignore', invalid='ignore'):
            lx, ly = np.log(k), np.log(t)
        ok = np.isfinite(lx) & np.isfinite(ly)
        self.spline = NaturalSpline(lx[ok], ly[ok])
        self.kpoints = k
        self.ns = cosmo['ns']
        a = 1.0 / (cosmo['redshift'] + 1.0)
        d = growth_factor(a, cosmo['omega_m'], cosmo['omega_lambda'])
        d0 = growth_factor(1.0, cosmo['omega_m'], cosmo['omega_lambda'])
        self.sigma8_pre = self.sigma_in_sphere(8.0)
        renorm = (cosmo['sigma8'] / self.sigma8_pre) * (d / d0)
        self.amplitude = renorm * renorm

    def transfer(self, k):
        k = np.asarray(k, float)
        with np.errstate(divide='ignore'):
            lk = np.log(k)
        inside = (lk >= self.spline.x[0]) & (lk <= self.spline.x[-1])
        return np.where(inside, np.exp(self.spline(np.where(inside, lk, self.spline.x[0]))), 0.0)

    def sigma_in_sphere(self, radius):
        """camb.hpp:300-328: Riemann sum, k accumulated by repeated addition."""
        kmax = min(self.kpoints[-1], 200.0 / radius) * 0.999999
        kmin = self.kpoints[0] * 1.000001
        dk = (kmax - kmin) / 50000.
        ks = []
        k = kmin
        while k < kmax:
            ks.append(k)
            k += dk
        ks = np.array(ks)
        t = self.transfer(ks)
        kr = ks * radius
        w = (np.sin(kr) - kr * np.cos(kr)) / (kr * kr * kr)
        s = float(np.sum(ks ** (self.ns + 2.) * w * w * t * t))
        return np.sqrt(s * 9. / 2. / np.pi / np.pi * dk)

    def __call__(self, k):
        k = np.asarray(k, float)
        t = np.where(k != 0, self.transfer(np.where(k != 0, k, 1.0)), 0.0)
        return self.amplitude * np.where(k != 0, k, 1.0) ** self.ns * t * t


def kgrid(n, box):
    """Integer and physical wavenumbers of the (n, n, n/2+1) half spectrum."""
    i = np.arange(n)
    ki = np.where(i > n // 2, i - n, i)
    kz = np.arange(n // 2 + 1)
    kmin = 2. * np.pi / box
    return ki, kz, kmin


def sqrt_power_grid(power, n, box):
    """sqrt(P_grid) on every stored mode (camb.hpp:101-139, field.hpp:394-412)."""
    ki, kz, kmin = kgrid(n, box)
    kx = (ki * kmin)[:, None, None]
    ky = (ki * kmin)[None, :, None]
    kzz = (kz * kmin)[None, None, :]
    k = np.sqrt(kx * kx + ky * ky + kzz * kzz)
    kw = 2. * np.pi / box
    norm = kw ** 3 / (2. * np.pi) ** 3 * n ** 3
    spec = power(k) * norm
    return np.sqrt(spec)


def zeldovich_fields(noise, power, box):
    """delta, psi_x, psi_y, psi_z in real space for one level (zeldovich.hpp:152-253)."""
    n = noise.shape[0]
    delta_k = noise * sqrt_power_grid(power, n, box)
    ki, kz, kmin = kgrid(n, box)
    kx = (ki * kmin)[:, None, None]
    ky = (ki * kmin)[None, :, None]
    kzz = (kz * kmin)[None, None, :]
    kk = kx * kx + ky * ky + kzz * kzz
    with np.errstate(divide='ignore', invalid='ignore'):
        base = 1j * delta_k / kk
    base[0, 0, 0] = 0
    nyq = n // 2
    out = [fft_c2r(delta_k)]
    for comp, kc, ic in ((0, kx, ki[:, None, None]), (1, ky, ki[None, :, None]), (2, kzz, kz[None, None, :])):
        psi_k = base * kc
        psi_k = np.where(ic == nyq, 0.0, psi_k)
        psi_k[0, 0, 0] = 0
        out.append(fft_c2r(psi_k))
    return out


def velocity_to_offset_ratio(cosmo):
    """parameters.hpp:84-106 (f = 1)."""
    a = 1.0 / (cosmo['redshift'] + 1.0)
    return 100. * np.sqrt(cosmo['omega_m'] / (a * a * a) + cosmo['omega_lambda']) * np.sqrt(a)


def particles(psi, box, offset, periodic, ratio):
    """Positions (wrapped) and velocities of every cell (zeldovich.hpp:87-124, generator.hpp:49-53)."""
    n = psi[0].shape[0]
    dx = box / n
    idx = np.arange(n, dtype=np.float64)
    cx = idx * dx + offset[0] + dx / 2
    cy = idx * dx + offset[1] + dx / 2
    cz = idx * dx + offset[2] + dx / 2
    X, Y, Z = np.meshgrid(cx, cy, cz, indexing='ij')
    pos = np.stack([psi[0] + X, psi[1] + Y, psi[2] + Z], axis=-1).reshape(-1, 3)
    pos = np.fmod(pos, periodic)
    pos = np.where(pos < 0, pos + periodic, pos)
    vel = np.stack([p * ratio for p in psi], axis=-1).reshape(-1, 3)
    return pos, vel


# --- zoom levels (multilevelgenerator.hpp:78-128, field.hpp:816-831, filter.hpp) ----

def fermi_lowpass(k, kcut):
    """LowPassFermiFilter (filter.hpp:208-239), temperature 0.1 k_cut."""
    return 1. / (1. + np.exp((k - kcut) / (kcut * 0.1)))


def kmag(n, box):
    ki, kz, kmin = kgrid(n, box)
    kx = (ki * kmin)[:, None, None]
    ky = (ki * kmin)[None, :, None]
    kzz = (kz * kmin)[None, None, :]
    return np.sqrt(kx * kx + ky * ky + kzz * kzz)


def displacement_spectra(delta_k, box):
    """psi_k = i k delta_k / k^2 with the Nyquist and k = 0 zeroing (zeldovich.hpp:155-181)."""
    n = delta_k.shape[0]
    ki, kz, kmin = kgrid(n, box)
    kx = (ki * kmin)[:, None, None]
    ky = (ki * kmin)[None, :, None]
    kzz = (kz * kmin)[None, None, :]
    kk = kx * kx + ky * ky + kzz * kzz
    with np.errstate(divide='ignore', invalid='ignore'):
        base = 1j * delta_k / kk
    base[0, 0, 0] = 0
    out = []
    for kc, ic in ((kx, ki[:, None, None]), (ky, ki[None, :, None]), (kzz, kz[None, None, :])):
        p = np.where(ic == n // 2, 0.0, base * kc)
        p[0, 0, 0] = 0
        out.append(p)
    return out


def catmull_rom_weights(t):
    t2, t3 = t * t, t * t * t
    return np.stack([-(t - 1) ** 2 * t / 2, (2 - 5 * t2 + 3 * t3) / 2, t * (1 + 4 * t - 3 * t2) / 2,
                     (t - 1) * t2 / 2], axis=-1)


def interpolate_to(coarse, cbox, coffset, periodic, fbox, fn, foffset):
    """Tricubic (Catmull-Rom tensor product) values of a coarse real field at the
    centroids of the fine grid's cells (field.hpp:483-509, 598-617): wrap on the
    periodic base grid, clamp on a zoom grid."""
    nc = coarse.shape[0]
    dxc, dxf = cbox / nc, fbox / fn
    wrap = cbox == periodic
    idx, wts = [], []
    for a in range(3):
        loc = np.arange(fn) * dxf + foffset[a] + dxf / 2 - coffset[a]
        loc = np.fmod(loc, periodic)
        loc = np.where(loc < 0, loc + periodic, loc)
        u = loc / dxc - 0.5
        i0 = np.floor(u)
        w = catmull_rom_weights(u - i0)
        ii = i0.astype(int)[:, None] + np.arange(-1, 3)[None, :]
        ii = ii % nc if wrap else np.clip(ii, 0, nc - 1)
        idx.append(ii)
        wts.append(w)
    g = np.einsum('xa,xayz->xyz', wts[0], coarse[idx[0]])
    g = np.einsum('yb,xybz->xyz', wts[1], g[:, idx[1]])
    g = np.einsum('zc,xyzc->xyz', wts[2], g[:, :, idx[2]])
    return g


def zoom_realisation(noises, levels, power):
    """Real-space delta, psi_x, psi_y, psi_z of every level after combination.
    levels: [(box, n, (x0, y0, z0))], level 0 periodic."""
    periodic = levels[0][0]
    raw_k = []  # per level: unfiltered delta_k
    out = []
    for (box, n, off), w in zip(levels, noises):
        raw_k.append(w * sqrt_power_grid(power, n, box))
    for li, ((box, n, off), dk) in enumerate(zip(levels, raw_k)):
        specs = [dk] + displacement_spectra(dk, box)
        if li > 0:
            cbox, cn, coff = levels[li - 1]
            kcut = 0.3 * (cn * 2. * np.pi / cbox)
            hp = np.sqrt(1. - fermi_lowpass(kmag(n, box), kcut) ** 2)
            specs = [s * hp for s in specs]
        fields = [fft_c2r(s) for s in specs]
        if li > 0:
            lp = fermi_lowpass(kmag(cn, cbox), kcut)
            src = [fft_r2c(f) * lp for f in out[li - 1]]
            for f, s in zip(fields, src):
                f += interpolate_to(fft_c2r(s), cbox, coff, periodic, box, n, off)
        out.append(fields)
    return out


# --- operations on the white noise (ic.hpp:1342-1344, 1652-1705) ---------------------------

def noise_reverse_small_k(noise, box, kmax):
    """-w where 0 < k^2 < kmax^2, k = integer * 2 pi / box per component (reverseSmallK)."""
    n = noise.shape[0]
    ki, kz, kmin = kgrid(n, box)
    kx = (ki * kmin)[:, None, None]
    ky = (ki * kmin)[None, :, None]
    kzz = (kz * kmin)[None, None, :]
    k2 = kx * kx + ky * ky + kzz * kzz
    return np.where((k2 < kmax * kmax) & (k2 != 0), -noise, noise)


def noise_unit_modulus(noise):
    """w / |w| where w != 0 (enforcePowerSpectrumOneGrid, multilevelfield.hpp:498-510)."""
    a = np.abs(noise)
    with np.errstate(invalid='ignore', divide='ignore'):
        return np.where(a == 0, 0, noise / np.where(a == 0, 1, a))


# --- second-order LPT (no counterpart in genetIC: Scoccimarro 1998, Crocce, Pueblas &
# Scoccimarro 2006, with Einstein-de Sitter growth: D2 = -3/7 D1^2, f2 = 2) -------------

LPT2_FACTOR = 3.0 / 7.0
_PAIRS = ((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))


def potential_hessian_spectra(delta_k, box):
    """phi_ij = k_i k_j delta_k / k^2 for ij = xx, yy, zz, xy, xz, yz (nabla^2 phi = delta);
    zero at k = 0, and the mixed ones where either component is the Nyquist mode
    (the first-derivative rule of zeldovich.hpp:173-178 applied twice)."""
    n = delta_k.shape[0]
    ki, kz, kmin = kgrid(n, box)
    comps = [((ki * kmin)[:, None, None], ki[:, None, None]), ((ki * kmin)[None, :, None], ki[None, :, None]),
             ((kz * kmin)[None, None, :], kz[None, None, :])]
    kk = comps[0][0] ** 2 + comps[1][0] ** 2 + comps[2][0] ** 2
    with np.errstate(divide='ignore', invalid='ignore'):
        base = delta_k / kk
    base[0, 0, 0] = 0
    out = []
    for a, b in _PAIRS:
        p = base * comps[a][0] * comps[b][0]
        if a != b:
            p = np.where((comps[a][1] == n // 2) | (comps[b][1] == n // 2), 0.0, p)
        p[0, 0, 0] = 0
        out.append(p)
    return out


def lpt2_source(phi):
    """S = sum_{i<j} (phi_ii phi_jj - phi_ij^2), so that nabla^2 phi2 = S."""
    xx, yy, zz, xy, xz, yz = phi
    return xx * yy + xx * zz + yy * zz - xy * xy - xz * xz - yz * yz


def _combine_levels(levels, own_specs, kcuts_hp):
    """Real fields per level: own spectra (x HP on zoom levels) to real space, plus the
    coarser level's combined fields low-passed and interpolated in (as zoom_realisation)."""
    periodic = levels[0][0]
    out = []
    for li, (box, n, off) in enumerate(levels):
        specs = own_specs[li]
        if li > 0:
            cbox, cn, coff = levels[li - 1]
            kcut = 0.3 * (cn * 2. * np.pi / cbox)
            hp = np.sqrt(1. - fermi_lowpass(kmag(n, box), kcut) ** 2)
            specs = [s * hp for s in specs]
        fields = [fft_c2r(s) for s in specs]
        if li > 0:
            lp = fermi_lowpass(kmag(cn, cbox), kcut)
            for f, c in zip(fields, out[li - 1]):
                f += interpolate_to(fft_c2r(fft_r2c(c) * lp), cbox, coff, periodic, box, n, off)
        out.append(fields)
    return out


def lpt2_realisation(noises, levels, power):
    """Second-order displacements (x, y, z) of every level: psi2 = (3/7) i k S_k / k^2
    from the combined potential Hessian of each level, combined across levels like
    the first-order fields."""
    hess = _combine_levels(levels, [potential_hessian_spectra(w * sqrt_power_grid(power, n, box), box)
                                    for (box, n, off), w in zip(levels, noises)], None)
    sources = [fft_r2c(lpt2_source(h)) * LPT2_FACTOR for h in hess]
    return _combine_levels(levels, [displacement_spectra(sk, box) for (box, n, off), sk in zip(levels, sources)],
                           None)


def particles_lpt2(psi1, psi2, box, offset, periodic, ratio):
    """Positions q + psi1 + psi2 (wrapped) and velocities ratio (psi1 + 2 psi2)."""
    pos, _ = particles([a + b for a, b in zip(psi1, psi2)], box, offset, periodic, ratio)
    vel = np.stack([(a + 2. * b) * ratio for a, b in zip(psi1, psi2)], axis=-1).reshape(-1, 3)
    return pos, vel


# --- modifications (modifications/*.hpp, multilevelfield.hpp, multilevelgrid.hpp) --------

class Levels:
    """Geometry of a multi-level context: [(box, n, (x0, y0, z0))], level 0 periodic."""

    def __init__(self, levels):
        self.levels = [(float(b), int(n), tuple(float(o) for o in off)) for b, n, off in levels]
        self.periodic = self.levels[0][0]
        dx0 = self.levels[0][0] / self.levels[0][1]
        # cell-volume weights relative to level 0 (multilevelgrid.hpp:121-124)
        self.weights = [(b / n / dx0) ** 3 for b, n, _ in self.levels]

    def __len__(self):
        return len(self.levels)

    def kcut(self, l):
        box, n, _ = self.levels[l]
        return 0.3 * (n * (2. * np.pi / box))

    def filter(self, l, k):
        """The family filter of level l (filterfamily.hpp:106-140): LP_0 on the base, HP_0 LP_1 ... HP_{l-1} LP_l."""
        f = np.ones_like(k)
        for m in range(l):
            f = f * np.sqrt(1. - fermi_lowpass(k, self.kcut(m)) ** 2)
        if l < len(self.levels) - 1:
            f = f * fermi_lowpass(k, self.kcut(l))
        return f

    def centroids(self, l, axis):
        box, n, off = self.levels[l]
        dx = box / n
        return np.arange(n) * dx + off[axis] + dx / 2

    def window_mask(self, l, window_level):
        """Cells of level l whose centroids lie in the box of level window_level (window.hpp)."""
        wbox, wn, woff = self.levels[window_level]
        masks = []
        for a in range(3):
            c = self.centroids(l, a)
            lo = np.fmod(woff[a], self.periodic)
            hi = np.fmod(woff[a] + wbox, self.periodic)
            if lo <= hi:
                masks.append((c >= lo) & (c < hi))
            else:
                masks.append((c >= lo) | (c < hi))
        return masks[0][:, None, None] & masks[1][None, :, None] & masks[2][None, None, :]


def flag_cells(levels, l, centre, kind, size):
    """Cells of level l selected by select_sphere / select_cube around `centre` (ic.hpp:1458-1524)."""
    box, n, off = levels.levels[l]
    L = levels.periodic
    d = []
    for a in range(3):
        x = levels.centroids(l, a) - centre[a]
        x = np.where(x > L / 2, x - L, np.where(x < -L / 2, x + L, x))
        d.append(x)
    X, Y, Z = np.meshgrid(d[0], d[1], d[2], indexing='ij')
    if kind == 'sphere':
        r2 = float(np.float32(size) * np.float32(size))
        sel = X * X + Y * Y + Z * Z < r2
    elif kind == 'ellipse':
        a2, b2, c2 = (float(np.float32(v) * np.float32(v)) for v in size)
        sel = X * X / a2 + Y * Y / b2 + Z * Z / c2 < 1.
    else:
        h = float(np.float32(size) / np.float32(2))
        sel = (np.abs(X) < h) & (np.abs(Y) < h) & (np.abs(Z) < h)
    return np.flatnonzero(sel.ravel())


def localisation_covector(levels, flagged, kind, direction=0):
    """Top-hat average over the flagged cells of the finest level, or the 4th-order
    -gradient stencil for velocity modifications (linearmodification.hpp:78-90, 202-240)."""
    box, n, _ = levels.levels[-1]
    out = np.zeros(n ** 3)
    w = 1.0 / len(flagged)
    if kind == 'overdensity':
        np.add.at(out, flagged, w)
        return out.reshape(n, n, n)
    dx = box / n
    a, b = -w / 12. / dx, w * 2. / 3. / dx
    coords = np.array(np.unravel_index(flagged, (n, n, n)))
    def idx(step):
        c = coords.copy()
        c[direction] = (c[direction] + step) % n
        return np.ravel_multi_index(c, (n, n, n))
    np.add.at(out, idx(-2), a)
    np.add.at(out, idx(-1), b)
    np.add.at(out, idx(1), -b)
    np.add.at(out, idx(2), -a)
    return out.reshape(n, n, n)


def flagged_centre(levels, flagged):
    """Grid::getCentreWrapped (grid.hpp:466-494) on the finest level: the mean of the
    wrapped offsets from the first cell, added back and wrapped."""
    box, n, off = levels.levels[-1]
    L = levels.periodic
    dx = box / n
    coords = np.array(np.unravel_index(np.asarray(flagged, dtype=np.int64), (n, n, n)), dtype=np.float64)
    cen = []
    for a in range(3):
        c = coords[a] * dx + off[a] + dx / 2
        d = c[1:] - c[0]
        d = np.where(d > L / 2, d - L, np.where(d < -L / 2, d + L, d))
        run = 0.0
        for v in d:  # the reference's running sum, in order
            run += v
        v = run / len(c) + c[0]
        cen.append(np.fmod(v, L) + (L if np.fmod(v, L) < 0 else 0))
    return np.array(cen)


def localisation_covector_am(levels, flagged, direction):
    """AngMomentumModification::calculateLocalisationCovector (linearmodification.hpp:333-383)."""
    box, n, off = levels.levels[-1]
    L = levels.periodic
    dx = box / n
    cen = flagged_centre(levels, flagged)
    norm = len(flagged) * dx
    a, b = 1. / 12. / norm, -2. / 3. / norm
    out = np.zeros(n ** 3)
    coords = np.array(np.unravel_index(np.asarray(flagged, dtype=np.int64), (n, n, n)))
    q = coords * dx + np.array(off)[:, None] + dx / 2
    dq = cen[:, None] - q
    dq = np.where(dq > L / 2, dq - L, np.where(dq < -L / 2, dq + L, dq))
    d1, d2 = (direction + 1) % 3, (direction + 2) % 3
    coeff = np.zeros_like(dq)
    coeff[d2] = dq[d1]
    coeff[d1] = -dq[d2]
    for ax in range(3):
        if ax == direction:
            continue
        def idx(step):
            c = coords.copy()
            c[ax] = (c[ax] + step) % n
            return np.ravel_multi_index(c, (n, n, n))
        np.add.at(out, idx(-2), coeff[ax] * a)
        np.add.at(out, idx(-1), coeff[ax] * b)
        np.add.at(out, idx(1), -coeff[ax] * b)
        np.add.at(out, idx(2), -coeff[ax] * a)
    return out.reshape(n, n, n)


def density_to_potential(field_k, box, cosmo):
    """cosmology::densityToPotential (cosmology/parameters.hpp:209-225), including its
    k = 0 guard that tests the y component, so modes with ky = 0 become zero."""
    n = field_k.shape[0]
    ki, kz, kmin = kgrid(n, box)
    kx = (ki * kmin)[:, None, None]
    ky = (ki * kmin)[None, :, None]
    kzz = (kz * kmin)[None, None, :]
    ksq = kx * kx + ky * ky + kzz * kzz
    a = 1.0 / (cosmo['redshift'] + 1.0)
    prefac = 3. / 2. * cosmo['omega_m'] / a * 100. * 100. / (299792.) / (299792.)
    with np.errstate(divide='ignore'):
        inv = np.where(ky == 0.0, 0.0, 1.0 / ksq)
    return -prefac * field_k * inv


def _axis_geometry(levels, fine, coarse, axis):
    cbox, cn, coff = levels.levels[coarse]
    dxc = cbox / cn
    loc = levels.centroids(fine, axis) - coff[axis]
    loc = np.fmod(loc, levels.periodic)
    loc = np.where(loc < 0, loc + levels.periodic, loc)
    u = loc / dxc - 0.5
    i0 = np.floor(u)
    return i0.astype(int), catmull_rom_weights(u - i0)


def deinterpolate(levels, hires, fine, coarse):
    """Transpose of the tricubic interpolation, fine real field -> coarse real field
    (field.hpp:420-480 via multilevelgrid.hpp:245-306); stencil indices wrap."""
    cn = levels.levels[coarse][1]
    out = hires
    for axis in range(3):
        i0, w = _axis_geometry(levels, fine, coarse, axis)
        shape = list(out.shape)
        shape[axis] = cn
        acc = np.zeros(shape)
        moved = np.moveaxis(out, axis, 0)
        accm = np.moveaxis(acc, axis, 0)
        for a in range(4):
            idx = (i0 + a - 1) % cn
            np.add.at(accm, idx, w[:, a].reshape((-1,) + (1,) * (moved.ndim - 1)) * moved)
        out = acc
    return out


def subsample_average(levels, fine_real, fine, coarse):
    """Average of the fine cells inside each coarse cell covered by the fine grid, 0
    elsewhere (SubSampleEvaluator, evaluator.hpp:180-207)."""
    fbox, fn, foff = levels.levels[fine]
    cbox, cn, coff = levels.levels[coarse]
    r = int(round((cbox / cn) / (fbox / fn)))
    m = fn // r
    avg = fine_real.reshape(m, r, m, r, m, r).mean(axis=(1, 3, 5))
    out = np.zeros((cn, cn, cn))
    start = [int(round((foff[a] - coff[a]) / (cbox / cn))) for a in range(3)]
    ix = [(start[a] + np.arange(m)) % cn for a in range(3)]
    out[np.ix_(ix[0], ix[1], ix[2])] += avg
    return out


def _kmag_level(levels, l):
    box, n, _ = levels.levels[l]
    return kmag(n, box)


def multilevel_covector(levels, hires_real, power_dm, velocity_scale=None, potential_cosmo=None):
    """ConstraintField of a modification in Fourier space on every level
    (multilevelgrid.hpp:245-321, linearmodification.hpp:64-75, 134-141, 242-297).
    velocity_scale: None for an overdensity, else the velocity-to-offset ratio
    (velocity and angular-momentum modifications); potential_cosmo: the cosmology of
    a potential modification (linearmodification.hpp:160-167)."""
    nl = len(levels)
    real = [None] * nl
    real[-1] = fft_c2r(fft_r2c(hires_real))
    for l in range(nl - 2, -1, -1):
        ratio = int(round((levels.levels[l][0] / levels.levels[l][1]) /
                          (levels.levels[l + 1][0] / levels.levels[l + 1][1])))
        real[l] = deinterpolate(levels, real[l + 1] / ratio ** 3, l + 1, l)
    out = []
    for l in range(nl):
        box, n, _ = levels.levels[l]
        f = fft_r2c(real[l] * (levels.weights[l] / levels.weights[-1])) * levels.filter(l, _kmag_level(levels, l))
        f = fft_r2c(fft_c2r(f))  # toReal then back to Fourier, as the reference does
        f = f * sqrt_power_grid(power_dm, n, box)
        if velocity_scale is not None:
            kk = _kmag_level(levels, l) ** 2
            with np.errstate(divide='ignore', invalid='ignore'):
                v = -velocity_scale * f / kk
            v[0, 0, 0] = 0
            f = v
        if potential_cosmo is not None:
            f = density_to_potential(f, box, potential_cosmo)
        out.append(f)
    return out


def inner(a, b):
    """Hermitian-weighted sum over levels of Re(conj a b) (multilevelfield.hpp:248-294)."""
    s = 0.0
    for x, y in zip(a, b):
        n = x.shape[0]
        w = np.full(x.shape[2], 2.0)
        w[0] = 1.0
        w[n // 2] = 1.0
        s += float(np.sum(np.real(np.conj(x) * y) * w[None, None, :]))
    return s


def cross_level_term(levels, field_k, target, source):
    """addFieldFromDifferentGridWithFilter(source, f_t f_s sqrt(w_t/w_s)) onto the
    target's real grid (multilevelfield.hpp:362-378, field.hpp:816-831)."""
    k = _kmag_level(levels, source)
    filt = levels.filter(target, k) * levels.filter(source, k) * np.sqrt(levels.weights[target] / levels.weights[source])
    src_real = fft_c2r(field_k[source] * filt)
    if source < target:
        tbox, tn, toff = levels.levels[target]
        sbox, sn, soff = levels.levels[source]
        return interpolate_to(src_real, sbox, soff, levels.periodic, tbox, tn, toff)
    return subsample_average(levels, src_real, source, target)


def apply_metric(levels, field_k, to_covector):
    """MultiLevelField::applyMetric (multilevelfield.hpp:344-384); fields in Fourier space."""
    nl = len(levels)
    out = []
    for l in range(nl):
        k = _kmag_level(levels, l)
        f = levels.filter(l, k)
        x = field_k[l].copy()
        if to_covector and l < nl - 1:
            mask = levels.window_mask(l, l + 1)
            # applyFilterInWindow(f, window, windowFirst=true) then (.., false) (field.hpp:752-775)
            xr = fft_c2r(x)
            inw = fft_r2c(np.where(mask, xr, 0.0)) * f
            x = fft_r2c(np.where(mask, 0.0, xr)) + inw
            xr = fft_c2r(x)
            inw_r = np.where(mask, fft_c2r(x * f), 0.0)
            x = fft_r2c(np.where(mask, 0.0, xr) + inw_r)
        else:
            x = x * f * f
        xr = fft_c2r(x)
        for s in range(nl):
            if s != l:
                xr = xr + cross_level_term(levels, field_k, l, s)
        out.append(fft_r2c(xr))
    return out


def chi2_levels(levels, noise_k):
    return inner(apply_metric(levels, noise_k, True), noise_k)


def apply_linear_modifications(levels, noise_k, covectors, targets, return_vectors=False):
    """Gram-Schmidt + correction (modificationmanager.hpp:199-217, 288-312), restated
    with the same operation order; returns the modified noise (and, with
    return_vectors, the orthonormalised covectors converted to vectors)."""
    alphas = [[c.copy() for c in cv] for cv in covectors]
    t = list(targets)
    n = len(alphas)
    for i in range(n):
        for j in range(i):
            r = inner(alphas[i], apply_metric(levels, alphas[j], False))
            alphas[i] = [a - r * b for a, b in zip(alphas[i], alphas[j])]
            t[i] -= r * t[j]
        nrm = np.sqrt(inner(alphas[i], apply_metric(levels, alphas[i], False)))
        alphas[i] = [a / nrm for a in alphas[i]]
        t[i] /= nrm
    existing = [inner(a, noise_k) for a in alphas]
    out = [w.copy() for w in noise_k]
    vectors = []
    for i in range(n):
        vec = apply_metric(levels, alphas[i], False)
        vectors.append(vec)
        d = t[i] - existing[i]
        out = [o + d * v for o, v in zip(out, vec)]
    if return_vectors:
        return out, vectors
    return out


# --- quadratic (variance) modification (quadraticmodification.hpp, modificationmanager.hpp) ---

def variance_highpass(k, scale):
    """1 - LP_Fermi(k; 2 pi / scale) (ComplementaryFilterAdaptor, quadraticmodification.hpp:187-195)."""
    return 1. - fermi_lowpass(k, 2. * np.pi / scale)


def push_variance(levels, field_k, flagged, scale, power_dm):
    """<field| Q as a covector (QuadraticModification::pushMultiLevelFieldThroughMatrix,
    quadraticmodification.hpp:59-92, and FilteredVarianceModification::
    pushOneLevelFieldThroughMatrix, :152-221): per level x = sqrt(P_dm) w, then
    window, high-pass, variance (window, minus the region mean, / n), high-pass,
    window; the covector metric; sqrt(P_dm) again.  flagged: cells per level."""
    pushed = []
    sp = []
    for l in range(len(levels)):
        box, n, _ = levels.levels[l]
        sp.append(sqrt_power_grid(power_dm, n, box))
        hp = variance_highpass(kmag(n, box), scale)
        fl = np.asarray(flagged[l], dtype=np.int64)

        def window(v):
            out = np.zeros(n ** 3)
            out[fl] = v.ravel()[fl]
            return out.reshape(n, n, n)

        xr = window(fft_c2r(field_k[l] * sp[l]))
        xr = window(fft_c2r(fft_r2c(xr) * hp))
        flat = xr.ravel()
        mean = float(np.sum(flat[fl])) / len(fl)
        flat[fl] = (flat[fl] - mean) / len(fl)
        xr = window(fft_c2r(fft_r2c(flat.reshape(n, n, n)) * hp))
        pushed.append(fft_r2c(xr))
    cov = apply_metric(levels, pushed, True)
    return [c * s for c, s in zip(cov, sp)]


def variance_value(levels, field_k, flagged, scale, power_dm):
    """QuadraticModification::calculateCurrentValue (quadraticmodification.hpp:51-57)."""
    return inner(push_variance(levels, field_k, flagged, scale, power_dm), field_k)


def linspace_targets(start, end, n):
    """tools::linspace (util_functions.hpp:77-92): n+1 points for n > 1."""
    if n in (0, 1) or start == end:
        return [end]
    step = (end - start) / n
    return [start + c * step for c in range(n + 1)]


def perform_quadratic_iterations(levels, field_k, lin_vectors, flagged, scale, power_dm, target, n_steps):
    """ModificationManager::performIterations (modificationmanager.hpp:249-275) with
    addToOrthonormalFamily (:318-333).  lin_vectors are the orthonormalised linear
    covectors after applyLinearModif converted them to vectors in place (:168-182),
    so the projection uses plain products with them."""
    field = [f.copy() for f in field_k]
    start = variance_value(levels, field, flagged, scale, power_dm)
    targets = linspace_targets(start, target, n_steps)
    for i in range(n_steps):
        p = push_variance(levels, field, flagged, scale, power_dm)
        current = inner(p, field)
        norm = np.sqrt(inner(p, apply_metric(levels, p, False)))
        for v in lin_vectors:
            r = inner(p, v)
            p = [a - r * b for a, b in zip(p, v)]
        n2 = np.sqrt(inner(p, apply_metric(levels, p, False)))
        p = [a / n2 for a in p]
        mult = 0.5 * (targets[i + 1] - current) / norm
        vec = apply_metric(levels, p, False)
        field = [f + mult * v for f, v in zip(field, vec)]
    return field


def apply_quadratic_modification(levels, field_k, lin_vectors, flagged, scale, power_dm, target,
                                 init_steps=10, precision=0.001):
    """applyLinQuadModif (modificationmanager.hpp:221-246) with calculateCorrectNumberSteps
    (:278-285): a trial on a copy fixes the number of steps.  Returns (field, steps)."""
    test = perform_quadratic_iterations(levels, field_k, lin_vectors, flagged, scale, power_dm, target, init_steps)
    achieved = abs(variance_value(levels, test, flagged, scale, power_dm) - target)
    n_steps = init_steps * int(np.ceil(np.sqrt(achieved / (target * precision))))
    steps = n_steps if n_steps > init_steps else init_steps
    return perform_quadratic_iterations(levels, field_k, lin_vectors, flagged, scale, power_dm, target, steps), steps


# --- splicing (modifications/splice.hpp:37-118, tools/numerics/cg.hpp:13-59) -----------------

def power_grid(power, n, box):
    """P_grid on every stored mode (the covariance genetIC keeps per level, camb.hpp:101-139)."""
    return sqrt_power_grid(power, n, box) ** 2


def apply_transfer(field_k, cov, p):
    """Field::applyTransferFunction (field.hpp:394-412): times cov^p, cov^p = cov where p = 1,
    and 0 where cov = 0."""
    with np.errstate(divide='ignore', invalid='ignore'):
        t = np.where(cov != 0.0, np.power(cov, p), 0.0) if p != 1.0 else cov
    return field_k * t


def c2r_with_tail(c):
    """Field::toReal as genetIC stores the result: the n^3 values compact at the front of
    the padded buffer (fourier.hpp:388-404, 479-518), and behind them the padded c2r
    output that the compaction did not overwrite -- the last rows' values and their
    padding slots, which hold the kz = n/2 coefficient after the x and y passes -- all
    divided by n^1.5.  Returns (real field, tail of 2 n^2 values)."""
    n = c.shape[0]
    m = mirror(c)
    xy = np.fft.ifft(np.fft.ifft(m, axis=0), axis=1) * n * n
    real = np.fft.irfftn(m, s=(n, n, n), axes=(0, 1, 2)) * n ** 3
    padded = np.zeros((n, n, n + 2))
    padded[:, :, :n] = real
    padded[:, :, n] = xy[:, :, n // 2].real
    padded[:, :, n + 1] = xy[:, :, n // 2].imag
    flat = padded.ravel() / n ** 1.5
    return real / n ** 1.5, flat[n ** 3:].copy()


class StoredReal:
    """A real field as genetIC holds it: values plus the buffer's tail.  Field's +=, -=,
    addScaled, negation and innerProduct run over the whole buffer (field.hpp:331-383);
    the mask multiply over the n^3 values only (field.hpp:306-318)."""

    def __init__(self, r, t):
        self.r, self.t = r, t

    def __add__(self, o):
        return StoredReal(self.r + o.r, self.t + o.t)

    def __sub__(self, o):
        return StoredReal(self.r - o.r, self.t - o.t)

    def __neg__(self):
        return StoredReal(-self.r, -self.t)

    def scaled(self, a):
        return StoredReal(self.r * a, self.t * a)

    def masked(self, m):
        return StoredReal(self.r * m, self.t.copy())

    def dot(self, o):
        return float(np.sum(self.r * o.r) + np.sum(self.t * o.t))


def conjugate_gradient(Q, b, rtol=1e-6, atol=1e-12):
    """tools::numerics::conjugateGradient on StoredReal fields; returns (x, iterations)."""
    residual = StoredReal(b.r.copy(), b.t.copy())
    direction = -residual
    x = StoredReal(np.zeros_like(b.r), np.zeros_like(b.t))
    scale = np.sqrt(b.dot(b))
    if scale == 0.0:
        return x, 0
    for i in range(b.r.size + 1):
        q_dir = Q(direction)
        alpha = -residual.dot(direction) / direction.dot(q_dir)
        x = x + direction.scaled(alpha)
        residual = Q(x) - b
        norm = np.sqrt(residual.dot(residual))
        if norm < rtol * scale or norm < atol:
            break
        beta = residual.dot(q_dir) / direction.dot(q_dir)
        direction = direction.scaled(beta) - residual
    return x, i


def splice_one_level(a_k, b_k, cov, flagged):
    """spliceOneLevel(a, b, cov): the field equal to a on the flagged cells and closest
    to b elsewhere in the C^-1 norm (splice.hpp:37-118); Fourier in, Fourier out; also
    the CG iterations.  The CG's scalars include the buffers' tails, as in the reference."""
    n = a_k.shape[0]
    mask = np.zeros(n ** 3)
    mask[np.asarray(flagged, dtype=np.int64)] = 1.0
    mask = mask.reshape(n, n, n)
    compl = 1.0 - mask
    pre = cov.copy()
    pre[0, 0, 0] = 1.0

    def P(f, p):
        return StoredReal(*c2r_with_tail(apply_transfer(fft_r2c(f.r), pre, p)))

    delta_diff = StoredReal(*c2r_with_tail(apply_transfer(b_k - a_k, pre, 0.5)))
    z = P(P(delta_diff.masked(mask), -1.0).masked(compl), 0.5)

    def X(v):
        return P(P(P(v, 0.5).masked(compl), -1.0).masked(compl), 0.5)

    alpha, its = conjugate_gradient(X, z)
    alpha = P(alpha, 0.5)
    b_delta = StoredReal(*c2r_with_tail(apply_transfer(b_k, pre, 0.5)))
    result = alpha.masked(compl) + b_delta - delta_diff.masked(mask)
    return apply_transfer(fft_r2c(result.r), pre, -0.5), its


def splice_levels(levels, original, new, power, flagged):
    """ICGenerator::splice (ic.hpp:1658-1688) per level: the new field on the flagged cells."""
    out, its = [], []
    for (box, n, off), w_old, w_new, fl in zip(levels, original, new, flagged):
        s, i = splice_one_level(w_new, w_old, power_grid(power, n, box), fl)
        out.append(s)
        its.append(i)
    return out, its


# --- tipsy output (genetIC/src/io/tipsy.hpp:109-145, 200-262) ---------------------------

def block_cells(parents, np_, nc, ratio, origin):
    """For every parent cell (ids on a grid of np_ per side), the ratio^3 cells it covers on
    the grid of nc per side whose corner is parent cell `origin`, x, y, z ascending
    (Grid::insertCubeIdsIntoVector, grid.hpp:704-729; iterateOverCube, coordinate.hpp:197-208)."""
    parents = np.asarray(parents, dtype=np.int64)
    px, py, pz = parents // (np_ * np_), (parents // np_) % np_, parents % np_
    px, py, pz = ((px - origin[0]) % np_, (py - origin[1]) % np_, (pz - origin[2]) % np_)
    s = np.arange(ratio ** 3)
    sx, sy, sz = s // (ratio * ratio), (s // ratio) % ratio, s % ratio
    fx = px[:, None] * ratio + sx[None, :]
    fy = py[:, None] * ratio + sy[None, :]
    fz = pz[:, None] * ratio + sz[None, :]
    return ((fx * nc + fy) * nc + fz).ravel()


def mapper_order_levels(levels, replaced):
    """(level, cell) of every particle in genetIC's mapper order for any number of levels:
    a OneLevelParticleMapper of level 0 wrapped in one TwoLevelParticleMapper per zoom level
    (ic.hpp:1150-1185; particles/mapper/twolevelmapper.hpp:262-320, 869-893).  Each wrapping
    drops the replaced cells of the level above from the order so far, then appends the
    blocks of those cells in ascending cell id.  levels: [(n, ratio, origin)];
    replaced[l]: level-l cell ids replaced by level l+1."""
    n0 = levels[0][0]
    lev = np.zeros(n0 ** 3, dtype=np.int64)
    cells = np.arange(n0 ** 3, dtype=np.int64)
    for l in range(1, len(levels)):
        pn = levels[l - 1][0]
        n, ratio, origin = levels[l]
        rep = np.sort(np.asarray(replaced[l - 1], dtype=np.int64))
        drop = (lev == l - 1) & np.isin(cells, rep)
        lev, cells = lev[~drop], cells[~drop]
        fine = block_cells(rep, pn, n, ratio, origin)
        lev = np.concatenate([lev, np.full(len(fine), l, dtype=np.int64)])
        cells = np.concatenate([cells, fine])
    return lev, cells


def mapper_order(n0, replaced=(), n1=0, ratio=1, origin=(0, 0, 0)):
    """The mapper order of one level, or of two when `replaced` level-0 cells are given."""
    if len(replaced) == 0:
        return mapper_order_levels([(n0, 1, (0, 0, 0))], [])
    return mapper_order_levels([(n0, 1, (0, 0, 0)), (n1, ratio, origin)], [replaced])


def tipsy_factors(levels, cosmo, order_levels, soft_scale=None):
    """Per-level particle mass and softening (zeldovich.hpp:55-62, 112-121, grid.hpp:112)
    and TipsyOutput's factors (tipsy.hpp:200-239): mass_factor = Om / (masses summed in
    mapper order), pos_factor = 1 / box, vel_factor = a^-1/2 / dKmsUnit.  soft_scale: per
    level the grid's cellSofteningScale (1; a supersampled virtual grid's is its factor,
    virtualgrid.hpp:139-146)."""
    L = levels[0][0]
    om, h = cosmo['omega_m'], cosmo['hubble']
    a = 1.0 / (1.0 + cosmo['redshift'])
    box_mass = 27.744948 * om * pow(L, 3.0)
    mass = [box_mass * pow((b / n) / L, 3.0) for b, n, _ in levels]
    soft_scale = soft_scale or [1.0] * len(levels)
    eps = [(b / n) * float(sc) * 0.01075 for (b, n, _), sc in zip(levels, soft_scale)]
    tot = 0.0
    for lv in order_levels:  # the reference's running double sum
        tot += mass[lv]
    mass_factor = om / tot
    pos_factor = 1. / L
    kpc = L * 1000 / h
    msol = 1e10 / h / mass_factor
    kms = np.sqrt(4.3022682e-6 * msol / kpc)
    vel_factor = pow(a, -0.5) / kms
    return mass, eps, pos_factor, vel_factor, mass_factor


def resample_displacements(psi, box, n, offset, periodic, factor):
    """A level's displacement fields on genetIC's supersampled (factor >= 2) or subsampled
    (factor <= -2) virtual grid of the same region (SuperSampleEvaluator / SubSampleEvaluator,
    evaluator.hpp:96-207; virtualgrid.hpp:126-160, 528-605): the tricubic of the level's
    fields at the virtual centroids (wrapped on the periodic base level, clamped on a zoom
    level), or the mean of each block of |factor|^3 cells.  Returns (fields, cells per side)."""
    if factor > 1:
        nv = n * factor
        return [interpolate_to(p, box, offset, periodic, box, nv, offset) for p in psi], nv
    s = -factor
    nv = n // s
    return [p.reshape(nv, s, nv, s, nv, s).sum(axis=(1, 3, 5)) / float(s ** 3) for p in psi], nv


def matched_displacements(psi_fine, fine, psi_coarse, coarse, periodic):
    """A zoom level's displacements on its resolution-matching grid, the output grid of a
    zoom level with stray particles on (ResolutionMatchingGrid / ResolutionMatchingEvaluator,
    virtualgrid.hpp:217-300, evaluator.hpp:208-256): the zoom's resolution over the whole
    region of the level above; the coarse level's fields supersampled (tricubic at the fine
    centroids), overwritten by the zoom's own inside its window.  fine, coarse: (box, n, offset).
    Returns (fields, cells per side, the matching grid's (box, n, offset))."""
    fbox, fn, foff = fine
    cbox, cn, coff = coarse
    r = int(round((cbox / cn) / (fbox / fn)))
    nv = cn * r
    out = [interpolate_to(p, cbox, coff, periodic, cbox, nv, coff) for p in psi_coarse]
    w0 = [int(round((foff[a] - coff[a]) / (fbox / fn))) for a in range(3)]
    ix = [(w0[a] + np.arange(fn)) % nv for a in range(3)]
    for o, p in zip(out, psi_fine):
        o[np.ix_(ix[0], ix[1], ix[2])] = p
    return out, nv, (cbox, nv, coff)


def grafic_slabs(fields, box, n, offset, periodic, factor, roll, ratio, vel_factor, pos_factor, id_offset):
    """genetIC's grafic writer on one grid of its stack (GraficOutput::writeGrid,
    io/grafic.hpp:160-200): the level's fields (delta, psi_x, psi_y, psi_z) on the grid
    (the level itself, or its supersampled / subsampled virtual grid), seen through a
    CenteredGrid (virtualgrid.hpp:680-800: output cell (x, y, z) is the grid's cell
    (x, y, z) - roll, periodically).  Per cell as the files hold them, each [z][y][x]:
    velocities (psi * ratio * vel_factor, in double, then float), displacements
    (psi * pos_factor), the overdensity, and ids (the grid cell's index + id_offset)."""
    if factor == 1:
        f, nv = list(fields), n
    else:
        f, nv = resample_displacements(fields, box, n, offset, periodic, factor)
    idx = [(np.arange(nv) - roll[a]) % nv for a in range(3)]
    # out[z][y][x] = field[ux][uy][uz]
    pick = lambda a: a[np.ix_(idx[0], idx[1], idx[2])].transpose(2, 1, 0)
    ux, uy, uz = np.meshgrid(idx[0], idx[1], idx[2], indexing='ij')
    ids = (((ux.astype(np.uint64) * nv + uy) * nv + uz) + np.uint64(id_offset)).transpose(2, 1, 0)
    vel = [(pick(p).astype(np.float64) * ratio * vel_factor).astype(np.float32) for p in f[1:]]
    pos = [(pick(p).astype(np.float64) * pos_factor).astype(np.float32) for p in f[1:]]
    return vel, pos, pick(f[0]).astype(np.float32), ids


def tipsy_records(order, pos, vel, mass, eps, pos_factor, vel_factor, mass_factor):
    """Dark records (mass, x, y, z, vx, vy, vz, eps, phi) as float32 (tipsy.hpp:61-63,
    123-131): products and differences in double, then rounded to float."""
    lev, cells = order
    out = np.zeros((len(cells), 9), dtype=np.float32)
    for l in range(len(pos)):
        sel = lev == l
        c = cells[sel]
        out[sel, 0] = np.float32(mass[l] * mass_factor)
        out[sel, 1:4] = (pos[l][c] * pos_factor - 0.5).astype(np.float32)
        out[sel, 4:7] = (vel[l][c] * vel_factor).astype(np.float32)
        out[sel, 7] = np.float32(eps[l] * pos_factor)
    return out


def gadget_blocks(order, pos, vel, mass):
    """Position, velocity and mass blocks of a gadget file whose particles are all of
    one type (io/gadget.hpp:481-520): Coordinate<float> of pos and vel, float masses, in
    mapper order."""
    lev, cells = order
    n = len(cells)
    p = np.zeros((n, 3), dtype=np.float32)
    v = np.zeros((n, 3), dtype=np.float32)
    m = np.zeros(n, dtype=np.float32)
    for l in range(len(pos)):
        sel = lev == l
        p[sel] = pos[l][cells[sel]].astype(np.float32)
        v[sel] = vel[l][cells[sel]].astype(np.float32)
        m[sel] = np.float32(mass[l])
    return p, v, m
