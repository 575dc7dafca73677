"""torch.autograd bindings of the realisation maps.

The forward maps and their adjoints are CUDA kernels in libgicgpu (gic_field_from_noise,
gic_field_from_noise_adjoint, gic_variance_gradient); this module only passes torch
device tensors through the C ABI.  genetIC has no counterpart: it does not
differentiate its realisations.

The differentiable input is each level's white noise as a real field w (unit
gaussians, shape (n, n, n), the context's precision: float64 for 'fp64', float32 for
'mixed'); `noise_real` returns the drawn noise in that form.  The maps follow
gic_zeldovich: a level's delta or displacement is its own noise times sqrt(P) (and the
level's high-pass filter), plus on the first zoom level the base level's low-passed
field interpolated in.  Gradients through the zoom combination cover levels 0 and 1.

  noise = [noise_real(gen, l) for l in range(len(gen.levels))]
  noise = [w.requires_grad_() for w in noise]
  delta = NoiseToDelta.apply(gen, 1, *noise)           # w -> delta on level 1
  x = zeldovich_positions(gen, 1, noise)               # w -> q + psi, (n^3, 3)
  v = VarianceObjective.apply(gen, 3.0, *noise)        # w -> <Q delta, delta>
"""
import ctypes

import numpy as np
import torch

from . import _lib


def _dtype(gen):
    return torch.float64 if gen.precision == 'fp64' else torch.float32


def _device(gen):
    return torch.device('cuda', _device_index(gen))


def _device_index(gen):
    return getattr(gen, 'device', 0)


def _ptr_array(tensors):
    return (ctypes.c_void_p * len(tensors))(*[t.data_ptr() for t in tensors])


def _prepare(gen, tensors):
    """Contiguous tensors of the context's dtype on its device; torch's queued work on
    them is finished before the library's stream reads them."""
    out = []
    for t in tensors:
        if t.dtype != _dtype(gen):
            raise TypeError('expected %s tensors for a %s context' % (_dtype(gen), gen.precision))
        out.append(t.detach().contiguous())
    torch.cuda.current_stream(_device(gen)).synchronize()
    return out


def noise_real(gen, level):
    """The drawn white noise of `level` as a real (n, n, n) tensor."""
    n = gen.levels[level][1]
    out = torch.empty((n, n, n), dtype=_dtype(gen), device=_device(gen))
    torch.cuda.current_stream(_device(gen)).synchronize()
    gen._call('gic_noise_real', level, ctypes.c_void_p(out.data_ptr()))
    return out


class _FieldFromNoise(torch.autograd.Function):
    """One field (delta or a displacement component) of a level from every level's
    real white noise; backward runs the hand-written adjoint kernels."""

    @staticmethod
    def forward(ctx, gen, level, what, *noise):
        noise = _prepare(gen, noise)
        n = gen.levels[level][1]
        out = torch.empty((n, n, n), dtype=_dtype(gen), device=_device(gen))
        gen._call('gic_field_from_noise', level, what, _ptr_array(noise), ctypes.c_void_p(out.data_ptr()))
        ctx.gen, ctx.level, ctx.what = gen, level, what
        ctx.shapes = [w.shape for w in noise]
        return out

    @staticmethod
    def backward(ctx, grad):
        gen = ctx.gen
        (grad,) = _prepare(gen, [grad])
        grads = [torch.empty(s, dtype=_dtype(gen), device=_device(gen)) for s in ctx.shapes]
        gen._call('gic_field_from_noise_adjoint', ctx.level, ctx.what, ctypes.c_void_p(grad.data_ptr()),
                  _ptr_array(grads))
        return (None, None, None) + tuple(grads)


class NoiseToDelta:
    """w -> delta of one level: NoiseToDelta.apply(gen, level, *noise) (an autograd
    Function application; backward is the adjoint kernel)."""

    @staticmethod
    def apply(gen, level, *noise):
        return _FieldFromNoise.apply(gen, level, _lib.GIC_FIELD_DELTA, *noise)


def displacement(gen, level, noise):
    """w -> (psi_x, psi_y, psi_z) of one level, stacked as (3, n, n, n)."""
    return torch.stack([_FieldFromNoise.apply(gen, level, w, *noise)
                        for w in (_lib.GIC_FIELD_PSI_X, _lib.GIC_FIELD_PSI_Y, _lib.GIC_FIELD_PSI_Z)])


def cell_centroids(gen, level):
    """Lagrangian positions q of the level's cells, (n^3, 3), genetIC's centroid
    offset + (i + 1/2) dx (grid.hpp:662-669)."""
    box, n, off = gen.levels[level]
    dx = box / n
    axes = [torch.arange(n, dtype=torch.float64) * dx + off[a] + dx / 2 for a in range(3)]
    X, Y, Z = torch.meshgrid(*axes, indexing='ij')
    return torch.stack([X, Y, Z], -1).reshape(-1, 3).to(device=_device(gen), dtype=_dtype(gen))


def zeldovich_positions(gen, level, noise):
    """w -> Zel'dovich positions q + psi of the level's particles, (n^3, 3), unwrapped
    (the periodic wrap is not differentiable)."""
    psi = displacement(gen, level, noise)
    return cell_centroids(gen, level) + psi.reshape(3, -1).t()


class ZeldovichPositions:
    """w -> Zel'dovich positions: ZeldovichPositions.apply(gen, level, *noise)."""

    @staticmethod
    def apply(gen, level, *noise):
        return zeldovich_positions(gen, level, list(noise))


def _variance(gen, filterscale, noise, exact):
    noise = _prepare(gen, noise)
    grads = [torch.empty_like(w) for w in noise]
    ptrs, counts = gen._level_cells()
    value = ctypes.c_double()
    gen._call('gic_variance_gradient', ptrs, counts, float(filterscale), _ptr_array(noise), _ptr_array(grads),
              int(exact), ctypes.byref(value))
    return value.value, grads


class VarianceObjective(torch.autograd.Function):
    """<A w|w>, genetIC's variance functional (A w = the pushed covector of the variance
    modification over the flagged cells of the generator's last selection, every
    level, high-passed at `filterscale`); VarianceObjective.apply(gen, filterscale,
    *noise) -> scalar.  The gradient is exact, (A + A^T) w, from the forward and
    transposed kernels.  On one level A is symmetric and it equals 2 A w, the
    direction genetIC's quadratic solver steps along (`solver_direction`)."""

    @staticmethod
    def forward(ctx, gen, filterscale, *noise):
        value, grads = _variance(gen, filterscale, noise, True)
        ctx.save_for_backward(*grads)
        return torch.tensor(value, dtype=torch.float64, device=_device(gen))

    @staticmethod
    def backward(ctx, gout):
        grads = ctx.saved_tensors
        return (None, None) + tuple(g * gout.to(g.dtype) for g in grads)


def solver_direction(gen, filterscale, noise):
    """2 A w per level: the step direction of genetIC's quadratic solver (twice the
    pushed covector in real space, modificationmanager.hpp:249-275)."""
    return _variance(gen, filterscale, noise, False)[1]


def mode_direction(n, kx, ky, kz, phase=0.0, dtype=np.float64):
    """The real field of one Fourier mode (kx, ky, kz) with unit half-spectrum
    amplitude e^{i phase} (and its Hermitian partner), under genetIC's unitary
    normalisation: a noise 'mode' direction for finite-difference checks."""
    c = np.zeros((n, n, n // 2 + 1), dtype=np.complex128)
    c[kx % n, ky % n, kz] = np.exp(1j * phase)
    return (np.fft.irfftn(c, s=(n, n, n), axes=(0, 1, 2)) * n ** 1.5).astype(dtype)
