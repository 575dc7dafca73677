"""Gradients through the realisation: the hand-written adjoint kernels behind the
torch.autograd bindings, checked by the adjoint identity, by central finite
differences on random noise modes (FP64, eps = 1e-3), and against the direction
the reference's quadratic solver uses (twice the pushed covector, from the oracle)."""
import numpy as np
import pytest

import field_oracle as fo
from conftest import COSMO, make_generator

pytestmark = pytest.mark.gpu
torch = pytest.importorskip('torch')

LEVELS = [('base', 50.0, 32), ('zoom', 8, 8, 8, 2, 32)]
ORACLE_LEVELS = [(50.0, 32, (0.0, 0.0, 0.0)), (25.0, 32, (12.5, 12.5, 12.5))]


@pytest.fixture(scope='module')
def gen(bbks):
    g = make_generator('fp64', bbks, LEVELS, 8896131, 'random_seed')
    g.draw()
    yield g
    g.close()


def _noise(gen):
    from genetic_gb300.autograd import noise_real
    return [noise_real(gen, l) for l in range(len(gen.levels))]


def test_forward_maps_match_zeldovich(built, gen):
    from genetic_gb300.autograd import NoiseToDelta, displacement
    noise = _noise(gen)
    gen.done(apply_modifications=False)
    for l in range(2):
        d = NoiseToDelta.apply(gen, l, *noise).cpu().numpy()
        ref = gen.field(l, 'delta')
        assert np.abs(d - ref).max() <= 1e-12 * np.abs(ref).max(), l
        psi = displacement(gen, l, noise).cpu().numpy()
        for a, name in enumerate(('psi_x', 'psi_y', 'psi_z')):
            ref = gen.field(l, name)
            assert np.abs(psi[a] - ref).max() <= 1e-12 * np.abs(ref).max(), (l, name)


@pytest.mark.parametrize('level', [0, 1])
@pytest.mark.parametrize('what', ['delta', 'psi_x', 'psi_z'])
def test_adjoint_identity(built, gen, level, what):
    """<A w, g> = <w, A^T g> for random w, g."""
    from genetic_gb300 import _lib
    from genetic_gb300.autograd import _FieldFromNoise
    code = {'delta': _lib.GIC_FIELD_DELTA, 'psi_x': _lib.GIC_FIELD_PSI_X, 'psi_z': _lib.GIC_FIELD_PSI_Z}[what]
    rng = torch.Generator(device='cpu').manual_seed(7)
    w = [torch.randn((32, 32, 32), generator=rng, dtype=torch.float64).cuda().requires_grad_() for _ in range(2)]
    g = torch.randn((32, 32, 32), generator=rng, dtype=torch.float64).cuda()
    out = _FieldFromNoise.apply(gen, level, code, *w)
    lhs = float((out.detach() * g).sum())
    grads = torch.autograd.grad(out, w, grad_outputs=g)
    rhs = float(sum((a.detach() * b).sum() for a, b in zip(w, grads)))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1e-30)
    if level == 0:
        assert float(grads[1].abs().max()) == 0.0


def _mode_directions(count, seed=12345, levels=2):
    """Random interior Fourier modes of random levels, as real-field directions."""
    from genetic_gb300.autograd import mode_direction
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        lev = int(rng.integers(levels))
        kx, ky = (int(v) for v in rng.integers(-15, 16, size=2))
        kz = int(rng.integers(1, 16))
        d = mode_direction(32, kx, ky, kz, float(rng.uniform(0, 2 * np.pi)))
        out.append((lev, torch.from_numpy(d).cuda()))
    return out


def _fd_check(loss_fn, noise, eps=1e-3, count=64, levels=2):
    """Directional derivatives along `count` random modes, analytic vs central
    differences.  Returns the norm-wise relative error ||fd - an|| / ||an|| and the
    largest per-direction error relative to the largest directional derivative.
    (Modes the low-pass filters suppress have derivatives near the differences'
    rounding floor, |loss| u / eps, so a per-direction relative error says nothing there.)"""
    w = [x.clone().requires_grad_() for x in noise]
    loss = loss_fn(w)
    grads = torch.autograd.grad(loss, w)
    an, fd = [], []
    for lev, d in _mode_directions(count, levels=levels):
        an.append(float((grads[lev] * d).sum()))
        wp = [x.clone() for x in noise]
        wm = [x.clone() for x in noise]
        wp[lev] += eps * d
        wm[lev] -= eps * d
        with torch.no_grad():
            fd.append((float(loss_fn(wp)) - float(loss_fn(wm))) / (2 * eps))
    an, fd = np.array(an), np.array(fd)
    return (float(np.linalg.norm(fd - an) / np.linalg.norm(an)),
            float(np.abs(fd - an).max() / np.abs(an).max()))


def test_positions_loss_matches_finite_differences(built, gen):
    """sum |x_i - x0|^2 over the 8^3 zoom particles nearest the centre."""
    from genetic_gb300.autograd import cell_centroids, zeldovich_positions
    noise = _noise(gen)
    q = cell_centroids(gen, 1)
    x0 = torch.tensor([25.0, 25.0, 25.0], dtype=torch.float64, device='cuda')
    idx = torch.argsort(((q - x0) ** 2).sum(1))[:8 ** 3]

    def loss(w):
        x = zeldovich_positions(gen, 1, w)[idx]
        return ((x - x0) ** 2).sum()

    norm_err, worst = _fd_check(loss, noise)
    print('positions loss: FD mismatch norm-wise %.3g, worst direction %.3g' % (norm_err, worst))
    assert norm_err < 1e-6 and worst < 1e-6


def test_variance_objective_matches_finite_differences(built, gen):
    from genetic_gb300.autograd import VarianceObjective
    gen.centre(25, 25, 25)
    gen.select_sphere(4)
    noise = _noise(gen)
    norm_err, worst = _fd_check(lambda w: VarianceObjective.apply(gen, 3.0, *w), noise)
    print('variance objective: FD mismatch norm-wise %.3g, worst direction %.3g' % (norm_err, worst))
    assert norm_err < 1e-6 and worst < 1e-6


def test_variance_solver_direction_is_twice_the_pushed_covector(built, gen, bbks):
    """The reference's quadratic-solver direction (2 x the oracle's pushed covector),
    and how far it is from the exact gradient on two levels."""
    from genetic_gb300.autograd import VarianceObjective, solver_direction
    gen.centre(25, 25, 25)
    gen.select_sphere(4)
    noise = [x.requires_grad_() for x in _noise(gen)]
    v = VarianceObjective.apply(gen, 3.0, *noise)
    exact = torch.autograd.grad(v, noise)
    direction = solver_direction(gen, 3.0, [x.detach() for x in noise])
    L = fo.Levels(ORACLE_LEVELS)
    fl = [fo.flag_cells(L, l, (25., 25., 25.), 'sphere', 4) for l in range(2)]
    w_k = [fo.fft_r2c(x.detach().cpu().numpy()) for x in noise]
    p_dm = fo.CambPower(bbks, COSMO, column=1)
    np.seterr(over='ignore')
    p = fo.push_variance(L, w_k, fl, 3.0, p_dm)
    assert abs(float(v) / fo.inner(p, w_k) - 1) < 1e-10
    num = den = 0.0
    for l in range(2):
        want = 2 * fo.fft_c2r(p[l])
        got = direction[l].cpu().numpy()
        assert np.abs(got - want).max() <= 1e-10 * np.abs(want).max(), l
        num += float(((exact[l] - direction[l]) ** 2).sum())
        den += float((exact[l] ** 2).sum())
    print('two levels: |exact gradient - solver direction| / |exact gradient| = %.3g' % np.sqrt(num / den))


def test_variance_gradient_one_level_equals_solver_direction(built, bbks):
    """On one level A is symmetric: the exact gradient is the solver's direction."""
    from genetic_gb300.autograd import VarianceObjective, noise_real, solver_direction
    g = make_generator('fp64', bbks, [('base', 50.0, 32)], 8896131, 'random_seed')
    g.draw()
    g.centre(25, 25, 25)
    g.select_sphere(6)
    noise = [noise_real(g, 0).requires_grad_()]
    v = VarianceObjective.apply(g, 4.0, *noise)
    (exact,) = torch.autograd.grad(v, noise)
    (direction,) = solver_direction(g, 4.0, [noise[0].detach()])
    assert float((exact - direction).abs().max()) <= 1e-10 * float(direction.abs().max())
    norm_err, worst = _fd_check(lambda w: VarianceObjective.apply(g, 4.0, *w), [noise[0].detach()], count=16,
                                levels=1)
    assert norm_err < 1e-6 and worst < 1e-6
    g.close()
