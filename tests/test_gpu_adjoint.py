"""Adjoint gradients of the differentiable forward model vs float64 central
finite differences of the oracle (the same model restated in float64).

Bar: each directional derivative <g, v>_w (Hermitian-weighted inner product)
within 1e-2 relative of the float64 central difference, and dL/dOm0 likewise.
"""
import numpy
import pytest
import torch

from oracle import pmesh_np, fastpm_np
from tests.helpers import tonp

pytestmark = pytest.mark.gpu


def _hermitian_direction(n, seed):
    rng = numpy.random.RandomState(seed)
    return numpy.fft.rfftn(rng.normal(size=(n, n, n))) / n ** 1.5


def _wdot(g, v, n):
    w = numpy.full(g.shape, 2.0)
    w[:, :, 0] = 1
    w[:, :, n // 2] = 1
    return float((w * (numpy.conj(g) * v).real).sum())


@pytest.mark.parametrize('nc,B,ck', [(16, 2, 1), (16, 1, 4)])
def test_adjoint_matches_finite_differences(nc, B, ck):
    import fastpm_gb300 as G
    from fastpm_gb300.adjoint import ForwardModel
    box, s8, Om0 = 64.0, 0.8, 0.31
    stages = numpy.linspace(0.1, 1.0, 4)
    n = nc * B
    wn_t = pmesh_np.whitenoise([nc] * 3, 3)
    wn = pmesh_np.whitenoise([nc] * 3, 5)
    target = fastpm_np.model_density(wn_t, Om0, s8, nc, B, box, stages)
    model = ForwardModel(nc, B, box, stages, sigma8=s8, checkpoint_every=ck,
                         target=torch.from_numpy(target.astype('f4')).cuda())
    loss = model.forward(model.pm.complex_from(wn), Om0)
    ref = fastpm_np.model_loss(wn, Om0, s8, nc, B, box, stages, target)
    assert abs(loss - ref) <= 1e-3 * ref
    g, dOm = model.backward()
    g = tonp(g.value).astype('c16')
    for seed in range(4):
        v = _hermitian_direction(nc, 100 + seed)
        eps = 1e-4   # small enough that few particles cross a CIC weight kink
        lp = fastpm_np.model_loss(wn + eps * v, Om0, s8, nc, B, box, stages, target)
        lm = fastpm_np.model_loss(wn - eps * v, Om0, s8, nc, B, box, stages, target)
        fd = (lp - lm) / (2 * eps)
        ad = _wdot(g, v, nc)
        assert abs(ad - fd) <= 1e-2 * abs(fd) + 1e-6 * ref, (seed, ad, fd)
    h = 1e-4
    fdo = (fastpm_np.model_loss(wn, Om0 + h, s8, nc, B, box, stages, target)
           - fastpm_np.model_loss(wn, Om0 - h, s8, nc, B, box, stages, target)) / (2 * h)
    assert abs(dOm - fdo) <= 1e-2 * abs(fdo), (dOm, fdo)


def test_autograd_function_wraps_the_adjoint():
    from fastpm_gb300.adjoint import ForwardModel, FastPMLoss
    nc, B, box = 16, 2, 64.0
    stages = numpy.linspace(0.1, 1.0, 3)
    model = ForwardModel(nc, B, box, stages)
    wn = model.pm.complex_from(pmesh_np.whitenoise([nc] * 3, 5))
    x = wn.data.clone().requires_grad_(True)
    om = torch.tensor(0.3, dtype=torch.float64, requires_grad=True)
    loss = FastPMLoss.apply(x, om, model)
    loss.backward()
    assert x.grad is not None and torch.isfinite(x.grad).all()
    assert om.grad is not None and torch.isfinite(om.grad)
    # the Euclidean gradient is the Hermitian-weighted half-mode gradient
    g, dom = model.backward()
    assert abs(float(om.grad) - dom) <= 1e-6 * abs(dom)


def test_c4_adjoint_against_float64_finite_differences():
    """The differentiable-model configuration in full: 128^3 particles, 256^3
    CIC mesh, box 256 Mpc/h, 2LPT at 0.1 and 10 KDK steps, loss = sum (rho /
    nbar - target)^2 with the seed-3 target, gradient at the seed-5
    whitenoise by the adjoint with 1-in-4 step checkpoints, against float64
    central finite differences of the same model (tests/golden/c4_fd.npz,
    made by tests/golden/make_c4_fd.py) along 64 random Hermitian mode
    directions and along Om0.  Bars: cosine >= 0.999 between the 64 adjoint
    and finite-difference directional derivatives, median relative error
    <= 3 %, dL/dOm0 within 5 %.  (Single directions of this chaotic model
    carry finite-difference noise of a few per cent, hence the aggregate
    bars.)"""
    import os
    from fastpm_gb300.adjoint import ForwardModel
    from tests.golden import make_c4_fd as C
    g = numpy.load(os.path.join(os.path.dirname(__file__), 'golden', 'c4_fd.npz'))
    dev = 'cuda'
    target = C.density(torch.from_numpy(pmesh_np.whitenoise([C.NC] * 3, 3)).to(dev), C.OM0)
    model = ForwardModel(C.NC, C.B, C.BOX, C.STAGES, sigma8=C.S8, checkpoint_every=4,
                         target=target.float().contiguous())
    del target
    wn = pmesh_np.whitenoise([C.NC] * 3, 5)
    loss = model.forward(model.pm.complex_from(wn), C.OM0)
    assert abs(loss - float(g['loss'])) <= 1e-3 * float(g['loss'])
    grad, dom = model.backward()
    gh = tonp(grad.value).astype('c16')
    proj = numpy.array([_wdot(gh, C.direction(i), C.NC) for i in range(C.NDIR)])
    fd = g['fd']
    cos = float(proj @ fd / numpy.linalg.norm(proj) / numpy.linalg.norm(fd))
    rel = numpy.abs(proj - fd) / numpy.abs(fd)
    print('c4 adjoint: cosine %.6f, median rel %.3e, rms err / rms fd %.3e, dL/dOm0 %.6e vs %.6e'
          % (cos, numpy.median(rel), numpy.sqrt(((proj - fd) ** 2).mean() / (fd ** 2).mean()), dom,
             float(g['fdo'])))
    assert cos >= 0.999
    assert numpy.median(rel) <= 0.03
    assert abs(dom - float(g['fdo'])) <= 0.05 * abs(float(g['fdo']))
