"""Generate tests/golden/c4_fd.npz: float64 central finite differences of the
differentiable forward model's loss at the 128^3-particle configuration.

Configuration: 128^3 particles, 256^3 CIC mesh (B = 2), box 256 Mpc/h, 2LPT
at a = 0.1 then 10 KDK steps linear in a to 1, Om0 = 0.3089, sigma8 = 0.8159.
Loss = sum (rho / nbar - target)^2 over the CIC-painted final mesh, target =
the same model's density from the seed-3 whitenoise; the derivatives are
taken at the seed-5 whitenoise (the oracle's whitenoise stream):

  fd[i] = (L(wn + eps v_i) - L(wn - eps v_i)) / (2 eps), i < 64, v_i the
          Hermitian direction rfftn(normal(seed 1000 + i)) / 128^1.5
  fdo   = (L(Om0 + h) - L(Om0 - h)) / (2 h), the P(k), growth and force
          factor all following Om0

Each loss is a float64 run of tests/f64_device.py (the reference algorithm in
torch float64 on the GPU, itself checked against the numpy oracle), so this
needs a CUDA device: about 130 runs.

    python tests/golden/make_c4_fd.py [output path, default tests/golden/c4_fd.npz]
"""
import os
import sys
import time

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

NC, B, BOX, OM0, S8 = 128, 2, 256.0, 0.3089, 0.8159
STAGES = numpy.linspace(0.1, 1.0, 11)
NDIR = 64
EPS = 1e-4
DOM = 1e-4


def direction(i, nc=NC):
    rng = numpy.random.RandomState(1000 + i)
    return numpy.fft.rfftn(rng.normal(size=(nc, nc, nc))) / nc ** 1.5


def density(wn, Om0, nc=NC, b=B, box=BOX, stages=STAGES, sigma8=S8):
    """rho / nbar of the CIC-painted final positions (float64, on the device)."""
    from oracle import cosmology_np
    from tests import f64_device as F
    cosmo = cosmology_np.Cosmology(Om0=Om0, sigma8=sigma8)
    st = F.run(wn, cosmology_np.EHPower(cosmo, 0), nc, b, box, 'cic', stages, Om0)
    n = nc * b
    return F.paint(st.X, n, box, 'cic') / (nc ** 3 / float(n) ** 3)


def loss(wn, Om0, target):
    d = density(wn, Om0)
    return float(((d - target) ** 2).sum())


def main():
    import torch
    from oracle import pmesh_np
    t0 = time.perf_counter()
    dev = 'cuda'
    target = density(torch.from_numpy(pmesh_np.whitenoise([NC] * 3, 3)).to(dev), OM0)
    wn = torch.from_numpy(pmesh_np.whitenoise([NC] * 3, 5)).to(dev)
    l0 = loss(wn, OM0, target)
    fd = numpy.empty(NDIR)
    for i in range(NDIR):
        v = torch.from_numpy(direction(i)).to(dev)
        fd[i] = (loss(wn + EPS * v, OM0, target) - loss(wn - EPS * v, OM0, target)) / (2 * EPS)
        print('direction %d fd %.9e (%.0f s)' % (i, fd[i], time.perf_counter() - t0), flush=True)
    fdo = (loss(wn, OM0 + DOM, target) - loss(wn, OM0 - DOM, target)) / (2 * DOM)
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, 'c4_fd.npz')
    numpy.savez_compressed(out, fd=fd, fdo=fdo, loss=l0, eps=EPS, dom=DOM,
                           nc=NC, B=B, box=BOX, Om0=OM0, sigma8=S8, stages=STAGES,
                           direction_seeds=numpy.arange(1000, 1000 + NDIR))
    print('loss %.9e dL/dOm0 %.9e, %.0f s' % (l0, fdo, time.perf_counter() - t0))


if __name__ == '__main__':
    main()
