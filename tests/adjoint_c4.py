"""Full-size check of the adjoint of the differentiable forward model.

Configuration: 128^3 particles, 256^3 CIC mesh (B = 2), box 256 Mpc/h, 10 KDK
steps linear in a from 0.1 to 1.0, float32 device state, 1-in-4 step
checkpoints.  Loss = sum (rho / nbar - target)^2 on the CIC-painted mesh with
the target from the seed-3 run; gradient at the seed-5 whitenoise w.r.t. the
modes and Om0, compared with float64 central finite differences of the oracle
along 64 random Hermitian mode directions (seeds 1000..1063) and along Om0.

    python -m tests.adjoint_c4 gpu OUT.npz        # on a GPU: loss, <g, v_i>_w, dL/dOm0
    python -m tests.adjoint_c4 fd OUT.npz [NPROC] # on CPU cores: finite differences + report
"""
import os
import sys
import time

import numpy

NC, B, BOX, OM0, S8 = 128, 2, 256.0, 0.3089, 0.8159
STAGES = numpy.linspace(0.1, 1.0, 11)
NDIR = 64
EPS = 1e-4
DOM = 1e-4


def direction(i):
    rng = numpy.random.RandomState(1000 + i)
    return numpy.fft.rfftn(rng.normal(size=(NC, NC, NC))) / NC ** 1.5


def wdot(g, v):
    w = numpy.full(g.shape, 2.0)
    w[:, :, 0] = 1
    w[:, :, NC // 2] = 1
    return float((w * (numpy.conj(g) * v).real).sum())


def run_gpu(out):
    import torch
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import pmesh_np
    from fastpm_gb300.adjoint import ForwardModel
    model = ForwardModel(NC, B, BOX, STAGES, sigma8=S8, checkpoint_every=4)
    wn_t = model.pm.complex_from(pmesh_np.whitenoise([NC] * 3, 3))
    model.forward(wn_t, OM0)
    target = model.resid.clone()              # rho / nbar of the seed-3 run (target was zero)
    model.target = target
    wn = model.pm.complex_from(pmesh_np.whitenoise([NC] * 3, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss = model.forward(wn, OM0)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    g, dom = model.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    gh = g.value.cpu().numpy().astype('c16')
    proj = numpy.array([wdot(gh, direction(i)) for i in range(NDIR)])
    numpy.savez(out, loss=loss, proj=proj, dom=dom, t_forward=t1 - t0, t_backward=t2 - t1)
    print('loss %.6e dL/dOm0 %.6e forward %.2f s backward %.2f s' % (loss, dom, t1 - t0, t2 - t1))


def _loss(args):
    which, i = args
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import fastpm_np, pmesh_np
    import oracle.pmesh_np as pn
    pn._FFT_KW = dict(workers=1)
    target = _loss.target
    wn = pmesh_np.whitenoise([NC] * 3, 5)
    if which == 'dir':
        v = direction(i // 2)
        s = EPS if i % 2 == 0 else -EPS
        return fastpm_np.model_loss(wn + s * v, OM0, S8, NC, B, BOX, STAGES, target)
    s = DOM if i == 0 else -DOM
    return fastpm_np.model_loss(wn, OM0 + s, S8, NC, B, BOX, STAGES, target)


def _init(target):
    _loss.target = target


def run_fd(path, nproc=8):
    import multiprocessing as mp
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from oracle import fastpm_np, pmesh_np
    res = numpy.load(path)
    target = fastpm_np.model_density(pmesh_np.whitenoise([NC] * 3, 3), OM0, S8, NC, B, BOX, STAGES)
    jobs = [('dir', i) for i in range(2 * NDIR)] + [('om', 0), ('om', 1)]
    ctx = mp.get_context('spawn')
    with ctx.Pool(nproc, initializer=_init, initargs=(target,)) as pool:
        vals = pool.map(_loss, jobs)
    fd = numpy.array([(vals[2 * i] - vals[2 * i + 1]) / (2 * EPS) for i in range(NDIR)])
    fdo = (vals[-2] - vals[-1]) / (2 * DOM)
    rel = numpy.abs(res['proj'] - fd) / numpy.abs(fd)
    print('directions: median rel err %.2e, 90%% %.2e, max %.2e' % (numpy.median(rel),
          numpy.percentile(rel, 90), rel.max()))
    print('Om0: adjoint %.6e fd %.6e rel %.2e' % (float(res['dom']), fdo, abs(float(res['dom']) - fdo) / abs(fdo)))
    numpy.savez(path.replace('.npz', '_fd.npz'), fd=fd, fdo=fdo, rel=rel)


if __name__ == '__main__':
    if sys.argv[1] == 'gpu':
        run_gpu(sys.argv[2])
    else:
        run_fd(sys.argv[2], int(sys.argv[3]) if len(sys.argv) > 3 else 8)
