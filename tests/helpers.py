"""Shared set-up for the parity tests (device engine vs CPU oracle)."""
import numpy
import torch

from oracle import pmesh_np, fastpm_np, cosmology_np, power_np


def rel_l2(a, b):
    a = numpy.asarray(a, dtype='c16' if numpy.iscomplexobj(a) or numpy.iscomplexobj(b) else 'f8')
    b = numpy.asarray(b, dtype=a.dtype)
    return float(numpy.linalg.norm((a - b).ravel()) / max(numpy.linalg.norm(b.ravel()), 1e-300))


def tonp(t):
    return t.detach().cpu().numpy() if torch.is_tensor(t) else numpy.asarray(t)


def run_pair(nc, B, box, resampler, seed, a0, stages, order=2, shift=0.0, unitary=False, monitor=True,
             permute=None):
    """Same whitenoise into the oracle (float64) and the device solver.

    monitor=False runs the device nbody without a monitor (its fused
    kick-drift + brick-count path; no delta_k is returned then).  permute=seed
    shuffles the particle grid Q the same way on both sides, so the device
    works in explicit-position mode (no lattice)."""
    import fastpm_gb300 as G
    Plin = cosmology_np.EHPower(cosmology_np.Planck15, 0)
    # oracle
    opm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, dtype='f8', resampler=resampler)
    osolver = fastpm_np.Solver(opm, cosmology_np.Planck15, B=B)
    oQ = opm.generate_uniform_particle_grid(shift=shift)
    perm = None
    if permute is not None:
        perm = numpy.random.RandomState(permute).permutation(len(oQ))
        oQ = oQ[perm]
    wn = osolver.whitenoise(seed, unitary=unitary)
    odlin = osolver.linear(wn, lambda k: Plin(k))
    ostate = osolver.lpt(odlin, oQ, a=a0, order=order)
    olpt = {k: getattr(ostate, k).copy() for k in ('S', 'P', 'F')}
    odk = {}

    def omon(action, ai, ac, af, st, ev):
        if action == 'F':
            odk['last'] = ev['delta_k'].value.copy()

    ostate = osolver.nbody(ostate, fastpm_np.leapfrog(stages), monitor=omon)
    # device
    pm = G.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, dtype='f4', resampler=resampler)
    solver = G.Solver(pm, G.Planck15, B=B)
    Q = pm.generate_uniform_particle_grid(shift=shift)
    if perm is not None:
        Q = Q[torch.from_numpy(perm).to(Q.device)].clone()   # a plain tensor: explicit positions
    gwn = pm.complex_from(wn.value)
    dlin = solver.linear(gwn, lambda k: Plin(k))
    state = solver.lpt(dlin, Q, a=a0, order=order)
    glpt = {k: tonp(getattr(state, k)).copy() for k in ('S', 'P', 'F')}
    gdk = {}

    def gmon(action, ai, ac, af, st, ev):
        if action == 'F':
            gdk['last'] = ev['delta_k']

    state = solver.nbody(state, G.leapfrog(stages), monitor=gmon if monitor else None)
    torch.cuda.synchronize()
    return dict(oracle=ostate, olpt=olpt, odk=odk['last'], odlin=odlin.value,
                gpu=state, glpt=glpt, gdk=gdk.get('last'), gdlin=dlin, box=box, nc=nc, B=B)
