"""Generate the golden fixtures in this directory from the reference's OWN code.

Run where the reference source is available: its project root is the first
argument, or the REFERENCE_ROOT environment variable.  The GPU tests do not
need this script, only the .npz files it writes.

The reference's fastpm/core.py, fastpm/force/{lpt,gravity,kernels}.py,
fastpm/background.py and fastpm/utils.py are imported UNMODIFIED.  The
third-party modules they import and that are absent here are stood in for:
``pmesh.pm`` by oracle.pmesh_np and ``nbodykit.cosmology`` by
oracle.cosmology_np.  The fixtures therefore pin the oracle's restatement of
the reference's own Python (oracle/fastpm_np.py, oracle/power_np.py) to the
reference itself; the pmesh layer beneath both is the shared stand-in.

    python tests/golden/make_golden.py <reference project root>
"""
import os
import sys
import types

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REFERENCE_ROOT = sys.argv[1] if len(sys.argv) > 1 else os.environ.get('REFERENCE_ROOT')


def load_reference():
    sys.dont_write_bytecode = True
    sys.path.insert(0, REPO)
    from oracle import pmesh_np, cosmology_np
    pmesh = types.ModuleType('pmesh')
    pmesh.pm = pmesh_np
    nbodykit = types.ModuleType('nbodykit')
    nbodykit.cosmology = cosmology_np
    sys.modules.update({'pmesh': pmesh, 'pmesh.pm': pmesh_np,
                        'nbodykit': nbodykit, 'nbodykit.cosmology': cosmology_np})
    sys.path.insert(0, REFERENCE_ROOT)
    import fastpm.core as core
    import fastpm.background as background
    import fastpm.utils as utils
    import fastpm.ncdm as ncdm
    import fastpm.multi as multi
    import fastpm.state as state
    from fastpm.force import kernels, lpt, gravity
    return dict(core=core, background=background, utils=utils, kernels=kernels, ncdm=ncdm,
                multi=multi, state=state,
                lpt=lpt, gravity=gravity, pmesh_np=pmesh_np, cosmology_np=cosmology_np)


def background_case(ref):
    bg = ref['background']
    Om0 = 0.3089
    a = numpy.array([0.01, 0.05, 0.1, 0.1 * 2 ** 0.5, 0.2, 0.5, 0.75, 1.0])
    pt = bg.MatterDominated(Om0, a=a, a_normalize=1.0)
    out = dict(a=a)
    for name in ('D1', 'D2', 'f1', 'f2', 'E', 'Gp', 'gp', 'Gf', 'gf', 'gf2'):
        out['bg_' + name] = getattr(pt, name)(a)
    for order in (1, 2):
        out['bg_D1_o%d' % order] = pt.D1(a, order)
        out['bg_D2_o%d' % order] = pt.D2(a, order)
    # kick / drift factors of the 64^3 / 10-step schedule, computed the way
    # FastPMStep.Kick/Drift do (core.py:170-171, 177-178)
    stages = numpy.linspace(0.1, 1.0, 11)
    acts = list(ref['core'].leapfrog(stages))
    kd = []
    for action, ai, ac, af in acts:
        pt = bg.MatterDominated(Om0, a=[ai, ac, af], a_normalize=1.0)
        if action == 'K':
            kd.append(1 / (ac ** 2 * pt.E(ac)) * (pt.Gf(af) - pt.Gf(ai)) / pt.gf(ac))
        elif action == 'D':
            kd.append(1 / (ac ** 3 * pt.E(ac)) * (pt.Gp(af) - pt.Gp(ai)) / pt.gp(ac))
        else:
            kd.append(0.0)
    out['sched_actions'] = numpy.array([x[0] for x in acts])
    out['sched_a'] = numpy.array([x[1:] for x in acts])
    out['sched_fac'] = numpy.array(kd)
    return out


def kernels_case(ref):
    pmesh_np, K = ref['pmesh_np'], ref['kernels']
    pm = pmesh_np.ParticleMesh(BoxSize=128., Nmesh=[8, 8, 8])
    rng = numpy.random.RandomState(333)
    real = pm.create('real', value=rng.normal(size=(8, 8, 8)))
    ck = real.r2c()
    out = dict(kern_in=ck.value.copy())
    out['kern_laplace'] = ck.apply(K.laplace).value.copy()
    for d in range(3):
        out['kern_grad1_%d' % d] = ck.apply(K.gradient(d, order=1)).value.copy()
        out['kern_grad0_%d' % d] = ck.apply(K.gradient(d, order=0)).value.copy()
    out['kern_lr2'] = ck.apply(K.longrange(2.0)).value.copy()
    return out


def solver_case(ref, tag, nc, B, box, resampler, seed, a0, stages, order=2, shift=0.0,
                unitary=False):
    core, pmesh_np, cosmo = ref['core'], ref['pmesh_np'], ref['cosmology_np']
    pm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, dtype='f8', resampler=resampler)
    Plin = cosmo.EHPower(cosmo.Planck15, 0)
    solver = core.Solver(pm, cosmo.Planck15, B=B)
    Q = pm.generate_uniform_particle_grid(shift=shift)
    wn = solver.whitenoise(seed, unitary=unitary)
    dlin = solver.linear(wn, lambda k: Plin(k))
    state = solver.lpt(dlin, Q, a=a0, order=order)
    out = {}
    p = tag + '_'
    out[p + 'wn'] = wn.value.copy()
    out[p + 'dlin'] = dlin.value.copy()
    out[p + 'Q'] = Q.copy()
    for key in ('S', 'P', 'F'):
        out[p + 'lpt_' + key] = getattr(state, key).copy()
    deltas = []

    def monitor(action, ai, ac, af, st, event):
        if action == 'F':
            deltas.append(event['delta_k'].value.copy())

    state = solver.nbody(state, core.leapfrog(stages), monitor=monitor)
    for key in ('S', 'P', 'F', 'RHO', 'X', 'V'):
        out[p + 'nb_' + key] = getattr(state, key).copy()
    out[p + 'nb_a'] = numpy.array([state.a['S'], state.a['P'], state.a['F']])
    out[p + 'delta_k_last'] = deltas[-1]
    out[p + 'meta'] = numpy.array([nc, B, box, seed, a0, order, shift, unitary], dtype='f8')
    out[p + 'stages'] = numpy.asarray(stages, dtype='f8')
    out[p + 'resampler'] = numpy.array(resampler)
    # P(k) of the final density with the reference's own estimator (utils.py:77)
    k, pk = ref['utils'].power(deltas[-1].copy(), boxsize=box)
    out[p + 'pk_k'] = k
    out[p + 'pk_p'] = pk
    return out


def ncdm_case(ref, tag, nc, B, box, resampler, seed, a0, stages):
    """The reference's own fastpm/ncdm.py Solver (neutrino transfer on
    delta_k before the force) on the stand-in mesh, with the synthetic
    linear-response cosmology of oracle/cosmology_np.py."""
    ncdm, pmesh_np, cosmo = ref['ncdm'], ref['pmesh_np'], ref['cosmology_np']
    c = cosmo.LinearResponseNeutrinos()
    pm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, dtype='f8', resampler=resampler)
    Plin = cosmo.EHPower(c, 0)
    solver = ncdm.Solver(pm, c, B=B)
    Q = pm.generate_uniform_particle_grid(shift=0)
    wn = solver.whitenoise(seed)
    state = solver.lpt(solver.linear(wn, lambda k: Plin(k)), Q, a=a0, order=2)
    deltas = []

    def monitor(action, ai, ac, af, st, event):
        if action == 'F':
            deltas.append(event['delta_k'].value.copy())

    state = solver.nbody(state, ref['core'].leapfrog(stages), monitor=monitor)
    p = tag + '_'
    out = {p + 'wn': wn.value.copy(), p + 'stages': numpy.asarray(stages, dtype='f8'),
           p + 'meta': numpy.array([nc, B, box, seed, a0], dtype='f8'), p + 'resampler': numpy.array(resampler),
           p + 'delta_k_last': deltas[-1]}
    for key in ('X', 'V', 'F', 'RHO'):
        out[p + key] = getattr(state, key).copy()
    return out


def multi_case(ref, tag, nc, B, box, resampler, seed, a0, stages, order):
    """The reference's own fastpm/multi.py Solver with fastpm/state.py's
    species (baryons '0', CDM '1') on the stand-in mesh, with the synthetic
    primordial P(k) and species transfers of oracle/multi_np.py."""
    from oracle import multi_np
    multi, state, pmesh_np, cosmo = ref['multi'], ref['state'], ref['pmesh_np'], ref['cosmology_np']
    c = cosmo.Planck15
    pm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, dtype='f8', resampler=resampler)
    solver = multi.Solver(pm, c, B=B)
    P_prim, tf = multi_np.synthetic_species(c, a0)
    Q = pm.generate_uniform_particle_grid(shift=0)
    wn = solver.whitenoise(seed)
    prm = solver.primordial(wn, P_prim)
    st = solver.lpt(prm, {'0': (state.Baryon, tf['d_b'], tf['dd_b']),
                          '1': (state.CDM, tf['d_cdm'], tf['dd_cdm'])}, Q, a=a0, order=order)
    p = tag + '_'
    out = {p + 'meta': numpy.array([nc, B, box, seed, a0, order], dtype='f8'), p + 'stages': numpy.asarray(stages),
           p + 'resampler': numpy.array(resampler), p + 'prm': prm.value.copy()}
    for sp in ('0', '1'):
        for key in ('S', 'P'):
            out[p + 'lpt_%s_%s' % (sp, key)] = getattr(st.species[sp], key).copy()
    deltas = []

    def monitor(action, ai, ac, af, s_, event):
        if action == 'F':
            deltas.append(event['delta_k'].value.copy())

    st = solver.nbody(st, ref['core'].leapfrog(stages), monitor=monitor)
    for sp in ('0', '1'):
        for key in ('X', 'V', 'F'):
            out[p + '%s_%s' % (sp, key)] = getattr(st.species[sp], key).copy()
    out[p + 'delta_k_last'] = deltas[-1]
    return out


def lpt_relation_case(ref):
    """fastpm/tests/test_core.py:46-62 on the stand-in mesh: P(1) = P(0.01) + fac F(0.01)."""
    core, pmesh_np, cosmo, bg = ref['core'], ref['pmesh_np'], ref['cosmology_np'], ref['background']
    pm = pmesh_np.ParticleMesh(BoxSize=128., Nmesh=[8, 8, 8])
    Plin = cosmo.LinearPower(cosmo.Planck15, redshift=0, transfer='EisensteinHu')
    solver = core.Solver(pm, cosmo.Planck15, B=1)
    Q = pm.generate_uniform_particle_grid(shift=0)
    dlin = solver.linear(solver.whitenoise(1234), lambda k: Plin(k))
    s1 = solver.lpt(dlin, Q, a=0.01, order=1)
    s2 = solver.lpt(dlin, Q, a=1.0, order=1)
    pt = bg.MatterDominated(cosmo.Planck15.Om0, a=[0.01, 1.0], a_normalize=1.0)
    fac = 1 / (0.01 ** 2 * pt.E(0.01)) * (pt.Gf(1.0) - pt.Gf(0.01)) / pt.gf(0.01)
    numpy.testing.assert_allclose(s2.P, s1.P + fac * s1.F)
    return dict(lptrel_P1=s1.P.copy(), lptrel_F1=s1.F.copy(), lptrel_P2=s2.P.copy(),
                lptrel_fac=numpy.array(fac))


def schedule_case(ref):
    core = ref['core']
    out = {}
    for n, knots in enumerate([[0.1, 1.0], [1.0], [0.5], [0.1, 0.2, 1.0]]):
        out['auto_%d' % n] = core.autostages(knots, astart=0.1, N=12)
    out['auto_cli'] = core.autostages([0.5, 1.0], astart=0.1, N=5)
    lf = list(core.leapfrog(numpy.linspace(0.1, 1.0, 2, endpoint=True)))
    out['lf2_actions'] = numpy.array([x[0] for x in lf])
    out['lf2_a'] = numpy.array([x[1:] for x in lf])
    return out


def power_case(ref):
    rng = numpy.random.RandomState(17)
    f = 1.0 + 0.1 * rng.normal(size=(16, 16, 16))
    k, p = ref['utils'].power(f.copy(), boxsize=64.0)
    k2, p2, n2 = ref['utils'].power(f.copy(), boxsize=64.0, average=False)
    return dict(pow_in=f, pow_k=k, pow_p=p, pow_k2=k2, pow_p2=p2, pow_n2=n2)


def main():
    if not REFERENCE_ROOT:
        sys.exit('usage: make_golden.py <reference project root>  (or set REFERENCE_ROOT)')
    ref = load_reference()
    out = {}
    out.update(background_case(ref))
    out.update(kernels_case(ref))
    out.update(schedule_case(ref))
    out.update(power_case(ref))
    out.update(lpt_relation_case(ref))
    numpy.savez_compressed(os.path.join(HERE, 'reference_units.npz'), **out)

    runs = {}
    # 8^3 particles / 8^3 mesh, CIC, the reference test's mesh (test_core.py:9)
    runs.update(solver_case(ref, 'c8', 8, 1, 128.0, 'cic', 1234, 0.1, [0.1, 0.5, 1.0]))
    # 16^3 / 32^3 (B=2) CIC: the 64^3 / 128^3 CIC run's shape at 1/4 linear size, 4 KDK steps
    runs.update(solver_case(ref, 'c16', 16, 2, 64.0, 'cic', 42, 0.1,
                            numpy.linspace(0.1, 1.0, 5)))
    # 16^3 / 32^3 TSC, log-spaced, shifted lattice, unitary noise
    runs.update(solver_case(ref, 't16', 16, 2, 64.0, 'tsc', 11, 0.05,
                            numpy.geomspace(0.05, 1.0, 5), shift=0.5, unitary=True))
    # 12^3 / 24^3 (radix-3 sizes), first-order LPT
    runs.update(solver_case(ref, 'c12', 12, 2, 48.0, 'cic', 7, 0.1,
                            numpy.linspace(0.1, 1.0, 4), order=1))
    numpy.savez_compressed(os.path.join(HERE, 'reference_runs.npz'), **runs)

    nc_runs = {}
    # fastpm/ncdm.py: 16^3 / 32^3 CIC, and TSC, 3 KDK steps
    nc_runs.update(ncdm_case(ref, 'n16', 16, 2, 64.0, 'cic', 42, 0.1, numpy.linspace(0.1, 1.0, 4)))
    nc_runs.update(ncdm_case(ref, 'n16t', 16, 2, 96.0, 'tsc', 7, 0.1, numpy.linspace(0.1, 1.0, 4)))
    numpy.savez_compressed(os.path.join(HERE, 'reference_ncdm.npz'), **nc_runs)

    mruns = {}
    # fastpm/multi.py + state.py: baryons and CDM, 16^3 / 32^3, 3 KDK steps
    mruns.update(multi_case(ref, 'm16', 16, 2, 64.0, 'cic', 42, 0.1, numpy.linspace(0.1, 1.0, 4), 1))
    mruns.update(multi_case(ref, 'm16o2', 16, 2, 96.0, 'tsc', 7, 0.1, numpy.linspace(0.1, 1.0, 4), 2))
    numpy.savez_compressed(os.path.join(HERE, 'reference_multi.npz'), **mruns)
    print('wrote', sorted(os.listdir(HERE)))


if __name__ == '__main__':
    main()
