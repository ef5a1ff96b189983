"""The oracle's float64 restatement against the reference's own outputs.

tests/golden/*.npz were written by tests/golden/make_golden.py, which runs the
reference's unmodified fastpm/core.py, force/*.py, background.py and utils.py.
"""
import numpy
import pytest
from numpy.testing import assert_allclose, assert_array_equal

from oracle import fastpm_np as F
from oracle import pmesh_np, cosmology_np, power_np

RTOL = 1e-12


def test_background_factors(golden_units):
    g = golden_units
    pt = F.MatterDominated(0.3089, a=g['a'], a_normalize=1.0)
    for name in ('D1', 'D2', 'f1', 'f2', 'E', 'Gp', 'gp', 'Gf', 'gf', 'gf2'):
        assert_allclose(getattr(pt, name)(g['a']), g['bg_' + name], rtol=RTOL, err_msg=name)
    for o in (1, 2):
        assert_allclose(pt.D1(g['a'], o), g['bg_D1_o%d' % o], rtol=RTOL)
        assert_allclose(pt.D2(g['a'], o), g['bg_D2_o%d' % o], rtol=RTOL)


def test_kick_drift_schedule(golden_units):
    g = golden_units
    stages = numpy.linspace(0.1, 1.0, 11)
    acts = list(F.leapfrog(stages))
    assert_array_equal(numpy.array([x[0] for x in acts]), g['sched_actions'])
    assert_allclose(numpy.array([x[1:] for x in acts]), g['sched_a'], rtol=0, atol=0)
    for (action, ai, ac, af), ref in zip(acts, g['sched_fac']):
        if action == 'K':
            assert_allclose(F.kick_factor(0.3089, ai, ac, af), ref, rtol=RTOL)
        elif action == 'D':
            assert_allclose(F.drift_factor(0.3089, ai, ac, af), ref, rtol=RTOL)


def test_kernels(golden_units):
    g = golden_units
    pm = pmesh_np.ParticleMesh(BoxSize=128., Nmesh=[8, 8, 8])
    ck = pm.create('complex', value=g['kern_in'])
    assert_allclose(ck.apply(F.laplace).value, g['kern_laplace'], rtol=RTOL, atol=0)
    for d in range(3):
        assert_allclose(ck.apply(F.gradient(d, 1)).value, g['kern_grad1_%d' % d], rtol=RTOL, atol=1e-300)
        assert_allclose(ck.apply(F.gradient(d, 0)).value, g['kern_grad0_%d' % d], rtol=RTOL, atol=1e-300)
    assert_allclose(ck.apply(F.longrange_kernel(2.0)).value, g['kern_lr2'], rtol=RTOL)


def test_schedules(golden_units):
    g = golden_units
    for n, knots in enumerate([[0.1, 1.0], [1.0], [0.5], [0.1, 0.2, 1.0]]):
        s = F.autostages(knots, astart=0.1, N=12)
        assert_array_equal(s, g['auto_%d' % n])
        assert len(s) == 12 and all(k in s for k in knots)     # test_core.py:11-23
    assert_array_equal(F.autostages([0.5, 1.0], astart=0.1, N=5), g['auto_cli'])
    lf = list(F.leapfrog(numpy.linspace(0.1, 1.0, 2)))
    assert len(lf) == 1 + 4 * (2 - 1)                            # test_core.py:25-30
    assert_array_equal(numpy.array([x[0] for x in lf]), g['lf2_actions'])
    assert_array_equal(numpy.array([x[1:] for x in lf]), g['lf2_a'])
    assert len(list(F.leapfrog([1.0]))) == 1
    assert list(F.leapfrog([])) == []


def test_power(golden_units):
    g = golden_units
    k, p = power_np.power(g['pow_in'].copy(), boxsize=64.0)
    assert_allclose(k, g['pow_k'], rtol=RTOL)
    assert_allclose(p, g['pow_p'], rtol=RTOL)
    k2, p2, n2 = power_np.power(g['pow_in'].copy(), boxsize=64.0, average=False)
    assert_allclose(p2, g['pow_p2'], rtol=RTOL)
    assert_array_equal(n2, g['pow_n2'])


def test_lpt_relation(golden_units):
    """fastpm/tests/test_core.py:46-62 re-run on the oracle."""
    g = golden_units
    pm = pmesh_np.ParticleMesh(BoxSize=128., Nmesh=[8, 8, 8])
    Plin = cosmology_np.LinearPower(cosmology_np.Planck15, redshift=0, transfer='EisensteinHu')
    solver = F.Solver(pm, cosmology_np.Planck15, B=1)
    Q = pm.generate_uniform_particle_grid(shift=0)
    dlin = solver.linear(solver.whitenoise(1234), lambda k: Plin(k))
    s1 = solver.lpt(dlin, Q, a=0.01, order=1)
    s2 = solver.lpt(dlin, Q, a=1.0, order=1)
    fac = F.kick_factor(cosmology_np.Planck15.Om0, 0.01, 0.01, 1.0)
    assert_allclose(fac, g['lptrel_fac'], rtol=RTOL)
    assert_allclose(s2.P, s1.P + fac * s1.F, rtol=1e-7)
    assert_allclose(s1.P, g['lptrel_P1'], rtol=RTOL, atol=1e-14)
    assert_allclose(s1.F, g['lptrel_F1'], rtol=RTOL, atol=1e-14)
    assert_allclose(s2.P, g['lptrel_P2'], rtol=RTOL, atol=1e-14)


@pytest.mark.parametrize('tag', ['c8', 'c16', 't16', 'c12'])
def test_solver_runs(golden_runs, tag):
    g = golden_runs
    p = tag + '_'
    nc, B, box, seed, a0, order, shift, unitary = g[p + 'meta']
    nc, B, seed, order = int(nc), int(B), int(seed), int(order)
    resampler = str(g[p + 'resampler'])
    pm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, dtype='f8', resampler=resampler)
    Plin = cosmology_np.EHPower(cosmology_np.Planck15, 0)
    solver = F.Solver(pm, cosmology_np.Planck15, B=B)
    Q = pm.generate_uniform_particle_grid(shift=shift)
    assert_array_equal(Q, g[p + 'Q'])
    wn = solver.whitenoise(seed, unitary=bool(unitary))
    assert_array_equal(wn.value, g[p + 'wn'])
    dlin = solver.linear(wn, lambda k: Plin(k))
    assert_allclose(dlin.value, g[p + 'dlin'], rtol=RTOL, atol=0)
    state = solver.lpt(dlin, Q, a=a0, order=order)
    scale = numpy.abs(g[p + 'lpt_S']).max()
    for key in ('S', 'P', 'F'):
        ref = g[p + 'lpt_' + key]
        assert_allclose(getattr(state, key), ref, rtol=1e-10, atol=1e-12 * numpy.abs(ref).max(),
                        err_msg=key)
    last = {}

    def monitor(action, ai, ac, af, st, event):
        if action == 'F':
            last['dk'] = event['delta_k'].value

    state = F.Solver.nbody(solver, state, F.leapfrog(g[p + 'stages']), monitor=monitor)
    for key in ('S', 'P', 'F', 'RHO', 'X', 'V'):
        ref = g[p + 'nb_' + key]
        assert_allclose(getattr(state, key), ref, rtol=1e-9, atol=1e-11 * numpy.abs(ref).max(),
                        err_msg=key)
    assert_allclose([state.a['S'], state.a['P'], state.a['F']], g[p + 'nb_a'], rtol=0)
    assert_allclose(last['dk'], g[p + 'delta_k_last'], rtol=1e-9, atol=1e-11)
    k, pk = power_np.power(last['dk'].copy(), boxsize=box)
    assert_allclose(pk, g[p + 'pk_p'], rtol=1e-8)
    assert scale > 0


@pytest.mark.parametrize('tag', ['n16', 'n16t'])
def test_ncdm_runs(tag):
    """oracle NCDMSolver (fastpm/ncdm.py restated) against the reference's own
    ncdm.Solver run over the same stand-ins (tests/golden/reference_ncdm.npz)."""
    import os
    g = numpy.load(os.path.join(os.path.dirname(__file__), 'golden', 'reference_ncdm.npz'))
    p = tag + '_'
    nc, B, box, seed, a0 = g[p + 'meta']
    nc, B, seed = int(nc), int(B), int(seed)
    c = cosmology_np.LinearResponseNeutrinos()
    pm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, dtype='f8', resampler=str(g[p + 'resampler']))
    Plin = cosmology_np.EHPower(c, 0)
    solver = F.NCDMSolver(pm, c, B=B)
    wn = solver.whitenoise(seed)
    assert_array_equal(wn.value, g[p + 'wn'])
    state = solver.lpt(solver.linear(wn, lambda k: Plin(k)), pm.generate_uniform_particle_grid(shift=0),
                       a=a0, order=2)
    last = {}

    def monitor(action, ai, ac, af, st, event):
        if action == 'F':
            last['dk'] = event['delta_k'].value

    state = solver.nbody(state, F.leapfrog(g[p + 'stages']), monitor=monitor)
    for key in ('X', 'V', 'F', 'RHO'):
        ref = g[p + key]
        assert_allclose(getattr(state, key), ref, rtol=1e-9, atol=1e-11 * numpy.abs(ref).max(), err_msg=key)
    assert_allclose(last['dk'], g[p + 'delta_k_last'], rtol=1e-9, atol=1e-11)
    # the transfer changes the force: the plain core solver differs
    plain = F.Solver(pm, c, B=B)
    st2 = plain.nbody(plain.lpt(plain.linear(wn, lambda k: Plin(k)), pm.generate_uniform_particle_grid(shift=0),
                                a=a0, order=2), F.leapfrog(g[p + 'stages']))
    assert numpy.abs(st2.F - state.F).max() > 1e-3 * numpy.abs(state.F).max()


@pytest.mark.parametrize('tag', ['m16', 'm16o2'])
def test_multi_runs(tag):
    """oracle multi_np (fastpm/multi.py + state.py restated) against the
    reference's own multi-species Solver over the same stand-ins
    (tests/golden/reference_multi.npz): baryons and CDM, LPT then 3 KDK steps."""
    import os
    from oracle import multi_np
    g = numpy.load(os.path.join(os.path.dirname(__file__), 'golden', 'reference_multi.npz'))
    p = tag + '_'
    nc, B, box, seed, a0, order = g[p + 'meta']
    nc, B, seed, order = int(nc), int(B), int(seed), int(order)
    c = cosmology_np.Planck15
    pm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, dtype='f8', resampler=str(g[p + 'resampler']))
    solver = multi_np.Solver(pm, c, B=B)
    P_prim, tf = multi_np.synthetic_species(c, a0)
    with numpy.errstate(divide='ignore', invalid='ignore'):
        prm = solver.primordial(solver.whitenoise(seed), P_prim)
    assert_allclose(prm.value, g[p + 'prm'], rtol=1e-12, atol=0)
    st = solver.lpt(prm, {'0': (multi_np.Baryon, tf['d_b'], tf['dd_b']),
                          '1': (multi_np.CDM, tf['d_cdm'], tf['dd_cdm'])},
                    pm.generate_uniform_particle_grid(shift=0), a=a0, order=order)
    for sp in ('0', '1'):
        for key in ('S', 'P'):
            ref = g[p + 'lpt_%s_%s' % (sp, key)]
            assert_allclose(getattr(st.species[sp], key), ref, rtol=1e-10, atol=1e-12 * numpy.abs(ref).max())
    last = {}
    st = solver.nbody(st, F.leapfrog(g[p + 'stages']),
                      monitor=lambda a, ai, ac, af, s_, ev: last.update(dk=ev['delta_k'].value)
                      if a == 'F' else None)
    for sp in ('0', '1'):
        for key in ('X', 'V', 'F'):
            ref = g[p + '%s_%s' % (sp, key)]
            assert_allclose(getattr(st.species[sp], key), ref, rtol=1e-9, atol=1e-11 * numpy.abs(ref).max(),
                            err_msg=sp + key)
    assert_allclose(last['dk'], g[p + 'delta_k_last'], rtol=1e-9, atol=1e-11)
    assert numpy.abs(st.species['0'].F - st.species['1'].F).max() > 0   # species differ


def test_radiation_dominated_growth_matches_reference():
    """background.py:258-325 PerturbationGrowth (RadiationDominated) of the
    engine's host module against the oracle restatement (both with the same
    cosmology methods)."""
    import fastpm_gb300 as G
    from oracle import multi_np
    a = [0.05, 0.1, 0.3, 1.0]
    o = multi_np.RadiationDominated(cosmology_np.Planck15, a=a)
    d = G.background.RadiationDominated(G.Planck15, a=a)
    for name in ('D1', 'D2', 'f1', 'f2', 'Gf', 'gf', 'Gp', 'gp', 'E'):
        assert_allclose(getattr(d, name)(numpy.array(a)), getattr(o, name)(numpy.array(a)), rtol=1e-12)
    assert G.background.PerturbationGrowth is G.background.RadiationDominated
