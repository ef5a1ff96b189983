"""End-to-end parity of the device Solver against the float64 oracle.

Both codes get the same whitenoise (the oracle's), the same P(k) callable and
the same schedule.  Bars (from the engine's stated accuracy targets):
  rms |X_gpu - X_oracle| <= 1e-4 of the mean interparticle spacing L / Nc,
  P(k) of the final density within 1e-3 relative for k < k_Nyq / 2,
  V and F within 1e-3 relative rms.
"""
import numpy
import pytest
import torch
from numpy.testing import assert_allclose

from oracle import fastpm_np, power_np, cosmology_np, pmesh_np
from tests.helpers import run_pair, tonp, rel_l2

pytestmark = pytest.mark.gpu

CASES = {
    # nc, B, box, resampler, seed, a0, stages, order, shift, unitary
    'cic16': (16, 2, 64.0, 'cic', 42, 0.1, numpy.linspace(0.1, 1.0, 5), 2, 0.0, False),
    'tsc16': (16, 2, 64.0, 'tsc', 11, 0.05, numpy.geomspace(0.05, 1.0, 5), 2, 0.5, True),
    'cic24': (24, 2, 48.0, 'cic', 7, 0.1, numpy.linspace(0.1, 1.0, 4), 1, 0.0, False),
    'cic32': (32, 2, 128.0, 'cic', 42, 0.1, numpy.linspace(0.1, 1.0, 11), 2, 0.0, False),
    'tsc32b1': (32, 1, 64.0, 'tsc', 3, 0.1, numpy.linspace(0.1, 1.0, 6), 2, 0.0, False),
}


@pytest.mark.parametrize('name', sorted(CASES))
def test_solver_matches_oracle(name):
    nc, B, box, res, seed, a0, stages, order, shift, unitary = CASES[name]
    r = run_pair(nc, B, box, res, seed, a0, stages, order, shift, unitary)
    o, g = r['oracle'], r['gpu']
    # linear field and LPT initial conditions
    assert rel_l2(tonp(r['gdlin'].value), r['odlin']) < 1e-6
    for k in ('S', 'P', 'F'):
        assert rel_l2(r['glpt'][k], r['olpt'][k]) < 2e-5, k
    # final state
    spacing = box / nc
    dx = tonp(g.X) - o.X
    dx -= box * numpy.round(dx / box)
    rms = numpy.sqrt((dx ** 2).sum(axis=1).mean())
    assert rms <= 1e-4 * spacing, (rms, spacing)
    assert rel_l2(tonp(g.V), o.V) < 1e-3
    assert rel_l2(tonp(g.F), o.F) < 1e-3
    assert rel_l2(tonp(g.RHO), o.RHO) < 1e-4
    assert g.a == o.a
    # P(k) of the last force's delta_k
    n = nc * B
    k, pg = power_np.power(tonp(r['gdk'].value).astype('c16'), boxsize=box)
    k, po = power_np.power(r['odk'].copy(), boxsize=box)
    knyq = numpy.pi * n / box
    sel = (k < 0.5 * knyq) & numpy.isfinite(po) & (po > 0)
    assert numpy.abs(pg[sel] / po[sel] - 1).max() < 1e-3


def test_lpt_relation_on_device():
    """fastpm/tests/test_core.py:46-62 on the device solver."""
    import fastpm_gb300 as G
    pm = G.ParticleMesh(BoxSize=128., Nmesh=[16, 16, 16])
    Plin = G.LinearPower(G.Planck15, redshift=0, transfer='EisensteinHu')
    solver = G.Solver(pm, G.Planck15, B=1)
    Q = pm.generate_uniform_particle_grid(shift=0)
    dlin = solver.linear(solver.whitenoise(1234), lambda k: Plin(k))
    s1 = solver.lpt(dlin, Q, a=0.01, order=1)
    s2 = solver.lpt(dlin, Q, a=1.0, order=1)
    fac = G.background.kick_factor(G.Planck15.Om0, 0.01, 0.01, 1.0)
    assert_allclose(tonp(s2.P), tonp(s1.P) + fac * tonp(s1.F), rtol=1e-5,
                    atol=1e-5 * float(s2.P.abs().max()))


def test_janus_reversibility():
    """examples/janus.py:65-71: leapfrog(stages) then leapfrog(stages[::-1]) returns to the IC."""
    import fastpm_gb300 as G
    pm = G.ParticleMesh(BoxSize=64., Nmesh=[32, 32, 32])
    solver = G.Solver(pm, G.Planck15, B=2)
    Q = pm.generate_uniform_particle_grid()
    stages = numpy.linspace(0.1, 1.0, 10, endpoint=True)
    dlin = solver.linear(solver.whitenoise(400), G.EHPower(G.Planck15, 0))
    lpt = solver.lpt(dlin, Q, stages[0])
    state = solver.nbody(lpt.copy(), G.leapfrog(stages))
    back = solver.nbody(state, G.leapfrog(stages[::-1]))
    dx = tonp(back.X) - tonp(lpt.X)
    # float32 state with compensated updates: reversible to ~1e-5 of the spacing
    assert numpy.abs(dx).max() < 1e-3 * (64. / 32)


@pytest.mark.parametrize('permute', [None, 7])
@pytest.mark.parametrize('name', ['cic16', 'tsc32b1', 'cic32'])
def test_solver_without_monitor_matches_oracle(name, permute):
    """Without a monitor the device runs its fused path (one kick-drift pass
    that also counts the new positions into the sorted paint's bricks); with
    a shuffled particle grid it runs in explicit-position mode.  Same bars."""
    nc, B, box, res, seed, a0, stages, order, shift, unitary = CASES[name]
    r = run_pair(nc, B, box, res, seed, a0, stages, order, shift, unitary, monitor=False, permute=permute)
    o, g = r['oracle'], r['gpu']
    spacing = box / nc
    dx = tonp(g.X) - o.X
    dx -= box * numpy.round(dx / box)
    rms = numpy.sqrt((dx ** 2).sum(axis=1).mean())
    assert rms <= 1e-4 * spacing, (rms, spacing)
    assert rel_l2(tonp(g.V), o.V) < 1e-3
    assert rel_l2(tonp(g.F), o.F) < 1e-3
    assert rel_l2(tonp(g.RHO), o.RHO) < 1e-4
    assert g.a == o.a


FORCE_PATHS = {
    'fused-readout': dict(fused_readout=True),
    'particle-order-readout': dict(brick_readout=False),
    'three-mesh': dict(packed_force=False),
    'atomic-paint': dict(sorted_paint=False),
    'unbinned-drift': dict(binned_drift=False),
    'blocked-packed-readout': dict(blocked_force=True),
}


@pytest.mark.parametrize('path', sorted(FORCE_PATHS))
@pytest.mark.parametrize('name', ['tsc16', 'cic32'])
def test_solver_other_force_paths(name, path):
    """The other force paths (forces read out from the potential by brick;
    packed readout in particle order; three force meshes + four-mesh readout;
    atomic scatter paint; the packed mesh in 2x2x2-cell blocks read out by
    four threads per particle) meet the same bars as the default (cell-sorted
    paint, stencil into the packed mesh, packed readout in brick order)."""
    import fastpm_gb300 as G
    cls = G.core.FastPMStep
    old = {k: getattr(cls, k) for k in FORCE_PATHS[path]}
    for k, v in FORCE_PATHS[path].items():
        setattr(cls, k, v)
    try:
        test_solver_matches_oracle(name)
    finally:
        for k, v in old.items():
            setattr(cls, k, v)


@pytest.mark.parametrize('path', ['default', 'fused-readout', 'blocked-packed-readout'])
def test_solver_list_modes_bit_identical(path):
    """Without a monitor the fused kick-drift prepares the paint's brick lists:
    through per-brick buckets (option 26 = 1, the default), through buckets so
    small that every brick overflows and the paint recounts (2), or as brick
    keys and ranks that a pass of its own fills (0).  A whole solve gives the
    same bits in every mode, for each readout that reads the lists."""
    import fastpm_gb300 as G
    from fastpm_gb300 import _lib
    cls = G.core.FastPMStep
    over = {} if path == 'default' else FORCE_PATHS[path]
    old = {k: getattr(cls, k) for k in over}
    old26 = _lib.query('fpm_get_option', 26)
    res = []
    try:
        for k, v in over.items():
            setattr(cls, k, v)
        for mode in (0, 1, 2):
            _lib.call('fpm_set_option', 26, mode)
            pm = G.ParticleMesh(BoxSize=128., Nmesh=[32] * 3, resampler='tsc')
            solver = G.Solver(pm, G.Planck15, B=2)
            Q = pm.generate_uniform_particle_grid(shift=0)
            dlin = solver.linear(solver.whitenoise(77), G.EHPower(G.Planck15, 0))
            st = solver.lpt(dlin, Q, a=0.1, order=2)
            st = solver.nbody(st, G.leapfrog(numpy.linspace(0.1, 1.0, 6)))
            torch.cuda.synchronize()
            res.append([t.clone() for t in (st.S, st.P, st.F, st.RHO)])
    finally:
        _lib.call('fpm_set_option', 26, old26)
        for k, v in old.items():
            setattr(cls, k, v)
    for r in res[1:]:
        for x, y in zip(res[0], r):
            assert torch.equal(x, y)


def test_batch_invariance():
    """The rank-invariance test (test_core.py:64-93) becomes: a solve gives the
    same bits alone and after another, unrelated solve on the same device."""
    import fastpm_gb300 as G

    def solve(seed):
        pm = G.ParticleMesh(BoxSize=128., Nmesh=[16] * 3)
        solver = G.Solver(pm, G.Planck15, B=2)
        Q = pm.generate_uniform_particle_grid(shift=0)
        dlin = solver.linear(solver.whitenoise(seed), G.EHPower(G.Planck15, 0))
        st = solver.lpt(dlin, Q, a=0.1, order=2)
        st = solver.nbody(st, G.leapfrog([0.1, 0.5, 1.0]))
        return tonp(st.X), tonp(st.P), tonp(st.F)

    a = solve(1234)
    solve(99)
    b = solve(1234)
    for x, y in zip(a, b):
        assert_allclose(x, y, rtol=1e-6, atol=1e-6 * numpy.abs(y).max())


def test_monitor_protocol():
    import fastpm_gb300 as G
    pm = G.ParticleMesh(BoxSize=64., Nmesh=[16] * 3)
    solver = G.Solver(pm, G.Planck15, B=1)
    Q = pm.generate_uniform_particle_grid(shift=0)
    st = solver.lpt(solver.linear(solver.whitenoise(1), G.EHPower(G.Planck15, 0)), Q, a=0.1)
    seen = []

    def monitor(action, ai, ac, af, state, event):
        seen.append((action, ai, ac, af, state.synchronized, None if event is None else sorted(event)))

    solver.nbody(st, G.leapfrog([0.1, 0.5]), monitor=monitor)
    assert [s[0] for s in seen] == ['F', 'K', 'D', 'F', 'K']
    assert seen[0][5] == ['delta_k'] and seen[3][5] == ['delta_k']
    assert seen[-1][4] is True
    with pytest.raises(AssertionError):
        solver.nbodystep.Kick(st, 0.5, 0.3, 0.6)   # time tag mismatch (core.py:169)


def test_state_save_round_trip(tmp_path):
    """StateVector.save (core.py:65-89) from the device state: the columns
    read back equal state.X, state.V and state.RHO in Q's dtype."""
    import fastpm_gb300 as G
    from fastpm_gb300 import snapshot
    pm = G.ParticleMesh(BoxSize=64., Nmesh=[16] * 3)
    solver = G.Solver(pm, G.Planck15, B=2)
    Q = pm.generate_uniform_particle_grid(shift=0)
    st = solver.lpt(solver.linear(solver.whitenoise(5), G.EHPower(G.Planck15, 0)), Q, a=0.1)
    st = solver.nbody(st, G.leapfrog([0.1, 0.4, 1.0]))
    path = str(tmp_path / 'snap')
    st.save(path, attrs={'seed': 5})
    header, cols = snapshot.read(path)
    numpy.testing.assert_array_equal(cols['Position'], tonp(st.X))
    # V = P H0 / a in Q's dtype (the reference's P shares Q's float64 dtype)
    numpy.testing.assert_array_equal(cols['Velocity'], tonp(st.P).astype('f8') * (100. / st.a['P']))
    numpy.testing.assert_array_equal(cols['Density'], tonp(st.RHO).astype('f8'))
    assert header['Time'] == 1.0 and header['seed'] == 5 and header['Om0'] == G.Planck15.Om0
