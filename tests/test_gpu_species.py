"""The species / transfer variants against the float64 oracle.

* fastpm/ncdm.py: the force with the linear-response neutrino transfer
  r(k) = d_m / d_cb on delta_k (ncdm.py:45-70), fused into the x pass
  (fpm_force_mesh_packed_transfer).  The cosmology is the synthetic
  linear-response stand-in of oracle/cosmology_np.py (CLASS is absent); the
  oracle's NCDMSolver is pinned to the reference's own ncdm.py by
  tests/golden/reference_ncdm.npz.
* fastpm/multi.py + state.py: several species in the potential of their
  Omega-weighted total density (the sorted paint adding species to one
  mesh, fpm_paint_sorted_add), against oracle/multi_np.py, pinned to the
  reference by tests/golden/reference_multi.npz.
"""
import numpy
import pytest
import torch

from oracle import cosmology_np, fastpm_np, pmesh_np, power_np
from tests.helpers import rel_l2, tonp

pytestmark = pytest.mark.gpu


def _device_nu():
    """The synthetic neutrino cosmology as a device-side Cosmology (the
    engine's Solver accepts its own Cosmology type, as the reference accepts
    nbodykit's)."""
    import fastpm_gb300 as G

    class DeviceNu(G.Cosmology):
        def __init__(self):
            G.Cosmology.__init__(self)
            self._o = cosmology_np.LinearResponseNeutrinos()

        def get_transfer(self, z):
            return self._o.get_transfer(z)

        def Omega_cdm(self, z):
            return self._o.Omega_cdm(z)

        def Omega_b(self, z):
            return self._o.Omega_b(z)

        def Omega_ncdm(self, z):
            return self._o.Omega_ncdm(z)

    return DeviceNu()


@pytest.mark.parametrize('n,box', [(64, 128.0), (512, 512.0)])
def test_transfer_force_mesh_vs_oracle(n, box):
    """The packed force mesh with the shell transfer (at n = 512 through the
    TMA-pipelined x pass) against the oracle: delta_k and forces."""
    import fastpm_gb300 as G
    from fastpm_gb300 import _lib, ncdm
    c = _device_nu()
    ac = 0.4
    rng = numpy.random.RandomState(n)
    rho = 1.0 + 0.3 * rng.normal(size=(n, n, n))
    pm = G.ParticleMesh(BoxSize=box, Nmesh=[n] * 3)
    table = ncdm.shell_table(c, ac, n, box, pm.device)
    ws = _lib.query('fpm_force_workspace', n)
    work = pm._scratch('force_ws', ws)
    packed = torch.empty((n, n, n, 4), dtype=torch.float32, device='cuda')
    dk = G.ComplexField(pm, empty=True)
    r = torch.from_numpy(rho.astype('f4')).cuda()
    _lib.call('fpm_force_mesh_packed_transfer', _lib.ptr(r), n, box, 1.0 / 0.125, 0.45, _lib.ptr(table),
              table.numel(), _lib.ptr(packed), _lib.ptr(dk.data), _lib.ptr(work), ws, _lib.stream_ptr())
    torch.cuda.synchronize()
    assert _lib.query('fpm_workspace_status', _lib.ptr(work), n, 0, 1) == 0
    opm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[n] * 3)
    odk = opm.create('real', value=rho / 0.125).r2c()
    odk = fastpm_np.phase_space_linear_ncdm(odk, c._o, ac)
    assert rel_l2(tonp(dk.value), odk.value) < 2e-6
    pot = odk.apply(fastpm_np.laplace)
    for d in range(3):
        ref = pot.apply(fastpm_np.gradient(d, order=1)).c2r().value * 0.45
        assert rel_l2(tonp(packed[..., d]), ref) < (1e-5 if n >= 512 else 5e-6), d
    # too short a table is refused
    with pytest.raises(_lib.FastPMError):
        _lib.call('fpm_force_mesh_packed_transfer', _lib.ptr(r), n, box, 1.0, 0.45, _lib.ptr(table),
                  table.numel() - 1, _lib.ptr(packed), None, _lib.ptr(work), ws, _lib.stream_ptr())


@pytest.mark.parametrize('nc,B,box,res', [(32, 2, 128.0, 'cic'), (16, 2, 96.0, 'tsc')])
def test_ncdm_solver_matches_oracle(nc, B, box, res):
    """ncdm.Solver on the device against the oracle's NCDMSolver (float64),
    the same whitenoise, 2LPT at 0.1 and 3 KDK steps: the engine's accuracy
    bars (rms |dX| <= 1e-4 of the spacing, P(k) within 1e-3 below k_Nyq / 2)."""
    import fastpm_gb300 as G
    from fastpm_gb300 import ncdm
    c = _device_nu()
    stages = numpy.linspace(0.1, 1.0, 4)
    Plin = cosmology_np.EHPower(c._o, 0)
    opm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, dtype='f8', resampler=res)
    osolver = fastpm_np.NCDMSolver(opm, c._o, B=B)
    wn = osolver.whitenoise(42)
    odk = {}
    ost = osolver.nbody(osolver.lpt(osolver.linear(wn, lambda k: Plin(k)),
                                    opm.generate_uniform_particle_grid(shift=0), a=0.1),
                        fastpm_np.leapfrog(stages),
                        monitor=lambda a, ai, ac, af, s, ev: odk.update(v=ev['delta_k'].value.copy())
                        if a == 'F' else None)
    pm = G.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, resampler=res)
    solver = ncdm.Solver(pm, c, B=B)
    gdk = {}
    st = solver.nbody(solver.lpt(solver.linear(pm.complex_from(wn.value), lambda k: Plin(k)),
                                 pm.generate_uniform_particle_grid(shift=0), a=0.1),
                      G.leapfrog(stages),
                      monitor=lambda a, ai, ac, af, s, ev: gdk.update(v=ev['delta_k']) if a == 'F' else None)
    torch.cuda.synchronize()
    dx = tonp(st.X) - ost.X
    dx -= box * numpy.round(dx / box)
    assert numpy.sqrt((dx ** 2).sum(axis=1).mean()) <= 1e-4 * box / nc
    assert rel_l2(tonp(st.F), ost.F) < 1e-3
    assert rel_l2(tonp(gdk['v'].value), odk['v']) < 1e-4
    k, pg = power_np.power(tonp(gdk['v'].value).astype('c16'), boxsize=box)
    k, po = power_np.power(odk['v'].copy(), boxsize=box)
    sel = (k < 0.5 * numpy.pi * nc * B / box) & numpy.isfinite(po) & (po > 0)
    assert numpy.abs(pg[sel] / po[sel] - 1).max() < 1e-3


@pytest.mark.parametrize('nc,B,box,res,order', [(16, 2, 64.0, 'cic', 1), (16, 2, 96.0, 'tsc', 2),
                                                (32, 2, 128.0, 'cic', 2)])
def test_multi_species_solver_matches_oracle(nc, B, box, res, order):
    """fastpm/multi.py on the device (baryons '0' and CDM '1': the
    Omega-weighted sorted paint of both species onto one mesh, one packed
    force mesh with the factor 1.5 E^2 a^3, a readout per species) against
    the oracle's restatement (pinned to the reference by
    tests/golden/reference_multi.npz): same whitenoise, LPT at 0.1, 3 KDK
    steps; the engine's accuracy bars per species."""
    import fastpm_gb300 as G
    from fastpm_gb300 import multi
    from oracle import multi_np
    stages = numpy.linspace(0.1, 1.0, 4)
    oc = cosmology_np.Planck15
    P_prim, tf = multi_np.synthetic_species(oc, 0.1)
    opm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, dtype='f8', resampler=res)
    osolver = multi_np.Solver(opm, oc, B=B)
    wn = osolver.whitenoise(42)
    with numpy.errstate(divide='ignore', invalid='ignore'):
        oprm = osolver.primordial(wn, P_prim)
    ost = osolver.lpt(oprm, {'0': (multi_np.Baryon, tf['d_b'], tf['dd_b']),
                             '1': (multi_np.CDM, tf['d_cdm'], tf['dd_cdm'])},
                      opm.generate_uniform_particle_grid(shift=0), a=0.1, order=order)
    olpt = {(sp, key): getattr(ost.species[sp], key).copy() for sp in ('0', '1') for key in ('S', 'P')}
    odk = {}
    ost = osolver.nbody(ost, fastpm_np.leapfrog(stages),
                        monitor=lambda a, ai, ac, af, s, ev: odk.update(v=ev['delta_k'].value.copy())
                        if a == 'F' else None)
    pm = G.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, resampler=res)
    solver = multi.Solver(pm, G.Planck15, B=B)
    prm = solver.primordial(pm.complex_from(wn.value), P_prim)
    assert rel_l2(tonp(prm.value), oprm.value) < 1e-6
    st = solver.lpt(prm, {'0': (multi.Baryon, tf['d_b'], tf['dd_b']), '1': (multi.CDM, tf['d_cdm'], tf['dd_cdm'])},
                    pm.generate_uniform_particle_grid(shift=0), a=0.1, order=order)
    for sp in ('0', '1'):
        for key in ('S', 'P'):
            assert rel_l2(tonp(getattr(st.species[sp], key)), olpt[sp, key]) < 2e-5, (sp, key)
    gdk = {}
    st = solver.nbody(st, G.leapfrog(stages),
                      monitor=lambda a, ai, ac, af, s, ev: gdk.update(v=ev['delta_k']) if a == 'F' else None)
    torch.cuda.synchronize()
    for sp in ('0', '1'):
        g, o = st.species[sp], ost.species[sp]
        dx = tonp(g.X) - o.X
        dx -= box * numpy.round(dx / box)
        assert numpy.sqrt((dx ** 2).sum(axis=1).mean()) <= 1e-4 * box / nc, sp
        assert rel_l2(tonp(g.V), o.V) < 1e-3 and rel_l2(tonp(g.F), o.F) < 1e-3, sp
        assert g.a == o.a
    assert rel_l2(tonp(gdk['v'].value), odk['v']) < 1e-4
