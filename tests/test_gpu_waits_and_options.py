"""Two library contracts that need a GPU but no fault:

* A bounded in-kernel wait that runs out returns an error status the host can
  read, and the context stays usable.  Option 21 lowers the limit of each
  tile's first wait in the TMA-pipelined y / x passes to one poll, so those
  waits give up before their copies land; the kernels drain the copies in
  flight (full limit), flag the workspace and return.  The next force, with
  the limit restored, is clean and correct.
* Tuning options are per host thread: two threads on distinct streams with
  different variants each get their own single-variant results.
"""
import threading

import numpy
import pytest
import torch

from oracle import fastpm_np, pmesh_np
from tests.helpers import rel_l2, tonp

pytestmark = pytest.mark.gpu

FPM_ERR_TIMEOUT = 6


def test_first_wait_time_out_is_reported_and_recovered():
    import fastpm_gb300 as G
    from fastpm_gb300 import _lib
    from fastpm_gb300.force import longrange_mesh
    n, box = 512, 512.0
    pm = G.ParticleMesh(BoxSize=box, Nmesh=[n] * 3)
    rng = numpy.random.RandomState(5)
    rho_np = 1.0 + 0.3 * rng.normal(size=(n, n, n))
    rho = G.RealField(pm, torch.from_numpy(rho_np.astype('f4')).cuda())
    assert _lib.query('fpm_get_option', 11) == 1   # the pipelined passes are the default
    _lib.call('fpm_set_option', 21, 1)
    try:
        longrange_mesh(rho, 0.125, factor=0.45)
        torch.cuda.synchronize()                    # the kernels returned
    finally:
        _lib.call('fpm_set_option', 21, 0)
    work = pm._bufs['force_ws']
    assert _lib.query('fpm_workspace_status', _lib.ptr(work), n, 0, 1) == FPM_ERR_TIMEOUT
    assert _lib.query('fpm_workspace_status', _lib.ptr(work), n, 0, 0) == 0   # cleared
    # the limit restored: the next force on the same workspace is correct
    fmesh, dk = longrange_mesh(rho, 0.125, factor=0.45)
    torch.cuda.synchronize()
    assert _lib.query('fpm_workspace_status', _lib.ptr(work), n, 0, 0) == 0
    opm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[n] * 3)
    odk = opm.create('real', value=rho_np / 0.125).r2c()
    assert rel_l2(tonp(dk.value), odk.value) < 2e-6
    pot = odk.apply(fastpm_np.laplace)
    ref = pot.apply(fastpm_np.gradient(0, order=1)).c2r().value * 0.45
    assert rel_l2(tonp(fmesh[0]), ref) < 1e-5


def test_solver_check_raises_on_flagged_workspace():
    """FastPMStep.check (run at the end of every nbody) turns the status word
    into an exception instead of returning invalid forces silently."""
    import fastpm_gb300 as G
    from fastpm_gb300 import _lib
    pm = G.ParticleMesh(BoxSize=512., Nmesh=[256] * 3, resampler='cic')
    solver = G.Solver(pm, G.Planck15, B=2)
    dlin = solver.linear(solver.whitenoise(3), G.EHPower(G.Planck15, 0))
    Q = pm.generate_uniform_particle_grid(shift=0)
    _lib.call('fpm_set_option', 21, 1)
    try:
        with pytest.raises(_lib.FastPMError) as e:
            solver.nbody(solver.lpt(dlin, Q, a=0.1), G.leapfrog([0.1, 0.2]))
        assert e.value.code == FPM_ERR_TIMEOUT
    finally:
        _lib.call('fpm_set_option', 21, 0)
    # the check cleared the status word: a new run is clean and repeatable
    a = solver.nbody(solver.lpt(dlin, Q, a=0.1), G.leapfrog([0.1, 0.2]))
    b = solver.nbody(solver.lpt(dlin, Q, a=0.1), G.leapfrog([0.1, 0.2]))
    torch.cuda.synchronize()
    assert torch.equal(a.S, b.S) and bool(torch.isfinite(a.S).all())


def test_options_are_per_thread():
    """Thread A runs the force with the gradient stencil (option 12 = 1),
    thread B with three gradient c2r's (option 12 = 0), concurrently on their
    own streams, several times each; every result is bitwise the result of
    its variant computed alone, and the main thread's options are unchanged."""
    import fastpm_gb300 as G
    from fastpm_gb300 import _lib
    from fastpm_gb300.force import longrange_mesh
    n = 128
    g = torch.Generator(device='cuda').manual_seed(9)
    rho = 1 + 0.2 * torch.randn((n, n, n), generator=g, device='cuda')
    alone = {}
    for v in (0, 1):
        pm = G.ParticleMesh(BoxSize=float(n), Nmesh=[n] * 3)
        old = _lib.query('fpm_get_option', 12)
        _lib.call('fpm_set_option', 12, v)
        try:
            alone[v] = longrange_mesh(G.RealField(pm, rho), 0.125, 0.45)[0].clone()
        finally:
            _lib.call('fpm_set_option', 12, old)
    torch.cuda.synchronize()
    assert not torch.equal(alone[0], alone[1])   # the variants are distinguishable
    main_opt = _lib.query('fpm_get_option', 12)
    results = {0: [], 1: []}
    errors = []
    barrier = threading.Barrier(2)

    def worker(v):
        try:
            stream = torch.cuda.Stream()
            pm = G.ParticleMesh(BoxSize=float(n), Nmesh=[n] * 3)
            _lib.call('fpm_set_option', 12, v)   # this thread only
            barrier.wait()
            with torch.cuda.stream(stream):
                for _ in range(6):
                    f, _ = longrange_mesh(G.RealField(pm, rho), 0.125, 0.45)
                    results[v].append(f.clone())
            stream.synchronize()
        except Exception as exc:   # reported on the main thread
            errors.append(exc)

    threads = [threading.Thread(target=worker, args=(v,)) for v in (0, 1)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for v in (0, 1):
        assert len(results[v]) == 6
        for f in results[v]:
            assert torch.equal(f, alone[v])
    assert _lib.query('fpm_get_option', 12) == main_opt
