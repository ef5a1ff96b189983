"""fastpm.force on the device: lpt1 / lpt2source (force/lpt.py) and the
long-range PM force (force/gravity.py:5-29) as fused mesh pipelines."""
import torch

from . import _lib
from .pm import ComplexField


def _lpt_work(pm):
    nbytes = _lib.query('fpm_lpt_workspace', pm.n)
    return pm._scratch('lpt_ws', nbytes), nbytes


def lpt1(dlin_k, state, resampler='cic'):
    """force/lpt.py:4-23: psi_d = readout_CIC(c2r(i a_d lap dlin_k)) at the state's Q.

    `state` is a StateVector (positions Q, lattice or explicit) of the base mesh.
    Returns float32 [Np, 3] on the device.
    """
    pm = dlin_k.pm
    n = pm.n
    work, nbytes = _lpt_work(pm)
    meshes = pm._scratch('lpt_mesh', 3 * n ** 3 * 4).view(torch.float32).view(3, n, n, n)
    _lib.call('fpm_lpt1_mesh', _lib.ptr(dlin_k.data), n, pm.L, _lib.ptr(meshes[0]),
              _lib.ptr(meshes[1]), _lib.ptr(meshes[2]), _lib.ptr(work), nbytes, _lib.stream_ptr())
    out = torch.empty((state.csize, 3), dtype=torch.float32, device=pm.device)
    pm._readout([meshes[0], meshes[1], meshes[2]], [out[:, 0], out[:, 1], out[:, 2]], [3, 3, 3],
                [1.0, 1.0, 1.0], q=state.q32, disp=None, lattice=state.lattice, resampler=resampler)
    return out


def lpt2source(dlin_k):
    """force/lpt.py:25-64: r2c(3/7 [sum phi_ii phi_jj - sum phi_ij^2]) (pmesh normalisation)."""
    pm = dlin_k.pm
    work, nbytes = _lpt_work(pm)
    out = ComplexField(pm, empty=True)
    _lib.call('fpm_lpt2_source', _lib.ptr(dlin_k.data), pm.n, pm.L, _lib.ptr(out.data),
              _lib.ptr(work), nbytes, _lib.stream_ptr())
    return out


def longrange_mesh(rho, nbar, factor, want_delta_k=True):
    """The mesh part of force/gravity.py:10-29 for rho = paint(X) (unnormalised):
    returns (three force meshes [3, n, n, n], delta_k or None)."""
    pm = rho.pm
    n = pm.n
    ws = _lib.query('fpm_force_workspace', n)
    work = pm._scratch('force_ws', ws)
    fmesh = torch.empty((3, n, n, n), dtype=torch.float32, device=pm.device)
    dk = ComplexField(pm, empty=True) if want_delta_k else None
    _lib.call('fpm_force_mesh', _lib.ptr(rho.value), n, pm.L, 1.0 / nbar, float(factor),
              _lib.ptr(fmesh[0]), _lib.ptr(fmesh[1]), _lib.ptr(fmesh[2]),
              _lib.ptr(dk.data) if dk is not None else None, _lib.ptr(work), ws, _lib.stream_ptr())
    return fmesh, dk
