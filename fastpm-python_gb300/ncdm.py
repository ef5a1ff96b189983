"""fastpm/ncdm.py on the device: the core solver whose force sees the total
matter density of a cosmology with massive neutrinos in linear response.

The reference (ncdm.py:10-41) paints the cold particles, forms delta_k, and
multiplies it by the ratio of the total-matter to the cold-matter transfer
function, r(k) = d_m(k) / d_cb(k), interpolated from the Boltzmann code's
tables at the force time (phase_space_linear_ncdm, ncdm.py:45-70), before the
long-range force.  Here r(k) is tabulated once per force time on the integer
shells |n|^2 of the mesh (every |k| on the mesh is 2 pi sqrt(q) / L) and the
device applies it inside the force's x pass (fpm_force_mesh_packed_transfer):
no extra pass over the complex mesh.

The cosmology must provide what the reference reads from nbodykit's CLASS
cosmology: get_transfer(z) -> {'k', 'd_cdm', 'd_b', 'd_ncdm[0]'} and
Omega_cdm(z), Omega_b(z), Omega_ncdm(z), plus Om0.
"""
import numpy
import torch

from . import _lib
from . import core


def transfer_ratio(cosmology, ac):
    """(k, d_m / d_cb) at a = ac, as ncdm.py:46-62 forms them."""
    z = 1 / ac - 1
    tf = cosmology.get_transfer(z=z)
    ktf = numpy.asarray(tf['k'], dtype='f8')
    d_cdm = numpy.asarray(tf['d_cdm'], dtype='f8')
    d_b = numpy.asarray(tf['d_b'], dtype='f8')
    d_ncdm = numpy.asarray(tf['d_ncdm[0]'], dtype='f8')
    Ocdm = cosmology.Omega_cdm(z)
    Ob = cosmology.Omega_b(z)
    Oncdm = cosmology.Omega_ncdm(z)
    d_m = (d_cdm * Ocdm + d_b * Ob + d_ncdm * Oncdm) / (Ob + Ocdm + Oncdm)
    d_cb = (d_cdm * Ocdm + d_b * Ob) / (Ob + Ocdm)
    return ktf, d_m / d_cb


def shell_table(cosmology, ac, n, boxsize, device):
    """r(|k|) on the integer shells q = 0 .. 3 (n/2)^2 of an n^3 mesh (float32,
    on the device), numpy.interp as ncdm.py:67 evaluates it."""
    ktf, r = transfer_ratio(cosmology, ac)
    q = numpy.arange(3 * (n // 2) ** 2 + 1, dtype='f8')
    k = numpy.sqrt(q) * (2 * numpy.pi / boxsize)
    return torch.from_numpy(numpy.interp(k, ktf, r).astype('f4')).to(device)


class Solver(core.Solver):
    """ncdm.py:5-8."""

    @property
    def nbodystep(self):
        return FastPMStep(self)


class FastPMStep(core.FastPMStep):
    """ncdm.py:10-41: the core step with the neutrino transfer on delta_k.

    The transfer is fused into the packed force mesh, so this step always
    takes the packed force path (row-major float4 mesh)."""
    packed_force = True
    fused_readout = False
    blocked_force = False

    def __init__(self, solver):
        core.FastPMStep.__init__(self, solver)
        self._tables = {}

    def _packed_force_mesh(self, rho, nbar, packed, delta_k, work, ws_bytes, blocked, ac):
        pm = self.pm
        t = self._tables.get(ac)
        if t is None:
            t = self._tables[ac] = shell_table(self.cosmology, ac, pm.n, pm.L, pm.device)
        _lib.call('fpm_force_mesh_packed_transfer', _lib.ptr(rho), pm.n, pm.L, 1.0 / nbar,
                  1.5 * self.cosmology.Om0, _lib.ptr(t), t.numel(), _lib.ptr(packed),
                  _lib.ptr(delta_k.data) if delta_k is not None else None, _lib.ptr(work), ws_bytes,
                  _lib.stream_ptr())
