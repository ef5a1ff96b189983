"""Integer-shell power spectrum on the device (fastpm/utils.py:77-164 ``power``).

Float64 shell sums in the kernel; the normalisation by |f(k=0)| (utils.py:95-96,
103-104) is applied on the host from the k = 0 mode.
"""
import numpy
import torch

from . import _lib
from .pm import ComplexField, RealField


def power(f1, f2=None, boxsize=None, average=True):
    """k, P(k) (or k, P*N, N with average=False) of ComplexField/RealField inputs."""
    def tocomplex(f):
        return f.r2c() if isinstance(f, RealField) else f

    f1 = tocomplex(f1)
    f2 = tocomplex(f2) if f2 is not None else None
    pm = f1.pm
    n = pm.n
    L = pm.L if boxsize is None else float(boxsize)
    nb = n // 2
    sums = torch.zeros((3, nb), dtype=torch.float64, device=pm.device)
    _lib.call('fpm_power_accumulate', _lib.ptr(f1.data), _lib.ptr(f2.data) if f2 is not None else None,
              n, L, _lib.ptr(sums[0]), _lib.ptr(sums[1]), _lib.ptr(sums[2]), _lib.stream_ptr())
    z1 = abs(complex(f1.value[0, 0, 0].item()))
    z2 = abs(complex(f2.value[0, 0, 0].item())) if f2 is not None else z1
    ksum, psum, wsum = sums.cpu().numpy()
    norm = (z1 if z1 != 0 else 1.0) * (z2 if z2 != 0 else 1.0)
    # pmesh's r2c carries 1/N; utils.power's own rfftn does not, but it divides
    # by |f(0)| which cancels the convention for density (1 + delta) fields.
    psum = psum / norm
    with numpy.errstate(invalid='ignore', divide='ignore'):
        center = ksum / wsum
        if not average:
            return center, psum * L ** 3, wsum
        return center, psum / wsum * L ** 3


def format_power(k, p, N, D):
    """The columns fastpm/main.py:81-92 writes for a power spectrum: k, P(k),
    the number of modes in the bin and P(k) / D^2 (D the linear growth
    factor at the output time), bins without modes dropped."""
    k, p, N = numpy.asarray(k), numpy.asarray(p), numpy.asarray(N)
    ok = N > 0
    return numpy.array([k[ok], p[ok], N[ok], p[ok] / D ** 2]).T


def write_power(path, field, a=1.0, cosmology=None, boxsize=None):
    """Write the power spectrum of `field` as fastpm/main.py:81-92 does
    (numpy.savetxt with comments='# k p N p/D**2' and no header, so, as in the
    reference's files, no comment line is written).  D is the growth factor
    D1(a) of `cosmology` normalised to 1 at a = 1 (1 when no cosmology is
    given).  The estimator is utils.power's integer-shell binning (bin width
    2 pi / L, modes counted over the full complex mesh)."""
    from .background import MatterDominated
    k, pn, N = power(field, boxsize=boxsize, average=False)
    with numpy.errstate(invalid='ignore', divide='ignore'):
        p = pn / N
    D = float(MatterDominated(cosmology.Om0, a=[a, 1.0]).D1(a)) if cosmology is not None else 1.0
    numpy.savetxt(path, format_power(k, p, N, D), comments='# k p N p/D**2')
    return path
