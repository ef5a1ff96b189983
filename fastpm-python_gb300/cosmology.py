"""Cosmology parameters and the linear power spectrum used by the solver.

Mirrors what the reference takes from ``nbodykit.cosmology``: a Cosmology
object exposing Om0 (fastpm/core.py:18,99-100,127) and a linear P(k) callable
(fastpm/tests/test_core.py:35, fastpm/main.py:30).  P(k) is the Eisenstein &
Hu (1998, ApJ 496, 605) no-wiggle fit, eqs. (26), (28)-(31), normalised to
sigma8 with a top-hat of radius 8 Mpc/h.  Host-side float64; it is evaluated
once per linear field on the integer |n|^2 shells of the mesh.
"""
import numpy


class Cosmology(object):
    def __init__(self, h=0.6774, Omega0_b=0.0486, Omega0_cdm=None, Om0=0.3089, n_s=0.9667,
                 sigma8=0.8159, T0_cmb=2.7255, N_eff=3.046):
        self.h = float(h)
        self.Ob0 = float(Omega0_b)
        self.Om0 = float(Om0) if Omega0_cdm is None else float(Omega0_cdm) + self.Ob0
        self.Ode0 = 1.0 - self.Om0
        self.n_s = float(n_s)
        self.sigma8 = float(sigma8)
        self.Tcmb0 = float(T0_cmb)
        self.Neff = float(N_eff)
        self.H0 = 100.0 * self.h
        self.m_nu = None

    # flat LambdaCDM without radiation: the nbodykit methods the reference's
    # multi-species solver and species read (fastpm/state.py:95-113,
    # background.py:258-322)
    Ogamma0 = 0.0

    def efunc(self, z):
        a = 1.0 / (1.0 + numpy.asarray(z, dtype='f8'))
        return (self.Om0 / a ** 3 + self.Ode0) ** 0.5

    def efunc_prime(self, z):
        """dE / da at redshift z."""
        a = 1.0 / (1.0 + numpy.asarray(z, dtype='f8'))
        return 0.5 / self.efunc(z) * (-3 * self.Om0 / a ** 4)

    def Omega_b(self, z):
        return self.Ob0 * (1 + numpy.asarray(z, dtype='f8')) ** 3 / self.efunc(z) ** 2

    def Omega_cdm(self, z):
        return (self.Om0 - self.Ob0) * (1 + numpy.asarray(z, dtype='f8')) ** 3 / self.efunc(z) ** 2

    def Om(self, z):
        return self.Om0 * (1 + numpy.asarray(z, dtype='f8')) ** 3 / self.efunc(z) ** 2

    def Ob(self, z):
        return self.Omega_b(z)

    def Odm(self, z):
        return self.Omega_cdm(z)

    def Onu(self, z):
        return 0.0 * numpy.asarray(z, dtype='f8')

    def clone(self, **kw):
        d = dict(h=self.h, Omega0_b=self.Ob0, Om0=self.Om0, n_s=self.n_s, sigma8=self.sigma8,
                 T0_cmb=self.Tcmb0, N_eff=self.Neff)
        d.update(kw)
        return Cosmology(**d)

    def __repr__(self):
        return 'Cosmology(Om0=%g, h=%g, Ob0=%g, n_s=%g, sigma8=%g)' % (
            self.Om0, self.h, self.Ob0, self.n_s, self.sigma8)


Planck15 = Cosmology()


def _transfer_nowiggle(k, c):
    k = numpy.asarray(k, dtype='f8')
    h = c.h
    wm, wb = c.Om0 * h * h, c.Ob0 * h * h
    fb = c.Ob0 / c.Om0
    theta = c.Tcmb0 / 2.7
    s = 44.5 * numpy.log(9.83 / wm) / numpy.sqrt(1.0 + 10.0 * wb ** 0.75)          # eq. 26
    alpha = 1.0 - 0.328 * numpy.log(431.0 * wm) * fb + 0.38 * numpy.log(22.3 * wm) * fb ** 2
    gamma = c.Om0 * h * (alpha + (1.0 - alpha) / (1.0 + (0.43 * k * h * s) ** 4))  # eq. 30-31
    q = k * theta ** 2 / gamma                                                        # eq. 28
    L0 = numpy.log(2.0 * numpy.e + 1.8 * q)
    C0 = 14.2 + 731.0 / (1.0 + 62.5 * q)
    return L0 / (L0 + C0 * q * q)                                                     # eq. 29


_SIGMA8_GRID = None


def _sigma8_grid():
    """ln k grid, k and the cosmology-independent factors of the sigma8
    integrand (k^3 / 2 pi^2 times the squared top-hat window of R = 8 Mpc/h),
    computed once."""
    global _SIGMA8_GRID
    if _SIGMA8_GRID is None:
        lnk = numpy.linspace(numpy.log(1e-5), numpy.log(1e3), 20001)
        k = numpy.exp(lnk)
        x = 8.0 * k
        w = 3.0 * (numpy.sin(x) - x * numpy.cos(x)) / x ** 3
        _SIGMA8_GRID = (lnk, k, w)
    return _SIGMA8_GRID


class EHPower(object):
    """Linear matter P(k) in (Mpc/h)^3 at redshift 0; k in h/Mpc."""

    def __init__(self, cosmo, redshift=0.0):
        if redshift != 0:
            raise NotImplementedError('only redshift 0 is provided')
        self.cosmo = cosmo
        lnk, k, w = _sigma8_grid()
        integrand = k ** 3 * k ** cosmo.n_s * _transfer_nowiggle(k, cosmo) ** 2 / (2 * numpy.pi ** 2) * w ** 2
        self.A = cosmo.sigma8 ** 2 / numpy.trapezoid(integrand, lnk)

    def __call__(self, k):
        k = numpy.asarray(k, dtype='f8')
        with numpy.errstate(divide='ignore', invalid='ignore'):
            p = self.A * k ** self.cosmo.n_s * _transfer_nowiggle(k, self.cosmo) ** 2
        return numpy.where(k > 0, p, 0.0)


def LinearPower(cosmo, redshift=0.0, transfer='EisensteinHu'):
    return EHPower(cosmo, redshift)
