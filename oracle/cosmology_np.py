"""``nbodykit.cosmology`` stand-in for the oracle — TEST INFRASTRUCTURE ONLY.

The reference only needs ``Cosmology`` as a type to check against
(fastpm/core.py:99-100) and ``cosmology.Om0`` (core.py:18,127,170,177,207);
its tests draw P(k) from ``LinearPower(Planck15, transfer='EisensteinHu')``
(fastpm/tests/test_core.py:35) and the CLI from ``EHPower(Planck15, 0)``
(fastpm/main.py:30).  nbodykit/CLASS are absent, so the linear power spectrum
is restated from the published Eisenstein & Hu (1998, ApJ 496, 605) no-wiggle
transfer function, eqs. (26), (28)-(31), normalised to sigma8 with a real-space
top-hat of radius 8 Mpc/h.
"""
import numpy


class Cosmology(object):
    """Flat LambdaCDM parameter set (the attributes the reference reads)."""

    def __init__(self, h=0.6774, Omega0_b=0.0486, Omega0_cdm=None, Om0=0.3089,
                 n_s=0.9667, sigma8=0.8159, T0_cmb=2.7255, N_eff=3.046):
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
        d = dict(h=self.h, Omega0_b=self.Ob0, Om0=self.Om0, n_s=self.n_s,
                 sigma8=self.sigma8, T0_cmb=self.Tcmb0, N_eff=self.Neff)
        d.update(kw)
        return Cosmology(**d)


Planck15 = Cosmology()


def eh_nowiggle_transfer(k, cosmo):
    """EH98 zero-baryon-oscillation transfer T0(k); k in h/Mpc (eqs. 26, 28-31)."""
    k = numpy.asarray(k, dtype='f8')
    h = cosmo.h
    om = cosmo.Om0 * h * h
    ob = cosmo.Ob0 * h * h
    fb = cosmo.Ob0 / cosmo.Om0
    theta = cosmo.Tcmb0 / 2.7
    s = 44.5 * numpy.log(9.83 / om) / numpy.sqrt(1.0 + 10.0 * ob ** 0.75)        # Mpc
    alpha = 1.0 - 0.328 * numpy.log(431.0 * om) * fb + 0.38 * numpy.log(22.3 * om) * fb ** 2
    kmpc = k * h
    gamma = cosmo.Om0 * h * (alpha + (1.0 - alpha) / (1.0 + (0.43 * kmpc * s) ** 4))
    q = k * theta ** 2 / gamma
    L0 = numpy.log(2.0 * numpy.e + 1.8 * q)
    C0 = 14.2 + 731.0 / (1.0 + 62.5 * q)
    return L0 / (L0 + C0 * q * q)


def _tophat(x):
    x = numpy.asarray(x, dtype='f8')
    return 3.0 * (numpy.sin(x) - x * numpy.cos(x)) / x ** 3


class EHPower(object):
    """Callable linear P(k) [(Mpc/h)^3] at redshift 0, sigma8-normalised."""

    def __init__(self, cosmo, redshift=0.0, transfer='NoWiggleEisensteinHu'):
        if redshift != 0:
            raise NotImplementedError("only redshift 0 is needed on this path")
        self.cosmo = cosmo
        lnk = numpy.linspace(numpy.log(1e-5), numpy.log(1e3), 20001)
        kk = numpy.exp(lnk)
        unnorm = kk ** cosmo.n_s * eh_nowiggle_transfer(kk, cosmo) ** 2
        integrand = kk ** 3 * unnorm / (2 * numpy.pi ** 2) * _tophat(8.0 * kk) ** 2
        sig2 = numpy.trapezoid(integrand, lnk)
        self.A = cosmo.sigma8 ** 2 / sig2

    def __call__(self, k):
        k = numpy.asarray(k, dtype='f8')
        with numpy.errstate(divide='ignore', invalid='ignore'):
            p = self.A * k ** self.cosmo.n_s * eh_nowiggle_transfer(k, self.cosmo) ** 2
        return numpy.where(k > 0, p, 0.0)


def LinearPower(cosmo, redshift=0.0, transfer='EisensteinHu'):
    return EHPower(cosmo, redshift, transfer)


class LinearResponseNeutrinos(Cosmology):
    """A cosmology with a massive-neutrino component for the NCDM force
    (fastpm/ncdm.py:45-70), standing in for nbodykit's CLASS cosmology, which
    is absent: the same methods (get_transfer(z) -> {'k', 'd_cdm', 'd_b',
    'd_ncdm[0]'}, Omega_cdm(z), Omega_b(z), Omega_ncdm(z)) with SYNTHETIC
    tables.  Matter splits into CDM, baryons and a neutrino fraction fnu; the
    neutrino density contrast follows the cold one on large scales and is
    suppressed below the free-streaming length,
        d_ncdm(k, z) = d_cdm(k, z) / (1 + (k / k_fs(z))^2),  k_fs = k_fs0 / (1 + z)^0.5,
    the baryons trail the CDM by a smooth factor.  These shapes exercise the
    interpolation and the weighting of ncdm.py; they are not a physical
    neutrino transfer function."""

    def __init__(self, fnu=0.05, k_fs0=0.08, **kw):
        Cosmology.__init__(self, **kw)
        self.fnu = float(fnu)
        self.k_fs0 = float(k_fs0)
        self.Oncdm0 = self.fnu * self.Om0
        self.Ocdm0 = self.Om0 - self.Ob0 - self.Oncdm0

    def _E2(self, z):
        return self.Om0 * (1 + z) ** 3 + self.Ode0

    def Omega_cdm(self, z):
        return self.Ocdm0 * (1 + z) ** 3 / self._E2(z)

    def Omega_b(self, z):
        return self.Ob0 * (1 + z) ** 3 / self._E2(z)

    def Omega_ncdm(self, z):
        return self.Oncdm0 * (1 + z) ** 3 / self._E2(z)

    def get_transfer(self, z):
        k = numpy.logspace(-4, 1.5, 300)
        d_cdm = -1.0 / (1.0 + (k / 0.05) ** 1.5) / (1 + z)
        d_b = d_cdm * (1.0 - 0.2 * k ** 2 / (k ** 2 + 0.3 ** 2))
        kfs = self.k_fs0 / (1.0 + z) ** 0.5
        d_ncdm = d_cdm / (1.0 + (k / kfs) ** 2)
        return {'k': k, 'd_cdm': d_cdm, 'd_b': d_b, 'd_ncdm[0]': d_ncdm}
