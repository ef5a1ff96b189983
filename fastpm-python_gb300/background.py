"""Host-side float64 growth factors (fastpm/background.py:4-256).

The ODE in ln a for D1 / D2 (background.py:175-184) is integrated with
scipy's odeint on the same grid the reference builds (the requested a values,
a_normalize and a = 1e-7, background.py:19-36), so every factor equals the
reference's to rounding.  The kick / drift factors of FastPMStep
(fastpm/core.py:170-171, 177-178) are cached per (Om0, ai, ac, af, a_normalize):
the reference solves the ODE once per action, which dominates the host time of
small meshes.
"""
import functools

import numpy
from scipy.integrate import odeint


class MatterDominated(object):
    def __init__(self, Omega0_m, Omega0_lambda=None, Omega0_k=0, a=None, a_normalize=1.0):
        if Omega0_lambda is None:
            Omega0_lambda = 1 - Omega0_k - Omega0_m
        self.Om0 = self.Omega0_m = Omega0_m
        self.Omega0_lambda = Omega0_lambda
        self.Omega0_k = Omega0_k
        if a is None:
            lna = numpy.log(numpy.logspace(-7, 0, 1024 * 10, endpoint=True))
        else:
            a = numpy.array(a, copy=True, dtype='f8').ravel()
            if a_normalize not in a:
                a = numpy.concatenate([[a_normalize], a])
            a.sort()
            if a[0] > 1e-7:
                a = numpy.concatenate([[1e-7], a])
            lna = numpy.log(a)
        self.lna = lna
        a0 = numpy.exp(lna[0])
        self._solve([a0, a0, -3. / 7 * a0 ** 2, -6. / 7 * a0 ** 2], a_normalize)

    def _solve(self, y0, a_normalize):
        """background.py:186-205: odeint on the ln a grid, normalised to 1 at
        the grid point nearest a_normalize."""
        lna = self.lna
        y = odeint(self.ode, y0, lna, tcrit=[0.], atol=0)
        v1 = numpy.empty((len(lna), 3))
        v2 = numpy.empty((len(lna), 3))
        for i, (yi, lnai) in enumerate(zip(y, lna)):
            d1p, f1p, d2p, f2p = self.ode(yi, lnai)
            v1[i] = (yi[0], yi[1], f1p)
            v2[i] = (yi[2], yi[3], f2p)
        ind = abs(lna - numpy.log(a_normalize)).argmin()
        self._D1 = v1 / v1[ind][0]
        self._D2 = v2 / v2[ind][0]

    def efunc(self, a):
        return (self.Omega0_m / a ** 3 + self.Omega0_k / a ** 2 + self.Omega0_lambda) ** 0.5

    def efunc_prime(self, a):
        return 0.5 / self.efunc(a) * (-3 * self.Omega0_m / (a ** 4) + -2 * self.Omega0_k / (a ** 3))

    def Om(self, a):
        return (self.Omega0_m / a ** 3) / self.efunc(a) ** 2

    def E(self, a, order=0):
        return self.efunc(a) if order == 0 else self.efunc_prime(a) * a

    def Hfac(self, a):
        return -2. - self.E(a, order=1) / self.E(a)

    def ode(self, y, lna):
        D1, F1, D2, F2 = y
        a = numpy.exp(lna)
        hfac = self.Hfac(a)
        omega = self.Om(a)
        return F1, hfac * F1 + 1.5 * omega * D1, F2, hfac * F2 + 1.5 * omega * D2 - 1.5 * omega * D1 ** 2

    def D1(self, a, order=0):
        return numpy.interp(numpy.log(a), self.lna, self._D1[:, order])

    def D2(self, a, order=0):
        return numpy.interp(numpy.log(a), self.lna, self._D2[:, order])

    def f1(self, a):
        return self.D1(a, order=1) / self.D1(a, order=0)

    def f2(self, a):
        return self.D2(a, order=1) / self.D2(a, order=0)

    def Gp(self, a):
        return self.D1(a)

    def Gp2(self, a):
        return self.D2(a)

    def gp(self, a):
        return self.D1(a, order=1) / a

    def gp2(self, a):
        return self.D2(a, order=1) / a

    def Gf(self, a):
        return self.D1(a, 1) * a ** 2 * self.E(a)

    def Gf2(self, a):
        return self.D2(a, 1) * a ** 2 * self.E(a)

    def gf(self, a):
        return 1 / a * (self.D1(a, 2) * a ** 2 * self.E(a)
                        + self.D1(a, 1) * (a ** 2 * self.E(a, order=1) + 2 * a ** 2 * self.E(a)))

    def gf2(self, a):
        return 1 / a * (self.D2(a, 2) * a ** 2 * self.E(a)
                        + self.D2(a, 1) * (a ** 2 * self.E(a, order=1) + 2 * a ** 2 * self.E(a)))


class RadiationDominated(MatterDominated):
    """background.py:258-322: the same growth equations with a cosmology's
    own E(z) and a radiation-dominated initial condition (a_H = 5.22281250e-05
    as the reference tunes it); the growth source is the non-relativistic
    matter Omega_b(z) + Omega_cdm(z).  The cosmology provides Om0, Ogamma0,
    efunc(z), efunc_prime(z) (dE/da), Omega_b(z) and Omega_cdm(z)."""

    def __init__(self, cosmo, a=None, a_normalize=1.0):
        self._cosmo = cosmo
        self.Om0 = self.Omega0_m = cosmo.Om0
        self.Omega0_gamma = cosmo.Ogamma0
        if a is None:
            lna = numpy.log(numpy.logspace(-7, 0, 1024 * 10, endpoint=True))
        else:
            a = numpy.array(a, copy=True, dtype='f8').ravel()
            if a_normalize not in a:
                a = numpy.concatenate([[a_normalize], a])
            a.sort()
            if a[0] > 1e-7:
                a = numpy.concatenate([[1e-7], a])
            lna = numpy.log(a)
        self.lna = lna
        a_H = 5.22281250e-05
        a0 = numpy.exp(lna[0])
        Om = self.Om(a0)
        D1i = numpy.log(a0 / a_H)
        y0 = [D1i, 1.0, -1.5 * Om * (D1i ** 2 - 4 * D1i + 6), -1.5 * Om * (D1i ** 2 - 2 * D1i + 2)]
        self._solve(y0, a_normalize)

    def efunc(self, a):
        return self._cosmo.efunc(1. / a - 1.0)

    def efunc_prime(self, a):
        return self._cosmo.efunc_prime(1. / a - 1.0)

    def Om(self, a):
        z = 1. / a - 1
        return self._cosmo.Omega_b(z) + self._cosmo.Omega_cdm(z)


# background.py:325 (the growth of fastpm/multi.py and main.py)
PerturbationGrowth = RadiationDominated


@functools.lru_cache(maxsize=4096)
def kick_factor(Om0, ai, ac, af, a_normalize=1.0):
    """(Gf(af) - Gf(ai)) / (ac^2 E(ac) gf(ac))   (fastpm/core.py:170-171)."""
    pt = MatterDominated(Om0, a=[ai, ac, af], a_normalize=a_normalize)
    return float(1 / (ac ** 2 * pt.E(ac)) * (pt.Gf(af) - pt.Gf(ai)) / pt.gf(ac))


@functools.lru_cache(maxsize=4096)
def drift_factor(Om0, ai, ac, af, a_normalize=1.0):
    """(Gp(af) - Gp(ai)) / (ac^3 E(ac) gp(ac))   (fastpm/core.py:177-178)."""
    pt = MatterDominated(Om0, a=[ai, ac, af], a_normalize=a_normalize)
    return float(1 / (ac ** 3 * pt.E(ac)) * (pt.Gp(af) - pt.Gp(ai)) / pt.gp(ac))
