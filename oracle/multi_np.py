"""float64 restatement of the multi-species solver — TEST INFRASTRUCTURE ONLY.

Restates, on top of oracle.pmesh_np and oracle.fastpm_np:
  fastpm/state.py   Species 6-91, Matter / Baryon / CDM / NCDM 93-111,
                    StateVector 114-140
  fastpm/multi.py   Solver 10-112 (whitenoise, primordial, lpt with a
                    species transfer spec, nbody), FastPMStep 115-182
                    (Kick / Drift per species, the Omega-weighted paint of
                    every species onto one mesh, the force with the factor
                    1.5 E(z)^2 a^3 read out for every species)
  fastpm/background.py  RadiationDominated 258-322 (PerturbationGrowth)
Pinned against the reference's own multi.py / state.py by
tests/golden/reference_multi.npz.
"""
from collections import OrderedDict

import numpy
from scipy.integrate import odeint

from .fastpm_np import MatterDominated, lpt1, lpt2source, longrange_batch_list
from .pmesh_np import ParticleMesh

H0 = 100.
G = 43007.1


class RadiationDominated(MatterDominated):
    """background.py:258-322."""

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
        y = odeint(self._ode, y0, lna, tcrit=[0.], atol=0)
        v1 = numpy.empty((len(lna), 3))
        v2 = numpy.empty((len(lna), 3))
        for n in range(len(lna)):
            d1, f1, d2, f2 = y[n]
            _, f1p, _, f2p = self._ode(y[n], lna[n])
            v1[n] = (d1, f1, f1p)
            v2[n] = (d2, f2, f2p)
        ind = abs(lna - numpy.log(a_normalize)).argmin()
        self._D1 = v1 / v1[ind][0]
        self._D2 = v2 / v2[ind][0]

    def efunc(self, a):
        return self._cosmo.efunc(1. / a - 1.0)

    def efunc_prime(self, a):
        return self._cosmo.efunc_prime(1. / a - 1.0)

    def Om(self, a):
        z = 1. / a - 1
        return self._cosmo.Omega_b(z) + self._cosmo.Omega_cdm(z)


PerturbationGrowth = RadiationDominated


class Species(object):
    """state.py:6-91 (I/O omitted)."""

    def __init__(self, cosmology, BoxSize, Q, comm=None):
        self.cosmology = cosmology
        self.BoxSize = numpy.zeros(Q.shape[-1], dtype='f8')
        self.BoxSize[...] = BoxSize
        self.Q = Q
        self.dtype = Q.dtype
        self.csize = len(Q)
        self.S = numpy.zeros_like(Q)
        self.P = numpy.zeros_like(Q)
        self.F = numpy.zeros_like(Q)
        self.RHO = numpy.zeros_like(Q[..., 0])
        self.a = dict(S=None, P=None, F=None)

    def Omega(self, a):
        raise NotImplementedError

    @property
    def X(self):
        return self.S + self.Q

    @property
    def V(self):
        return self.P * (H0 / self.a['P'])


class Matter(Species):
    def Omega(self, a):
        return self.cosmology.Om(z=1. / a - 1)


class Baryon(Species):
    def Omega(self, a):
        return self.cosmology.Ob(z=1. / a - 1)


class CDM(Species):
    def Omega(self, a):
        return self.cosmology.Odm(z=1. / a - 1)


class NCDM(Species):
    def Omega(self, a):
        return self.cosmology.Onu(z=1. / a - 1)


class StateVector(object):
    """state.py:114-140: species in name order."""

    def __init__(self, cosmology, species):
        self.cosmology = cosmology
        self.species = OrderedDict(sorted(species.items(), key=lambda t: t[0]))
        self.a = dict(S=None, P=None, F=None)

    def __getitem__(self, name):
        return self.species[name]


class Solver(object):
    """multi.py:10-112."""

    def __init__(self, pm, cosmology, B=1):
        self.pm = pm
        self.fpm = ParticleMesh(Nmesh=pm.Nmesh * B, BoxSize=pm.BoxSize, dtype=pm.dtype, comm=pm.comm,
                                resampler=pm.resampler)
        self.cosmology = cosmology

    @property
    def nbodystep(self):
        return FastPMStep(self)

    def whitenoise(self, seed, unitary=False):
        return self.pm.generate_whitenoise(seed, type='complex', unitary=unitary)

    def primordial(self, wn, Pk):
        """multi.py:31-38: wn (2 pi^2 k^-3 P(k))^1/2 / V^1/2, k = 0 -> 0."""
        def apply_primordial(k, v):
            k = sum(ki ** 2 for ki in k) ** 0.5
            with numpy.errstate(divide='ignore', invalid='ignore'):
                t = (2 * numpy.pi ** 2 * k ** -3 * Pk(k)) ** 0.5 / wn.BoxSize.prod() ** 0.5
            t[k == 0] = 0
            return t * v
        return wn.apply(apply_primordial)

    def lpt(self, primordial, species_spec, Q, a, order=1):
        """multi.py:40-103."""
        assert order in (1, 2)
        pt = PerturbationGrowth(self.cosmology, a=[a])
        z = 1. / a - 1
        get_k = lambda k: sum(ki ** 2 for ki in k) ** 0.5
        source1 = self.pm.create(type='complex', value=0)
        Omega_tot = 0
        species = {}
        for spname, (sptype, d, dd) in sorted(species_spec.items(), key=lambda t: t[0]):
            sp = sptype(self.cosmology, self.pm.BoxSize, Q)
            source = primordial.apply(lambda k, v: d(get_k(k)) * v)
            source1[...] += sp.Omega(a) * source
            Omega_tot += sp.Omega(a)
            sp.S[...] = lpt1(source, Q)
            source = primordial.apply(lambda k, v: a * self.cosmology.efunc(z) * dd(get_k(k)) * v)
            sp.P[...] = a ** 2 * lpt1(source, Q)
            sp.F[...] = 0
            sp.a['S'] = a
            sp.a['P'] = a
            species[spname] = sp
        if order == 2:
            source1[...] /= Omega_tot
            source1[...] /= pt.D1(a)
            source2 = lpt2source(source1)
            for spname, sp in species.items():
                DX2 = lpt1(source2, Q)
                sp.S[...] += pt.D2(a) * DX2
                # multi.py:96 adds to the velocity V (a property there, so the
                # addition is to a temporary and the state keeps its P)
        state = StateVector(self.cosmology, species)
        state.a['S'] = a
        state.a['P'] = a
        return state

    def nbody(self, state, stepping, monitor=None):
        step = self.nbodystep
        for action, ai, ac, af in stepping:
            step.run(action, ai, ac, af, state, monitor)
        return state


class FastPMStep(object):
    """multi.py:115-182."""

    def __init__(self, solver):
        self.cosmology = solver.cosmology
        self.pm = solver.fpm
        self.solver = solver

    def run(self, action, ai, ac, af, state, monitor):
        event = dict(K=self.Kick, D=self.Drift, F=self.Force)[action](state, ai, ac, af)
        if monitor is not None:
            monitor(action, ai, ac, af, state, event)

    def Kick(self, state, ai, ac, af):
        pt = PerturbationGrowth(self.cosmology, a=[ai, ac, af])
        fac = 1 / (ac ** 2 * pt.E(ac)) * (pt.Gf(af) - pt.Gf(ai)) / pt.gf(ac)
        for spname, sp in state.species.items():
            sp.P[...] = sp.P[...] + fac * sp.F[...]
            sp.a['P'] = af
        state.a['P'] = af

    def Drift(self, state, ai, ac, af):
        pt = PerturbationGrowth(self.cosmology, a=[ai, ac, af])
        fac = 1 / (ac ** 3 * pt.E(ac)) * (pt.Gp(af) - pt.Gp(ai)) / pt.gp(ac)
        for spname, sp in state.species.items():
            sp.S[...] = sp.S[...] + fac * sp.P[...]
            sp.a['S'] = af
        state.a['S'] = af

    def prepare_force(self, state, smoothing):
        rho = self.pm.create(type='real', value=0)
        X1 = []
        for spname, sp in state.species.items():
            X = sp.X
            nbar = sp.csize / self.pm.Nmesh.prod()
            rho[...] += self.pm.paint(X) * (sp.Omega(sp.a['S']) / nbar)
            X1.append(X)
        return X1, rho

    def Force(self, state, ai, ac, af):
        X1, rho = self.prepare_force(state, smoothing=None)
        delta_k = rho.r2c(out=Ellipsis)
        zc = 1. / ac - 1
        F1 = longrange_batch_list(X1, delta_k, split=0,
                                  factor=1.5 * self.cosmology.efunc(zc) ** 2 * ac ** 3)
        for (spname, sp), F1_sp in zip(state.species.items(), F1):
            sp.F[...] = F1_sp
            sp.a['F'] = af
        state.a['F'] = af
        return dict(delta_k=delta_k)


def synthetic_species(cosmo, a):
    """A primordial P(k) and species transfer functions standing in for
    CLASS's (get_species_transfer_function_from_class, multi.py:184-214, needs
    CLASS, which is absent): with P_prim(k) = k^3 P_EH(k) / (2 pi^2) the
    primordial field is the z = 0 linear field of the Eisenstein-Hu P(k); the
    cold dark matter follows it with the growth factor D(a) and the baryons
    trail it on small scales; the velocity transfers are the growth rate
    times those.  Smooth test shapes, not a physical baryon transfer.
    Returns (P_prim, {'d_cdm', 'dd_cdm', 'd_b', 'dd_b'})."""
    from .cosmology_np import EHPower
    Plin = EHPower(cosmo, 0)
    pt = RadiationDominated(cosmo, a=[a])
    D, f = float(pt.D1(a)), float(pt.f1(a))

    def P_prim(k):
        k = numpy.asarray(k, dtype='f8')
        return k ** 3 * Plin(k) / (2 * numpy.pi ** 2)

    supp = lambda k: 1.0 / (1.0 + (numpy.asarray(k) / 0.4) ** 2)
    tf = {
        'd_cdm': lambda k: -D * numpy.ones_like(numpy.asarray(k, dtype='f8')),
        'dd_cdm': lambda k: -D * f / a * numpy.ones_like(numpy.asarray(k, dtype='f8')),
        'd_b': lambda k: -D * supp(k),
        'dd_b': lambda k: -D * f / a * supp(k),
    }
    return P_prim, tf
