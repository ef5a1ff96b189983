"""fastpm/multi.py and fastpm/state.py on the device: several particle species
(baryons, CDM, massive neutrinos, ...) moving in the potential of their
Omega-weighted total density.

Same classes, signatures and semantics as the reference:
  state.py:6-140   Species (Q, S, P, F, RHO, a tags, X, V, Omega(a)), Matter /
                   Baryon / CDM / NCDM, StateVector (species in name order)
  multi.py:10-112  Solver: whitenoise, primordial, lpt(primordial,
                   species_spec, Q, a, order) with species_spec =
                   {name: (species type, d(k), dd(k))}, nbody
  multi.py:115-182 FastPMStep: Kick / Drift of every species with the
                   PerturbationGrowth (RadiationDominated) factors; the force
                   from rho = sum_s Omega_s(a) / nbar_s paint(X_s), with the
                   factor 1.5 E(z)^2 a^3, read out for every species.

On the device the species' densities accumulate in one mesh through the
cell-sorted paint (the first species overwrites the mesh, fpm_paint_sorted;
the others add to it, fpm_paint_sorted_add), the force is one packed force
mesh (rho_scale 1: the mesh is already 1 + delta), and each species reads it
out.  The transfer functions d(k), dd(k) and the primordial P(k) are the
caller's callables of |k| (the reference takes them from CLASS), evaluated on
the integer shells of the mesh.  As in the reference (multi.py:96), the
second-order LPT term changes the displacements only: its velocity term is
added to a temporary there.
"""
from collections import OrderedDict

import numpy
import torch

from . import _lib
from .background import PerturbationGrowth
from .core import _is_cosmology
from .force import lpt1, lpt2source
from .pm import ComplexField, ParticleMesh

H0 = 100.
G = 43007.1


class Species(object):
    """state.py:6-91, on the device (float32 S, P, F with Kahan terms)."""

    def __init__(self, cosmology, BoxSize, Q, comm=None, pm=None):
        self.cosmology = cosmology
        self.comm = comm
        self.BoxSize = numpy.zeros(3, dtype='f8')
        self.BoxSize[...] = BoxSize
        if isinstance(Q, numpy.ndarray):
            Q = torch.from_numpy(Q).cuda()
        self.Q = Q
        self.dtype = Q.dtype
        self.csize = len(Q)
        lat = getattr(Q, '_fpm_lattice', None)
        if lat is not None and (pm is None or lat[0] != pm.n or lat[2] != pm.L):
            lat = None
        self.lattice = (lat[0], lat[1]) if lat is not None else None
        self.q32 = None if lat is not None else Q.to(dtype=torch.float32).contiguous()
        z = lambda *s: torch.zeros(*s, dtype=torch.float32, device=Q.device)
        n = len(Q)
        self.S, self.P, self.F, self.RHO = z(n, 3), z(n, 3), z(n, 3), z(n)
        # Kahan compensation terms, bfloat16 (the kernels' storage format)
        self.S_c = torch.zeros(n, 3, dtype=torch.bfloat16, device=Q.device)
        self.P_c = torch.zeros(n, 3, dtype=torch.bfloat16, device=Q.device)
        self.a = dict(S=None, P=None, F=None)

    def Omega(self, a):
        raise NotImplementedError

    def M1(self, a):
        """state.py:33-38: mass of a particle."""
        z = 1.0 / a - 1
        rhoc = 3 * self.cosmology.efunc(z) ** 2 * H0 ** 2 / (8 * numpy.pi * G)
        return rhoc * self.Omega(a) * self.BoxSize.prod() / self.csize

    def copy(self):
        obj = object.__new__(type(self))
        obj.__dict__.update(self.__dict__)
        obj.a = dict(self.a)
        for key in ('S', 'P', 'F', 'RHO', 'S_c', 'P_c'):
            setattr(obj, key, getattr(self, key).clone())
        return obj

    @property
    def synchronized(self):
        a = self.a['S']
        return a == self.a['P'] and a == self.a['F']

    @property
    def X(self):
        return self.S.to(self.Q.dtype) + self.Q

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
    """state.py:114-140: a dict of species in name order."""

    def __init__(self, cosmology, species, comm=None):
        self.cosmology = cosmology
        self.species = OrderedDict(sorted(species.items(), key=lambda t: t[0]))
        self.comm = comm
        self.a = dict(S=None, P=None, F=None)

    def __getitem__(self, spname):
        return self.species[spname]

    def __iter__(self):
        return iter(self.species)

    def __contains__(self, name):
        return name in self.species

    def copy(self):
        s = StateVector(self.cosmology, {k: v.copy() for k, v in self.species.items()}, self.comm)
        s.a = dict(self.a)
        return s


def _isotropic(field, fn):
    """field * fn(|k|), fn evaluated once per integer shell of the mesh (a new field)."""
    pm = field.pm
    n = pm.n
    q = numpy.arange(3 * (n // 2) ** 2 + 1, dtype='f8')
    k = numpy.sqrt(q) * (2 * numpy.pi / pm.L)
    with numpy.errstate(divide='ignore', invalid='ignore'):
        t = numpy.asarray(fn(k), dtype='f8') * numpy.ones_like(k)
    t = torch.from_numpy(t.astype('f4')).to(pm.device)
    out = field.copy()
    _lib.call('fpm_apply_isotropic', _lib.ptr(out.data), n, _lib.ptr(t), len(t), _lib.stream_ptr())
    return out


class Solver(object):
    """multi.py:10-112."""

    def __init__(self, pm, cosmology, B=1):
        if not _is_cosmology(cosmology):
            raise TypeError("only nbodykit.cosmology object is supported")
        _lib.require_cuda()
        self.pm = pm
        self.fpm = ParticleMesh(Nmesh=pm.Nmesh * B, BoxSize=pm.BoxSize, dtype=pm.dtype, comm=pm.comm,
                                resampler=pm.resampler, device=pm.device)
        self.cosmology = cosmology

    @property
    def nbodystep(self):
        return FastPMStep(self)

    def whitenoise(self, seed, unitary=False):
        return self.pm.generate_whitenoise(seed, type='complex', unitary=unitary)

    def primordial(self, wn, Pk):
        """multi.py:31-38: wn (2 pi^2 k^-3 P(k))^1/2 / V^1/2, 0 at k = 0."""
        V = float(numpy.prod(wn.pm.BoxSize))

        def t(k):
            with numpy.errstate(divide='ignore', invalid='ignore'):
                r = (2 * numpy.pi ** 2 * k ** -3 * Pk(k)) ** 0.5 / V ** 0.5
            r[k == 0] = 0
            return r
        return _isotropic(wn, t)

    def lpt(self, primordial, species_spec, Q, a, order=1):
        """multi.py:40-103."""
        assert order in (1, 2)
        pt = PerturbationGrowth(self.cosmology, a=[a])
        z = 1. / a - 1
        source1 = ComplexField(self.pm)
        Omega_tot = 0
        species = {}
        for spname, (sptype, d, dd) in sorted(species_spec.items(), key=lambda t: t[0]):
            sp = sptype(self.cosmology, self.pm.BoxSize, Q, self.pm.comm, pm=self.pm)
            source = _isotropic(primordial, d)
            source1.data += float(sp.Omega(a)) * source.data
            Omega_tot += float(sp.Omega(a))
            sp.S[...] = lpt1(source, sp)
            efz = float(self.cosmology.efunc(z))
            source = _isotropic(primordial, lambda k: a * efz * dd(k))
            sp.P[...] = a ** 2 * lpt1(source, sp)
            sp.F.zero_()
            sp.a['S'] = a
            sp.a['P'] = a
            species[spname] = sp
        if order == 2:
            source1.data /= Omega_tot
            source1.data /= float(pt.D1(a))
            source2 = lpt2source(source1)
            for spname, sp in species.items():
                sp.S += float(pt.D2(a)) * lpt1(source2, sp)
        state = StateVector(self.cosmology, species, self.pm.comm)
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
        self._pt = {}

    def _growth(self, ai, ac, af):
        key = (ai, ac, af)
        if key not in self._pt:
            self._pt[key] = PerturbationGrowth(self.cosmology, a=[ai, ac, af])
        return self._pt[key]

    def run(self, action, ai, ac, af, state, monitor):
        event = dict(K=self.Kick, D=self.Drift, F=self.Force)[action](state, ai, ac, af)
        if monitor is not None:
            monitor(action, ai, ac, af, state, event)

    def Kick(self, state, ai, ac, af):
        pt = self._growth(ai, ac, af)
        fac = float(1 / (ac ** 2 * pt.E(ac)) * (pt.Gf(af) - pt.Gf(ai)) / pt.gf(ac))
        for spname, sp in state.species.items():
            _lib.call('fpm_kick', _lib.ptr(sp.P), _lib.ptr(sp.P_c), _lib.ptr(sp.F), sp.P.numel(), fac,
                      _lib.stream_ptr())
            sp.a['P'] = af
        state.a['P'] = af

    def Drift(self, state, ai, ac, af):
        pt = self._growth(ai, ac, af)
        fac = float(1 / (ac ** 3 * pt.E(ac)) * (pt.Gp(af) - pt.Gp(ai)) / pt.gp(ac))
        for spname, sp in state.species.items():
            _lib.call('fpm_drift', _lib.ptr(sp.S), _lib.ptr(sp.S_c), _lib.ptr(sp.P), sp.S.numel(), fac,
                      _lib.stream_ptr())
            sp.a['S'] = af
        state.a['S'] = af

    def prepare_force(self, state, smoothing):
        """multi.py:145-157: rho = sum_s Omega_s(a) / nbar_s paint(X_s) in one
        mesh (the first species overwrites it, the others add)."""
        pm = self.pm
        rho = pm._scratch('rho', pm.n ** 3 * 4).view(torch.float32).view(pm.n, pm.n, pm.n)
        for i, (spname, sp) in enumerate(state.species.items()):
            nbar = sp.csize / float(pm.n) ** 3
            pm._paint_sorted(rho, q=sp.q32, disp=sp.S, lattice=sp.lattice,
                             mass=float(sp.Omega(sp.a['S'])) / nbar, add=i > 0)
        return rho

    def Force(self, state, ai, ac, af):
        """multi.py:159-182."""
        pm = self.pm
        n = pm.n
        rho = self.prepare_force(state, smoothing=None)
        ws = _lib.query('fpm_force_workspace', n)
        work = pm._scratch('force_ws', ws)
        packed = pm._scratch('force_packed', 4 * n ** 3 * 4)
        delta_k = ComplexField(pm, empty=True)
        zc = 1. / ac - 1
        factor = 1.5 * float(self.cosmology.efunc(zc)) ** 2 * ac ** 3
        _lib.call('fpm_force_mesh_packed', _lib.ptr(rho), n, pm.L, 1.0, factor, _lib.ptr(packed),
                  _lib.ptr(delta_k.data), _lib.ptr(work), ws, _lib.stream_ptr())
        for spname, sp in state.species.items():
            qp, np_, nc, shift = pm._geom(sp.q32, sp.S, sp.lattice)
            _lib.call('fpm_readout_packed', _lib.ptr(packed), n, pm.L, _lib.ptr(sp.S), qp, np_, nc, shift,
                      _lib.FPM_WINDOW[pm.resampler], _lib.ptr(sp.F), None, _lib.stream_ptr())
            sp.a['F'] = af
        state.a['F'] = af
        return dict(delta_k=delta_k)
