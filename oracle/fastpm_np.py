"""float64 restatement of the FastPM hot path — TEST INFRASTRUCTURE ONLY.

Restates, on top of oracle.pmesh_np, the reference's
  fastpm/core.py            StateVector 7-89, Solver 91-152, FastPMStep 155-210,
                            autostages 212-259, leapfrog 261-288
  fastpm/force/kernels.py   laplace 3-9, gradient 11-25, longrange 27-35
  fastpm/force/gravity.py   longrange 5-8, longrange_batch 10-29
  fastpm/force/lpt.py       lpt1 4-23, lpt2source 25-64
  fastpm/background.py      Perturbation 4-205, MatterDominated 207-256
  fastpm/ncdm.py            Solver 5-8, FastPMStep 10-41, phase_space_linear_ncdm 45-70
Pinned against the reference's own modules by tests/golden (float64, 1e-12).
"""
import numpy
from scipy.integrate import odeint

from .pmesh_np import ParticleMesh


# ---------------------------------------------------------------------------
# background.py
# ---------------------------------------------------------------------------
class MatterDominated(object):
    """Growth factors D1/D2 and FastPM factors (background.py:4-256).

    ODE in ln a (background.py:175-184), matter-dominated start at a = 1e-7
    (242-247), normalised to D = 1 at the grid point nearest a_normalize
    (201-204); values off the grid are linear interpolations in ln a (53-54).
    """

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
        y0 = [a0, a0, -3. / 7 * a0 ** 2, -6. / 7 * a0 ** 2]
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
        return (self.Omega0_m / a ** 3 + self.Omega0_k / a ** 2 + self.Omega0_lambda) ** 0.5

    def efunc_prime(self, a):
        return 0.5 / self.efunc(a) * (-3 * self.Omega0_m / (a ** 4) + -2 * self.Omega0_k / (a ** 3))

    def Om(self, a):
        return (self.Omega0_m / a ** 3) / self.efunc(a) ** 2

    def E(self, a, order=0):
        return self.efunc(a) if order == 0 else self.efunc_prime(a) * a

    def _ode(self, y, lna):
        d1, f1, d2, f2 = y
        a = numpy.exp(lna)
        hfac = -2. - self.E(a, order=1) / self.E(a)
        om = self.Om(a)
        return f1, hfac * f1 + 1.5 * om * d1, f2, hfac * f2 + 1.5 * om * d2 - 1.5 * om * d1 ** 2

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

    def gp(self, a):
        return self.D1(a, order=1) / a

    def Gf(self, a):
        return self.D1(a, 1) * a ** 2 * self.E(a)

    def gf(self, a):
        return 1 / a * (self.D1(a, 2) * a ** 2 * self.E(a)
                        + self.D1(a, 1) * (a ** 2 * self.E(a, order=1) + 2 * a ** 2 * self.E(a)))

    def gf2(self, a):
        return 1 / a * (self.D2(a, 2) * a ** 2 * self.E(a)
                        + self.D2(a, 1) * (a ** 2 * self.E(a, order=1) + 2 * a ** 2 * self.E(a)))


def kick_factor(Om0, ai, ac, af, a_normalize=1.0):
    """core.py:170-171: (Gf(af) - Gf(ai)) / (ac^2 E(ac) gf(ac))."""
    pt = MatterDominated(Om0, a=[ai, ac, af], a_normalize=a_normalize)
    return 1 / (ac ** 2 * pt.E(ac)) * (pt.Gf(af) - pt.Gf(ai)) / pt.gf(ac)


def drift_factor(Om0, ai, ac, af, a_normalize=1.0):
    """core.py:177-178: (Gp(af) - Gp(ai)) / (ac^3 E(ac) gp(ac))."""
    pt = MatterDominated(Om0, a=[ai, ac, af], a_normalize=a_normalize)
    return 1 / (ac ** 3 * pt.E(ac)) * (pt.Gp(af) - pt.Gp(ai)) / pt.gp(ac)


# ---------------------------------------------------------------------------
# force/kernels.py
# ---------------------------------------------------------------------------
def laplace(k, v):
    """kernels.py:3-9: v / k^2 with the k = 0 mode set to 0."""
    kk = sum(ki ** 2 for ki in k)
    zero = kk == 0
    kk = numpy.where(zero, 1, kk)
    return numpy.where(zero, 0, v / kk)


def gradient(dir, order=0):
    """kernels.py:11-25: order 0 = i k (Nyquist cleared), order 1 = 4-point FD."""
    if order == 0:
        def kernel(k, v):
            mask = v.i[dir] != v.Nmesh[dir] // 2
            return v * (1j * k[dir]) * mask
    else:
        def kernel(k, v):
            h = v.BoxSize[dir] / v.Nmesh[dir]
            w = k[dir] * h
            return v * (1j * (1 / (6.0 * h) * (8 * numpy.sin(w) - numpy.sin(2 * w))))
    return kernel


def longrange_kernel(r_split):
    """kernels.py:27-35: Gaussian long-range filter; identity for r_split = 0."""
    if r_split != 0:
        def kernel(k, v):
            return v * numpy.exp(-sum(ki ** 2 for ki in k) * r_split ** 2)
    else:
        def kernel(k, v):
            return v
    return kernel


# ---------------------------------------------------------------------------
# force/gravity.py, force/lpt.py
# ---------------------------------------------------------------------------
def longrange(x, delta_k, split, factor):
    """gravity.py:5-29: F_d = factor * readout(c2r(grad_d laplace delta_k))."""
    f = numpy.empty_like(x)
    pot_k = delta_k.apply(laplace).apply(longrange_kernel(split), out=Ellipsis)
    for d in range(delta_k.ndim):
        force_d = pot_k.apply(gradient(d, order=1)).c2r(out=Ellipsis)
        force_d.readout(x, out=f[..., d])
    f[...] *= factor
    return f


def longrange_batch_list(xs, delta_k, split, factor):
    """gravity.py:10-29: the long-range force read out at each of several
    position arrays from one delta_k."""
    fs = [numpy.empty_like(x) for x in xs]
    pot_k = delta_k.apply(laplace).apply(longrange_kernel(split), out=Ellipsis)
    for d in range(delta_k.ndim):
        force_d = pot_k.apply(gradient(d, order=1)).c2r(out=Ellipsis)
        for x, f in zip(xs, fs):
            force_d.readout(x, out=f[..., d])
    for f in fs:
        f[...] *= factor
    return fs


def lpt1(dlin_k, q, resampler='cic'):
    """lpt.py:4-23: first-order displacement read out (CIC) at q."""
    source = numpy.zeros((len(q), 3), dtype=q.dtype)
    for d in range(3):
        disp = dlin_k.apply(laplace).apply(gradient(d, order=1), out=Ellipsis).c2r(out=Ellipsis)
        source[..., d] = disp.readout(q, resampler=resampler)
    return source


def lpt2source(dlin_k):
    """lpt.py:25-64: 3/7 [sum_i<j phi_ii phi_jj - sum_i<j phi_ij^2], returned in k space."""
    source = dlin_k.pm.create('real')
    D1 = [1, 2, 0]
    D2 = [2, 0, 1]
    phi_ii = []
    for d in range(3):
        phi_ii.append(dlin_k.apply(laplace).apply(gradient(d, order=1), out=Ellipsis)
                      .apply(gradient(d, order=1), out=Ellipsis).c2r(out=Ellipsis))
    for d in range(3):
        source[...] += phi_ii[D1[d]].value * phi_ii[D2[d]].value
    for d in range(3):
        phi_ij = dlin_k.apply(laplace).apply(gradient(D1[d], order=1), out=Ellipsis) \
            .apply(gradient(D2[d], order=1), out=Ellipsis).c2r(out=Ellipsis)
        source[...] -= phi_ij[...] ** 2
    source[...] *= 3.0 / 7
    return source.r2c(out=Ellipsis)


# ---------------------------------------------------------------------------
# core.py
# ---------------------------------------------------------------------------
class StateVector(object):
    """core.py:7-89 (save/to_catalog omitted: I/O is outside the path)."""

    def __init__(self, solver, Q):
        self.solver = solver
        self.pm = solver.pm
        self.Q = Q
        self.csize = solver.pm.comm.allreduce(len(self.Q))
        self.dtype = self.Q.dtype
        self.cosmology = solver.cosmology
        self.H0 = 100.
        self.GM0 = self.H0 ** 2 / (4 * numpy.pi) * 1.5 * self.cosmology.Om0 \
            * self.pm.BoxSize.prod() / self.csize
        self.S = numpy.zeros_like(self.Q)
        self.P = numpy.zeros_like(self.Q)
        self.F = numpy.zeros_like(self.Q)
        self.RHO = numpy.zeros_like(self.Q[..., 0])
        self.a = dict(S=None, P=None, F=None)

    def copy(self):
        obj = object.__new__(type(self))
        obj.__dict__.update(self.__dict__)
        obj.a = dict(self.a)
        for key in ('S', 'P', 'F', 'RHO'):
            setattr(obj, key, getattr(self, key).copy())
        return obj

    @property
    def synchronized(self):
        a = self.a['S']
        return a == self.a['P'] and a == self.a['F']

    @property
    def X(self):
        return self.S + self.Q

    @property
    def V(self):
        return self.P * (self.H0 / self.a['P'])


class Solver(object):
    """core.py:91-152."""

    def __init__(self, pm, cosmology, B=1, a_linear=1.0):
        if not hasattr(cosmology, 'Om0'):
            raise TypeError("only nbodykit.cosmology object is supported")
        self.pm = pm
        self.fpm = ParticleMesh(Nmesh=pm.Nmesh * B, BoxSize=pm.BoxSize, dtype=pm.dtype,
                                comm=pm.comm, resampler=pm.resampler)
        self.cosmology = cosmology
        self.a_linear = a_linear

    @property
    def nbodystep(self):
        return FastPMStep(self)

    def whitenoise(self, seed, unitary=False):
        return self.pm.generate_whitenoise(seed, type='complex', unitary=unitary)

    def linear(self, whitenoise, Pk):
        return whitenoise.apply(lambda k, v:
                                Pk(sum(ki ** 2 for ki in k) ** 0.5) ** 0.5 * v / v.BoxSize.prod() ** 0.5)

    def lpt(self, linear, Q, a, order=2):
        assert order in (1, 2)
        state = StateVector(self, Q)
        pt = MatterDominated(self.cosmology.Om0, a=[a], a_normalize=self.a_linear)
        DX1 = pt.D1(a) * lpt1(linear, Q)
        V1 = a ** 2 * pt.f1(a) * pt.E(a) * DX1
        if order == 2:
            DX2 = pt.D2(a) * lpt1(lpt2source(linear), Q)
            V2 = a ** 2 * pt.f2(a) * pt.E(a) * DX2
            state.S[...] = DX1 + DX2
            state.P[...] = V1 + V2
            state.F[...] = a ** 2 * pt.E(a) * (pt.gf(a) / pt.D1(a) * DX1 + pt.gf2(a) / pt.D2(a) * DX2)
        else:
            state.S[...] = DX1
            state.P[...] = V1
            state.F[...] = a ** 2 * pt.E(a) * (pt.gf(a) / pt.D1(a) * DX1)
        state.a['S'] = a
        state.a['P'] = a
        return state

    def nbody(self, state, stepping, monitor=None):
        step = self.nbodystep
        for action, ai, ac, af in stepping:
            step.run(action, ai, ac, af, state, monitor)
        return state


class FastPMStep(object):
    """core.py:155-210."""

    def __init__(self, solver):
        self.cosmology = solver.cosmology
        self.pm = solver.fpm
        self.solver = solver

    def run(self, action, ai, ac, af, state, monitor):
        event = dict(K=self.Kick, D=self.Drift, F=self.Force)[action](state, ai, ac, af)
        if monitor is not None:
            monitor(action, ai, ac, af, state, event)

    def Kick(self, state, ai, ac, af):
        assert ac == state.a['F']
        fac = kick_factor(self.cosmology.Om0, ai, ac, af, self.solver.a_linear)
        state.P[...] = state.P[...] + fac * state.F[...]
        state.a['P'] = af

    def Drift(self, state, ai, ac, af):
        assert ac == state.a['P']
        fac = drift_factor(self.cosmology.Om0, ai, ac, af, self.solver.a_linear)
        state.S[...] = state.S[...] + fac * state.P[...]
        state.a['S'] = af

    def prepare_force(self, state, smoothing):
        nbar = 1.0 * state.csize / self.pm.Nmesh.prod()
        X = state.X
        rho = self.pm.paint(X)
        rho /= nbar
        return X, rho

    def Force(self, state, ai, ac, af):
        assert ac == state.a['S']
        X, rho = self.prepare_force(state, smoothing=None)
        state.RHO[...] = rho.readout(X)
        delta_k = rho.r2c(out=Ellipsis)
        state.F[...] = longrange(X, delta_k, split=0, factor=1.5 * self.cosmology.Om0)
        state.a['F'] = af
        return dict(delta_k=delta_k)


def autostages(knots, N, astart=None, N0=None):
    """core.py:212-259."""
    knots = numpy.sort(numpy.array(knots, dtype='f8'))
    stages = numpy.array([], dtype='f8')
    if astart is not None and astart != knots.min():
        assert astart < knots.min()
        if N0 is None:
            N0 = 1
        knots = numpy.append([astart], knots)
    else:
        N0 = 1
    for i in range(len(knots) - 1):
        da = (knots[-1] - knots[i]) / (N - len(stages) - 1)
        n = int((knots[i + 1] - knots[i]) / da + 0.5)
        if i == 0 and n < N0:
            n = N0
        stages = numpy.append(stages, numpy.linspace(knots[i], knots[i + 1], n, endpoint=False))
    return numpy.append(stages, [knots[-1]])


def leapfrog(stages):
    """core.py:261-288: F first, then K(half) D F K(full) per interval."""
    if len(stages) == 0:
        return
    ai = stages[0]
    yield 'F', ai, ai, ai
    x = p = f = ai
    for i in range(len(stages) - 1):
        a0, a1 = stages[i], stages[i + 1]
        ah = (a0 * a1) ** 0.5
        yield 'K', p, f, ah
        p = ah
        yield 'D', x, p, a1
        x = a1
        yield 'F', f, x, a1
        f = a1
        yield 'K', p, f, a1
        p = a1


# ---------------------------------------------------------------------------
# ncdm.py: the core step with the linear-response neutrino transfer on delta_k
# ---------------------------------------------------------------------------
def phase_space_linear_ncdm(delta_k, cosmology, ac):
    """ncdm.py:45-70: delta_k *= interp(|k|, k_tf, d_m / d_cb) at z = 1/ac - 1."""
    z = 1 / ac - 1
    tf = cosmology.get_transfer(z=z)
    ktf = tf['k']
    d_cdm, d_b, d_ncdm = tf['d_cdm'], tf['d_b'], tf['d_ncdm[0]']
    Ocdm, Ob, Oncdm = cosmology.Omega_cdm(z), cosmology.Omega_b(z), cosmology.Omega_ncdm(z)
    d_m = (d_cdm * Ocdm + d_b * Ob + d_ncdm * Oncdm) / (Ob + Ocdm + Oncdm)
    d_cb = (d_cdm * Ocdm + d_b * Ob) / (Ob + Ocdm)

    def transfer(k, v):
        k = sum(ki ** 2 for ki in k) ** 0.5
        return numpy.interp(k, ktf, d_m / d_cb) * v
    return delta_k.apply(transfer, out=Ellipsis)


class NCDMSolver(Solver):
    """ncdm.py:5-8."""

    @property
    def nbodystep(self):
        return NCDMStep(self)


class NCDMStep(FastPMStep):
    """ncdm.py:10-41."""

    def Force(self, state, ai, ac, af):
        assert ac == state.a['S']
        X, rho = self.prepare_force(state, smoothing=None)
        state.RHO[...] = rho.readout(X)
        delta_k = rho.r2c(out=Ellipsis)
        delta_k = phase_space_linear_ncdm(delta_k, self.cosmology, ac)
        state.F[...] = longrange(X, delta_k, split=0, factor=1.5 * self.cosmology.Om0)
        state.a['F'] = af
        return dict(delta_k=delta_k)


# ---------------------------------------------------------------------------
# loss of the differentiable forward model (float64), for finite differences
# ---------------------------------------------------------------------------
def model_density(wn_value, Om0, sigma8, nc, B, box, stages, resampler='cic'):
    """rho / nbar of the CIC-painted final positions of a 2LPT + leapfrog run
    started from whitenoise modes wn_value (complex [nc, nc, nc//2+1])."""
    from .cosmology_np import Cosmology, EHPower
    pm = ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, dtype='f8', resampler=resampler)
    cosmo = Cosmology(Om0=Om0, sigma8=sigma8)
    solver = Solver(pm, cosmo, B=B)
    wn = pm.create('complex', value=wn_value)
    dlin = solver.linear(wn, EHPower(cosmo, 0))
    Q = pm.generate_uniform_particle_grid(shift=0)
    state = solver.lpt(dlin, Q, a=stages[0], order=2)
    state = solver.nbody(state, leapfrog(stages))
    n = nc * B
    from .pmesh_np import paint
    rho = paint(state.X, [n] * 3, [box] * 3, 'cic')
    return rho / (nc ** 3 / float(n) ** 3)


def model_loss(wn_value, Om0, sigma8, nc, B, box, stages, target, resampler='cic'):
    d = model_density(wn_value, Om0, sigma8, nc, B, box, stages, resampler)
    return float(((d - target) ** 2).sum())
