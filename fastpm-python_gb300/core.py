"""Drop-in for fastpm.core: Solver / StateVector / FastPMStep / leapfrog.

Same classes, signatures, time-tag assertions and monitor protocol as the
reference's fastpm/core.py (cited per method).  State lives on the GPU:
S, P, F are float32 [Np, 3] torch tensors, RHO float32 [Np]; positions are the
particle's lattice point plus the float32 displacement S, and the kicks and
drifts carry Kahan compensation terms.  All mesh and particle arithmetic runs
in the libfastpm_gb300 kernels; the host does the float64 background factors
(fastpm/background.py) and the Python control flow.
"""
import numpy
import torch

from . import _lib
from .background import MatterDominated, kick_factor, drift_factor
from .cosmology import Cosmology
from .pm import ParticleMesh, ComplexField, RealField


def _is_cosmology(c):
    if isinstance(c, Cosmology):
        return True
    try:  # an nbodykit Cosmology, when nbodykit is installed
        from nbodykit.cosmology import Cosmology as NBCosmology
        return isinstance(c, NBCosmology)
    except Exception:
        return False


class StateVector(object):
    """fastpm/core.py:7-89."""

    def __init__(self, solver, Q):
        self.solver = solver
        self.pm = solver.pm
        device = solver.pm.device
        if isinstance(Q, numpy.ndarray):
            Q = torch.from_numpy(Q).to(device)
        self.Q = Q
        self.csize = solver.pm.comm.allreduce(len(self.Q))
        self.dtype = Q.dtype
        self.cosmology = solver.cosmology
        self.H0 = 100.
        self.GM0 = self.H0 ** 2 / (4 * numpy.pi) * 1.5 * self.cosmology.Om0 \
            * self.pm.BoxSize.prod() / self.csize
        lat = getattr(Q, '_fpm_lattice', None)
        if lat is not None and (lat[0] != solver.pm.n or lat[2] != solver.pm.L):
            lat = None
        # lattice mode: (nc, shift); explicit mode: float32 copy of Q for the kernels
        self.lattice = (lat[0], lat[1]) if lat is not None else None
        self.q32 = None if lat is not None else Q.to(device=device, dtype=torch.float32).contiguous()
        np_ = len(Q)
        z = lambda *s: torch.zeros(*s, dtype=torch.float32, device=device)
        self.S = z(np_, 3)
        self.P = z(np_, 3)
        self.F = z(np_, 3)
        self.RHO = z(np_)
        # Kahan compensation of S and P, bfloat16 (the kernels' storage format)
        self.S_c = torch.zeros(np_, 3, dtype=torch.bfloat16, device=device)
        self.P_c = torch.zeros(np_, 3, dtype=torch.bfloat16, device=device)
        self.a = dict(S=None, P=None, F=None)

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
        return self.P * (self.H0 / self.a['P'])

    def to_mesh(self):
        """Painted (unnormalised) density on the base mesh (core.py:50-55)."""
        real = RealField(self.pm)
        self.pm._paint(real.value, q=self.q32, disp=self.S,
                       lattice=self._lattice_on(self.pm))
        return real

    def _lattice_on(self, pm):
        return self.lattice

    def save(self, filename, attrs={}):
        """core.py:65-89: a snapshot directory with a Header block (Om0, Tcmb0,
        Neff, Ob0, Ode0, Time, h, RSDFactor, attrs) and the columns
        1/Position (X), 1/Velocity (V), 1/Density (RHO); see snapshot.py."""
        from .snapshot import save_state
        save_state(self, filename, attrs)


class Solver(object):
    """fastpm/core.py:91-152."""

    def __init__(self, pm, cosmology, B=1, a_linear=1.0):
        if not _is_cosmology(cosmology):
            raise TypeError("only nbodykit.cosmology object is supported")
        _lib.require_cuda()
        fpm = ParticleMesh(Nmesh=pm.Nmesh * B, BoxSize=pm.BoxSize, dtype=pm.dtype, comm=pm.comm,
                           resampler=pm.resampler, device=pm.device)
        self.pm = pm
        self.fpm = fpm
        self.B = int(B)
        self.cosmology = cosmology
        self.a_linear = a_linear

    @property
    def nbodystep(self):
        return FastPMStep(self)

    def whitenoise(self, seed, unitary=False):
        return self.pm.generate_whitenoise(seed, type='complex', unitary=unitary)

    def linear(self, whitenoise, Pk):
        """dlin = whitenoise * sqrt(P(|k|) / V)   (core.py:116-118).

        P is evaluated on the host once per integer shell n^2 = |n|^2 of the
        mesh (every |k| on the mesh is 2 pi sqrt(n^2) / L), the device kernel
        applies the table.
        """
        pm = whitenoise.pm
        n = pm.n
        qmax = 3 * (n // 2) ** 2
        k = numpy.sqrt(numpy.arange(qmax + 1, dtype='f8')) * (2 * numpy.pi / pm.L)
        with numpy.errstate(invalid='ignore', divide='ignore'):
            table = numpy.asarray(Pk(k), dtype='f8') ** 0.5 / pm.BoxSize.prod() ** 0.5
        # pinned and asynchronous: a pageable copy would make the host wait for
        # everything queued on the stream before it
        t = torch.from_numpy(table.astype('f4')).pin_memory().to(pm.device, non_blocking=True)
        out = whitenoise.copy()
        _lib.call('fpm_apply_isotropic', _lib.ptr(out.data), n, _lib.ptr(t), len(table),
                  _lib.stream_ptr())
        return out

    def lpt(self, linear, Q, a, order=2):
        """2LPT displacement, momentum and force at a (core.py:120-145)."""
        return self._lpt(linear, Q, a, order, check=True)

    def _lpt(self, linear, Q, a, order=2, check=True, growth=None):
        """lpt; check=False leaves the time-out status word of the LPT
        workspace (meshes of n >= 512) for the caller to read later instead of
        waiting for the stream here; growth: a MatterDominated of this
        cosmology (normalised at a_linear) already solved on a grid holding a."""
        assert order in (1, 2)
        from .force import lpt1, lpt2source
        state = StateVector(self, Q)
        pt = growth if growth is not None else MatterDominated(self.cosmology.Om0, a=[a],
                                                               a_normalize=self.a_linear)
        D1, D2 = float(pt.D1(a)), float(pt.D2(a))
        f1, f2, E = float(pt.f1(a)), float(pt.f2(a)), float(pt.E(a))
        gf, gf2 = float(pt.gf(a)), float(pt.gf2(a))
        dx1 = lpt1(linear, state)
        if order == 2:
            dx2 = lpt1(lpt2source(linear), state)
            state.S[...] = D1 * dx1 + D2 * dx2
            state.P[...] = (a ** 2 * f1 * E * D1) * dx1 + (a ** 2 * f2 * E * D2) * dx2
            state.F[...] = (a ** 2 * E * gf) * dx1 + (a ** 2 * E * gf2) * dx2
        else:
            state.S[...] = D1 * dx1
            state.P[...] = (a ** 2 * f1 * E * D1) * dx1
            state.F[...] = (a ** 2 * E * gf) * dx1
        state.a['S'] = a
        state.a['P'] = a
        work = self.pm._bufs.get('lpt_ws')
        if check and work is not None and self.pm.n >= 512:
            # the status word is read on the host: after this stream's kernels
            torch.cuda.current_stream().synchronize()
            rc = _lib.workspace_status(work, self.pm.n, 1, 1)
            if rc != 0:
                raise _lib.FastPMError('fpm_workspace_status', rc, _lib.load().fpm_strerror(rc).decode())
        return state

    def nbody(self, state, stepping, monitor=None):
        """core.py:147-152.  Without a monitor nothing can observe the state
        between actions, so runs of Kick / Kick / Drift go to the device as one
        fused pass (same arithmetic, same order as separate launches)."""
        step = self.nbodystep
        if monitor is not None:
            for action, ai, ac, af in stepping:
                step.run(action, ai, ac, af, state, monitor)
            step.check()
            return state
        pending = []
        for act in stepping:
            if act[0] == 'F':
                step.flush(pending, state)
                pending = []
                step.run(*act, state, None)
            elif act[0] == 'D':
                pending.append(act)
                step.flush(pending, state)
                pending = []
            else:
                pending.append(act)
                if len(pending) > 2:
                    step.flush(pending[:1], state)
                    pending = pending[1:]
        step.flush(pending, state)
        step.check()
        return state


class FastPMStep(object):
    """fastpm/core.py:155-210 on the device."""

    # forces and density interleaved in one float4 mesh for the readout
    packed_force = True
    # cell-sorted paint (binned by mesh brick, stored once) for the force
    sorted_paint = True
    # the force readout in mesh-brick order, from the sorted paint's lists
    # (each CTA's gathers stay within its brick's window cells)
    brick_readout = True
    # with the brick readout: the float4 mesh in 2x2x2-cell blocks of one
    # cache line, read by four threads per particle (8 lines per TSC window
    # instead of 9-18): fewer L1 wavefronts but twice the instructions and a
    # slower blocked stencil store; measured 9.9 ms against 7.3 ms for the
    # row-major readout at 512^3 particles / 1024^3 cells, off
    blocked_force = False
    # forces read out straight from the potential by mesh brick (no force
    # mesh; needs the sorted paint's lists): instruction-bound, measured
    # slower than the stencil + packed readout, off
    fused_readout = False
    # the fused kick-drift also counts the new positions into the sorted
    # paint's brick lists (the paint then skips its counting pass)
    binned_drift = True

    def __init__(self, solver):
        self.cosmology = solver.cosmology
        self.pm = solver.fpm
        self.solver = solver
        self.want_event = True
        self._counted = None    # (state, S buffer) whose brick counts are in the paint workspace

    def run(self, action, ai, ac, af, state, monitor):
        actions = dict(K=self.Kick, D=self.Drift, F=self.Force)
        # without a monitor the event (delta_k) is never seen: skip writing it
        self.want_event = monitor is not None
        event = actions[action](state, ai, ac, af)
        self.want_event = True
        if monitor is not None:
            monitor(action, ai, ac, af, state, event)

    def Kick(self, state, ai, ac, af):
        assert ac == state.a['F']
        fac = kick_factor(self.cosmology.Om0, ai, ac, af, self.solver.a_linear)
        _lib.call('fpm_kick', _lib.ptr(state.P), _lib.ptr(state.P_c), _lib.ptr(state.F),
                  state.P.numel(), fac, _lib.stream_ptr())
        state.a['P'] = af

    def Drift(self, state, ai, ac, af):
        assert ac == state.a['P']
        fac = drift_factor(self.cosmology.Om0, ai, ac, af, self.solver.a_linear)
        _lib.call('fpm_drift', _lib.ptr(state.S), _lib.ptr(state.S_c), _lib.ptr(state.P),
                  state.S.numel(), fac, _lib.stream_ptr())
        self._counted = None
        state.a['S'] = af

    def check(self):
        """Raise if a bounded wait inside a fused FFT kernel gave up (the
        kernels flag it in the workspace instead of hanging)."""
        pm = self.pm
        work = pm._bufs.get('force_ws')
        if work is not None and pm.n >= 512:
            rc = _lib.workspace_status(work, pm.n, 0, 1)
            if rc != 0:
                raise _lib.FastPMError('fpm_workspace_status', rc, _lib.load().fpm_strerror(rc).decode())

    def flush(self, acts, state):
        """Apply a run of kicks optionally ending with one drift (at most two
        kicks) in one device pass; the time tags advance as action by action."""
        if not acts:
            return
        kicks = [a for a in acts if a[0] == 'K']
        drift = acts[-1] if acts[-1][0] == 'D' else None
        if drift is None or len(kicks) > 2:
            for a in acts:
                self.run(*a, state, None)
            return
        fk = []
        for _, ai, ac, af in kicks:
            assert ac == state.a['F']
            fk.append(kick_factor(self.cosmology.Om0, ai, ac, af, self.solver.a_linear))
            state.a['P'] = af
        _, ai, ac, af = drift
        assert ac == state.a['P']
        fd = drift_factor(self.cosmology.Om0, ai, ac, af, self.solver.a_linear)
        fk += [0.0] * (2 - len(fk))
        self._counted = None
        if self.sorted_paint and self.binned_drift:
            # the new positions' brick counts go straight into the paint workspace
            pm = self.pm
            qp, np_, nc, shift = pm._geom(state.q32, state.S, self._lattice(state))
            work, ws = pm._paint_work(np_)
            _lib.call('fpm_kick_drift_bin', _lib.ptr(state.P), _lib.ptr(state.P_c), _lib.ptr(state.S),
                      _lib.ptr(state.S_c), _lib.ptr(state.F), np_, fk[0], fk[1], len(kicks), fd,
                      pm.n, pm.L, qp, nc, shift, _lib.FPM_WINDOW[pm.resampler], _lib.ptr(work), ws,
                      _lib.stream_ptr())
            self._counted = (id(state), state.S.data_ptr())
        else:
            _lib.call('fpm_kick_drift', _lib.ptr(state.P), _lib.ptr(state.P_c), _lib.ptr(state.S),
                      _lib.ptr(state.S_c), _lib.ptr(state.F), state.P.numel(), fk[0], fk[1],
                      len(kicks), fd, _lib.stream_ptr())
        state.a['S'] = af

    def _lattice(self, state):
        """Lattice on the force mesh: same (nc, shift); B = n_force / nc."""
        return state.lattice

    def prepare_force(self, state, smoothing):
        """rho = paint(X) / nbar, here kept unnormalised; nbar folded into the FFT."""
        pm = self.pm
        rho = pm._scratch('rho', pm.n ** 3 * 4).view(torch.float32).view(pm.n, pm.n, pm.n)
        self._bins = None
        if self.sorted_paint:
            counted = self._counted == (id(state), state.S.data_ptr())
            self._counted = None
            self._bins = pm._paint_sorted(rho, q=state.q32, disp=state.S, lattice=self._lattice(state),
                                          counted=counted)
        else:
            rho.zero_()
            pm._paint(rho, q=state.q32, disp=state.S, lattice=self._lattice(state))
        return rho

    def _packed_force_mesh(self, rho, nbar, packed, delta_k, work, ws_bytes, blocked, ac):
        """r2c, Poisson + gradient transfer, force mesh (core.py:205-207,
        force/gravity.py:10-29) into the packed float4 mesh; subclasses that
        act on delta_k first override this."""
        pm = self.pm
        _lib.call('fpm_force_mesh_blocked' if blocked else 'fpm_force_mesh_packed', _lib.ptr(rho), pm.n,
                  pm.L, 1.0 / nbar, 1.5 * self.cosmology.Om0, _lib.ptr(packed),
                  _lib.ptr(delta_k.data) if delta_k is not None else None,
                  _lib.ptr(work), ws_bytes, _lib.stream_ptr())

    def Force(self, state, ai, ac, af):
        assert ac == state.a['S']
        pm = self.pm
        n = pm.n
        nbar = 1.0 * state.csize / float(n) ** 3
        rho = self.prepare_force(state, smoothing=None)
        ws_bytes = _lib.query('fpm_force_workspace', n)
        work = pm._scratch('force_ws', ws_bytes)
        delta_k = ComplexField(pm, empty=True) if self.want_event else None
        if self.fused_readout and self._bins is not None:
            # forces at the particles straight from the potential (no force mesh)
            qp, np_, nc, shift = pm._geom(state.q32, state.S, self._lattice(state))
            bins = self._bins
            _lib.call('fpm_force_readout_sorted', _lib.ptr(rho), n, pm.L, 1.0 / nbar,
                      1.5 * self.cosmology.Om0,
                      _lib.ptr(delta_k.data) if delta_k is not None else None,
                      _lib.ptr(work), ws_bytes, _lib.ptr(state.S), qp, np_, nc, shift,
                      _lib.FPM_WINDOW[pm.resampler], _lib.ptr(state.F), _lib.ptr(state.RHO),
                      bins['brick'], _lib.ptr(bins['work']), bins['bytes'], _lib.stream_ptr())
            state.a['F'] = af
            return dict(delta_k=delta_k)
        if self.packed_force:
            # one float4 mesh {F_x, F_y, F_z, rho / nbar}: the readout gathers
            # 16 bytes per window cell instead of four scattered floats
            packed = pm._scratch('force_packed', 4 * n ** 3 * 4)
            bins = self._bins if self.brick_readout else None
            blocked = bins is not None and self.blocked_force
            self._packed_force_mesh(rho, nbar, packed, delta_k, work, ws_bytes, blocked, ac)
            qp, np_, nc, shift = pm._geom(state.q32, state.S, self._lattice(state))
            if blocked:
                _lib.call('fpm_readout_blocked_sorted', _lib.ptr(packed), n, pm.L, _lib.ptr(state.S),
                          qp, np_, nc, shift, _lib.FPM_WINDOW[pm.resampler], _lib.ptr(state.F),
                          _lib.ptr(state.RHO), bins['brick'], _lib.ptr(bins['work']), bins['bytes'],
                          _lib.stream_ptr())
            elif bins is not None:
                # in mesh-brick order, from the paint's particle lists
                _lib.call('fpm_readout_packed_sorted', _lib.ptr(packed), n, pm.L, _lib.ptr(state.S),
                          qp, np_, nc, shift, _lib.FPM_WINDOW[pm.resampler], _lib.ptr(state.F),
                          _lib.ptr(state.RHO), bins['brick'], _lib.ptr(bins['work']), bins['bytes'],
                          _lib.stream_ptr())
            else:
                _lib.call('fpm_readout_packed', _lib.ptr(packed), n, pm.L, _lib.ptr(state.S), qp, np_,
                          nc, shift, _lib.FPM_WINDOW[pm.resampler], _lib.ptr(state.F),
                          _lib.ptr(state.RHO), _lib.stream_ptr())
            state.a['F'] = af
            return dict(delta_k=delta_k)
        fmesh = pm._scratch('force_mesh', 3 * n ** 3 * 4).view(torch.float32).view(3, n, n, n)
        _lib.call('fpm_force_mesh', _lib.ptr(rho), n, pm.L, 1.0 / nbar, 1.5 * self.cosmology.Om0,
                  _lib.ptr(fmesh[0]), _lib.ptr(fmesh[1]), _lib.ptr(fmesh[2]),
                  _lib.ptr(delta_k.data) if delta_k is not None else None,
                  _lib.ptr(work), ws_bytes, _lib.stream_ptr())
        F = state.F
        pm._readout([fmesh[0], fmesh[1], fmesh[2], rho],
                    [F[:, 0], F[:, 1], F[:, 2], state.RHO], [3, 3, 3, 1],
                    [1.0, 1.0, 1.0, 1.0 / nbar],
                    q=state.q32, disp=state.S, lattice=self._lattice(state))
        state.a['F'] = af
        return dict(delta_k=delta_k)


def autostages(knots, N, astart=None, N0=None):
    """fastpm/core.py:212-259: N stages including every knot."""
    knots = numpy.array(knots, dtype='f8')
    knots.sort()
    stages = numpy.array([], dtype='f8')
    if astart is not None and astart != knots.min():
        assert astart < knots.min()
        if N0 is None:
            N0 = 1
        knots = numpy.append([astart], knots)
    else:
        N0 = 1
    for i in range(0, len(knots) - 1):
        da = (knots[-1] - knots[i]) / (N - len(stages) - 1)
        n_span = int((knots[i + 1] - knots[i]) / da + 0.5)
        if i == 0 and n_span < N0:
            n_span = N0
        stages = numpy.append(stages, numpy.linspace(knots[i], knots[i + 1], n_span, endpoint=False))
    return numpy.append(stages, [knots[-1]])


def leapfrog(stages):
    """fastpm/core.py:261-288: F at the first stage, then K D F K per interval."""
    if len(stages) == 0:
        return
    ai = stages[0]
    yield 'F', ai, ai, ai
    x, p, f = ai, ai, ai
    for i in range(len(stages) - 1):
        a0 = stages[i]
        a1 = stages[i + 1]
        ah = (a0 * a1) ** 0.5
        yield 'K', p, f, ah
        p = ah
        yield 'D', x, p, a1
        x = a1
        yield 'F', f, x, a1
        f = a1
        yield 'K', p, f, a1
        p = a1


def leapfrog_with_lpt(stages):
    """fastpm/core.py:290-317: as leapfrog, without the first force."""
    if len(stages) == 0:
        return
    ai = stages[0]
    x, p, f = ai, ai, ai
    for i in range(len(stages) - 1):
        a0 = stages[i]
        a1 = stages[i + 1]
        ah = (a0 * a1) ** 0.5
        yield 'K', p, f, ah
        p = ah
        yield 'D', x, p, a1
        x = a1
        yield 'F', f, x, a1
        f = a1
        yield 'K', p, f, a1
        p = a1
