"""Continuous-batching serving of many small FastPM simulations on one GPU.

Each request is one reference-style run: whitenoise(seed) -> linear(P(k) of its
own cosmology) -> 2LPT at a0 -> leapfrog KDK to a = 1 (fastpm/core.py:113-210),
ending with the P(k) of its final density (fastpm/utils.py:77 estimator).

GB300 design:
  * requests are grouped by shape class (Nc, B): a class owns slot pools
    [slot][...] for particles, meshes and FFT workspace, sized at start-up from
    an HBM budget (admission = a free slot of the request's class);
  * one engine round advances every active slot of every class by one action
    group: the kick(s)/drift of its own schedule (per-slot factors) then a force,
    as ONE batched launch per kernel (fpm_*_batch: grid dimension = slot), each
    class on its own CUDA stream so small classes overlap;
  * with use_graphs, a class's round (KD, paint, 5 FFT passes, readout) is a
    captured CUDA graph replayed with per-slot parameters refreshed by one small
    host-to-device copy;
  * requests that arrive while others run are admitted as soon as a slot frees
    up (continuous batching); results leave the device as P(k) shells.

The host computes each request's kick/drift factors once at admission from a
single MatterDominated solve over all its stage times (background.py), instead
of one ODE solve per action as core.py does; the factors agree to ~1e-9
relative, far inside the float32 state.
"""
import ctypes
import heapq
import math
import time

import numpy
import torch

from . import _lib, autotune
from .background import MatterDominated
from .core import Solver, leapfrog
from .cosmology import Cosmology, EHPower
from .pm import ParticleMesh
from .power import power


class Request(object):
    """One simulation request (a configuration of the serving stream)."""

    def __init__(self, rid, nc, B, Om0, sigma8, nsteps, arrival=0.0, seed=None, box=None,
                 a0=0.1, a1=1.0, resampler='cic'):
        self.rid = int(rid)
        self.nc = int(nc)
        self.B = int(B)
        self.box = float(box) if box is not None else 4.0 * nc
        self.Om0 = float(Om0)
        self.sigma8 = float(sigma8)
        self.nsteps = int(nsteps)
        self.arrival = float(arrival)
        self.seed = int(rid if seed is None else seed)
        self.a0, self.a1 = float(a0), float(a1)
        self.resampler = resampler
        # filled by the engine
        self.admitted = None
        self.done = None
        self.k = None
        self.pk = None
        self.X = None
        # 'pending' -> 'done', or 'rejected' (no shape class / not admissible),
        # 'failed' (an exception while preparing or collecting it), 'cancelled'
        self.status = 'pending'
        self.error = None

    @property
    def key(self):
        return (self.nc, self.B, self.box, self.resampler)

    @property
    def stages(self):
        return numpy.linspace(self.a0, self.a1, self.nsteps + 1)

    def cosmology(self):
        return Cosmology(Om0=self.Om0, sigma8=self.sigma8)

    @property
    def latency(self):
        return None if self.done is None else self.done - self.arrival


def schedule_factors(Om0, stages, a_normalize=1.0, with_growth=False):
    """Kick / drift factors of leapfrog(stages) from one growth solve.

    Returns (k1, d, k2) arrays over the intervals: the first half kick
    (a_i -> sqrt(a_i a_{i+1}), force at a_i), the drift (a_i -> a_{i+1}, momentum
    at the half step) and the second half kick (force at a_{i+1}); the formulas
    of fastpm/core.py:170-171 and 177-178.  with_growth: also the solved
    MatterDominated, whose grid holds every stage (the initial conditions at
    stages[0] take their growth factors from it).
    """
    st = numpy.asarray(stages, dtype='f8')
    ah = numpy.sqrt(st[:-1] * st[1:])
    pt = MatterDominated(Om0, a=numpy.concatenate([st, ah]), a_normalize=a_normalize)
    E, Gf, gf, Gp, gp = pt.E, pt.Gf, pt.gf, pt.Gp, pt.gp
    a0, a1 = st[:-1], st[1:]
    k1 = 1 / (a0 ** 2 * E(a0)) * (Gf(ah) - Gf(a0)) / gf(a0)
    d = 1 / (ah ** 3 * E(ah)) * (Gp(a1) - Gp(a0)) / gp(ah)
    k2 = 1 / (a1 ** 2 * E(a1)) * (Gf(a1) - Gf(ah)) / gf(a1)
    if with_growth:
        return k1, d, k2, pt
    return k1, d, k2


class _KD(ctypes.Structure):
    _fields_ = [('fk1', ctypes.c_float), ('fk2', ctypes.c_float), ('fd', ctypes.c_float),
                ('nkick', ctypes.c_int), ('drift', ctypes.c_int)]


def class_slot_bytes(nc, B):
    """Device bytes one slot of shape (nc, B) needs (admission accounting)."""
    n = nc * B
    np_ = nc ** 3
    zp = _lib.query('fpm_complex_row', n)
    particles = np_ * (3 * 4 * 3 + 3 * 2 * 2 + 4)  # S P F, S_c P_c (bfloat16), RHO
    meshes = 5 * n ** 3 * 4                     # rho + force pool (3 meshes or packed float4)
    work = 3 * n * n * zp * 8                   # complex FFT workspace
    sort = 10 * np_ * 4 + 5 * 4 * (n // 4) ** 3  # sorted-paint particle ids, keys, ranks, brick counters
    return particles + meshes + work + sort


DEFAULT_VARIANT = dict(paint='sorted', paint_brick=0, tile_el=0, force='packed')


class ShapeClass(object):
    """Slot pools and the batched round of one (nc, B, box, window) shape."""

    def __init__(self, key, nslots, device, use_graphs=False, variant=None):
        nc, B, box, res = key
        self.key = key
        self.nc, self.B, self.box, self.res = nc, B, box, res
        self.n = n = nc * B
        self.np = nc ** 3
        self.S = nslots
        self.device = device
        self.stream = torch.cuda.Stream(device=device)
        self.pm = ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, resampler=res, device=device)
        z = lambda *s: torch.zeros(*s, dtype=torch.float32, device=device)
        S = nslots
        self.Sd, self.P, self.F = z(S, self.np, 3), z(S, self.np, 3), z(S, self.np, 3)
        # Kahan compensation terms, bfloat16 (the kernels' storage format)
        self.Sc = torch.zeros(S, self.np, 3, dtype=torch.bfloat16, device=device)
        self.Pc = torch.zeros(S, self.np, 3, dtype=torch.bfloat16, device=device)
        self.RHO = z(S, self.np)
        self.rho = z(S, n, n, n)
        # force pool: three meshes [3][slot][n^3] or one packed [slot][n^3] float4
        self.fpool = z(4 * S * n ** 3)
        self.fmesh = self.fpool[:3 * S * n ** 3].view(3, S, n, n, n)
        self.packed = self.fpool.view(S, n ** 3, 4)
        self.work_bytes = _lib.query('fpm_force_batch_workspace', n, S)
        # zeroed: the packed batch force keeps a time-out status word in it
        self.work = torch.zeros(self.work_bytes, dtype=torch.uint8, device=device)
        zp = _lib.query('fpm_complex_row', n)
        self.force_status_at = 2 * S * n * n * zp * 8 if n >= 512 else None
        # sorted-paint workspace: enough for the smallest brick (the most bricks)
        with autotune.options(paint_brick=4 if n % 4 == 0 else 0):
            self.pwork_bytes = _lib.query('fpm_paint_sorted_batch_workspace', n, self.np, S)
        self.pwork = torch.empty(max(self.pwork_bytes, 256), dtype=torch.uint8, device=device)
        self.variant = dict(DEFAULT_VARIANT, **(variant or {}))
        self.tune_timings = None
        # per-slot parameters: device copies and a ring of pinned host staging
        # buffers (a buffer is rewritten only after its copy has completed)
        self.ring = [dict(kd=torch.zeros(S * 5, dtype=torch.int32).pin_memory(),
                          act=torch.zeros(S, dtype=torch.int32).pin_memory(),
                          fac=torch.zeros(S, dtype=torch.float32).pin_memory(),
                          ev=None) for _ in range(3)]
        self.ring_i = 0
        self.inflight = []          # events of enqueued rounds
        self.d_active_f = torch.zeros(S, dtype=torch.int32, device=device)
        self.d_factor = torch.zeros(S, dtype=torch.float32, device=device)
        self.d_kd = torch.zeros(S * 5, dtype=torch.int32, device=device)
        self.slots = [None] * S     # request per slot
        self.phase = [None] * S     # ('init',) / ('step', i) / ('final',)
        self.sched = [None] * S
        self.use_graphs = use_graphs
        self.graph = None
        self.Q = None          # the lattice, shared by every request of the class
        self.served = []       # requests whose initial conditions ran since the last check_status

    # -- slot management -------------------------------------------------
    def free_slot(self):
        for s, r in enumerate(self.slots):
            if r is None:
                return s
        return None

    @property
    def busy(self):
        return any(r is not None for r in self.slots)

    def release(self, s):
        """Free slot s (a cancelled or failed request): the next round treats
        it as inactive; rounds already enqueued still compute it, on the
        class's stream, before any later admission writes the slot."""
        self.slots[s] = None
        self.phase[s] = None
        self.sched[s] = None

    def admit(self, req, s):
        """Initial conditions of req into slot s (single-simulation kernels)."""
        cosmo = req.cosmology()
        solver = Solver(self.pm, cosmo, B=self.B)
        if self.Q is None:
            self.Q = self.pm.generate_uniform_particle_grid(shift=0, dtype='f4')
        Q = self.Q
        dlin = solver.linear(solver.whitenoise(req.seed), EHPower(cosmo, 0))
        # one growth solve for the schedule and the initial conditions (its
        # grid holds a0); the LPT's time-out status word is read after the run
        # (check_status): reading it here would wait for the rounds queued on
        # the class stream
        k1, d, k2, pt = schedule_factors(req.Om0, req.stages, with_growth=True)
        st = solver._lpt(dlin, Q, a=req.a0, order=2, check=False, growth=pt)
        self.served.append(req)
        self.Sd[s].copy_(st.S)
        self.P[s].copy_(st.P)
        self.F[s].copy_(st.F)
        self.Sc[s].zero_()
        self.Pc[s].zero_()
        self.slots[s] = req
        self.phase[s] = ('init',)
        self.sched[s] = (k1, d, k2)

    def check_status(self):
        """After the class's stream has drained: requests served since the
        last check, and the error if a bounded wait timed out among them (the
        LPT of the initial conditions or the pipelined passes of the batched
        force, meshes of n >= 512), else None; the status words are cleared."""
        reqs, self.served = self.served, []
        why = []
        # the initial conditions run on the base mesh (nc^3), whose workspace
        # this is: its size and status word follow that mesh
        work = self.pm._bufs.get('lpt_ws')
        if work is not None and self.pm.n >= 512:
            rc = _lib.workspace_status(work, self.pm.n, 1, 1)
            if rc != 0:
                why.append('a bounded wait of the LPT timed out (status %d)' % rc)
        if self.force_status_at is not None and self.variant['force'] == 'packed':
            word = self.work[self.force_status_at:self.force_status_at + 4].view(torch.int32)
            if int(word.item()) != 0:
                word.zero_()
                why.append('a bounded wait of the batched force timed out')
        return reqs, ('; '.join(why) if why else None)

    # -- one round -------------------------------------------------------
    def _params(self):
        """Host-side per-slot parameters of this round; returns slots that finish."""
        kd = numpy.zeros((self.S, 5), dtype='i4')
        kdf = kd.view('f4')
        act = numpy.zeros(self.S, dtype='i4')
        fac = numpy.zeros(self.S, dtype='f4')
        finishing = []
        for s, r in enumerate(self.slots):
            if r is None:
                continue
            ph = self.phase[s]
            k1, d, k2 = self.sched[s]
            fac[s] = 1.5 * r.Om0
            if ph[0] == 'init':
                act[s] = 1                       # first force at a0
            elif ph[0] == 'step':
                i = ph[1]
                kicks = ([k2[i - 1]] if i > 0 else []) + [k1[i]]
                kdf[s, 0] = kicks[0]
                kdf[s, 1] = kicks[1] if len(kicks) > 1 else 0.0
                kdf[s, 2] = d[i]
                kd[s, 3] = len(kicks)
                kd[s, 4] = 1
                act[s] = 1                       # force at a_{i+1}
            else:                                # last half kick, no force
                kdf[s, 0] = k2[-1]
                kd[s, 3] = 1
                finishing.append(s)
        buf = self.ring[self.ring_i]
        self.ring_i = (self.ring_i + 1) % len(self.ring)
        if buf['ev'] is not None:
            buf['ev'].synchronize()
        buf['kd'].numpy()[:] = kd.ravel()
        buf['act'].numpy()[:] = act
        buf['fac'].numpy()[:] = fac
        return finishing, buf

    def _launch_round(self):
        v = self.variant
        with autotune.options(paint_brick=v.get('paint_brick'), tile_el=v.get('tile_el')):
            self._launch_round_variant(v)

    def _launch_round_variant(self, v):
        n, S, np_ = self.n, self.S, self.np
        sp = ctypes.c_void_p(self.stream.cuda_stream)
        act = _lib.ptr(self.d_active_f)
        _lib.call('fpm_kick_drift_batch', _lib.ptr(self.P), _lib.ptr(self.Pc), _lib.ptr(self.Sd),
                  _lib.ptr(self.Sc), _lib.ptr(self.F), 3 * np_, 3 * np_, _lib.ptr(self.d_kd), S, sp)
        win = _lib.FPM_WINDOW[self.res]
        nbar = 1.0 * np_ / float(n) ** 3
        if v['paint'] == 'sorted':
            _lib.call('fpm_paint_sorted_batch', _lib.ptr(self.rho), n ** 3, n, self.box, _lib.ptr(self.Sd),
                      3 * np_, np_, self.nc, 0.0, win, 1.0, S, act, _lib.ptr(self.pwork),
                      self.pwork.numel(), sp)
        else:
            self.rho.zero_()
            _lib.call('fpm_paint_batch', _lib.ptr(self.rho), n ** 3, n, self.box, _lib.ptr(self.Sd),
                      3 * np_, np_, self.nc, 0.0, win, 1.0, S, act, sp)
        if v['force'] == 'packed':
            _lib.call('fpm_force_mesh_batch_packed', _lib.ptr(self.rho), n ** 3, n, self.box, 1.0 / nbar,
                      _lib.ptr(self.d_factor), _lib.ptr(self.packed), n ** 3, _lib.ptr(self.work),
                      self.work_bytes, S, act, sp)
            _lib.call('fpm_readout_packed_batch', _lib.ptr(self.packed), n ** 3, n, self.box,
                      _lib.ptr(self.Sd), 3 * np_, np_, self.nc, 0.0, win, _lib.ptr(self.F), 3 * np_,
                      _lib.ptr(self.RHO), np_, S, act, sp)
            return
        _lib.call('fpm_force_mesh_batch', _lib.ptr(self.rho), n ** 3, n, self.box, 1.0 / nbar,
                  _lib.ptr(self.d_factor), _lib.ptr(self.fmesh[0]), _lib.ptr(self.fmesh[1]),
                  _lib.ptr(self.fmesh[2]), n ** 3, _lib.ptr(self.work), self.work_bytes, S, act, sp)
        m_arr, k1 = _lib.ptr_array([self.fmesh[0], self.fmesh[1], self.fmesh[2], self.rho])
        F = self.F
        o_arr, k2 = _lib.ptr_array([F[:, :, 0], F[:, :, 1], F[:, :, 2], self.RHO])
        strides = (ctypes.c_int * 4)(3, 3, 3, 1)
        # RHO's slot stride is np, F's is 3 np: read out F and RHO in two passes
        scales3 = (ctypes.c_float * 3)(1.0, 1.0, 1.0)
        _lib.call('fpm_readout_batch', m_arr, n ** 3, 3, n, self.box, _lib.ptr(self.Sd), 3 * np_, np_,
                  self.nc, 0.0, win, o_arr, strides, 3 * np_, scales3, S, act, sp)
        m1, k3 = _lib.ptr_array([self.rho])
        o1, k4 = _lib.ptr_array([self.RHO])
        _lib.call('fpm_readout_batch', m1, n ** 3, 1, n, self.box, _lib.ptr(self.Sd), 3 * np_, np_,
                  self.nc, 0.0, win, o1, (ctypes.c_int * 1)(1), np_, (ctypes.c_float * 1)(1.0 / nbar),
                  S, act, sp)

    def autotune(self, reps=3):
        """Pick this class's paint variant / brick and force variant by timing
        full batched rounds (every slot active, a synthetic displacement field
        of 0.3 cells rms); the pools are cleared afterwards."""
        key = autotune.cache_key('serving-round', (self.nc, self.B, self.box, self.res, self.S), self.device)
        hit = autotune.lookup(key)
        if hit is not None:
            self.variant = dict(DEFAULT_VARIANT, **hit['variant'])
            self.tune_timings = hit['timings']
            return self.variant
        g = torch.Generator(device=self.device).manual_seed(self.nc * 7 + self.B)
        with torch.cuda.stream(self.stream):
            self.Sd.copy_(torch.randn(self.Sd.shape, generator=g, device=self.device)
                          * (0.3 * self.box / self.n))
            self.d_kd.zero_()
            self.d_active_f.fill_(1)
            self.d_factor.fill_(0.45)

        def run(cand):
            self.variant = dict(DEFAULT_VARIANT, **cand)
            self._launch_round()

        best_paint, t1 = autotune.pick(autotune.paint_candidates(self.n, self.B),
                                       lambda c: run(dict(c, force='packed')), self.stream, reps)
        best_force, t2 = autotune.pick(autotune.force_candidates(),
                                       lambda c: run(dict(best_paint, **c)), self.stream, reps)
        self.variant = dict(DEFAULT_VARIANT, **best_paint)
        self.variant.update(best_force)
        self.tune_timings = dict(t1, **{'force:' + k: v for k, v in t2.items()})
        with torch.cuda.stream(self.stream):
            # the force workspace too: the three-mesh candidate's meshes cover the
            # packed force's time-out word
            for t in (self.Sd, self.P, self.F, self.Sc, self.Pc, self.RHO, self.rho, self.fpool, self.work):
                t.zero_()
            self.d_active_f.zero_()
        self.stream.synchronize()
        autotune.store(key, {'variant': {k: self.variant[k] for k in DEFAULT_VARIANT},
                             'timings': self.tune_timings})
        return self.variant

    def round(self, max_inflight=3):
        """Enqueue one action group for every active slot; returns the slots
        whose simulation this round completes."""
        if not self.busy:
            return []
        while len(self.inflight) >= max_inflight:
            self.inflight.pop(0).synchronize()
        finishing, buf = self._params()
        with torch.cuda.stream(self.stream):
            self.d_kd.copy_(buf['kd'], non_blocking=True)
            self.d_active_f.copy_(buf['act'], non_blocking=True)
            self.d_factor.copy_(buf['fac'], non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(self.stream)
            buf['ev'] = ev
            if self.use_graphs:
                if self.graph is None:
                    self._launch_round()          # first round un-captured (tables, attributes)
                    self.graph = torch.cuda.CUDAGraph()
                    self.stream.synchronize()
                    with torch.cuda.graph(self.graph, stream=self.stream):
                        self._launch_round()
                else:
                    self.graph.replay()
            else:
                self._launch_round()
            rev = torch.cuda.Event()
            rev.record(self.stream)
            self.inflight.append(rev)
        # advance the host-side phases
        for s, r in enumerate(self.slots):
            if r is None:
                continue
            ph = self.phase[s]
            if ph[0] == 'init':
                self.phase[s] = ('step', 0) if r.nsteps > 0 else ('final',)
            elif ph[0] == 'step':
                i = ph[1] + 1
                self.phase[s] = ('step', i) if i < r.nsteps else ('final',)
        return finishing

    def finish(self, s, keep_state=False):
        """Enqueue the P(k) of slot s's final density (device shell sums copied
        to pinned host memory) and free the slot; returns (request, event,
        host buffers) to collect once the event has completed."""
        r = self.slots[s]
        n = self.n
        with torch.cuda.stream(self.stream):
            sp = ctypes.c_void_p(self.stream.cuda_stream)
            mesh = self.rho[s]
            mesh.zero_()
            _lib.call('fpm_paint_batch', _lib.ptr(mesh), n ** 3, n, self.box, _lib.ptr(self.Sd[s]),
                      3 * self.np, self.np, self.nc, 0.0, _lib.FPM_WINDOW[self.res], 1.0, 1, None, sp)
            zp = _lib.query('fpm_complex_row', n)
            ck = torch.empty((n, n, zp, 2), dtype=torch.float32, device=self.device)
            _lib.call('fpm_r2c', _lib.ptr(mesh), _lib.ptr(ck), n, 1.0 / float(n) ** 3, sp)
            sums = torch.zeros((3, n // 2), dtype=torch.float64, device=self.device)
            _lib.call('fpm_power_accumulate', _lib.ptr(ck), None, n, self.box, _lib.ptr(sums[0]),
                      _lib.ptr(sums[1]), _lib.ptr(sums[2]), sp)
            h_sums = torch.empty((3, n // 2), dtype=torch.float64).pin_memory()
            h_k0 = torch.empty(2, dtype=torch.float32).pin_memory()
            h_sums.copy_(sums, non_blocking=True)
            h_k0.copy_(ck[0, 0, 0], non_blocking=True)
            r.X = self.Sd[s].clone() if keep_state else None
            ev = torch.cuda.Event()
            ev.record(self.stream)
        self.slots[s] = None
        self.phase[s] = None
        self.sched[s] = None
        return (r, ev, h_sums, h_k0, self.box)

    @staticmethod
    def collect(item):
        """k, P(k) of a finished request once its event has completed
        (fastpm/utils.py:77-164 normalisation by |f(0)|^2)."""
        r, ev, h_sums, h_k0, box = item
        ksum, psum, wsum = h_sums.numpy()
        z = float(abs(complex(float(h_k0[0]), float(h_k0[1]))))
        norm = z * z if z != 0 else 1.0
        with numpy.errstate(invalid='ignore', divide='ignore'):
            r.k = ksum / wsum
            r.pk = psum / norm / wsum * box ** 3
        return r


def check_request(r):
    """Reason a request cannot run on this engine at all, or None."""
    if r.nc < 1 or r.B < 1 or not _lib.query('fpm_fft_supported', r.nc * r.B) \
            or not _lib.query('fpm_fft_supported', r.nc):
        return 'unsupported shape: Nc = %d, B = %d (mesh sizes %s)' % (
            r.nc, r.B, '16 24 32 48 64 96 128 192 256 384 512 1024')
    if r.nsteps < 0 or not (0 < r.a0 < r.a1):
        return 'bad schedule: %d steps from a = %g to %g' % (r.nsteps, r.a0, r.a1)
    if not (0 < r.Om0 <= 1) or not (r.sigma8 > 0) or not (r.box > 0):
        return 'bad cosmology or box: Om0 = %g, sigma8 = %g, box = %g' % (r.Om0, r.sigma8, r.box)
    if r.resampler not in ('cic', 'tsc'):
        return 'bad resampler %r' % (r.resampler,)
    return None


class ServingEngine(object):
    """Continuous batching over shape classes with HBM-budget admission.

    Failures stay with the request that caused them: a request of a shape the
    engine has no class for, or whose class got no slot within the HBM
    budget, is rejected at arrival; an exception while admitting it (its
    P(k), growth factors or initial conditions) or collecting its result fails
    it; cancel(rid) withdraws it, freeing its slot at the next round.  The
    other requests run on unchanged (slots are independent: their results do
    not depend on which other slots are active)."""

    def __init__(self, classes, hbm_budget=None, max_slots=32, use_graphs=True, device='cuda',
                 keep_state=False, tune=True, variant=None, admit_budget_s=0.01):
        self.device = torch.device(device)
        free, total = torch.cuda.mem_get_info(self.device)
        budget = hbm_budget if hbm_budget is not None else 0.6 * free
        keys = sorted(set(classes))
        share = budget / max(len(keys), 1)
        self.classes = {}
        self.refused = {}   # key -> why the class has no slot
        for key in keys:
            nc, B = key[0], key[1]
            per = class_slot_bytes(nc, B)
            S = int(min(max_slots, share // per))
            if S < 1:
                self.refused[key] = ('admission refused: one slot of %dx%d needs %.3g GB, the HBM '
                                     'budget share is %.3g GB' % (nc, B, per / 1e9, share / 1e9))
                continue
            self.classes[key] = ShapeClass(key, S, self.device, use_graphs=use_graphs, variant=variant)
            if tune and variant is None:
                self.classes[key].autotune()
        self.keep_state = keep_state
        self.capacity = {k: c.S for k, c in self.classes.items()}
        self._cancel = set()
        # host seconds of admissions (initial conditions, growth solves) per
        # engine round: admitting a whole burst before the next round would
        # leave the GPU idle once the queued rounds have run
        self.admit_budget_s = admit_budget_s

    def cancel(self, rid):
        """Withdraw request rid: if it waits it is dropped, if it runs its
        slot is freed before the next round (work already enqueued for it
        completes on the device and is discarded)."""
        self._cancel.add(int(rid))

    def run(self, requests, realtime=True, on_round=None):
        """Serve requests (arrival times in seconds from start); returns them
        all, each with its final status (done / rejected / failed / cancelled).

        Nothing synchronises the whole device: each class runs at most three
        rounds ahead of the GPU, finished requests are collected by polling
        their events, so host bookkeeping, admissions and the GPU overlap.
        on_round(engine, i), if given, is called after engine round i (the
        tests use it to cancel requests mid-batch)."""
        pending = sorted(requests, key=lambda r: (r.arrival, r.rid))
        waiting = {k: [] for k in self.classes}
        done, collecting = [], []
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0

        def close(r, status, error=None):
            r.status, r.error, r.done = status, error, now()
            done.append(r)

        i = 0
        it = 0
        while len(done) < len(requests):
            t = now() if realtime else float('inf')
            while i < len(pending) and pending[i].arrival <= t:
                r = pending[i]
                i += 1
                why = check_request(r)
                if why is None and r.key not in self.classes:
                    why = self.refused.get(r.key, 'no shape class for Nc = %d, B = %d, box = %g, %s'
                                           % r.key)
                if why is not None:
                    close(r, 'rejected', why)
                else:
                    waiting[r.key].append(r)
            if self._cancel:
                for key, q in waiting.items():
                    for r in [r for r in q if r.rid in self._cancel]:
                        q.remove(r)
                        close(r, 'cancelled')
                for cls in self.classes.values():
                    for s, r in enumerate(cls.slots):
                        if r is not None and r.rid in self._cancel:
                            cls.release(s)
                            close(r, 'cancelled')
            # admissions: one request per class per pass, round robin; the
            # first pass always completes (every class with a free slot gets
            # one), later passes run until this round's host budget is spent
            ta = time.perf_counter()
            admitted_any = True
            first = True
            while admitted_any:
                admitted_any = False
                for key, q in waiting.items():
                    cls = self.classes[key]
                    if not q:
                        continue
                    s = cls.free_slot()
                    if s is None:
                        continue
                    r = q.pop(0)
                    admitted_any = True
                    try:
                        with torch.cuda.stream(cls.stream):
                            cls.admit(r, s)
                    except Exception as e:   # this request only: its slot stays free
                        cls.release(s)
                        close(r, 'failed', '%s: %s' % (type(e).__name__, e))
                        continue
                    r.admitted = now()
                    if not first and time.perf_counter() - ta > self.admit_budget_s:
                        break
                first = False
                if time.perf_counter() - ta > self.admit_budget_s:
                    break
            busy = [c for c in self.classes.values() if c.busy]
            for cls in busy:
                for s in cls.round():
                    collecting.append(cls.finish(s, keep_state=self.keep_state))
            if busy:
                if on_round is not None:
                    on_round(self, it)
                it += 1
            still = []
            for item in collecting:
                if item[1].query():
                    try:
                        r = ShapeClass.collect(item)
                    except Exception as e:
                        close(item[0], 'failed', '%s: %s' % (type(e).__name__, e))
                        continue
                    close(r, 'done')
                else:
                    still.append(item)
            collecting = still
            if not busy:
                if collecting:
                    collecting[0][1].synchronize()
                elif i < len(pending) and realtime:
                    time.sleep(max(0.0, min(pending[i].arrival - now(), 0.005)))
        torch.cuda.synchronize(self.device)
        for cls in self.classes.values():
            reqs, err = cls.check_status()
            if err is not None:
                for r in reqs:
                    if r.status == 'done':
                        r.status, r.error = 'failed', err
        return done


def run_plain(requests, realtime=True, keep_state=False, device='cuda'):
    """One request at a time through the single-simulation Solver (FIFO)."""
    out = []
    lattice = {}
    t0 = time.perf_counter()
    for r in sorted(requests, key=lambda r: (r.arrival, r.rid)):
        if realtime:
            wait = r.arrival - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
        cosmo = r.cosmology()
        if r.key not in lattice:
            pm = ParticleMesh(BoxSize=r.box, Nmesh=[r.nc] * 3, resampler=r.resampler, device=device)
            lattice[r.key] = (pm, pm.generate_uniform_particle_grid(shift=0, dtype='f4'))
        pm, Q = lattice[r.key]
        solver = Solver(pm, cosmo, B=r.B)
        dlin = solver.linear(solver.whitenoise(r.seed), EHPower(cosmo, 0))
        st = solver.lpt(dlin, Q, a=r.a0, order=2)
        st = solver.nbody(st, leapfrog(r.stages))
        from .pm import RealField
        mesh = RealField(solver.fpm)
        solver.fpm._paint(mesh.value, disp=st.S, lattice=st.lattice)
        r.k, r.pk = power(mesh)
        r.X = st.S.clone() if keep_state else None
        torch.cuda.synchronize()
        r.done = time.perf_counter() - t0
        out.append(r)
    return out


def make_stream(nreq, rate, seed=0, nc_choices=(64, 96, 128, 192, 256), B_choices=(1, 2),
                steps=(5, 20)):
    """The serving workload: Poisson arrivals at `rate` per second, per request
    Nc in nc_choices, B in B_choices, box 4 Nc, Om0 ~ U[0.25, 0.35],
    sigma8 ~ U[0.70, 0.90], seed = request id, 5-20 KDK steps from a = 0.1."""
    rng = numpy.random.RandomState(seed)
    t = numpy.cumsum(rng.exponential(1.0 / rate, size=nreq))
    reqs = []
    for i in range(nreq):
        reqs.append(Request(i, nc=int(rng.choice(nc_choices)), B=int(rng.choice(B_choices)),
                            Om0=rng.uniform(0.25, 0.35), sigma8=rng.uniform(0.70, 0.90),
                            nsteps=int(rng.randint(steps[0], steps[1] + 1)), arrival=float(t[i])))
    return reqs


def summarize(done):
    """Throughput and latency of the completed requests (status 'done'; the
    plain path's requests count as done)."""
    ok = [r for r in done if r.status in ('done', 'pending')]
    lat = numpy.array([r.latency for r in ok])
    first = min(r.arrival for r in ok)
    last = max(r.done for r in ok)
    return {'completed': len(ok), 'sims_per_s': len(ok) / (last - first),
            'p50_s': float(numpy.percentile(lat, 50)), 'p99_s': float(numpy.percentile(lat, 99)),
            'makespan_s': last - first}
