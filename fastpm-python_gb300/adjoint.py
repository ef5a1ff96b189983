"""Differentiable FastPM forward model with hand-written adjoint kernels.

Forward model (fastpm/core.py:113-210 with a loss on top):
    d   = T(k) wn                        T = sqrt(P(k; Om0) / V)     (core.py:116-118)
    psi1 = lpt1(d),  psi2 = lpt1(lpt2source(d))                      (force/lpt.py)
    S0 = D1 psi1 + D2 psi2,  P0 = A1 psi1 + A2 psi2                  (core.py:128-135)
    leapfrog(stages): F, then K D F K per interval                   (core.py:261-288)
    L  = sum_cells (rho(X_final) / nbar - target)^2,  rho = CIC paint of X = Q + S

Reverse mode, written out (lambda_Y = dL/dY):
    loss:   lambda_S += readout_vjp(2 (rho / nbar - target) / nbar)          (CIC weight derivative)
    K  (P += fk F):  lambda_F += fk lambda_P;   dL/dfk = <lambda_P, F>
    D  (S += fd P):  lambda_P += fd lambda_S;   dL/dfd = <lambda_S, P>
    F  (F_d = readout(phi_d), phi_d = factor/nbar G_d rho, G_d = c2r (i a_d / k^2) r2c):
        lambda_S += readout_vjp(phi_d; weights lambda_F_d)                  (moving the window)
                  + readout_vjp(nu; factor / nbar),  nu = -sum_d G_d paint(lambda_F_d)
                  (G_d is antisymmetric: its transpose is -G_d)
        dL/dfactor = <lambda_F, F> / factor,  then lambda_F = 0
    LPT (Q fixed): g_d = -sum_d K_d FFT(paint_Q(lambda_psi1_d))        K_d = i a_d / k^2
                   g_s = -sum_d K_d FFT(paint_Q(lambda_psi2_d)),  lambda_s = c2r(g_s) / N^3
                   lambda_phi_ii = 3/7 lambda_s (phi_jj + phi_kk), lambda_phi_ij = -6/7 lambda_s phi_ij
                   g_d += sum_ij K_ij FFT(lambda_phi_ij),  K_ij = (i a_i)(i a_j) / k^2
    linear: g_wn = T g_d;   dL/dOm0 collects <.,.> contractions times the float64
    host derivatives of every Om0-dependent scalar (kick / drift factors, D1, D2,
    A1, A2, 1.5 Om0, T(k)).
Half-complex gradients g satisfy dL = sum_half w Re(conj(g) dmode), w = 1 on the
l = 0 and l = n/2 planes and 2 elsewhere (the real field's Hermitian weighting,
fastpm/operators.py:94-96); the torch wrapper returns w g as the Euclidean
gradient of the float32 mode array.

Positions for the reverse pass are recomputed from checkpoints of (S, P, F and
their Kahan terms) taken every `checkpoint_every` steps (default 4).
"""
import ctypes

import numpy
import torch

from . import _lib
from .background import MatterDominated, kick_factor, drift_factor
from .cosmology import Cosmology, EHPower
from .pm import ParticleMesh, ComplexField, RealField
from .force import lpt1, lpt2source


def _cls_ptrs(ts):
    arr, keep = _lib.ptr_array(ts)
    return arr, keep


class ForwardModel(object):
    """wn (whitenoise modes on the base mesh) and Om0 -> loss, with adjoints."""

    def __init__(self, nc, B, box, stages, sigma8=0.8159, target=None, checkpoint_every=4,
                 resampler='cic', device='cuda', dOm=1e-5):
        self.nc, self.B, self.box = int(nc), int(B), float(box)
        self.n = self.nc * self.B
        self.stages = numpy.asarray(stages, dtype='f8')
        self.sigma8 = float(sigma8)
        self.ck = int(checkpoint_every)
        self.res = resampler
        self.device = torch.device(device)
        self.pm = ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, resampler='cic', device=device)
        self.fpm = ParticleMesh(BoxSize=box, Nmesh=[self.n] * 3, resampler=resampler, device=device)
        self.np = self.nc ** 3
        self.nbar = self.np / float(self.n) ** 3
        self.target = target      # float32 [n, n, n] device tensor of rho / nbar, or None (zero)
        self.dOm = dOm
        self.lattice = (self.nc, 0.0)

    # -- host scalars ----------------------------------------------------------
    def _table(self, Om0):
        n, L = self.nc, self.box
        q = numpy.arange(3 * (n // 2) ** 2 + 1, dtype='f8')
        k = numpy.sqrt(q) * (2 * numpy.pi / L)
        P = EHPower(Cosmology(Om0=Om0, sigma8=self.sigma8), 0)(k)
        return P ** 0.5 / L ** 1.5

    def _lpt_coefs(self, Om0):
        a = self.stages[0]
        pt = MatterDominated(Om0, a=[a], a_normalize=1.0)
        D1, D2 = float(pt.D1(a)), float(pt.D2(a))
        A1 = a ** 2 * float(pt.f1(a)) * float(pt.E(a)) * D1
        A2 = a ** 2 * float(pt.f2(a)) * float(pt.E(a)) * D2
        return numpy.array([D1, D2, A1, A2])

    def _actions(self):
        st = self.stages
        acts = [('F', st[0], st[0], st[0])]
        for i in range(len(st) - 1):
            a0, a1 = st[i], st[i + 1]
            ah = (a0 * a1) ** 0.5
            acts += [('K', a0, a0, ah), ('D', a0, ah, a1), ('F', a0, a1, a1), ('K', ah, a1, a1)]
        return acts

    def _factor(self, Om0, act):
        t, ai, ac, af = act
        if t == 'K':
            return kick_factor(Om0, ai, ac, af)
        if t == 'D':
            return drift_factor(Om0, ai, ac, af)
        return 1.5 * Om0

    # -- device helpers -------------------------------------------------------
    def _force(self, S, F, want_meshes=False):
        pm, n = self.fpm, self.n
        rho = torch.zeros((n, n, n), dtype=torch.float32, device=self.device)
        pm._paint(rho, disp=S, lattice=self.lattice)
        ws = _lib.query('fpm_force_workspace', n)
        work = pm._scratch('force_ws', ws)
        fm = torch.empty((3, n, n, n), dtype=torch.float32, device=self.device)
        _lib.call('fpm_force_mesh', _lib.ptr(rho), n, pm.L, 1.0 / self.nbar, 1.5 * self.Om0,
                  _lib.ptr(fm[0]), _lib.ptr(fm[1]), _lib.ptr(fm[2]), None, _lib.ptr(work), ws,
                  _lib.stream_ptr())
        pm._readout([fm[0], fm[1], fm[2]], [F[:, 0], F[:, 1], F[:, 2]], [3, 3, 3], [1.0, 1.0, 1.0],
                    disp=S, lattice=self.lattice)
        return fm if want_meshes else None

    def _run(self, state, acts, fac, record=False):
        """Apply actions to state = dict(S, Sc, P, Pc, F); optionally record pre-action copies."""
        rec = []
        for act, f in zip(acts, fac):
            t = act[0]
            if record:
                rec.append({k: state[k].clone() for k in ('S', 'P', 'F')})
            if t == 'K':
                _lib.call('fpm_kick', _lib.ptr(state['P']), _lib.ptr(state['Pc']), _lib.ptr(state['F']),
                          state['P'].numel(), f, _lib.stream_ptr())
            elif t == 'D':
                _lib.call('fpm_drift', _lib.ptr(state['S']), _lib.ptr(state['Sc']), _lib.ptr(state['P']),
                          state['S'].numel(), f, _lib.stream_ptr())
            else:
                fm = self._force(state['S'], state['F'], want_meshes=record)
                if record:
                    rec[-1]['meshes'] = fm
                    rec[-1]['Fout'] = state['F'].clone()
        return rec

    def _final_density(self, S):
        n = self.n
        rho = torch.zeros((n, n, n), dtype=torch.float32, device=self.device)
        self.fpm._paint(rho, disp=S, lattice=self.lattice, resampler='cic')
        return rho / self.nbar

    # -- forward ----------------------------------------------------------------
    def forward(self, wn, Om0):
        """Loss at whitenoise wn (ComplexField on the base mesh) and Om0; keeps checkpoints."""
        self.Om0 = float(Om0)
        self.wn = wn
        pm = self.pm
        T = self._table(self.Om0)
        self.T = torch.from_numpy(T.astype('f4')).to(self.device)
        d = wn.copy()
        _lib.call('fpm_apply_isotropic', _lib.ptr(d.data), pm.n, _lib.ptr(self.T), len(T), _lib.stream_ptr())
        self.d = d

        class _St(object):
            pass
        st = _St()
        st.csize, st.lattice, st.q32 = self.np, (self.nc, 0.0), None
        self.psi1 = lpt1(d, st)
        self.psi2 = lpt1(lpt2source(d), st)
        D1, D2, A1, A2 = self.coefs = self._lpt_coefs(self.Om0)
        z = lambda: torch.zeros((self.np, 3), dtype=torch.float32, device=self.device)
        zc = lambda: torch.zeros((self.np, 3), dtype=torch.bfloat16, device=self.device)
        state = dict(S=D1 * self.psi1 + D2 * self.psi2, P=A1 * self.psi1 + A2 * self.psi2, F=z(),
                     Sc=zc(), Pc=zc())
        self.acts = self._actions()
        self.fac = [self._factor(self.Om0, a) for a in self.acts]
        # checkpoints at action indices 0, 1 + 4 ck, 1 + 8 ck, ... (step boundaries)
        bounds = [0] + list(range(1, len(self.acts), 4 * self.ck)) + [len(self.acts)]
        bounds = sorted(set(bounds))
        self.segments = list(zip(bounds[:-1], bounds[1:]))
        self.ckpt = []
        for a, b in self.segments:
            self.ckpt.append({k: v.clone() for k, v in state.items()})
            self._run(state, self.acts[a:b], self.fac[a:b])
        self.S_final = state['S']
        rho = self._final_density(state['S'])
        tgt = self.target if self.target is not None else torch.zeros_like(rho)
        self.resid = rho - tgt
        return float((self.resid.double() ** 2).sum())

    # -- reverse ------------------------------------------------------------------
    def _dot(self, x, y):
        return float((x.double() * y.double()).sum())

    def _vjp_force(self, S, lamF, meshes, Fout, lamS):
        pm, n = self.fpm, self.n
        win = self.res
        # term 1: the window moves with the particle
        w_arr, k1 = _cls_ptrs([lamF[:, 0], lamF[:, 1], lamF[:, 2]])
        m_arr, k2 = _cls_ptrs([meshes[0], meshes[1], meshes[2]])
        _lib.call('fpm_readout_vjp', m_arr, 3, n, pm.L, _lib.ptr(S), None, self.np, self.nc, 0.0,
                  _lib.FPM_WINDOW[win], w_arr, (ctypes.c_int * 3)(3, 3, 3),
                  (ctypes.c_float * 3)(1.0, 1.0, 1.0), _lib.ptr(lamS), 1, _lib.stream_ptr())
        # term 2: the density moves with the particle
        mu = torch.zeros((3, n, n, n), dtype=torch.float32, device=self.device)
        mp, k3 = _cls_ptrs([mu[0], mu[1], mu[2]])
        vp, k4 = _cls_ptrs([lamF[:, 0], lamF[:, 1], lamF[:, 2]])
        _lib.call('fpm_paint_values', mp, 3, n, pm.L, _lib.ptr(S), None, self.np, self.nc, 0.0,
                  _lib.FPM_WINDOW[win], vp, (ctypes.c_int * 3)(3, 3, 3), 1.0, _lib.stream_ptr())
        mk = [RealField(pm, mu[d]).r2c() for d in range(3)]
        nuk = ComplexField(pm, empty=True)
        ip, k5 = _cls_ptrs([c.data for c in mk])
        _lib.call('fpm_kspace_combine', ip, 3, (ctypes.c_int * 9)(1, 0, 0, 0, 1, 0, 0, 0, 1),
                  (ctypes.c_int * 3)(1, 1, 1), _lib.ptr(nuk.data), n, pm.L, -1.0, _lib.stream_ptr())
        nu = nuk.c2r()
        factor = 1.5 * self.Om0
        m1, k6 = _cls_ptrs([nu.value])
        _lib.call('fpm_readout_vjp', m1, 1, n, pm.L, _lib.ptr(S), None, self.np, self.nc, 0.0,
                  _lib.FPM_WINDOW[win], None, None, (ctypes.c_float * 1)(factor / self.nbar),
                  _lib.ptr(lamS), 1, _lib.stream_ptr())
        return self._dot(lamF, Fout) / factor

    def _lpt1_T(self, lam):
        """g = -sum_d K_d FFT(paint_Q(lam[:, d])) on the base mesh (lpt1 transpose)."""
        pm, nc = self.pm, self.nc
        mu = torch.zeros((3, nc, nc, nc), dtype=torch.float32, device=self.device)
        mp, k1 = _cls_ptrs([mu[0], mu[1], mu[2]])
        vp, k2 = _cls_ptrs([lam[:, 0], lam[:, 1], lam[:, 2]])
        _lib.call('fpm_paint_values', mp, 3, nc, pm.L, None, None, self.np, self.nc, 0.0,
                  _lib.FPM_WINDOW['cic'], vp, (ctypes.c_int * 3)(3, 3, 3), 1.0, _lib.stream_ptr())
        fk = []
        for d in range(3):
            c = ComplexField(pm, empty=True)
            _lib.call('fpm_r2c', _lib.ptr(mu[d]), _lib.ptr(c.data), nc, 1.0, _lib.stream_ptr())
            fk.append(c)
        g = ComplexField(pm, empty=True)
        ip, k3 = _cls_ptrs([c.data for c in fk])
        _lib.call('fpm_kspace_combine', ip, 3, (ctypes.c_int * 9)(1, 0, 0, 0, 1, 0, 0, 0, 1),
                  (ctypes.c_int * 3)(1, 1, 1), _lib.ptr(g.data), nc, pm.L, -1.0, _lib.stream_ptr())
        return g

    def _combine(self, fields, powers, scale):
        g = ComplexField(self.pm, empty=True)
        ip, k = _cls_ptrs([f.data for f in fields])
        pw = (ctypes.c_int * (3 * len(fields)))(*[x for p in powers for x in p])
        _lib.call('fpm_kspace_combine', ip, len(fields), pw, (ctypes.c_int * len(fields))(*([1] * len(fields))),
                  _lib.ptr(g.data), self.pm.n, self.pm.L, scale, _lib.stream_ptr())
        return g

    def backward(self):
        """(g_wn: ComplexField on the base mesh, dL/dOm0)."""
        n, pm, fpm = self.n, self.pm, self.fpm
        dev = self.device
        lamS = torch.zeros((self.np, 3), dtype=torch.float32, device=dev)
        lamP = torch.zeros_like(lamS)
        lamF = torch.zeros_like(lamS)
        # loss -> final positions (CIC)
        lr = (2.0 / self.nbar) * self.resid
        m1, k1 = _cls_ptrs([lr])
        _lib.call('fpm_readout_vjp', m1, 1, n, fpm.L, _lib.ptr(self.S_final), None, self.np, self.nc,
                  0.0, _lib.FPM_WINDOW['cic'], None, None, (ctypes.c_float * 1)(1.0), _lib.ptr(lamS), 1,
                  _lib.stream_ptr())
        dfac = numpy.zeros(len(self.acts))       # dL/d(factor of action)
        for si in reversed(range(len(self.segments))):
            a, b = self.segments[si]
            state = {k: v.clone() for k, v in self.ckpt[si].items()}
            rec = self._run(state, self.acts[a:b], self.fac[a:b], record=True)
            for j in reversed(range(b - a)):
                act, f, r = self.acts[a + j], self.fac[a + j], rec[j]
                if act[0] == 'K':
                    dfac[a + j] = self._dot(lamP, r['F'])
                    lamF += f * lamP
                elif act[0] == 'D':
                    dfac[a + j] = self._dot(lamS, r['P'])
                    lamP += f * lamS
                else:
                    dfac[a + j] = self._vjp_force(r['S'], lamF, r['meshes'], r['Fout'], lamS)
                    lamF.zero_()
        D1, D2, A1, A2 = self.coefs
        # LPT
        lam1 = D1 * lamS + A1 * lamP
        lam2 = D2 * lamS + A2 * lamP
        dco = numpy.array([self._dot(lamS, self.psi1), self._dot(lamS, self.psi2),
                           self._dot(lamP, self.psi1), self._dot(lamP, self.psi2)])
        g_d = self._lpt1_T(lam1)
        g_s = self._lpt1_T(lam2)
        lam_s = g_s.c2r()
        lam_s.value *= 1.0 / float(self.nc) ** 3
        # second derivatives of the potential (base mesh)
        E = [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
        pairs_ii = [(2, 0, 0), (0, 2, 0), (0, 0, 2)]
        pairs_ij = [(1, 1, 0), (0, 1, 1), (1, 0, 1)]     # xy, yz, zx
        phi = {}
        for pw in pairs_ii + pairs_ij:
            phi[pw] = self._combine([self.d], [pw], 1.0).c2r().value
        ls = lam_s.value
        lam_phi = {
            (2, 0, 0): (3.0 / 7) * ls * (phi[(0, 2, 0)] + phi[(0, 0, 2)]),
            (0, 2, 0): (3.0 / 7) * ls * (phi[(2, 0, 0)] + phi[(0, 0, 2)]),
            (0, 0, 2): (3.0 / 7) * ls * (phi[(2, 0, 0)] + phi[(0, 2, 0)]),
        }
        for pw in pairs_ij:
            lam_phi[pw] = (-6.0 / 7) * ls * phi[pw]
        fk = []
        for pw in pairs_ii + pairs_ij:
            c = ComplexField(pm, empty=True)
            _lib.call('fpm_r2c', _lib.ptr(lam_phi[pw].contiguous()), _lib.ptr(c.data), pm.n, 1.0,
                      _lib.stream_ptr())
            fk.append(c)
        g2 = self._combine(fk, pairs_ii + pairs_ij, 1.0)
        gd = g_d.value + g2.value
        # linear field
        g_wn = ComplexField(pm)
        g_wn.value[...] = gd
        _lib.call('fpm_apply_isotropic', _lib.ptr(g_wn.data), pm.n, _lib.ptr(self.T), self.T.numel(),
                  _lib.stream_ptr())
        # Om0: host derivatives of every scalar
        h = self.dOm
        Om = self.Om0
        dfac_dOm = numpy.array([(self._factor(Om + h, act) - self._factor(Om - h, act)) / (2 * h)
                                for act in self.acts])
        dco_dOm = (self._lpt_coefs(Om + h) - self._lpt_coefs(Om - h)) / (2 * h)
        dT = (self._table(Om + h) - self._table(Om - h)) / (2 * h)
        dTt = torch.from_numpy(dT.astype('f4')).to(dev)
        wmode = self.mode_weights(pm)
        q = self._shell_index(pm)
        gT = (wmode * (gd.conj() * self.wn.value).real.double() * dTt.double()[q]).sum()
        dL_dOm = float((dfac * dfac_dOm).sum() + (dco * dco_dOm).sum() + float(gT))
        return g_wn, dL_dOm

    @staticmethod
    def mode_weights(pm):
        n = pm.n
        w = torch.full((n, n, n // 2 + 1), 2.0, dtype=torch.float64, device=pm.device)
        w[:, :, 0] = 1.0
        w[:, :, n // 2] = 1.0
        return w

    @staticmethod
    def _shell_index(pm):
        n = pm.n
        i = torch.arange(n, device=pm.device)
        s = torch.where(i < n // 2, i, i - n)
        l = torch.arange(n // 2 + 1, device=pm.device)
        return (s.view(-1, 1, 1) ** 2 + s.view(1, -1, 1) ** 2 + l.view(1, 1, -1) ** 2)


class FastPMLoss(torch.autograd.Function):
    """torch.autograd.Function over ForwardModel.

    forward(wn_data, om0, model): wn_data float32 [nc, nc, nzp, 2] (a
    ComplexField's .data), om0 a 0-d tensor.  backward returns the Euclidean
    gradient w g of the mode array (Hermitian weighting, see the module
    docstring) and dL/dOm0."""

    @staticmethod
    def forward(ctx, wn_data, om0, model):
        wn = ComplexField(model.pm, wn_data.detach())
        loss = model.forward(wn, float(om0))
        ctx.model = model
        return torch.tensor(loss, dtype=torch.float64, device=wn_data.device)

    @staticmethod
    def backward(ctx, gout):
        model = ctx.model
        g, dom = model.backward()
        w = ForwardModel.mode_weights(model.pm).float()
        gdata = torch.zeros_like(g.data)
        nz = model.pm.n // 2 + 1
        gv = torch.view_as_complex(gdata)[:, :, :nz]
        gv[...] = g.value * w
        s = float(gout)
        return gdata * s, torch.tensor(dom * s, dtype=torch.float64, device=gdata.device), None
