"""Float64 comparator on the GPU — TEST INFRASTRUCTURE ONLY.

The float64 oracle (oracle/fastpm_np.py over oracle/pmesh_np.py) is numpy on
the host: it finishes the 64^3-particle configuration in seconds but not the
256^3 / 512^3-particle ones.  This module restates the same algorithm with
torch float64 tensors on the device (cuFFT for the transforms, index_add_ for
the mass assignment), so the engine can be compared at those sizes:

  fastpm/core.py:113-118    whitenoise -> linear (P evaluated per integer shell)
  fastpm/core.py:120-145    lpt (2LPT S, P, F)
  fastpm/force/lpt.py:4-64  lpt1 (CIC readout at Q), lpt2source
  fastpm/core.py:168-180    Kick / Drift (float64, no compensation needed)
  fastpm/core.py:182-210    prepare_force (paint / nbar), Force (RHO readout,
                            r2c, longrange)
  fastpm/force/gravity.py:10-29, force/kernels.py:3-35  laplace, gradient(order=1)
  fastpm/utils.py:77-164    power (integer shells, Hermitian weights)

It is itself checked against the numpy oracle on a configuration the oracle
finishes quickly (tests/test_gpu_accuracy.py), so it stands in for the oracle
at the larger sizes.  It is never used by the package.
"""
import math

import numpy
import torch

from oracle import fastpm_np

C16 = torch.complex128


def _freqs(n, box, device):
    """k_x, k_y (fftfreq order) and k_z (0 .. n/2) in h/Mpc, float64, broadcastable."""
    f = torch.fft.fftfreq(n, 1.0 / n, dtype=torch.float64, device=device)
    fz = torch.arange(n // 2 + 1, dtype=torch.float64, device=device)
    s = 2 * math.pi / box
    return (f * s).view(n, 1, 1), (f * s).view(1, n, 1), (fz * s).view(1, 1, -1)


def _ints(n, device):
    f = torch.fft.fftfreq(n, 1.0 / n, dtype=torch.float64, device=device).round().long()
    fz = torch.arange(n // 2 + 1, device=device)
    return f.view(n, 1, 1), f.view(1, n, 1), fz.view(1, 1, -1)


def r2c(real):
    """pmesh RealField.r2c: forward transform with the 1/N normalisation."""
    n = real.shape[0]
    return torch.fft.rfftn(real) / float(n) ** 3


def c2r(cplx, n):
    """pmesh ComplexField.c2r: unnormalised inverse (c2r(r2c(x)) == x)."""
    return torch.fft.irfftn(cplx, s=(n, n, n)) * float(n) ** 3


def laplace_inplace(v, n, box):
    """force/kernels.py:3-9: v / k^2, k = 0 -> 0."""
    kx, ky, kz = _freqs(n, box, v.device)
    for i in range(n):   # plane by plane: no full-size k^2 temporary
        kk = kx[i] ** 2 + ky[0] ** 2 + kz[0] ** 2
        if i == 0:
            kk[0, 0] = 1.0
        p = v[i] / kk
        if i == 0:
            p[0, 0] = 0
        v[i] = p
    return v


def gradient_mult(d, n, box, device):
    """force/kernels.py:17-24 (order 1): i (8 sin w - sin 2w) / (6 h), w = k_d h,
    as a broadcastable complex multiplier along axis d."""
    h = box / n
    k = _freqs(n, box, device)[d]
    w = k * h
    return 1j * ((8 * torch.sin(w) - torch.sin(2 * w)) / (6.0 * h))


def _window(x, resampler):
    if resampler == 'cic':
        i0 = torch.floor(x)
        f = x - i0
        return i0.long(), (0, 1), (1.0 - f, f)
    i0 = torch.floor(x + 0.5)
    d = x - i0
    return i0.long(), (-1, 0, 1), (0.5 * (0.5 - d) ** 2, 0.75 - d ** 2, 0.5 * (0.5 + d) ** 2)


def _iter_window(pos, n, box, resampler, chunk=1 << 23):
    """(start, flat cell index, weight) for every window cell of every particle;
    pos float64 [Np, 3] in Mpc/h, cells at i L / n, periodic (pmesh semantics,
    restated in oracle/pmesh_np.py:_iter_window)."""
    scale = n / box
    for start in range(0, pos.shape[0], chunk):
        x = pos[start:start + chunk] * scale
        i0x, offs, wx = _window(x[:, 0], resampler)
        i0y, _, wy = _window(x[:, 1], resampler)
        i0z, _, wz = _window(x[:, 2], resampler)
        for a, oa in enumerate(offs):
            ix = torch.remainder(i0x + oa, n)
            for b, ob in enumerate(offs):
                iy = torch.remainder(i0y + ob, n)
                wab = wx[a] * wy[b]
                base = (ix * n + iy) * n
                for c, oc in enumerate(offs):
                    iz = torch.remainder(i0z + oc, n)
                    yield start, base + iz, wab * wz[c]


def paint(pos, n, box, resampler):
    out = torch.zeros(n ** 3, dtype=torch.float64, device=pos.device)
    for _, idx, w in _iter_window(pos, n, box, resampler):
        out.index_add_(0, idx, w)
    return out.view(n, n, n)


def readout(meshes, pos, box, resampler):
    """Window-weighted gather of each mesh at pos -> list of float64 [Np]."""
    n = meshes[0].shape[0]
    flats = [m.reshape(-1) for m in meshes]
    outs = [torch.zeros(pos.shape[0], dtype=torch.float64, device=pos.device) for _ in meshes]
    for start, idx, w in _iter_window(pos, n, box, resampler):
        for f, o in zip(flats, outs):
            o[start:start + len(w)] += w * f[idx]
    return outs


def lattice(nc, box, shift, device):
    """pmesh generate_uniform_particle_grid: (i + shift) L / nc, C order."""
    i = torch.arange(nc, dtype=torch.float64, device=device)
    g = (i + shift) * (box / nc)
    X, Y, Z = torch.meshgrid(g, g, g, indexing='ij')
    return torch.stack([X.reshape(-1), Y.reshape(-1), Z.reshape(-1)], dim=1)


def linear(wn, Pk, nc, box):
    """core.py:116-118: dlin = wn sqrt(P(|k|) / V); |k| = 2 pi sqrt(q) / L on
    integer shells q = nx^2 + ny^2 + nz^2, P evaluated once per shell."""
    dev = wn.device
    qmax = 3 * (nc // 2) ** 2
    k = numpy.sqrt(numpy.arange(qmax + 1, dtype='f8')) * (2 * numpy.pi / box)
    with numpy.errstate(invalid='ignore', divide='ignore'):
        table = numpy.asarray(Pk(k), dtype='f8') ** 0.5 / box ** 1.5
    table[0] = 0.0 if not numpy.isfinite(table[0]) else table[0]
    t = torch.from_numpy(table).to(dev)
    ix, iy, iz = _ints(nc, dev)
    out = torch.empty_like(wn)
    for i in range(nc):
        q = ix[i] ** 2 + iy[0] ** 2 + iz[0] ** 2
        out[i] = wn[i] * t[q]
    return out


def lpt1(dlin_k, q, nc, box):
    """force/lpt.py:4-23: c2r(i a_d(k) dlin / k^2) read out (CIC) at q, d = 0..2."""
    pot = laplace_inplace(dlin_k.clone(), nc, box)
    meshes = []
    for d in range(3):
        meshes.append(c2r(pot * gradient_mult(d, nc, box, pot.device), nc))
    del pot
    out = readout(meshes, q, box, 'cic')
    return torch.stack(out, dim=1)


def lpt2source(dlin_k, nc, box):
    """force/lpt.py:25-64: r2c(3/7 [sum phi_ii phi_jj - sum phi_ij^2])."""
    pot = laplace_inplace(dlin_k.clone(), nc, box)
    g = [gradient_mult(d, nc, box, pot.device) for d in range(3)]
    phi_ii = [c2r(pot * g[d] * g[d], nc) for d in range(3)]
    D1, D2 = [1, 2, 0], [2, 0, 1]
    source = torch.zeros((nc, nc, nc), dtype=torch.float64, device=pot.device)
    for d in range(3):
        source += phi_ii[D1[d]] * phi_ii[D2[d]]
    del phi_ii
    for d in range(3):
        source -= c2r(pot * g[D1[d]] * g[D2[d]], nc) ** 2
    source *= 3.0 / 7
    return r2c(source)


class State(object):
    def __init__(self, Q):
        self.Q = Q
        self.S = torch.zeros_like(Q)
        self.P = torch.zeros_like(Q)
        self.F = torch.zeros_like(Q)
        self.RHO = torch.zeros_like(Q[:, 0])
        self.a = dict(S=None, P=None, F=None)
        self.delta_k = None

    @property
    def X(self):
        return self.S + self.Q

    @property
    def V(self):
        return self.P * (100. / self.a['P'])


def force(state, n, box, resampler, Om0):
    """core.py:182-210 + force/gravity.py:10-29: RHO = readout(paint(X) / nbar),
    F = 1.5 Om0 readout(c2r(grad_d lap delta_k)); one window pass reads out
    the density and the three force meshes."""
    X = state.X
    nbar = state.Q.shape[0] / float(n) ** 3
    rho = paint(X, n, box, resampler)
    rho /= nbar
    delta_k = r2c(rho)
    state.delta_k = delta_k
    pot = laplace_inplace(delta_k.clone(), n, box)
    meshes = [rho] + [c2r(pot * gradient_mult(d, n, box, pot.device), n) for d in range(3)]
    del pot
    out = readout(meshes, X, box, resampler)
    del meshes
    state.RHO = out[0]
    state.F = torch.stack(out[1:], dim=1) * (1.5 * Om0)


def run(wn, Pk, nc, B, box, resampler, stages, Om0, shift=0.0, order=2, a_linear=1.0):
    """2LPT at stages[0] then leapfrog(stages) (core.py:120-152, 261-288), all
    float64 on the device.  wn: complex128 whitenoise on the base mesh."""
    dev = wn.device
    n = nc * B
    a0 = float(stages[0])
    Q = lattice(nc, box, shift, dev)
    state = State(Q)
    dlin = linear(wn, Pk, nc, box)
    pt = fastpm_np.MatterDominated(Om0, a=[a0], a_normalize=a_linear)
    D1, D2 = float(pt.D1(a0)), float(pt.D2(a0))
    f1, f2, E = float(pt.f1(a0)), float(pt.f2(a0)), float(pt.E(a0))
    gf, gf2 = float(pt.gf(a0)), float(pt.gf2(a0))
    DX1 = D1 * lpt1(dlin, Q, nc, box)
    if order == 2:
        DX2 = D2 * lpt1(lpt2source(dlin, nc, box), Q, nc, box)
        state.S = DX1 + DX2
        state.P = a0 ** 2 * f1 * E * DX1 + a0 ** 2 * f2 * E * DX2
        state.F = a0 ** 2 * E * (gf / D1 * DX1 + gf2 / D2 * DX2)
        del DX2
    else:
        state.S = DX1.clone()
        state.P = a0 ** 2 * f1 * E * DX1
        state.F = a0 ** 2 * E * (gf / D1 * DX1)
    del DX1, dlin
    state.a['S'] = state.a['P'] = a0
    for action, ai, ac, af in fastpm_np.leapfrog(stages):
        if action == 'K':
            assert ac == state.a['F']
            state.P = state.P + fastpm_np.kick_factor(Om0, ai, ac, af, a_linear) * state.F
            state.a['P'] = af
        elif action == 'D':
            assert ac == state.a['P']
            state.S = state.S + fastpm_np.drift_factor(Om0, ai, ac, af, a_linear) * state.P
            state.a['S'] = af
        else:
            assert ac == state.a['S']
            force(state, n, box, resampler, Om0)
            state.a['F'] = af
    return state


def power(f, box):
    """fastpm/utils.py:77-164 on a float64 half mesh: integer shells
    floor(sqrt(n^2)), weight 2 on the half axis except its first and last
    planes, normalised by |f(0)|.  Returns k, P (numpy, n/2 bins)."""
    n = f.shape[0]
    z = abs(complex(f[0, 0, 0].item()))
    ix, iy, iz = _ints(n, f.device)
    nb = n // 2
    w = torch.full((n // 2 + 1,), 2.0, dtype=torch.float64, device=f.device)
    w[0] = 1
    w[-1] = 1
    ksum = torch.zeros(n, dtype=torch.float64, device=f.device)
    wsum = torch.zeros_like(ksum)
    psum = torch.zeros_like(ksum)
    for i in range(n):
        kk = (ix[i] ** 2 + iy[0] ** 2 + iz[0] ** 2)
        d = torch.floor(torch.sqrt(kk.double())).long()
        d = d - ((d * d) > kk).long() + (((d + 1) * (d + 1)) <= kk).long()   # exact integer root
        ww = w.view(1, -1).expand(n, -1)
        ksum.index_add_(0, d.reshape(-1), (torch.sqrt(kk.double()) * (2 * math.pi / box) * ww).reshape(-1))
        wsum.index_add_(0, d.reshape(-1), ww.reshape(-1))
        psum.index_add_(0, d.reshape(-1), ((f[i].abs() ** 2) * ww).reshape(-1))
    norm = z * z if z != 0 else 1.0
    ksum, wsum, psum = ksum[:nb].cpu().numpy(), wsum[:nb].cpu().numpy(), psum[:nb].cpu().numpy() / norm
    with numpy.errstate(invalid='ignore', divide='ignore'):
        return ksum / wsum, psum / wsum * box ** 3


def errors(gx, gv, g_dk, ref, box, nc):
    """Error of a device (float32) state against a comparator state:
    rms |dX| in units of the mean spacing L / nc (periodic), relative rms dV,
    and max |P_gpu / P_ref - 1| over k < k_Nyq / 2 of the final delta_k."""
    dx = gx - ref.X
    dx -= box * torch.round(dx / box)
    rms_x = float(torch.sqrt((dx ** 2).sum(dim=1).mean())) / (box / nc)
    rel_v = float(torch.linalg.norm(gv - ref.V) / torch.linalg.norm(ref.V))
    n = ref.delta_k.shape[0]
    k, pr = power(ref.delta_k, box)
    _, pg = power(g_dk, box)
    knyq = math.pi * n / box
    sel = (k < 0.5 * knyq) & numpy.isfinite(pr) & (pr > 0)
    dp = float(numpy.abs(pg[sel] / pr[sel] - 1).max())
    return dict(rms_dx_over_spacing=rms_x, rel_rms_dv=rel_v, max_dp_over_p=dp)
