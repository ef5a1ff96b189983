"""Error of the float32 device engine against the float64 oracle on the
plain-run configurations (same whitenoise fed to both):

  c0: 64^3 particles, 128^3 CIC mesh, box 256 Mpc/h, seed 42, 2LPT at a = 0.1,
      10 KDK steps linear in a to 1.0
  c1: 256^3 particles, 512^3 CIC mesh, box 512 Mpc/h, seed 7, 2LPT at a = 0.1,
      20 KDK steps linear in a to 1.0

    python -m tests.accuracy_configs gpu OUTDIR [c0 c1]     # device runs
    python -m tests.accuracy_configs cpu OUTDIR [c0 c1]     # float64 oracle runs
    python -m tests.accuracy_configs compare GPUDIR CPUDIR  # report

Saved per run: P(k) of the final CIC density (integer shells), and X, V of
every 97th particle (a fixed subsample, small enough to move between hosts).
"""
import os
import sys
import time

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

CONFIGS = {
    'c0': dict(nc=64, B=2, box=256.0, seed=42, a0=0.1, nsteps=10),
    'c1': dict(nc=256, B=2, box=512.0, seed=7, a0=0.1, nsteps=20),
}
STRIDE = 97


def stages(c):
    return numpy.linspace(c['a0'], 1.0, c['nsteps'] + 1)


def run_gpu(outdir, names):
    import torch
    import fastpm_gb300 as G
    from oracle import pmesh_np
    from oracle.cosmology_np import EHPower, Planck15
    for name in names:
        c = CONFIGS[name]
        wn = pmesh_np.whitenoise([c['nc']] * 3, c['seed'])
        pm = G.ParticleMesh(BoxSize=c['box'], Nmesh=[c['nc']] * 3, resampler='cic')
        solver = G.Solver(pm, G.Planck15, B=c['B'])
        Q = pm.generate_uniform_particle_grid(shift=0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dlin = solver.linear(pm.complex_from(wn), EHPower(Planck15, 0))
        st = solver.lpt(dlin, Q, a=c['a0'], order=2)
        st = solver.nbody(st, G.leapfrog(stages(c)))
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        mesh = G.RealField(solver.fpm)
        solver.fpm._paint(mesh.value, disp=st.S, lattice=st.lattice)
        k, p = G.power(mesh)
        numpy.savez(os.path.join(outdir, 'acc_%s_gpu.npz' % name), k=k, p=p,
                    X=st.X[::STRIDE].cpu().numpy(), V=st.V[::STRIDE].cpu().numpy(), seconds=t)
        print(name, 'device run %.2f s' % t)


def run_cpu(outdir, names):
    from oracle import fastpm_np, pmesh_np, power_np
    from oracle.cosmology_np import EHPower, Planck15
    for name in names:
        c = CONFIGS[name]
        pm = pmesh_np.ParticleMesh(BoxSize=c['box'], Nmesh=[c['nc']] * 3, dtype='f8', resampler='cic')
        solver = fastpm_np.Solver(pm, Planck15, B=c['B'])
        t0 = time.perf_counter()
        wn = solver.whitenoise(c['seed'])
        dlin = solver.linear(wn, EHPower(Planck15, 0))
        st = solver.lpt(dlin, pm.generate_uniform_particle_grid(shift=0), a=c['a0'], order=2)
        st = solver.nbody(st, fastpm_np.leapfrog(stages(c)))
        t = time.perf_counter() - t0
        n = c['nc'] * c['B']
        rho = pmesh_np.paint(st.X, [n] * 3, [c['box']] * 3, 'cic')
        k, p = power_np.power(rho, boxsize=c['box'])
        numpy.savez(os.path.join(outdir, 'acc_%s_cpu.npz' % name), k=k, p=p, X=st.X[::STRIDE],
                    V=st.V[::STRIDE], seconds=t)
        print(name, 'oracle run %.1f s' % t)


def compare(gdir, cdir, names=('c0', 'c1')):
    rows = []
    for name in names:
        gp, cp = os.path.join(gdir, 'acc_%s_gpu.npz' % name), os.path.join(cdir, 'acc_%s_cpu.npz' % name)
        if not (os.path.exists(gp) and os.path.exists(cp)):
            continue
        g, o = numpy.load(gp), numpy.load(cp)
        c = CONFIGS[name]
        spacing = c['box'] / c['nc']
        dx = g['X'] - o['X']
        dx -= c['box'] * numpy.round(dx / c['box'])
        rms = numpy.sqrt((dx ** 2).sum(axis=1).mean())
        dv = numpy.sqrt(((g['V'] - o['V']) ** 2).sum(axis=1).mean() / (o['V'] ** 2).sum(axis=1).mean())
        n = c['nc'] * c['B']
        kny = numpy.pi * n / c['box']
        sel = (o['k'] < 0.5 * kny) & (o['p'] > 0) & numpy.isfinite(o['p'])
        dp = numpy.abs(g['p'][sel] / o['p'][sel] - 1).max()
        rows.append((name, rms / spacing, dv, dp, float(g['seconds']), float(o['seconds'])))
        print('%s: rms|dX| = %.2e spacing, rel rms dV = %.2e, max |dP/P| (k < kNyq/2) = %.2e; '
              'device %.2f s, oracle %.0f s' % rows[-1])
    return rows


if __name__ == '__main__':
    mode = sys.argv[1]
    if mode == 'gpu':
        run_gpu(sys.argv[2], sys.argv[3:] or ['c0', 'c1'])
    elif mode == 'cpu':
        run_cpu(sys.argv[2], sys.argv[3:] or ['c0', 'c1'])
    else:
        compare(sys.argv[2], sys.argv[3])
