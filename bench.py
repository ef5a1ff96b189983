"""Benchmark of the FastPM particle-mesh step on GB300.

Workload (default): 512^3 particles on a 1024^3 TSC mesh (B = 2), box
1024 Mpc/h, seed 11, 2LPT at a = 0.05, KDK steps log-spaced in a to 1.0 (the
large single-run configuration of the engine's accuracy targets), float32
mesh / FFT / forces, synthetic inputs (seeded whitenoise and an
Eisenstein-Hu no-wiggle P(k)).  A "step" is one KDK step: K(half) D F K(half)
through FastPMStep, i.e. paint -> 5 fused FFT passes -> readout of 3 force
meshes + density -> kick / drift.  Inputs (meshes of 4.3 GB and particle arrays
of 1.6 GB) are far larger than L2 (129 MB), so no flush is needed between
steps.

Metric: particle-steps/s = Np * steps / time (higher is better).

  value  device-resident state, CUDA events on the launching stream around
         exactly --steps KDK steps (default 0 = the workload's whole schedule,
         40 steps from a = 0.05 to 1 for the default) starting from the
         initial conditions; the --warmup untimed steps run first and the
         state is then restored to the initial conditions.  Max over ranks.
  e2e    the same steps through the public API (Solver.nbody) with the initial
         state copied in from pinned host memory and the final X (formed on
         the device in float64, as the reference's X) and V copied back, all
         inside the timed region (the device allocator is warm: X and V were
         formed once before).
  roofline  the dominant kernel's algorithmic bytes per launch / its mean
         event-timed duration (a separate traced run of the same steps, from
         the same initial conditions), against the measured HBM copy
         bandwidth.
  cpu_baseline  the CPU oracle (numpy restatement of the reference algorithm)
         on a bounded sample, on the host cores.

--impl reference runs the CPU oracle arm instead (the reference is pure
Python over pmesh, which is not installable here; the oracle is its
restatement).  Under torchrun (N > 1) each rank runs an independent replica
(a single simulation does not shard on this design: replicas only).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

WORKLOADS = {
    # name: nc, B, box, resampler, seed, a0, a1, nsteps, spacing
    'fastpm-512p-1024m-tsc': (512, 2, 1024.0, 'tsc', 11, 0.05, 1.0, 40, 'log'),
    'fastpm-256p-512m-cic': (256, 2, 512.0, 'cic', 7, 0.1, 1.0, 20, 'lin'),
    # the default workload at 1/8 the particles: small enough for ncu section captures
    'fastpm-256p-512m-tsc': (256, 2, 512.0, 'tsc', 11, 0.05, 1.0, 40, 'log'),
    'fastpm-64p-128m-cic': (64, 2, 256.0, 'cic', 42, 0.1, 1.0, 10, 'lin'),
    'fastpm-128p-256m-cic': (128, 2, 256.0, 'cic', 5, 0.1, 1.0, 10, 'lin'),
}
DEFAULT = 'fastpm-512p-1024m-tsc'
METRIC = 'particle-steps/s'


def schedule(a0, a1, nsteps, spacing, total):
    """Stages of the workload, extended with the same spacing past a1 if the
    benchmark asks for more steps than the schedule has."""
    if spacing == 'log':
        st = numpy.geomspace(a0, a1, nsteps + 1)
        r = st[1] / st[0]
        while len(st) < total + 1:
            st = numpy.append(st, st[-1] * r)
    else:
        st = numpy.linspace(a0, a1, nsteps + 1)
        d = st[1] - st[0]
        while len(st) < total + 1:
            st = numpy.append(st, st[-1] + d)
    return st


def step_actions(stages, i):
    """The K D F K actions of interval i of leapfrog(stages) (core.py:261-288)."""
    a0, a1 = stages[i], stages[i + 1]
    ah = (a0 * a1) ** 0.5
    return [('K', a0, a0, ah), ('D', a0, ah, a1), ('F', a0, a1, a1), ('K', ah, a1, a1)]


# ---------------------------------------------------------------------------
class ClockSampler(object):
    FIELDS = ('clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
              'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
              'clocks_event_reasons.sw_power_cap')

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.index), '--query-gpu=' + self.FIELDS,
                 '--format=csv,noheader,nounits', '-lms', '200'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(',')]
            if len(parts) == 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        if not self.samples:
            return None
        sm = [float(s[0]) for s in self.samples if s[0].replace('.', '').isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace('.', '').isdigit()]
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i] == 'Active'})
        return {'sm_mhz': float(numpy.median(sm)) if sm else None,
                'sm_max_mhz': max(mx) if mx else None, 'reasons': reasons,
                'samples': len(self.samples)}


# ---------------------------------------------------------------------------
def algorithmic_bytes(n, np_, resampler, with_dk=False, stencil=False, packed=False):
    """Bytes each pass must move per force (inputs read once, outputs written
    once; the Kahan terms excluded)."""
    M = float(n) ** 3
    Mc = float(n) * n * (n // 2 + 1)
    R, C = 4.0, 8.0
    if stencil:   # one potential mesh through the inverse passes, then the stencil
        return {
            'paint_' + resampler: np_ * 12 + M * R,
            'fft_z_r2c': M * R + Mc * C,
            'fft_y_fwd': 2 * Mc * C,
            'fft_x_fwd_transfer_inv': 2 * Mc * C + (Mc * C if with_dk else 0),
            'fft_y_inv': 2 * Mc * C,
            'fft_z_c2r': Mc * C + M * R,
            # packed: reads phi and rho, writes {F_x, F_y, F_z, rho} per cell
            'grad_stencil': (2 * M * R + 4 * M * R) if packed else (M * R + 3 * M * R),
            'readout4_' + resampler: 4 * M * R + np_ * 12 + np_ * 16,
            'kick': np_ * 36, 'drift': np_ * 36, 'kick_drift': np_ * 60,
            # the fused kick-drift also counts the new positions into the paint's bricks
            'kick_drift_bin': np_ * 60,
            # forces from the potential at the particles: phi and rho read, F and RHO written
            'force_readout_' + resampler: 2 * M * R + np_ * 12 + np_ * 16,
            # cell-sorted paint: binning passes (positions read, >= 1 id written)
            'paint_bin_count': np_ * 12, 'paint_bin_fill': np_ * 16,
        }
    return {
        'paint_' + resampler: np_ * 12 + M * R,
        'fft_z_r2c': M * R + Mc * C,
        'fft_y_fwd': 2 * Mc * C,
        'fft_x_fwd_transfer_inv': Mc * C + 2 * Mc * C + (Mc * C if with_dk else 0),
        'fft_y_inv': 2 * Mc * C + 3 * Mc * C,
        'fft_z_c2r': 3 * Mc * C + 3 * M * R,
        # plane-batched fused passes: the intermediate stays in L2
        'fft_z_r2c_y_fwd': M * R + Mc * C,
        'fft_y_inv_z_c2r': 2 * Mc * C + 3 * M * R,
        'readout4_' + resampler: 4 * M * R + np_ * 12 + np_ * 16,
        'grad_stencil': M * R + 3 * M * R,
        'kick': np_ * 36,
        'drift': np_ * 36,
        'kick_drift': np_ * 60,
    }


def kernel_table(kern, alg, peak, trace_steps, res, bucketed):
    """Per-kernel rows of the bench line from the tracer's {name: (launches,
    ms)} over trace_steps steps: share of the traced time, and for kernels with
    an algorithmic byte model the rate and fraction of peak; plus the whole
    paint stage and the whole FFT of a force.  bucketed: the brick lists went
    through the kick-drift's buckets (option 26), so the recount and fill
    launches carry no byte model."""
    total_ms = sum(v[1] for v in kern.values())
    kernels = {}
    for name, (cnt, tms) in kern.items():
        d = {'launches': cnt, 'ms_per_launch': tms / cnt, 'share': tms / total_ms}
        if name in alg:
            # alg[name] is the bytes of one pass per force; a pass may be split
            # into several launches, so rate = bytes of all its launches / time
            per_force = launches_per_force(name, kern, trace_steps)
            gbs = alg[name] * (cnt / per_force) / (tms / 1e3) / 1e9
            d.update({'alg_bytes_per_pass': alg[name], 'launches_per_pass': per_force, 'gbs': gbs,
                      'frac': gbs / peak})
        kernels[name] = d
    # with bucketed brick lists the recount and fill launches return at once
    # unless a spill list overflowed: no byte model for them (their time is in
    # the paint stage)
    if bucketed:
        for name in ('paint_bin_count', 'paint_bin_fill'):
            if name in kernels:
                for key in ('alg_bytes_per_pass', 'launches_per_pass', 'gbs', 'frac'):
                    kernels[name].pop(key, None)
                kernels[name]['note'] = ('returns at once unless the kick-drift\'s bucket spill list '
                                         'overflowed (the buckets hold the lists)')
    # the whole mass assignment (binning passes + brick deposit) against the
    # paint's algorithmic bytes: positions read once, the mesh written once
    stage = [k for k in kernels if k.startswith('paint_')]
    if any(k.startswith('paint_bin') for k in stage):
        pname = 'paint_' + res
        tms = sum(kern[k][1] for k in stage)
        gbs = alg[pname] * (kern[pname][0] / launches_per_force(pname, kern, trace_steps)) \
            / (tms / 1e3) / 1e9
        kernels['paint_stage'] = {'launches': sum(kern[k][0] for k in stage),
                                  'ms_per_launch': tms / kern[pname][0], 'share': tms / total_ms,
                                  'alg_bytes_per_pass': alg[pname], 'gbs': gbs, 'frac': gbs / peak,
                                  'kernels': stage}
    # the whole FFT of a force (z r2c, y forward, x forward + transfer +
    # inverse, y inverse, z c2r) against the sum of its passes' algorithmic bytes
    fft = [k for k in kernels if k.startswith('fft_') and 'alg_bytes_per_pass' in kernels[k]]
    if fft:
        tms = sum(kern[k][1] for k in fft)
        nbytes = sum(alg[k] * (kern[k][0] / launches_per_force(k, kern, trace_steps)) for k in fft)
        nforce = kern[fft[0]][0] / launches_per_force(fft[0], kern, trace_steps)
        gbs = nbytes / (tms / 1e3) / 1e9
        kernels['fft_stage'] = {'launches': sum(kern[k][0] for k in fft), 'ms_per_launch': tms / nforce,
                                'share': tms / total_ms, 'alg_bytes_per_pass': nbytes / nforce, 'gbs': gbs,
                                'frac': gbs / peak, 'kernels': fft}
    return kernels


def launches_per_force(name, kern, steps):
    """Launches one pass of `name` takes per force (passes may be split)."""
    per_step = {'kick': None, 'drift': None, 'kick_drift': None}
    if name in per_step:
        return 1
    cnt = kern[name][0]
    return max(1, int(round(cnt / float(steps))))


def load_peaks():
    path = os.path.join(HERE, 'MEASURED_PEAKS.json')
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d['hbm_gbs']), 'measured'
    return 6800.0, 'fallback'


def load_traffic():
    """Per-launch DRAM bytes of each kernel from the committed ncu summary."""
    path = os.path.join(HERE, 'profiles', 'ncu_traffic.txt')
    out = {}
    if os.path.exists(path):
        for line in open(path):
            line = line.strip()
            if not line or line.startswith('#'):
                continue
            parts = line.split()
            if len(parts) >= 3:
                out[(parts[0], parts[1])] = float(parts[2])
    return out


# ---------------------------------------------------------------------------
def build_state(G, workload, total_steps):
    import torch
    nc, B, box, res, seed, a0, a1, nsteps, spacing = WORKLOADS[workload]
    pm = G.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, resampler=res)
    solver = G.Solver(pm, G.Planck15, B=B)
    Q = pm.generate_uniform_particle_grid(shift=0)
    dlin = solver.linear(solver.whitenoise(seed), G.EHPower(G.Planck15, 0))
    state = solver.lpt(dlin, Q, a=a0, order=2)
    del dlin
    stages = schedule(a0, a1, nsteps, spacing, total_steps)
    step = solver.nbodystep
    step.want_event = False
    # the first force of leapfrog(stages)
    step.Force(state, a0, a0, a0)
    torch.cuda.synchronize()
    return pm, solver, state, stages, step


def run_steps(solver, state, stages, first, count):
    """count KDK steps through the public Solver.nbody (no monitor)."""
    acts = [a for i in range(first, first + count) for a in step_actions(stages, i)]
    solver.nbody(state, acts)


class PhaseTimers(object):
    """Per-phase wall time of the CPU oracle (paint / FFT / transfer / readout /
    kick-drift / host background), by wrapping its functions for the sample."""

    PHASES = {
        'paint': [('pmesh_np', 'paint')],
        'fft': [('pmesh_np.RealField', 'r2c'), ('pmesh_np.ComplexField', 'c2r')],
        'transfer': [('pmesh_np.ComplexField', 'apply')],
        'readout': [('pmesh_np', 'readout')],
        'kick_drift': [('fastpm_np.FastPMStep', 'Kick'), ('fastpm_np.FastPMStep', 'Drift')],
        'background': [('fastpm_np', 'kick_factor'), ('fastpm_np', 'drift_factor')],
    }

    def __init__(self):
        self.t = {k: 0.0 for k in self.PHASES}
        self.saved = []

    def __enter__(self):
        import oracle.pmesh_np as pmesh_np
        import oracle.fastpm_np as fastpm_np
        mods = {'pmesh_np': pmesh_np, 'fastpm_np': fastpm_np,
                'pmesh_np.RealField': pmesh_np.RealField, 'pmesh_np.ComplexField': pmesh_np.ComplexField,
                'fastpm_np.FastPMStep': fastpm_np.FastPMStep}
        for phase, targets in self.PHASES.items():
            for owner, name in targets:
                obj = mods[owner]
                fn = getattr(obj, name)
                self.saved.append((obj, name, fn))
                setattr(obj, name, self._wrap(phase, fn))
        return self

    def _wrap(self, phase, fn):
        timers = self

        def timed(*a, **kw):
            t0 = time.perf_counter()
            try:
                return fn(*a, **kw)
            finally:
                timers.t[phase] += time.perf_counter() - t0
        return timed

    def __exit__(self, *exc):
        for obj, name, fn in reversed(self.saved):
            setattr(obj, name, fn)
        return False


def cpu_sample(steps=1, nc=128, B=2, resampler='tsc', box=256.0):
    """The CPU oracle (reference algorithm, numpy, float32 state) on a bounded
    sample: `steps` KDK steps of an nc^3 / (B nc)^3 run; returns particle-steps/s,
    the time, and the per-phase split of that time."""
    from oracle import fastpm_np, pmesh_np, cosmology_np
    pm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3, dtype='f4', resampler=resampler)
    solver = fastpm_np.Solver(pm, cosmology_np.Planck15, B=B)
    Q = pm.generate_uniform_particle_grid(shift=0, dtype='f4')
    dlin = solver.linear(solver.whitenoise(11), cosmology_np.EHPower(cosmology_np.Planck15, 0))
    state = solver.lpt(dlin, Q, a=0.05, order=2)
    stages = numpy.geomspace(0.05, 1.0, 41)
    solver.nbody(state, [('F', 0.05, 0.05, 0.05)])
    acts = []
    for i in range(steps):
        acts += step_actions(stages, i)
    with PhaseTimers() as pt:
        t0 = time.perf_counter()
        solver.nbody(state, acts)
        dt = time.perf_counter() - t0
    t = dict(pt.t)
    t['kick_drift'] -= t['background']   # the factors are computed inside Kick / Drift
    split = {k: round(v / dt, 4) for k, v in t.items()}
    return nc ** 3 * steps / dt, dt, split


# ---------------------------------------------------------------------------
def dist_init():
    import torch
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local = int(os.environ.get('LOCAL_RANK', '0'))
    if world > 1:
        import torch.distributed as dist
        backend = 'nccl' if torch.cuda.is_available() else 'gloo'
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, x):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device='cuda' if torch.cuda.is_available() else 'cpu')
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main_reference(args, world, rank):
    """CPU oracle arm: each step is one KDK step of a bounded sample."""
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    nc, B = 128, 2
    from oracle import fastpm_np, pmesh_np, cosmology_np
    pm = pmesh_np.ParticleMesh(BoxSize=256.0, Nmesh=[nc] * 3, dtype='f4', resampler='tsc')
    solver = fastpm_np.Solver(pm, cosmology_np.Planck15, B=B)
    Q = pm.generate_uniform_particle_grid(shift=0, dtype='f4')
    dlin = solver.linear(solver.whitenoise(11), cosmology_np.EHPower(cosmology_np.Planck15, 0))
    state = solver.lpt(dlin, Q, a=0.05, order=2)
    # K steps after W warm-up steps of the 40-step schedule (default K = 10:
    # about 4-5 s of CPU time a step at this sample size)
    steps = args.steps if args.steps > 0 else 10
    stages = schedule(0.05, 1.0, 40, 'log', args.warmup + steps)
    solver.nbody(state, [('F', 0.05, 0.05, 0.05)])
    for i in range(args.warmup):
        solver.nbody(state, step_actions(stages, i))
    with PhaseTimers() as pt:
        t0 = time.perf_counter()
        for i in range(args.warmup, args.warmup + steps):
            solver.nbody(state, step_actions(stages, i))
        dt = time.perf_counter() - t0
    v = nc ** 3 * steps / dt
    ph = dict(pt.t)
    ph['kick_drift'] -= ph['background']
    sample = ('KDK steps of a %d^3-particle / %d^3-mesh TSC run (the benchmark workload at 1/64 '
              'the particles), numpy oracle restating the reference algorithm, float32 state, '
              'scipy.fft with %d workers' % (nc, nc * B, cores))
    line = {'impl': 'reference', 'metric': METRIC, 'value': v, 'unit': METRIC,
            'n_gpus': args.gpus, 'steps': steps, 'warmup': args.warmup,
            'ms_per_step': dt / steps * 1e3, 'higher_is_better': True, 'scaling': 'weak',
            'vs_baseline': None, 'dtype': 'f32', 'data': 'synthetic',
            'config': {'workload': args.workload, 'sample': '%dp-%dm-tsc' % (nc, nc * B)},
            'cpu_baseline': {'value': v, 'unit': METRIC, 'cores': cores, 'kind': 'port',
                             'sample': sample,
                             'phase_share': {k: round(x / dt, 4) for k, x in ph.items()}},
            'e2e': {'value': v, 'unit': METRIC, 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0}}
    print(json.dumps(line))


def serving_measure(requests=256, sample=32, loads=(1.0, 4.0, 'saturated'), seed=2):
    """Batched continuous serving against one-at-a-time GPU solves on the
    serving stream (Poisson arrivals; per request Nc in {64, 96, 128, 192,
    256}, B in {1, 2}, box 4 Nc, Om0 ~ U[0.25, 0.35], sigma8 ~ U[0.7, 0.9],
    seed = request id, 5-20 KDK steps from a = 0.1).

    The plain path's capacity (sims/s) is measured first on `sample` requests
    all queued at t = 0; the same seeded stream of `requests` is then offered
    to both paths at each multiple in `loads` of that capacity, and
    ('saturated') with every request queued at t = 0, which measures each
    path's throughput at its own capacity.  Reports sims/s (completed /
    makespan) and p50 / p99 latency (arrival to result on the host) of each
    path and load, and the largest relative difference of the batched P(k)
    from the plain P(k) of the same request (k < k_Nyq / 2)."""
    import torch
    from fastpm_gb300.serving import ServingEngine, run_plain, make_stream, summarize
    classes = [(nc, B) for nc in (64, 96, 128, 192, 256) for B in (1, 2)]
    warm = lambda: [make_stream(1, 1e9, seed=100 + i, nc_choices=(nc,), B_choices=(B,), steps=(2, 2))[0]
                    for i, (nc, B) in enumerate(classes)]
    t0 = time.perf_counter()
    eng = ServingEngine({w.key for w in warm()}, use_graphs=True)
    eng.run(warm(), realtime=False)          # allocation, plans, graph capture
    run_plain(warm(), realtime=False)
    setup_s = time.perf_counter() - t0
    smp = make_stream(sample, rate=1e9, seed=1)
    t0 = time.perf_counter()
    run_plain(smp, realtime=False)
    cap = sample / (time.perf_counter() - t0)
    out = {'requests': requests, 'arrivals': 'poisson', 'plain_capacity_sims_per_s': cap,
           'capacity_sample': sample, 'setup_s': setup_s,
           'slots': {'%dx%d' % (k[0], k[1]): v for k, v in eng.capacity.items()},
           'tuned_variants': {'%dx%d' % (k[0], k[1]): c.variant for k, c in eng.classes.items()},
           'loads': {}}
    worst = 0.0
    for load in loads:
        rate = 1e9 if load == 'saturated' else load * cap
        b = eng.run(make_stream(requests, rate, seed=seed), realtime=True)
        p = run_plain(make_stream(requests, rate, seed=seed), realtime=True)
        pb = {r.rid: r for r in p}
        for r in b:
            q = pb[r.rid]
            kmax = numpy.pi * r.nc * r.B / r.box / 2
            sel = numpy.isfinite(q.pk) & (q.pk > 0) & (q.k < kmax)
            worst = max(worst, float(numpy.abs(r.pk[sel] / q.pk[sel] - 1).max()))
        sb, sp = summarize(b), summarize(p)
        out['loads'][load if load == 'saturated' else '%gx' % load] = {
                                     'rate_per_s': rate, 'batched': sb, 'plain': sp,
                                     'speedup_sims_per_s': sb['sims_per_s'] / sp['sims_per_s']}
    out['pk_max_rel_diff_batched_vs_plain'] = worst
    del eng
    torch.cuda.empty_cache()
    return out


def main_serving(args, world, rank):
    """Serving stream alone (--mode serving): the serving_measure figures at
    --load times the plain capacity, with --requests requests."""
    import torch
    torch.cuda.set_device(int(os.environ.get('LOCAL_RANK', '0')))
    res = serving_measure(requests=args.requests, sample=args.sample, loads=(args.load,))
    lv = res['loads']['%gx' % args.load]
    if rank == 0:
        line = {'metric': 'sims/s (serving stream)', 'value': lv['batched']['sims_per_s'], 'unit': 'sims/s',
                'n_gpus': world, 'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None,
                'dtype': 'f32', 'data': 'synthetic',
                'config': {'workload': 'serving stream', 'requests': args.requests,
                           'offered_load_vs_plain_capacity': args.load, 'nc': [64, 96, 128, 192, 256],
                           'B': [1, 2], 'steps': [5, 20]},
                'serving': res}
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=0,
                    help='KDK steps timed (0: the whole schedule of the workload)')
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--workload', default=DEFAULT, choices=sorted(WORKLOADS))
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--trace-steps', type=int, default=0,
                    help='steps of the per-kernel trace (0: the timed steps)')
    ap.add_argument('--mode', default='step', choices=['step', 'serving'])
    ap.add_argument('--requests', type=int, default=4096, help='--mode serving: stream length')
    ap.add_argument('--sample', type=int, default=64, help='--mode serving: capacity sample')
    ap.add_argument('--load', type=float, default=4.0, help='--mode serving: offered load')
    ap.add_argument('--set-option', action='append', default=[], metavar='KEY=VALUE',
                    help='library tuning option (fpm_set_option) for this run, e.g. 22=1')
    ap.add_argument('--serving-requests', type=int, default=256,
                    help='requests per load level of the serving figures in the step line (0: skip)')
    args = ap.parse_args()
    world, rank, local = dist_init()
    if args.mode == 'serving':
        main_serving(args, world, rank)
        return
    if args.impl == 'reference':
        main_reference(args, world, rank)
        return

    import torch
    import fastpm_gb300 as G
    from fastpm_gb300 import _lib
    torch.cuda.set_device(local)
    for kv in args.set_option:
        k, v = kv.split('=')
        _lib.call('fpm_set_option', int(k), int(v))
    nc, B, box, res, seed, a0, a1, nsteps, spacing = WORKLOADS[args.workload]
    n = nc * B
    np_ = nc ** 3
    steps = args.steps if args.steps > 0 else nsteps
    total = max(steps, args.warmup)
    pm, solver, state, stages, step = build_state(G, args.workload, total)
    # every run below starts from the same initial conditions (2LPT at a0 and
    # the first force), so the timed steps are steps 0 .. K-1 of the schedule
    keys = ('S', 'P', 'F', 'RHO', 'S_c', 'P_c')
    snap = {k: getattr(state, k).clone() for k in keys}
    tags = dict(state.a)

    def restore():
        for k in keys:
            getattr(state, k).copy_(snap[k])
        state.a = dict(tags)

    # ---- device-resident timing -------------------------------------------
    run_steps(solver, state, stages, 0, args.warmup)
    restore()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    l0 = _lib.launch_count()
    ev0.record()
    run_steps(solver, state, stages, 0, steps)
    ev1.record()
    torch.cuda.synchronize()
    launches = _lib.launch_count() - l0
    clk = clocks.stop()
    barrier(world)
    ms = allmax(world, ev0.elapsed_time(ev1))
    value = np_ * steps * world / (ms / 1e3)

    # ---- per-kernel trace of the same steps --------------------------------
    trace_steps = min(args.trace_steps, steps) if args.trace_steps > 0 else steps
    restore()
    _lib.trace(True)
    run_steps(solver, state, stages, 0, trace_steps)
    torch.cuda.synchronize()
    _lib.trace(False)
    kern = _lib.trace_summary()
    from fastpm_gb300.core import FastPMStep
    alg = algorithmic_bytes(n, np_, res, stencil=bool(_lib.query('fpm_get_option', 12))
                            or FastPMStep.packed_force, packed=FastPMStep.packed_force)
    peak, peak_src = load_peaks()
    kernels = kernel_table(kern, alg, peak, trace_steps, res, _lib.query('fpm_get_option', 26) != 0)
    dom = max((k for k in kernels if not k.endswith('_stage')), key=lambda k: kernels[k]['share'])
    traffic = load_traffic().get((dom, args.workload))
    roof = {'bound': 'hbm', 'kernel': dom, 'achieved': kernels[dom].get('gbs'), 'peak': peak,
            'unit': 'GB/s', 'frac': kernels[dom].get('frac'), 'peak_source': peak_src,
            'traffic': traffic, 'alg_bytes_per_pass': kernels[dom].get('alg_bytes_per_pass'),
            'launches_per_pass': kernels[dom].get('launches_per_pass')}

    # ---- end to end through the public API ---------------------------------
    # the initial state comes from pinned host memory, X and V go back to it
    pin = {k: snap[k].cpu().pin_memory() for k in ('S', 'P', 'F')}
    # pinned host buffers for the results (X in Q's dtype, V), allocated before timing
    X = torch.empty(tuple(state.S.shape), dtype=state.Q.dtype).pin_memory()
    V = torch.empty(tuple(state.P.shape), dtype=torch.float32).pin_memory()
    acts = [a for i in range(0, steps) for a in step_actions(stages, i)]
    for k in ('RHO', 'S_c', 'P_c'):
        getattr(state, k).zero_()
    # warm the caching allocator for the float64 X and the V the API forms at
    # the end (the first 3.2 GB cudaMalloc of X alone took ~0.65 s); forming
    # and copying them stay inside the timed region
    xw, vw = state.X, state.V
    # and the pinned buffers: the first DMA through freshly pinned pages ran at
    # 32-41 GB/s against 190-210 GB/s once they had been used
    X.copy_(xw, non_blocking=True)
    V.copy_(vw, non_blocking=True)
    for k in ('S', 'P', 'F'):
        getattr(state, k).copy_(pin[k], non_blocking=True)
    del xw, vw
    torch.cuda.synchronize()
    barrier(world)
    ph = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    t0 = time.perf_counter()
    ph[0].record()
    for k in ('S', 'P', 'F'):
        getattr(state, k).copy_(pin[k], non_blocking=True)
    state.S_c.zero_()
    state.P_c.zero_()
    state.a = dict(tags)
    ph[1].record()
    solver.nbody(state, acts)
    ph[2].record()
    t_host = time.perf_counter() - t0       # host time to enqueue the copies and the steps
    X.copy_(state.X, non_blocking=True)
    V.copy_(state.V, non_blocking=True)
    ph[3].record()
    torch.cuda.synchronize()
    e2e_s = allmax(world, time.perf_counter() - t0)
    e2e = {'value': np_ * steps * world / e2e_s, 'unit': METRIC,
           'h2d_bytes_per_step': int(sum(p.numel() * 4 for p in pin.values()) / steps),
           'd2h_bytes_per_step': int((X.numel() * X.element_size() + V.numel() * V.element_size())
                                     / steps),
           # device time of each part (events on the launching stream) and the
           # host time until the last step was enqueued
           'phases_ms': {'h2d': ph[0].elapsed_time(ph[1]), 'steps': ph[1].elapsed_time(ph[2]),
                         'x_v_d2h': ph[2].elapsed_time(ph[3]), 'host_enqueue': 1e3 * t_host,
                         'wall': 1e3 * e2e_s}}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, dt, split = cpu_sample()
        cpu = {'value': v, 'unit': METRIC, 'cores': os.cpu_count(), 'kind': 'port',
               'phase_share': split,
               'sample': 'one KDK step of a 128^3-particle / 256^3-mesh TSC run (this workload at '
                         '1/64 the particles), numpy oracle restating the reference algorithm, '
                         'float32 state; %.1f s' % dt}
    serving = None
    if args.serving_requests > 0 and rank == 0:
        # the step workload's buffers go first: the engine sizes its slot
        # pools from the free HBM
        del state, solver, pm, step, snap, pin, X, V
        import gc
        gc.collect()
        torch.cuda.empty_cache()
        serving = serving_measure(requests=args.serving_requests)
    if rank == 0:
        line = {'metric': METRIC, 'value': value, 'unit': METRIC, 'n_gpus': world,
                'steps': steps, 'warmup': args.warmup, 'ms_per_step': ms / steps,
                'higher_is_better': True, 'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f32',
                'data': 'synthetic',
                'config': {'workload': args.workload, 'particles': np_, 'mesh': n, 'box': box,
                           'resampler': res, 'seed': seed, 'a0': a0, 'parallelism': 'replicas',
                           'timed': 'KDK steps 0..%d of the %d-step schedule from a = %g' % (
                               steps - 1, nsteps, a0),
                           'l2': 'inputs larger than L2 (mesh %.1f GB)' % (n ** 3 * 4 / 1e9),
                           'options': args.set_option},
                'e2e': e2e, 'roofline': roof, 'cpu_baseline': cpu, 'gpu_launches': launches,
                'clocks': clk, 'kernels': kernels, 'serving': serving}
        print(json.dumps(line))


if __name__ == '__main__':
    main()
