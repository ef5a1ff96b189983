"""Serving: batched continuous serving gives each request the result it gets alone."""
import numpy
import pytest
from numpy.testing import assert_allclose

from tests.helpers import tonp


def test_schedule_factors_match_per_action_factors():
    """One growth solve per request equals core.py's per-action solves (1e-7)."""
    import fastpm_gb300 as G
    from fastpm_gb300.serving import schedule_factors
    stages = numpy.linspace(0.1, 1.0, 8)
    k1, d, k2 = schedule_factors(0.27, stages)
    acts = list(G.leapfrog(stages))[1:]
    for i in range(len(stages) - 1):
        K1, D, _, K2 = acts[4 * i: 4 * i + 4]
        assert_allclose(k1[i], G.background.kick_factor(0.27, *K1[1:]), rtol=1e-7)
        assert_allclose(d[i], G.background.drift_factor(0.27, *D[1:]), rtol=1e-7)
        assert_allclose(k2[i], G.background.kick_factor(0.27, *K2[1:]), rtol=1e-7)


def test_schedule_growth_gives_the_lpt_factors():
    """The admission's one growth solve (schedule_factors with the growth
    returned) gives the 2LPT factors at a0 bit for bit as Solver.lpt's own
    solve on the grid [a0] does, so the batched initial conditions are the
    plain path's."""
    from fastpm_gb300.background import MatterDominated
    from fastpm_gb300.serving import make_stream, schedule_factors
    for r in make_stream(6, 1e9, seed=3):
        k1, d, k2, pt = schedule_factors(r.Om0, r.stages, with_growth=True)
        one = MatterDominated(r.Om0, a=[r.a0])
        a = r.a0
        for f in ('D1', 'D2', 'f1', 'f2', 'E', 'gf', 'gf2'):
            assert getattr(pt, f)(a) == getattr(one, f)(a), (f, r.rid)
        assert numpy.array_equal(k1, schedule_factors(r.Om0, r.stages)[0])


def test_stream_shape():
    from fastpm_gb300.serving import make_stream
    reqs = make_stream(200, rate=50.0, seed=1)
    assert len(reqs) == 200
    assert all(r.box == 4 * r.nc for r in reqs)
    assert all(5 <= r.nsteps <= 20 and 0.25 <= r.Om0 <= 0.35 and 0.7 <= r.sigma8 <= 0.9 for r in reqs)
    assert sorted(r.arrival for r in reqs) == [r.arrival for r in reqs]
    assert {r.seed for r in reqs} == set(range(200))


def test_slot_bytes_cover_the_library_workspaces():
    """Admission accounting: the per-slot estimate covers what one slot of a
    class allocates (particle pools, rho + force pool, the FFT and the sorted
    paint workspaces as the library sizes them, per slot of an S-slot class)."""
    from fastpm_gb300 import _lib
    from fastpm_gb300.serving import class_slot_bytes
    for nc, B in ((64, 1), (64, 2), (96, 2), (128, 2), (192, 1), (256, 2)):
        n, np_ = nc * B, nc ** 3
        for S in (1, 8):
            need = (np_ * (3 * 4 * 3 + 3 * 2 * 2 + 4) + 5 * n ** 3 * 4
                    + _lib.query('fpm_force_batch_workspace', n, S) / S
                    + _lib.query('fpm_paint_sorted_batch_workspace', n, np_, S) / S)
            assert class_slot_bytes(nc, B) >= need, (nc, B, S)


class _FakeEvent(object):
    def query(self):
        return True

    def synchronize(self):
        pass


class _FakeClass(object):
    """A shape class without a GPU: admissions take `cost` seconds of host
    time, a simulation runs `rounds` engine rounds; it logs every admission
    with the engine round it came before."""

    def __init__(self, key, nslots, cost, rounds, log):
        self.key, self.S, self.cost, self.rounds, self.log = key, nslots, cost, rounds, log
        self.slots = [None] * nslots
        self.left = [0] * nslots
        self.stream = None
        self.engine_round = 0

    def free_slot(self):
        return next((s for s, r in enumerate(self.slots) if r is None), None)

    @property
    def busy(self):
        return any(r is not None for r in self.slots)

    def admit(self, req, s):
        import time
        t = time.perf_counter()
        while time.perf_counter() - t < self.cost:
            pass
        self.slots[s] = req
        self.left[s] = self.rounds
        self.log.append((self.engine_round, self.key, req.rid))

    def release(self, s):
        self.slots[s] = None

    def round(self):
        done = []
        for s, r in enumerate(self.slots):
            if r is not None:
                self.left[s] -= 1
                if self.left[s] == 0:
                    done.append(s)
        self.engine_round += 1
        return done

    def finish(self, s, keep_state=False):
        r, self.slots[s] = self.slots[s], None
        return (r, _FakeEvent())

    def check_status(self):
        return [], None


def test_admissions_interleave_with_rounds(monkeypatch):
    """The engine's host loop without a GPU: a burst of requests is admitted a
    few per engine round (each round admits one request per class with a free
    slot, then more only while the round's host budget lasts), so the rounds
    of running simulations go on between admissions; every request finishes."""
    import torch
    from fastpm_gb300 import serving
    monkeypatch.setattr(torch.cuda, 'synchronize', lambda *a, **k: None)
    monkeypatch.setattr(serving.ShapeClass, 'collect', staticmethod(lambda item: item[0]))
    log = []
    eng = object.__new__(serving.ServingEngine)
    keys = [(32, 2, 128.0, 'cic'), (24, 2, 96.0, 'cic')]
    eng.classes = {k: _FakeClass(k, 16, 0.004, 3, log) for k in keys}
    eng.refused = {}
    eng.keep_state = False
    eng._cancel = set()
    eng.admit_budget_s = 0.01
    eng.device = 'cpu'
    reqs = [_req(i, 32 if i % 2 else 24, 2, 4) for i in range(40)]
    done = eng.run(reqs, realtime=False)
    assert sorted(r.rid for r in done) == list(range(40))
    assert all(r.status == 'done' for r in done)
    per_round = {}
    for rnd, key, rid in log:
        per_round.setdefault((rnd, key), []).append(rid)
    # the first round admits one request per class although the first
    # admission alone nearly spends the budget, and no round admits the whole
    # burst of 20 per class
    assert all((0, k) in per_round for k in keys)
    assert max(len(v) for v in per_round.values()) < 16
    # admissions of a class spread over several rounds
    assert all(len({rnd for (rnd, kk) in per_round if kk == k}) >= 3 for k in keys)


def _req(rid, nc, B, nsteps, Om0=0.3, s8=0.8):
    from fastpm_gb300.serving import Request
    return Request(rid, nc=nc, B=B, Om0=Om0, sigma8=s8, nsteps=nsteps, arrival=0.0)


VARIANTS = {
    'tuned': None,
    'tiled-three': dict(paint='tiled', force='three'),
    'sorted8-packed': dict(paint='sorted', paint_brick=8, force='packed'),
}


@pytest.mark.gpu
@pytest.mark.parametrize('variant', sorted(VARIANTS))
@pytest.mark.parametrize('graphs', [False, True])
def test_alone_equals_mix_equals_plain(graphs, variant):
    from fastpm_gb300.serving import ServingEngine, run_plain
    probe = lambda: _req(7, 32, 2, 4, Om0=0.28, s8=0.75)
    others = [_req(100 + i, 32, 2, 3 + i % 4, Om0=0.26 + 0.01 * i) for i in range(5)] + \
             [_req(200 + i, 24, 2, 5, Om0=0.33) for i in range(3)] + [_req(300, 16, 1, 6)]
    classes = [r.key for r in others] + [probe().key]
    eng = ServingEngine(classes, max_slots=4, use_graphs=graphs, keep_state=True,
                        hbm_budget=4e9, variant=VARIANTS[variant])
    alone = eng.run([probe()], realtime=False)[0]
    mix = [r for r in eng.run([probe()] + others, realtime=False) if r.rid == 7][0]
    plain = run_plain([probe()], realtime=False, keep_state=True)[0]
    a, m, p = tonp(alone.X), tonp(mix.X), tonp(plain.X)
    spacing = alone.box / alone.nc
    for x in (m, p):
        rms = numpy.sqrt(((x - a) ** 2).sum(axis=1).mean())
        assert rms <= 1e-4 * spacing, rms
    sel = numpy.isfinite(alone.pk) & (alone.pk > 0)
    for r in (mix, plain):
        assert numpy.abs(r.pk[sel] / alone.pk[sel] - 1).max() < 1e-3


@pytest.mark.gpu
def test_engine_completes_all_and_admits_by_slots():
    from fastpm_gb300.serving import ServingEngine, make_stream
    reqs = make_stream(24, rate=1000.0, seed=3, nc_choices=(16, 32), B_choices=(1, 2), steps=(2, 4))
    eng = ServingEngine({r.key for r in reqs}, max_slots=3, use_graphs=True, hbm_budget=4e9)
    done = eng.run(reqs, realtime=True)
    assert sorted(r.rid for r in done) == list(range(24))
    assert all(r.done >= r.arrival and numpy.isfinite(r.pk[1:]).all() for r in done)
    assert max(eng.capacity.values()) <= 3


@pytest.mark.gpu
def test_autotune_picks_a_timed_candidate(tmp_path, monkeypatch):
    """The tuner times every paint and force candidate of a class, keeps the
    fastest, and serves the next engine from its cache file."""
    from fastpm_gb300 import autotune
    from fastpm_gb300.serving import ServingEngine
    path = tmp_path / 'tune.json'
    monkeypatch.setenv('FASTPM_GB300_TUNE_CACHE', str(path))
    key = (32, 2, 128.0, 'cic')
    eng = ServingEngine([key], max_slots=2, hbm_budget=2e9)
    cls = eng.classes[key]
    t = cls.tune_timings
    paint = {k: v for k, v in t.items() if not k.startswith('force:')}
    assert len(paint) == len(autotune.paint_candidates(64, 2)) and all(v > 0 for v in t.values())
    chosen = autotune.describe({k: cls.variant[k] for k in ('paint', 'paint_brick')}) \
        if cls.variant['paint'] == 'sorted' else \
        autotune.describe({k: cls.variant[k] for k in ('paint', 'tile_el')})
    assert paint[chosen] == min(paint.values())
    assert path.exists()
    autotune._cache.clear()
    eng2 = ServingEngine([key], max_slots=2, hbm_budget=2e9)
    assert eng2.classes[key].variant == cls.variant


# ---------------------------------------------------------------------------
# host-side faults: each stays with its request; the other slots finish with
# the results they get in a run without the fault
def _faultless_results(keys, reqs):
    from fastpm_gb300.serving import ServingEngine
    eng = ServingEngine(keys, max_slots=3, use_graphs=True, keep_state=True, hbm_budget=4e9, tune=False)
    return {r.rid: r for r in eng.run(reqs, realtime=False)}


def _assert_unchanged(got, ref):
    """The final state bit for bit; P(k) to float32 rounding (the density it
    is measured on is painted with float atomics, whose order varies)."""
    assert got.status == 'done', (got.rid, got.status, got.error)
    assert numpy.array_equal(tonp(got.X), tonp(ref.X)), got.rid
    sel = numpy.isfinite(ref.pk)
    assert_allclose(got.pk[sel], ref.pk[sel], rtol=1e-6)


def _others():
    return [_req(10 + i, 32, 2, 3 + i % 3, Om0=0.26 + 0.01 * i) for i in range(6)] + \
           [_req(20 + i, 24, 2, 4, Om0=0.31) for i in range(4)]


@pytest.mark.gpu
def test_fault_invalid_shape_rejected():
    """A request of an unsupported mesh size (Nc = 20, B = 2: a 40^3 mesh) and
    one of a shape the engine has no class for arrive among the others: both
    are rejected with a reason, the others finish unchanged."""
    from fastpm_gb300.serving import ServingEngine
    keys = {r.key for r in _others()}
    ref = _faultless_results(keys, _others())
    bad = [_req(90, 20, 2, 3), _req(91, 16, 2, 3)]
    reqs = _others()
    reqs = reqs[:4] + bad + reqs[4:]
    eng = ServingEngine(keys, max_slots=3, use_graphs=True, keep_state=True, hbm_budget=4e9, tune=False)
    done = {r.rid: r for r in eng.run(reqs, realtime=False)}
    assert done[90].status == 'rejected' and 'unsupported shape' in done[90].error
    assert done[91].status == 'rejected' and 'no shape class' in done[91].error
    for rid, r in ref.items():
        _assert_unchanged(done[rid], r)


@pytest.mark.gpu
def test_fault_admission_refused_by_hbm_budget():
    """A class whose single slot does not fit its share of the HBM budget gets
    no slot: its requests are refused at arrival, the other class serves on."""
    from fastpm_gb300.serving import ServingEngine, class_slot_bytes
    small = [r for r in _others() if r.nc == 24]
    big = _req(95, 256, 2, 3)
    keys = {small[0].key, big.key}
    budget = 2.2 * class_slot_bytes(24, 2)          # share per class: 1.1 small slots
    ref = _faultless_results({small[0].key}, [r for r in _others() if r.nc == 24])
    eng = ServingEngine(keys, max_slots=3, use_graphs=True, keep_state=True, hbm_budget=budget, tune=False)
    assert big.key in eng.refused and big.key not in eng.classes
    assert eng.capacity == {small[0].key: 1}
    done = {r.rid: r for r in eng.run(small[:1] + [big] + small[1:], realtime=False)}
    assert done[95].status == 'rejected' and 'admission refused' in done[95].error
    for rid, r in ref.items():
        _assert_unchanged(done[rid], r)


@pytest.mark.gpu
def test_fault_cancelled_mid_batch():
    """Request 12 is cancelled while it runs (after engine round 2) and request
    23 while it still waits for a slot: both report 'cancelled', their slots
    go to the next requests, the others finish unchanged."""
    from fastpm_gb300.serving import ServingEngine
    keys = {r.key for r in _others()}
    ref = _faultless_results(keys, [r for r in _others() if r.rid not in (12, 23)])
    eng = ServingEngine(keys, max_slots=3, use_graphs=True, keep_state=True, hbm_budget=4e9, tune=False)
    seen = {}

    def on_round(engine, i):
        if i == 2:
            running = [r.rid for c in engine.classes.values() for r in c.slots if r is not None]
            seen['running'] = running
            engine.cancel(12)
            engine.cancel(23)

    done = {r.rid: r for r in eng.run(_others(), realtime=False, on_round=on_round)}
    assert 12 in seen['running'] and 23 not in seen['running']
    assert done[12].status == 'cancelled' and done[23].status == 'cancelled'
    for rid, r in ref.items():
        _assert_unchanged(done[rid], r)


@pytest.mark.gpu
def test_fault_worker_exception_mid_batch():
    """Preparing request 13 raises on the host (its cosmology cannot be
    built) when it is admitted into a slot freed mid-batch: it fails with the
    exception's message, the slot is reused, the others finish unchanged."""
    from fastpm_gb300.serving import ServingEngine, Request

    class Broken(Request):
        def cosmology(self):
            raise RuntimeError('cosmology worker failed')

    keys = {r.key for r in _others()}
    ref = _faultless_results(keys, [r for r in _others() if r.rid != 13])
    reqs = [r if r.rid != 13 else Broken(13, nc=32, B=2, Om0=0.29, sigma8=0.8, nsteps=4) for r in _others()]
    eng = ServingEngine(keys, max_slots=3, use_graphs=True, keep_state=True, hbm_budget=4e9, tune=False)
    done = {r.rid: r for r in eng.run(reqs, realtime=False)}
    assert done[13].status == 'failed' and 'cosmology worker failed' in done[13].error
    assert done[13].admitted is None
    for rid, r in ref.items():
        _assert_unchanged(done[rid], r)
