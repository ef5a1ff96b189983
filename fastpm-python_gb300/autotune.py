"""Autotuner for the engine's tile shapes and pass variants.

The kernels of libfastpm_gb300 expose their tunable shapes as options of
the calling host thread (fpm_set_option): the brick edge of the cell-sorted paint (key 14),
the lattice brick of the tiled atomic paint (15), the force as a gradient
stencil (12), the TMA-pipelined column passes (11).  A shape class of the
serving engine additionally chooses between pass variants (sorted or tiled
paint, packed or three-mesh force).  The tuner times every candidate on the
class's own batched round with CUDA events on the class's stream and keeps the
fastest; results are cached per (device, shape) in memory and, when the
environment variable FASTPM_GB300_TUNE_CACHE names a file, in that JSON file.
"""
import json
import os
import threading

import torch

from . import _lib

OPTION_KEYS = {'pipe': 11, 'stencil': 12, 'paint_brick': 14, 'tile_el': 15}

_cache = {}
_lock = threading.Lock()


class options(object):
    """Context manager: set library options (by name) for the calling thread
    and restore them on exit.

    The options are read when a kernel is launched (or captured into a CUDA
    graph), so a graph captured inside the context keeps them; other threads
    keep their own options meanwhile."""

    def __init__(self, **kw):
        self.kw = {k: v for k, v in kw.items() if k in OPTION_KEYS and v is not None}
        self.old = {}

    def __enter__(self):
        for k, v in self.kw.items():
            key = OPTION_KEYS[k]
            self.old[key] = _lib.query('fpm_get_option', key)
            _lib.call('fpm_set_option', key, int(v))
        return self

    def __exit__(self, *exc):
        for key, v in self.old.items():
            _lib.call('fpm_set_option', key, v)
        return False


def time_ms(fn, stream, reps=3, warmup=1):
    """Median CUDA-event time of fn() on `stream` (fn enqueues on it)."""
    for _ in range(warmup):
        fn()
    stream.synchronize()
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    times.sort()
    return times[len(times) // 2]


def _file():
    return os.environ.get('FASTPM_GB300_TUNE_CACHE')


def cache_key(kind, shape, device=None):
    dev = torch.cuda.get_device_name(device)
    return '%s|%s|%s' % (kind, dev, ','.join(str(s) for s in shape))


def lookup(key):
    with _lock:
        if key in _cache:
            return _cache[key]
        path = _file()
        if path and os.path.exists(path):
            try:
                with open(path) as f:
                    _cache.update(json.load(f))
            except (OSError, ValueError):
                pass
        return _cache.get(key)


def store(key, value):
    with _lock:
        _cache[key] = value
        path = _file()
        if path:
            data = {}
            if os.path.exists(path):
                try:
                    with open(path) as f:
                        data = json.load(f)
                except (OSError, ValueError):
                    data = {}
            data[key] = value
            tmp = path + '.tmp'
            with open(tmp, 'w') as f:
                json.dump(data, f, indent=1, sort_keys=True)
            os.replace(tmp, path)


def pick(candidates, run, stream, reps=3):
    """Time run(candidate) for every candidate; returns (best, {name: ms})."""
    timings = {}
    best, best_t = None, float('inf')
    for cand in candidates:
        t = time_ms(lambda: run(cand), stream, reps=reps)
        timings[describe(cand)] = t
        if t < best_t:
            best, best_t = cand, t
    return best, timings


def describe(cand):
    return ','.join('%s=%s' % kv for kv in sorted(cand.items()))


def paint_candidates(n, B):
    """Paint variants for an n^3 mesh of (n / B)^3 lattice particles."""
    out = [dict(paint='sorted', paint_brick=bs) for bs in (16, 8) if n % bs == 0]
    nc = n // B
    auto = max(4, 16 // B)          # the tiled paint's default lattice brick
    out.append(dict(paint='tiled', tile_el=0))
    out += [dict(paint='tiled', tile_el=el) for el in (4, 8) if el != auto and nc % el == 0]
    return out


def force_candidates():
    return [dict(force='packed'), dict(force='three')]
