"""CPU-side checks of the C ABI library and the host logic (no GPU calls)."""
import ctypes
import os
import re

import numpy
import pytest
from numpy.testing import assert_allclose, assert_array_equal

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, 'include', 'fastpm_gb300.h')


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(fpm_[a-z0-9_]+)\s*\(', text)))


def test_library_exports_every_declared_symbol():
    import fastpm_gb300
    lib = fastpm_gb300._lib.load()
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
    # every declared symbol has a ctypes signature, and vice versa
    assert set(syms) == set(fastpm_gb300._lib.SIGNATURES)


def test_host_queries():
    from fastpm_gb300 import _lib
    assert _lib.query('fpm_abi_version') == 1
    for n in (16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512, 1024):
        assert _lib.query('fpm_fft_supported', n) == 1
        zp = _lib.query('fpm_complex_row', n)
        assert zp >= n // 2 + 1 and zp % 16 == 0
        assert _lib.query("fpm_force_workspace", n) >= 3 * n * n * zp * 8
    for n in (0, 8, 10, 100, 2048):
        assert _lib.query('fpm_fft_supported', n) == 0
        assert _lib.query('fpm_complex_row', n) == -1
    assert b'workspace' in _lib.query('fpm_strerror', 4)


def test_argument_errors_without_gpu():
    """Argument checks run before any CUDA call, so they work on a CPU machine."""
    from fastpm_gb300 import _lib
    lib = _lib.load()
    assert lib.fpm_force_mesh(None, 64, 1.0, 1.0, 1.0, None, None, None, None, None, 0, None) == 1
    buf = ctypes.c_void_p(16)   # never dereferenced: the size check fails first
    assert lib.fpm_force_mesh(buf, 100, 1.0, 1.0, 1.0, buf, buf, buf, None, buf, 1 << 40, None) == 2
    assert lib.fpm_force_mesh(buf, 64, 1.0, 1.0, 1.0, buf, buf, buf, None, buf, 10, None) == 4
    assert lib.fpm_paint(buf, 64, 1.0, buf, None, 1000, 16, 0.0, 1, 1.0, None) == 1  # np != nc^3
    assert lib.fpm_paint(buf, 64, 1.0, buf, None, 16 ** 3, 16, 0.0, 7, 1.0, None) == 1  # window
    assert lib.fpm_kick(None, None, None, 3, 1.0, None) == 1


def test_layout_and_option_checks_without_gpu():
    """The blocked force mesh / readout refuse a mesh that is not 128-byte
    aligned and an odd n before any CUDA call; options 19, 20, 24, 25 and 26
    (layout, readout, line-plan, deposit and list variants) read back what was set."""
    from fastpm_gb300 import _lib
    lib = _lib.load()
    b16 = ctypes.c_void_p(16)     # 16-byte but not 128-byte aligned: never dereferenced
    b128 = ctypes.c_void_p(128)
    assert lib.fpm_force_mesh_blocked(b128, 64, 1.0, 1.0, 1.0, b16, None, b128, 1 << 40, None) == 1
    assert lib.fpm_force_mesh_blocked(b128, 64, 1.0, 1.0, 1.0, b128, None, b128, 10, None) == 4
    assert lib.fpm_force_mesh_blocked(b128, 100, 1.0, 1.0, 1.0, b128, None, b128, 1 << 40, None) == 2
    assert lib.fpm_readout_blocked_sorted(b16, 64, 1.0, b128, None, 16 ** 3, 16, 0.0, 2, b128, None, 16,
                                          b128, 1 << 40, None) == 1
    assert lib.fpm_readout_blocked_sorted(b128, 64, 1.0, b128, None, 16 ** 3, 16, 0.0, 7, b128, None, 16,
                                          b128, 1 << 40, None) == 1
    assert lib.fpm_readout_blocked_sorted(b128, 63, 1.0, b128, None, 16 ** 3, 16, 0.0, 2, b128, None, 16,
                                          b128, 1 << 40, None) == 2
    for key in (19, 20, 24, 25, 26):
        old = _lib.query('fpm_get_option', key)
        try:
            for v in (1, 0):
                _lib.call('fpm_set_option', key, v)
                assert _lib.query('fpm_get_option', key) == v
        finally:
            _lib.call('fpm_set_option', key, old)
    # the cell-sorted paint's workspace holds the brick counts, offsets and
    # cursors, the chunk sums of the brick scan, one key and up to 8 ids per particle
    n, np_ = 1024, 512 ** 3
    nbrick = (n // 16) ** 3
    assert _lib.query('fpm_paint_sorted_workspace', n, np_) >= 4 * (nbrick + 1) * 4 + 9 * np_ * 4 + nbrick // 256
    # the single-simulation workspace adds the fused kick-drift's buckets: a
    # mode block, home and tail buckets of 16 and 8 times the mean particles
    # per brick (512 here), and a spill list of np / 16 (brick, id) pairs
    single = _lib.query('fpm_paint_sorted_workspace', n, np_)
    batch1 = _lib.query('fpm_paint_sorted_batch_workspace', n, np_, 1)
    up = lambda x: (x + 255) // 256 * 256
    assert single - batch1 == 256 + up(nbrick * 8192 * 4) + up(nbrick * 4096 * 4) + up(np_ // 16 * 8)


def test_workspace_status_refuses_a_short_buffer():
    """The status word sits at an offset that follows from n: the helper the
    package calls refuses a buffer shorter than that workspace before the
    library reads anything (no GPU needed)."""
    import torch
    from fastpm_gb300 import _lib
    for kind, name in ((0, 'fpm_force_workspace'), (1, 'fpm_lpt_workspace')):
        short = torch.empty(_lib.query(name, 64) - 1, dtype=torch.uint8)
        with pytest.raises(ValueError):
            _lib.workspace_status(short, 64, kind)
        # a workspace sized for n = 32 is short for n = 64
        small = torch.empty(_lib.query(name, 32), dtype=torch.uint8)
        with pytest.raises(ValueError):
            _lib.workspace_status(small, 64, kind)


def test_schedules_and_background_match_reference(golden_units):
    import fastpm_gb300 as G
    g = golden_units
    for n, knots in enumerate([[0.1, 1.0], [1.0], [0.5], [0.1, 0.2, 1.0]]):
        assert_array_equal(G.autostages(knots, astart=0.1, N=12), g['auto_%d' % n])
    acts = list(G.leapfrog(numpy.linspace(0.1, 1.0, 11)))
    assert_array_equal(numpy.array([x[0] for x in acts]), g['sched_actions'])
    for (action, ai, ac, af), ref in zip(acts, g['sched_fac']):
        if action == 'K':
            assert_allclose(G.background.kick_factor(0.3089, ai, ac, af), ref, rtol=1e-12)
        elif action == 'D':
            assert_allclose(G.background.drift_factor(0.3089, ai, ac, af), ref, rtol=1e-12)
    pt = G.MatterDominated(0.3089, a=g['a'], a_normalize=1.0)
    for name in ('D1', 'D2', 'f1', 'f2', 'E', 'Gp', 'gp', 'Gf', 'gf', 'gf2'):
        assert_allclose(getattr(pt, name)(g['a']), g['bg_' + name], rtol=1e-12)
    assert list(G.leapfrog_with_lpt([0.1, 0.2]))[0][0] == 'K'


def test_linear_power_matches_oracle():
    import fastpm_gb300 as G
    from oracle import cosmology_np
    k = numpy.logspace(-3, 1, 200)
    assert_allclose(G.EHPower(G.Planck15, 0)(k),
                    cosmology_np.EHPower(cosmology_np.Planck15, 0)(k), rtol=1e-12)
    assert G.EHPower(G.Planck15, 0)(numpy.array([0.0]))[0] == 0.0


def test_solver_type_check():
    import fastpm_gb300 as G
    pm = object.__new__(G.ParticleMesh)
    with pytest.raises(TypeError):
        G.Solver(pm, object(), B=1)


def test_power_text_format():
    """format_power gives fastpm/main.py:81-92's columns (k, p, N, p/D^2),
    dropping empty bins; savetxt with its header round-trips."""
    import io
    from fastpm_gb300.power import format_power
    t = format_power([0.1, 0.2, 0.3], [1.0, 2.0, 3.0], [0, 4, 6], 0.5)
    assert t.shape == (2, 4)
    assert numpy.allclose(t[:, 0], [0.2, 0.3]) and numpy.allclose(t[:, 2], [4, 6])
    assert numpy.allclose(t[:, 3], [8.0, 12.0])
    buf = io.StringIO()
    numpy.savetxt(buf, t, comments='# k p N p/D**2', header='')
    back = numpy.loadtxt(io.StringIO(buf.getvalue()))
    assert numpy.allclose(back, t)
