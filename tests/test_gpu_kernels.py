"""Kernel-level parity: libfastpm_gb300 (through its C ABI) vs the CPU oracle.

Tolerances: FFTs and meshes are float32 (relative L2 error <= 2e-6 for an
n-point transform, about 10 float32 ulps); cell keys and wraps are integer and
must match bit for bit.
"""
import ctypes

import numpy
import pytest
import torch
from numpy.testing import assert_array_equal, assert_allclose

from oracle import pmesh_np, fastpm_np, power_np
from tests.helpers import rel_l2, tonp

pytestmark = pytest.mark.gpu

SIZES = [16, 24, 32, 48, 64, 96, 128, 192, 256]


@pytest.fixture(scope='module')
def G():
    import fastpm_gb300
    return fastpm_gb300


def device_pm(G, n, box=100.0, resampler='cic'):
    return G.ParticleMesh(BoxSize=box, Nmesh=[n] * 3, resampler=resampler)


@pytest.mark.parametrize('n', SIZES + [384, 512])
def test_r2c_c2r_vs_numpy(G, n):
    pm = device_pm(G, n)
    rng = numpy.random.RandomState(n)
    x = rng.normal(size=(n, n, n))
    real = G.RealField(pm, torch.from_numpy(x.astype('f4')).cuda())
    ck = real.r2c()
    ref = numpy.fft.rfftn(x) / n ** 3
    assert rel_l2(tonp(ck.value), ref) < 2e-6
    back = ck.c2r()
    assert rel_l2(tonp(back.value), x) < 2e-6
    # c2r of a reference spectrum
    ref_c = pm.complex_from(ref)
    assert rel_l2(tonp(ref_c.c2r().value), numpy.fft.irfftn(ref, s=(n, n, n), axes=(0, 1, 2)) * n ** 3) < 2e-6


@pytest.mark.parametrize('n', [16, 48, 64])
def test_gradient_hermitian(G, n):
    """fastpm/tests/test_kernel.py:7-13: a gradient survives c2r().r2c()."""
    pm = device_pm(G, n, box=128.0)
    data = pm.generate_whitenoise(seed=333, type='real')
    ck = data.r2c()
    kx = pm.k
    for d in range(3):
        g1 = ck.apply(lambda k, v: v * (1j * k[d]) * (pm.ic[d] != n // 2))
        g2 = g1.c2r().r2c()
        assert_allclose(tonp(g2.value), tonp(g1.value), atol=1e-5 * float(abs(tonp(g1.value)).max()))


@pytest.mark.parametrize('n', [16, 48, 64, 96])
@pytest.mark.parametrize('unitary', [False, True])
def test_whitenoise_matches_oracle(G, n, unitary):
    pm = device_pm(G, n)
    wn = pm.generate_whitenoise(1234 + n, unitary=unitary)
    ref = pmesh_np.whitenoise([n] * 3, 1234 + n, unitary=unitary)
    got = tonp(wn.value)
    assert_allclose(got, ref, rtol=1e-6, atol=1e-6)
    # the same float32 value in nearly every mode
    same = numpy.mean(got == ref.astype('c8'))
    assert same > 0.99


def _rand_disp(rng, np_, spread, dtype='f4'):
    d = rng.normal(scale=spread, size=(np_, 3)).astype(dtype)
    # exact cell boundaries, tiny negatives and far wraps
    d[:7] = numpy.array([[0, 0, 0], [1e-30, -1e-30, -0.0], [0.5, -0.5, 1.0], [-1, 1e-7, -1e-7],
                         [1e3, -1e3, 333.25], [2.0, 2.5, -2.5], [0.25, 0.75, -0.75]], dtype=dtype)
    return d


@pytest.mark.parametrize('resampler', ['cic', 'tsc'])
@pytest.mark.parametrize('nc,B,shift', [(16, 2, 0.0), (16, 1, 0.5), (32, 2, 0.5), (24, 2, 0.25)])
def test_cell_keys_bit_exact(G, resampler, nc, B, shift):
    from fastpm_gb300 import _lib
    n, box = nc * B, 64.0
    rng = numpy.random.RandomState(nc + B)
    disp = _rand_disp(rng, nc ** 3, 3.0)
    d = torch.from_numpy(disp).cuda()
    key = torch.empty(nc ** 3, dtype=torch.int64, device='cuda')
    frac = torch.empty((nc ** 3, 3), dtype=torch.float32, device='cuda')
    _lib.call('fpm_cell_keys', _lib.ptr(key), _lib.ptr(frac), n, box, _lib.ptr(d), None,
              nc ** 3, nc, shift, _lib.FPM_WINDOW[resampler], _lib.stream_ptr())
    rkey, rfrac = pmesh_np.cell_keys_lattice(disp, nc, shift, n, box, resampler)
    assert_array_equal(tonp(key), rkey)
    assert_array_equal(tonp(frac), rfrac)


def _positions(nc, box, shift, disp):
    q = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3).generate_uniform_particle_grid(shift=shift)
    return q + disp.astype('f8')


@pytest.mark.parametrize('resampler', ['cic', 'tsc'])
@pytest.mark.parametrize('nc,B', [(16, 2), (32, 1), (48, 2)])
def test_paint_readout_vs_oracle(G, resampler, nc, B):
    n, box, shift = nc * B, 96.0, 0.0
    rng = numpy.random.RandomState(7)
    disp = _rand_disp(rng, nc ** 3, 2.0)
    pm = device_pm(G, n, box, resampler)
    d = torch.from_numpy(disp).cuda()
    mesh = torch.zeros((n, n, n), dtype=torch.float32, device='cuda')
    pm._paint(mesh, disp=d, lattice=(nc, shift), resampler=resampler)
    pos = _positions(nc, box, shift, disp)
    ref = pmesh_np.paint(pos, [n] * 3, [box] * 3, resampler)
    assert rel_l2(tonp(mesh), ref) < 1e-6
    assert abs(float(mesh.double().sum()) - nc ** 3) < 1e-3 * nc ** 3 * 1e-3
    # readout of a smooth field, plus the painted mesh
    field = numpy.sin(2 * numpy.pi * numpy.arange(n) / n)[:, None, None] \
        * numpy.cos(4 * numpy.pi * numpy.arange(n) / n)[None, :, None] + 0 * numpy.arange(n)
    f = torch.from_numpy(field.astype('f4')).cuda().contiguous()
    out = torch.empty((nc ** 3, 2), dtype=torch.float32, device='cuda')
    pm._readout([f, mesh], [out[:, 0], out[:, 1]], [2, 2], [1.0, 0.5], disp=d, lattice=(nc, shift),
                resampler=resampler)
    r0 = pmesh_np.readout(field, pos, [box] * 3, resampler)
    r1 = pmesh_np.readout(ref, pos, [box] * 3, resampler) * 0.5
    assert_allclose(tonp(out[:, 0]), r0, atol=2e-6)
    assert rel_l2(tonp(out[:, 1]), r1) < 2e-6


@pytest.mark.parametrize('stencil', [0, 1])
@pytest.mark.parametrize('n,box', [(32, 64.0), (48, 100.0), (64, 128.0), (128, 256.0), (512, 512.0)])
def test_force_mesh_vs_oracle(G, n, box, stencil):
    """Force meshes: three gradient c2r's (stencil 0) or the 4-point gradient
    stencil of one potential mesh (stencil 1, the same operator)."""
    from fastpm_gb300 import _lib
    from fastpm_gb300.force import longrange_mesh
    old_opt = _lib.query('fpm_get_option', 12)
    _lib.call('fpm_set_option', 12, stencil)
    try:
        _check_force_mesh(G, n, box)
    finally:
        _lib.call('fpm_set_option', 12, old_opt)


def _check_force_mesh(G, n, box):
    from fastpm_gb300 import _lib
    from fastpm_gb300.force import longrange_mesh
    rng = numpy.random.RandomState(n)
    rho = 1.0 + 0.3 * rng.normal(size=(n, n, n))
    pm = device_pm(G, n, box)
    r = G.RealField(pm, torch.from_numpy(rho.astype('f4')).cuda())
    nbar = 0.125
    fmesh, dk = longrange_mesh(r, nbar, factor=1.5 * 0.3)
    opm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[n] * 3)
    odk = opm.create('real', value=rho / nbar).r2c()
    assert rel_l2(tonp(dk.value), odk.value) < 2e-6
    pot = odk.apply(fastpm_np.laplace)
    for d in range(3):
        ref = pot.apply(fastpm_np.gradient(d, order=1)).c2r().value * (1.5 * 0.3)
        assert rel_l2(tonp(fmesh[d]), ref) < (1e-5 if n >= 512 else 5e-6), d
    # the plane-batched kernels (n >= 512) report no timed-out wait
    work = pm._bufs['force_ws']
    assert _lib.query('fpm_workspace_status', _lib.ptr(work), n, 0, 1) == 0
    # a second call on the same workspace gives the same bits
    fmesh2, dk2 = longrange_mesh(r, nbar, factor=1.5 * 0.3)
    assert torch.equal(fmesh, fmesh2) and torch.equal(dk.value, dk2.value)


@pytest.mark.parametrize('resampler', ['cic', 'tsc'])
@pytest.mark.parametrize('nc,B,spread,brick', [(16, 2, 1.0, 0), (12, 2, 4.0, 0), (24, 1, 30.0, 0),
                                               (12, 2, 2.0, 4), (32, 2, 5.0, 8), (64, 2, 8.0, 0),
                                               (256, 2, 3.0, 0)])
@pytest.mark.parametrize('adaptive', [0, 1])
def test_sorted_paint_matches_scatter(G, resampler, nc, B, spread, brick, adaptive):
    """fpm_paint_sorted (binned by mesh brick, each brick stored once) gives the
    atomic scatter's mesh, overwriting what the mesh held; sizes cover bricks
    of 16 (n = 32, 128, 512), 8 (n = 24, and by option 14 at n = 64) and 4 (by
    option at n = 24), and displacements far beyond a brick (spread in cells);
    with the adaptive fixed-point scale (option 18) the bar is 3e-6."""
    from fastpm_gb300 import _lib
    from fastpm_gb300.autotune import options
    old18 = _lib.query('fpm_get_option', 18)
    _lib.call('fpm_set_option', 18, adaptive)
    try:
        with options(paint_brick=brick):
            _check_sorted_paint(G, resampler, nc, B, spread, 3e-6 if adaptive else 1e-6)
    finally:
        _lib.call('fpm_set_option', 18, old18)


def _check_sorted_paint(G, resampler, nc, B, spread, bar=1e-6):
    from fastpm_gb300 import _lib
    n = nc * B
    box = 2.0 * n
    rng = numpy.random.RandomState(nc + B)
    disp = torch.from_numpy(_rand_disp(rng, nc ** 3, spread * box / n)).cuda()
    pm = device_pm(G, n, box, resampler)
    ref = torch.zeros((n, n, n), dtype=torch.float32, device='cuda')
    pm._paint(ref, disp=disp, lattice=(nc, 0.5), resampler=resampler, mass=1.5)
    out = torch.full((n, n, n), float('nan'), dtype=torch.float32, device='cuda')
    pm._paint_sorted(out, disp=disp, lattice=(nc, 0.5), resampler=resampler, mass=1.5)
    assert rel_l2(tonp(out), tonp(ref)) < bar
    assert abs(float(out.double().sum()) - 1.5 * nc ** 3) < 1e-5 * nc ** 3
    # explicit positions (no lattice), outside the box as well
    q = torch.from_numpy(rng.uniform(-box, 2 * box, size=(5000, 3)).astype('f4')).cuda()
    ref.zero_()
    pm._paint(ref, q=q, resampler=resampler)
    pm._paint_sorted(out, q=q, resampler=resampler)
    assert rel_l2(tonp(out), tonp(ref)) < bar
    # no particles: the mesh is overwritten with zeros
    out.fill_(1.0)
    pm._paint_sorted(out, q=q[:0], resampler=resampler)
    assert float(out.abs().max()) == 0.0


@pytest.mark.parametrize('pitch', [1, 2, 3])
def test_sorted_paint_tile_pitch_is_bit_identical(G, pitch):
    """The brick deposit's tile layouts (option 23: 24-word rows for B = 2,
    17- and 19-word rows) hold the same integer sums: the same mesh, bit for
    bit, as the 16-word rows."""
    from fastpm_gb300 import _lib
    nc, B = 32, 2
    n = nc * B
    box = 2.0 * n
    rng = numpy.random.RandomState(41)
    disp = torch.from_numpy(_rand_disp(rng, nc ** 3, 3.0 * box / n)).cuda()
    pm = device_pm(G, n, box, 'tsc')
    ref = torch.full((n, n, n), float('nan'), dtype=torch.float32, device='cuda')
    pm._paint_sorted(ref, disp=disp, lattice=(nc, 0.0))
    old = _lib.query('fpm_get_option', 23)
    _lib.call('fpm_set_option', 23, pitch)
    try:
        out = torch.full((n, n, n), float('nan'), dtype=torch.float32, device='cuda')
        pm._paint_sorted(out, disp=disp, lattice=(nc, 0.0))
    finally:
        _lib.call('fpm_set_option', 23, old)
    assert torch.equal(out, ref)


@pytest.mark.parametrize('resampler', ['cic', 'tsc'])
@pytest.mark.parametrize('adaptive', [0, 1])
def test_sorted_paint_clustered(G, resampler, adaptive):
    """A late-time, halo-like distribution: 90 % of 32^3 particles (B = 2,
    64^3 cells) collapsed onto three points, one inside a brick, one at the
    mesh corner (its windows wrap across the periodic edges into eight
    bricks) and one on a brick corner, so a brick holds more than 10^4
    entries and single cells more than 10^3 full-weight contributions.  With
    option 18 on, the brick
    deposit picks a coarser fixed-point scale at which no cell can wrap; off,
    it accumulates at the finest scale with returning atomics, detects the
    wrap and redoes the brick with float atomics.  Both must match the float64
    oracle and conserve mass."""
    from fastpm_gb300 import _lib
    nc, B, box = 32, 2, 128.0
    n = nc * B
    h = box / n
    rng = numpy.random.RandomState(23)
    q = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3).generate_uniform_particle_grid(shift=0.0)
    targets = numpy.array([[8.4 * h, 7.7 * h, 40.2 * h], [0.0, 0.0, 0.0],
                           [16 * h + 0.3 * h, 32 * h - 0.2 * h, 48 * h]])
    np_ = nc ** 3
    which = rng.randint(0, 10, size=np_)            # 0..8: clustered (90 %), 9: in place
    group = numpy.where(which < 5, 0, numpy.where(which < 7, 1, 2))
    pos = q + rng.normal(scale=0.5 * h, size=(np_, 3))
    for k in range(3):
        sel = (which < 9) & (group == k)
        pos[sel] = targets[k] + rng.normal(scale=0.05 * h, size=(int(sel.sum()), 3))
    disp = (pos - q).astype('f4')
    # a brick of 16^3 cells holds more than 10^4 of these windows
    cells = numpy.floor((q + disp.astype('f8')) / h).astype('i8') % n
    per_brick = numpy.bincount(((cells // 16) * numpy.array([16, 4, 1])).sum(axis=1), minlength=64)
    assert per_brick.max() > 10000
    pm = device_pm(G, n, box, resampler)
    d = torch.from_numpy(disp).cuda()
    ref = pmesh_np.paint(q + disp.astype('f8'), [n] * 3, [box] * 3, resampler)
    old18 = _lib.query('fpm_get_option', 18)
    _lib.call('fpm_set_option', 18, adaptive)
    try:
        out = torch.full((n, n, n), float('nan'), dtype=torch.float32, device='cuda')
        pm._paint_sorted(out, disp=d, lattice=(nc, 0.0), resampler=resampler)
    finally:
        _lib.call('fpm_set_option', 18, old18)
    got = tonp(out).astype('f8')
    assert rel_l2(got, ref) < 1e-5
    assert abs(got.sum() - np_) < 1e-5 * np_
    # every cell, sparse ones next to a cluster included.  Adaptive: the scale
    # of a brick of E entries is about 2^32 / (E w_max), so a cell's rounding
    # error grows with the brick's density; bounded by 2e-7 of the densest
    # cell (measured 9e-8; a numpy emulation of the fixed-point sums gives
    # the same 4.2e-4 absolute).  Checked: the dense bricks wrap and are
    # redone with float32 atomics, whose rounding grows as sqrt(adds) ulps
    # of the cell (10^4 adds: 5e-6 of the densest cell; measured 2.2e-6)
    assert numpy.abs(got - ref).max() < (2e-7 if adaptive else 5e-6) * ref.max()


@pytest.mark.parametrize('resampler', ['cic', 'tsc'])
@pytest.mark.parametrize('case', ['gauss', 'clustered', 'whole', 'explicit'])
def test_sorted_paint_aggregated_is_bit_identical(G, resampler, case):
    """The warp-aggregated brick deposit (option 25: the lanes of a warp whose
    windows start in the same cell sum their contributions and one of them
    issues the shared atomic) holds the same integer sums as the one-atomic-
    per-lane deposit: the same mesh, bit for bit.  Cases: Gaussian
    displacements of 3 cells (few shared anchors), 90 % of the particles on
    three points (most warps aggregate), a mesh of one brick (n = 16: windows
    wrap inside the brick) and explicit positions (no lattice)."""
    from fastpm_gb300 import _lib
    nc, B = (8, 2) if case == 'whole' else (32, 2)
    n = nc * B
    box = 2.0 * n
    h = box / n
    rng = numpy.random.RandomState(57)
    disp = _rand_disp(rng, nc ** 3, 3.0 * h)
    if case == 'clustered':
        which = rng.randint(0, 10, size=nc ** 3)
        q = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[nc] * 3).generate_uniform_particle_grid(shift=0.0)
        targets = numpy.array([[8.4 * h, 7.7 * h, 40.2 * h], [0.0, 0.0, 0.0], [16.3 * h, 31.8 * h, 48 * h]])
        for k in range(3):
            sel = (which < 9) & (which % 3 == k)
            pos = targets[k] + rng.normal(scale=0.05 * h, size=(int(sel.sum()), 3))
            disp[sel] = (pos - q[sel]).astype('f4')
    pm = device_pm(G, n, box, resampler)
    kw = dict(disp=torch.from_numpy(disp).cuda(), lattice=(nc, 0.0))
    if case == 'explicit':
        kw = dict(q=torch.from_numpy(rng.uniform(-box, 2 * box, size=(20000, 3)).astype('f4')).cuda())
    ref = torch.full((n, n, n), float('nan'), dtype=torch.float32, device='cuda')
    pm._paint_sorted(ref, resampler=resampler, **kw)
    old = _lib.query('fpm_get_option', 25)
    _lib.call('fpm_set_option', 25, 1)
    try:
        out = torch.full((n, n, n), float('nan'), dtype=torch.float32, device='cuda')
        pm._paint_sorted(out, resampler=resampler, **kw)
    finally:
        _lib.call('fpm_set_option', 25, old)
    assert torch.equal(out, ref)


@pytest.mark.parametrize('resampler', ['cic', 'tsc'])
@pytest.mark.parametrize('n,box', [(32, 64.0), (48, 100.0), (128, 256.0), (512, 512.0)])
def test_packed_force_mesh_and_readout(G, n, box, resampler):
    """fpm_force_mesh_packed writes the stencil forces and rho * rho_scale
    interleaved (the same float32 values as the three-mesh path, bit for
    bit); fpm_readout_packed interpolates all four like fpm_readout."""
    from fastpm_gb300 import _lib
    from fastpm_gb300.force import longrange_mesh
    old_opt = _lib.query('fpm_get_option', 12)
    _lib.call('fpm_set_option', 12, 1)
    try:
        rng = numpy.random.RandomState(n + 1)
        rho = torch.from_numpy((1.0 + 0.3 * rng.normal(size=(n, n, n))).astype('f4')).cuda()
        pm = device_pm(G, n, box, resampler)
        nbar = 0.125
        fmesh, dk = longrange_mesh(G.RealField(pm, rho), nbar, factor=0.45)
        ws = _lib.query('fpm_force_workspace', n)
        work = pm._scratch('force_ws', ws)
        packed = torch.empty((n, n, n, 4), dtype=torch.float32, device='cuda')
        dk2 = G.ComplexField(pm, empty=True)
        _lib.call('fpm_force_mesh_packed', _lib.ptr(rho), n, box, 1.0 / nbar, 0.45,
                  _lib.ptr(packed), _lib.ptr(dk2.data), _lib.ptr(work), ws, _lib.stream_ptr())
    finally:
        _lib.call('fpm_set_option', 12, old_opt)
    for d in range(3):
        assert torch.equal(packed[..., d], fmesh[d]), d
    assert torch.equal(packed[..., 3], rho * numpy.float32(1.0 / nbar))
    assert torch.equal(dk2.value, dk.value)
    # readout at displaced lattice points (B = 2) and at explicit positions
    nc = n // 2
    disp = torch.from_numpy(_rand_disp(rng, nc ** 3, 1.5)).cuda()
    F0 = torch.empty((nc ** 3, 3), dtype=torch.float32, device='cuda')
    R0 = torch.empty(nc ** 3, dtype=torch.float32, device='cuda')
    pm._readout([fmesh[0], fmesh[1], fmesh[2], rho], [F0[:, 0], F0[:, 1], F0[:, 2], R0],
                [3, 3, 3, 1], [1.0, 1.0, 1.0, 1.0 / nbar], disp=disp, lattice=(nc, 0.25))
    F1 = torch.empty_like(F0)
    R1 = torch.empty_like(R0)
    _lib.call('fpm_readout_packed', _lib.ptr(packed), n, box, _lib.ptr(disp), None, nc ** 3, nc,
              0.25, _lib.FPM_WINDOW[resampler], _lib.ptr(F1), _lib.ptr(R1), _lib.stream_ptr())
    assert rel_l2(tonp(F1), tonp(F0)) < 1e-6
    assert rel_l2(tonp(R1), tonp(R0)) < 1e-6
    # in mesh-brick order from a sorted paint's particle lists: the same bits
    scratch = torch.empty((n, n, n), dtype=torch.float32, device='cuda')
    bins = pm._paint_sorted(scratch, disp=disp, lattice=(nc, 0.25))
    F4 = torch.full_like(F0, float('nan'))
    R4 = torch.full_like(R0, float('nan'))
    _lib.call('fpm_readout_packed_sorted', _lib.ptr(packed), n, box, _lib.ptr(disp), None, nc ** 3, nc,
              0.25, _lib.FPM_WINDOW[resampler], _lib.ptr(F4), _lib.ptr(R4), bins['brick'],
              _lib.ptr(bins['work']), bins['bytes'], _lib.stream_ptr())
    assert torch.equal(F4, F1) and torch.equal(R4, R1)
    # the same with each brick's cells staged in shared memory (option 16)
    old16 = _lib.query('fpm_get_option', 16)
    _lib.call('fpm_set_option', 16, 1 - old16)
    try:
        F4.fill_(float('nan'))
        R4.fill_(float('nan'))
        _lib.call('fpm_readout_packed_sorted', _lib.ptr(packed), n, box, _lib.ptr(disp), None, nc ** 3, nc,
                  0.25, _lib.FPM_WINDOW[resampler], _lib.ptr(F4), _lib.ptr(R4), bins['brick'],
                  _lib.ptr(bins['work']), bins['bytes'], _lib.stream_ptr())
    finally:
        _lib.call('fpm_set_option', 16, old16)
    assert torch.equal(F4, F1) and torch.equal(R4, R1)
    # each brick's particles sorted by window row or cell first (option 22):
    # the same per-particle sums, bit for bit
    old22 = _lib.query('fpm_get_option', 22)
    for srt in (1, 2):
        _lib.call('fpm_set_option', 22, srt)
        try:
            F4.fill_(float('nan'))
            R4.fill_(float('nan'))
            _lib.call('fpm_readout_packed_sorted', _lib.ptr(packed), n, box, _lib.ptr(disp), None, nc ** 3,
                      nc, 0.25, _lib.FPM_WINDOW[resampler], _lib.ptr(F4), _lib.ptr(R4), bins['brick'],
                      _lib.ptr(bins['work']), bins['bytes'], _lib.stream_ptr())
        finally:
            _lib.call('fpm_set_option', 22, old22)
        assert torch.equal(F4, F1) and torch.equal(R4, R1), srt
    # a force array that is only 4-byte aligned (three 32-bit stores per particle)
    Fm = torch.full((3 * nc ** 3 + 1,), float('nan'), dtype=torch.float32, device='cuda')[1:].view(nc ** 3, 3)
    _lib.call('fpm_readout_packed_sorted', _lib.ptr(packed), n, box, _lib.ptr(disp), None, nc ** 3, nc,
              0.25, _lib.FPM_WINDOW[resampler], _lib.ptr(Fm), None, bins['brick'],
              _lib.ptr(bins['work']), bins['bytes'], _lib.stream_ptr())
    assert torch.equal(Fm, F1)
    # two threads per particle (option 20): the same terms, summed in two halves
    old20 = _lib.query('fpm_get_option', 20)
    for pair in (0, 1):
        _lib.call('fpm_set_option', 20, pair)
        try:
            F4.fill_(float('nan'))
            R4.fill_(float('nan'))
            _lib.call('fpm_readout_packed_sorted', _lib.ptr(packed), n, box, _lib.ptr(disp), None, nc ** 3,
                      nc, 0.25, _lib.FPM_WINDOW[resampler], _lib.ptr(F4), _lib.ptr(R4), bins['brick'],
                      _lib.ptr(bins['work']), bins['bytes'], _lib.stream_ptr())
        finally:
            _lib.call('fpm_set_option', 20, old20)
        assert rel_l2(tonp(F4), tonp(F1)) < 1e-6 and rel_l2(tonp(R4), tonp(R1)) < 1e-6
    # forces straight from the potential by brick (no force mesh): the same
    # operator, summed in another order
    F5 = torch.full_like(F0, float('nan'))
    R5 = torch.full_like(R0, float('nan'))
    dk5 = G.ComplexField(pm, empty=True)
    _lib.call('fpm_force_readout_sorted', _lib.ptr(rho), n, box, 1.0 / nbar, 0.45, _lib.ptr(dk5.data),
              _lib.ptr(work), ws, _lib.ptr(disp), None, nc ** 3, nc, 0.25, _lib.FPM_WINDOW[resampler],
              _lib.ptr(F5), _lib.ptr(R5), bins['brick'], _lib.ptr(bins['work']), bins['bytes'],
              _lib.stream_ptr())
    assert rel_l2(tonp(F5), tonp(F1)) < 2e-6
    assert rel_l2(tonp(R5), tonp(R1)) < 1e-6
    assert torch.equal(dk5.value, dk.value)
    q = torch.from_numpy(rng.uniform(-box, 2 * box, size=(1000, 3)).astype('f4')).cuda()
    F2 = torch.empty((1000, 3), dtype=torch.float32, device='cuda')
    _lib.call('fpm_readout_packed', _lib.ptr(packed), n, box, None, _lib.ptr(q), 1000, 0, 0.0,
              _lib.FPM_WINDOW[resampler], _lib.ptr(F2), None, _lib.stream_ptr())
    F3 = torch.empty_like(F2)
    pm._readout([fmesh[0], fmesh[1], fmesh[2]], [F3[:, 0], F3[:, 1], F3[:, 2]], [3, 3, 3],
                [1.0, 1.0, 1.0], q=q)
    assert rel_l2(tonp(F2), tonp(F3)) < 1e-6
    # the blocked layout: the packed mesh's values, bit for bit, in 2x2x2-cell
    # blocks; its readout (four threads per particle, partial sums combined by
    # shuffles) sums the same terms in another order
    old12 = _lib.query('fpm_get_option', 12)
    _lib.call('fpm_set_option', 12, 1)
    try:
        blocked = torch.full((n ** 3, 4), float('nan'), dtype=torch.float32, device='cuda')
        dk6 = G.ComplexField(pm, empty=True)
        _lib.call('fpm_force_mesh_blocked', _lib.ptr(rho), n, box, 1.0 / nbar, 0.45, _lib.ptr(blocked),
                  _lib.ptr(dk6.data), _lib.ptr(work), ws, _lib.stream_ptr())
    finally:
        _lib.call('fpm_set_option', 12, old12)
    h = n // 2
    expect = packed.view(h, 2, h, 2, h, 2, 4).permute(0, 2, 4, 1, 3, 5, 6).reshape(n ** 3, 4)
    assert torch.equal(blocked, expect)
    assert torch.equal(dk6.value, dk.value)
    F6 = torch.full_like(F0, float('nan'))
    R6 = torch.full_like(R0, float('nan'))
    _lib.call('fpm_readout_blocked_sorted', _lib.ptr(blocked), n, box, _lib.ptr(disp), None, nc ** 3, nc,
              0.25, _lib.FPM_WINDOW[resampler], _lib.ptr(F6), _lib.ptr(R6), bins['brick'],
              _lib.ptr(bins['work']), bins['bytes'], _lib.stream_ptr())
    assert rel_l2(tonp(F6), tonp(F1)) < 1e-6
    assert rel_l2(tonp(R6), tonp(R1)) < 1e-6
    # explicit positions, most of them outside the box (wrapped)
    bq = pm._paint_sorted(scratch, q=q)
    F7 = torch.full_like(F2, float('nan'))
    _lib.call('fpm_readout_blocked_sorted', _lib.ptr(blocked), n, box, None, _lib.ptr(q), 1000, 0, 0.0,
              _lib.FPM_WINDOW[resampler], _lib.ptr(F7), None, bq['brick'], _lib.ptr(bq['work']),
              bq['bytes'], _lib.stream_ptr())
    assert rel_l2(tonp(F7), tonp(F2)) < 1e-6
    # argument checks: an odd offset (not 128-byte aligned) is refused
    rc = _lib.query('fpm_readout_blocked_sorted', ctypes.c_void_p(blocked.data_ptr() + 16), n, box,
                    _lib.ptr(disp), None, nc ** 3, nc, 0.25, _lib.FPM_WINDOW[resampler], _lib.ptr(F6), None,
                    bins['brick'], _lib.ptr(bins['work']), bins['bytes'], _lib.stream_ptr())
    assert rc == 1   # FPM_ERR_ARG


@pytest.mark.parametrize('resampler', ['cic', 'tsc'])
@pytest.mark.parametrize('nc,B', [(16, 2), (24, 2), (64, 1), (256, 2)])
def test_batched_sorted_paint_packed_force_readout(G, resampler, nc, B):
    """The slot-batched forms (serving) agree with the single-simulation calls
    slot by slot; an inactive slot is left untouched.  At n = 512 the batched
    force runs the TMA-pipelined y / x passes slot by slot, and its time-out
    status word stays clear."""
    from fastpm_gb300 import _lib
    n, S = nc * B, 3
    box = 3.0 * n
    np_ = nc ** 3
    rng = numpy.random.RandomState(nc)
    disp = torch.from_numpy(rng.normal(scale=2.0 * box / n, size=(S, np_, 3)).astype('f4')).cuda()
    active = torch.tensor([1, 0, 1], dtype=torch.int32, device='cuda')
    factor = torch.tensor([0.45, 0.5, 0.39], dtype=torch.float32, device='cuda')
    pm = device_pm(G, n, box, resampler)
    win = _lib.FPM_WINDOW[resampler]
    st = _lib.stream_ptr()
    # paint
    rho = torch.full((S, n, n, n), -7.0, dtype=torch.float32, device='cuda')
    ws = _lib.query('fpm_paint_sorted_batch_workspace', n, np_, S)
    work = torch.empty(ws, dtype=torch.uint8, device='cuda')
    _lib.call('fpm_paint_sorted_batch', _lib.ptr(rho), n ** 3, n, box, _lib.ptr(disp), 3 * np_, np_, nc,
              0.0, win, 1.0, S, _lib.ptr(active), _lib.ptr(work), ws, st)
    assert float(rho[1].min()) == -7.0 and float(rho[1].max()) == -7.0
    nbar = np_ / float(n) ** 3
    # force
    packed = torch.full((S, n ** 3, 4), -3.0, dtype=torch.float32, device='cuda')
    wb = _lib.query('fpm_force_batch_workspace', n, S)
    fw = torch.zeros(wb, dtype=torch.uint8, device='cuda')
    _lib.call('fpm_force_mesh_batch_packed', _lib.ptr(rho), n ** 3, n, box, 1.0 / nbar, _lib.ptr(factor),
              _lib.ptr(packed), n ** 3, _lib.ptr(fw), wb, S, _lib.ptr(active), st)
    assert float(packed[1].min()) == -3.0 and float(packed[1].max()) == -3.0
    at = 2 * S * n * n * _lib.query('fpm_complex_row', n) * 8    # the status word (n >= 512)
    assert int(fw[at:at + 4].view(torch.int32).item()) == 0
    # readout
    F = torch.zeros((S, np_, 3), dtype=torch.float32, device='cuda')
    R = torch.zeros((S, np_), dtype=torch.float32, device='cuda')
    _lib.call('fpm_readout_packed_batch', _lib.ptr(packed), n ** 3, n, box, _lib.ptr(disp), 3 * np_, np_,
              nc, 0.0, win, _lib.ptr(F), 3 * np_, _lib.ptr(R), np_, S, _lib.ptr(active), st)
    assert float(F[1].abs().max()) == 0.0
    single_ws = _lib.query('fpm_force_workspace', n)
    sw = torch.empty(single_ws, dtype=torch.uint8, device='cuda')
    for s in (0, 2):
        r1 = torch.zeros((n, n, n), dtype=torch.float32, device='cuda')
        pm._paint(r1, disp=disp[s], lattice=(nc, 0.0), resampler=resampler)
        # the sorted paint's fixed-point scale is 2^21 for these dense bricks (B = 1)
        assert rel_l2(tonp(rho[s]), tonp(r1)) < 3e-6
        p1 = torch.empty((n ** 3, 4), dtype=torch.float32, device='cuda')
        _lib.call('fpm_force_mesh_packed', _lib.ptr(rho[s]), n, box, 1.0 / nbar, float(factor[s]),
                  _lib.ptr(p1), None, _lib.ptr(sw), single_ws, st)
        assert rel_l2(tonp(packed[s]), tonp(p1)) < 1e-6
        F1 = torch.empty((np_, 3), dtype=torch.float32, device='cuda')
        R1 = torch.empty(np_, dtype=torch.float32, device='cuda')
        _lib.call('fpm_readout_packed', _lib.ptr(p1), n, box, _lib.ptr(disp[s]), None, np_, nc, 0.0, win,
                  _lib.ptr(F1), _lib.ptr(R1), st)
        assert rel_l2(tonp(F[s]), tonp(F1)) < 1e-6
        assert rel_l2(tonp(R[s]), tonp(R1)) < 1e-6


@pytest.mark.parametrize('n,box', [(32, 64.0), (48, 96.0), (64, 128.0), (512, 512.0)])
def test_lpt_meshes_vs_oracle(G, n, box):
    from fastpm_gb300 import _lib
    from fastpm_gb300.force import lpt2source
    opm = pmesh_np.ParticleMesh(BoxSize=box, Nmesh=[n] * 3)
    wn = opm.generate_whitenoise(5, type='complex')
    k2 = sum(k ** 2 for k in opm.k)
    dlin = opm.create('complex', value=wn.value * numpy.exp(-k2 * 4.0))
    pm = device_pm(G, n, box)
    gd = pm.complex_from(dlin.value)
    ws = _lib.query('fpm_lpt_workspace', n)
    work = torch.empty(ws, dtype=torch.uint8, device='cuda')
    m = torch.empty((3, n, n, n), dtype=torch.float32, device='cuda')
    _lib.call('fpm_lpt1_mesh', _lib.ptr(gd.data), n, box, _lib.ptr(m[0]), _lib.ptr(m[1]),
              _lib.ptr(m[2]), _lib.ptr(work), ws, _lib.stream_ptr())
    for d in range(3):
        ref = dlin.apply(fastpm_np.laplace).apply(fastpm_np.gradient(d, 1)).c2r().value
        assert rel_l2(tonp(m[d]), ref) < 5e-6
    src = lpt2source(gd)
    ref = fastpm_np.lpt2source(dlin)
    assert rel_l2(tonp(src.value), ref.value) < 1e-5


def test_kick_drift_kahan(G):
    """200 kick / drift pairs: the compensated float32 state tracks float64 sums."""
    from fastpm_gb300 import _lib
    rng = numpy.random.RandomState(3)
    n3 = 3 * 100000
    p0 = rng.normal(size=n3).astype('f4')
    s0 = (rng.normal(size=n3) * 10).astype('f4')
    f = rng.normal(size=n3).astype('f4')
    P, S, F = (torch.from_numpy(x).cuda() for x in (p0, s0, f))
    Pc = torch.zeros(n3, dtype=torch.bfloat16, device='cuda')   # bfloat16 compensation terms
    Sc = torch.zeros(n3, dtype=torch.bfloat16, device='cuda')
    pe, se = p0.astype('f8'), s0.astype('f8')
    for i in range(200):
        fk, fd = 1e-3 * (1 + i % 3), 2e-3
        _lib.call('fpm_kick', _lib.ptr(P), _lib.ptr(Pc), _lib.ptr(F), n3, fk, _lib.stream_ptr())
        _lib.call('fpm_drift', _lib.ptr(S), _lib.ptr(Sc), _lib.ptr(P), n3, fd, _lib.stream_ptr())
        pe = pe + float(numpy.float32(fk)) * f.astype('f8')
        se = se + float(numpy.float32(fd)) * pe
    # compensated sums stay within a few float32 ulps of the float64 sums
    assert numpy.abs(tonp(P) - pe).max() < 4 * numpy.spacing(numpy.float32(numpy.abs(pe).max()))
    assert numpy.abs(tonp(S) - se).max() < 8 * numpy.spacing(numpy.float32(numpy.abs(se).max()))
    # the fused kick+drift gives the same as kick then drift
    P2, S2, Pc2, Sc2 = P.clone(), S.clone(), Pc.clone(), Sc.clone()
    _lib.call('fpm_kick', _lib.ptr(P), _lib.ptr(Pc), _lib.ptr(F), n3, 1e-3, _lib.stream_ptr())
    _lib.call('fpm_drift', _lib.ptr(S), _lib.ptr(Sc), _lib.ptr(P), n3, 2e-3, _lib.stream_ptr())
    _lib.call('fpm_kick_drift', _lib.ptr(P2), _lib.ptr(Pc2), _lib.ptr(S2), _lib.ptr(Sc2), _lib.ptr(F),
              n3, 1e-3, 0.0, 1, 2e-3, _lib.stream_ptr())
    assert torch.equal(P, P2) and torch.equal(S, S2) and torch.equal(Sc, Sc2)
    # two kicks and a drift, fused, equal three separate launches bit for bit
    _lib.call('fpm_kick', _lib.ptr(P), _lib.ptr(Pc), _lib.ptr(F), n3, 3e-3, _lib.stream_ptr())
    _lib.call('fpm_kick', _lib.ptr(P), _lib.ptr(Pc), _lib.ptr(F), n3, 5e-3, _lib.stream_ptr())
    _lib.call('fpm_drift', _lib.ptr(S), _lib.ptr(Sc), _lib.ptr(P), n3, 7e-3, _lib.stream_ptr())
    _lib.call('fpm_kick_drift', _lib.ptr(P2), _lib.ptr(Pc2), _lib.ptr(S2), _lib.ptr(Sc2), _lib.ptr(F),
              n3, 3e-3, 5e-3, 2, 7e-3, _lib.stream_ptr())
    for a, b in ((P, P2), (Pc, Pc2), (S, S2), (Sc, Sc2)):
        assert torch.equal(a, b)


@pytest.mark.parametrize('n', [32, 48, 64])
def test_power_vs_oracle(G, n):
    from fastpm_gb300 import power
    rng = numpy.random.RandomState(n)
    f = 1.0 + 0.1 * rng.normal(size=(n, n, n))
    pm = device_pm(G, n, 64.0)
    r = G.RealField(pm, torch.from_numpy(f.astype('f4')).cuda())
    k, p = power(r.r2c(), boxsize=64.0)
    rk, rp = power_np.power(f.copy(), boxsize=64.0)
    ok = numpy.isfinite(rp)
    assert_allclose(k[ok], rk[ok], rtol=1e-10)
    assert_allclose(p[ok], rp[ok], rtol=2e-5)


def test_write_power_text(G, tmp_path):
    """write_power writes main.py:81-92's columns (k p N p/D**2) of the device P(k)."""
    from fastpm_gb300.power import write_power
    from fastpm_gb300.background import MatterDominated
    n = 32
    rng = numpy.random.RandomState(5)
    f = 1.0 + 0.1 * rng.normal(size=(n, n, n))
    pm = device_pm(G, n, 64.0)
    r = G.RealField(pm, torch.from_numpy(f.astype('f4')).cuda())
    path = write_power(str(tmp_path / 'power.txt'), r, a=0.5, cosmology=G.Planck15)
    # savetxt's `comments` prefixes a header only: like the reference's file, no comment line
    assert not open(path).readline().startswith('#')
    t = numpy.loadtxt(path)
    rk, rp = power_np.power(f.copy(), boxsize=64.0)
    ok = numpy.isfinite(rp) & (rp > 0)
    assert_allclose(t[:, 0], rk[ok], rtol=1e-10)
    assert_allclose(t[:, 1], rp[ok], rtol=2e-5)
    D = MatterDominated(G.Planck15.Om0, a=[0.5, 1.0]).D1(0.5)
    assert_allclose(t[:, 3], t[:, 1] / D ** 2, rtol=1e-12)
    assert (t[:, 2] > 0).all()


@pytest.mark.parametrize('resampler', ['cic', 'tsc'])
@pytest.mark.parametrize('nc,B', [(16, 2), (32, 1), (64, 2)])
@pytest.mark.parametrize('bucket', [0, 1, 2])
def test_kick_drift_bin_then_counted_paint(G, resampler, nc, B, bucket):
    """fpm_kick_drift_bin (kick-drift + brick counts of the new positions) then
    fpm_paint_sorted_counted gives the same state and mesh, bit for bit, as
    fpm_kick_drift then fpm_paint_sorted, and the particle lists it leaves give
    the brick-order readout the same forces: with the lists filled from brick
    keys and ranks (option 26 = 0), through buckets (1, the default), and
    through buckets of 2 home entries, which overflow in every brick and make
    the paint recount (2)."""
    from fastpm_gb300 import _lib
    old26 = _lib.query('fpm_get_option', 26)
    _lib.call('fpm_set_option', 26, bucket)
    try:
        _check_kick_drift_bin_then_counted_paint(G, resampler, nc, B)
    finally:
        _lib.call('fpm_set_option', 26, old26)


def _check_kick_drift_bin_then_counted_paint(G, resampler, nc, B):
    from fastpm_gb300 import _lib
    n = nc * B
    box = 2.0 * n
    np_ = nc ** 3
    rng = numpy.random.RandomState(nc * B)
    mk = lambda s: torch.from_numpy(rng.normal(scale=s, size=(np_, 3)).astype('f4')).cuda()
    S, P, F = mk(2.0), mk(1.0), mk(0.5)
    Sc, Pc = mk(1e-7).to(torch.bfloat16), mk(1e-7).to(torch.bfloat16)
    pm = device_pm(G, n, box, resampler)
    st = _lib.stream_ptr()
    a = [x.clone() for x in (S, P, Sc, Pc)]
    b = [x.clone() for x in (S, P, Sc, Pc)]
    _lib.call('fpm_kick_drift', _lib.ptr(a[1]), _lib.ptr(a[3]), _lib.ptr(a[0]), _lib.ptr(a[2]), _lib.ptr(F),
              3 * np_, 0.37, 0.21, 2, 0.83, st)
    m0 = torch.empty((n, n, n), dtype=torch.float32, device='cuda')
    bins = pm._paint_sorted(m0, disp=a[0], lattice=(nc, 0.0), resampler=resampler)
    # a packed mesh to read out in brick order from the paint's lists
    g = torch.Generator(device='cuda').manual_seed(nc)
    packed = torch.randn((n ** 3, 4), generator=g, device='cuda')

    def readout(disp):
        Fo = torch.full((np_, 3), float('nan'), device='cuda')
        Ro = torch.full((np_,), float('nan'), device='cuda')
        _lib.call('fpm_readout_packed_sorted', _lib.ptr(packed), n, box, _lib.ptr(disp), None, np_, nc, 0.0,
                  _lib.FPM_WINDOW[resampler], _lib.ptr(Fo), _lib.ptr(Ro), bins['brick'], _lib.ptr(bins['work']),
                  bins['bytes'], st)
        return Fo, Ro
    F0, R0 = readout(a[0])
    work, ws = pm._paint_work(np_)
    _lib.call('fpm_kick_drift_bin', _lib.ptr(b[1]), _lib.ptr(b[3]), _lib.ptr(b[0]), _lib.ptr(b[2]),
              _lib.ptr(F), np_, 0.37, 0.21, 2, 0.83, n, box, None, nc, 0.0, _lib.FPM_WINDOW[resampler],
              _lib.ptr(work), ws, st)
    m1 = torch.full((n, n, n), float('nan'), dtype=torch.float32, device='cuda')
    pm._paint_sorted(m1, disp=b[0], lattice=(nc, 0.0), resampler=resampler, counted=True)
    F1, R1 = readout(b[0])
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    assert torch.equal(m0, m1)
    assert torch.equal(F0, F1) and torch.equal(R0, R1)


@pytest.mark.parametrize('misaligned', [False, True])
@pytest.mark.parametrize('bucket', [0, 1, 2])
def test_kick_drift_bin_explicit_positions(G, misaligned, bucket):
    """fpm_kick_drift_bin at explicit positions for a particle count that is
    not a multiple of the warp (the vector path's scalar tail), and on arrays
    that are not 16-byte aligned (the scalar kernel): the same bits as
    fpm_kick_drift then fpm_paint_sorted, with each list mode of option 26."""
    from fastpm_gb300 import _lib
    old26 = _lib.query('fpm_get_option', 26)
    _lib.call('fpm_set_option', 26, bucket)
    try:
        _check_kick_drift_bin_explicit(G, misaligned)
    finally:
        _lib.call('fpm_set_option', 26, old26)


def _check_kick_drift_bin_explicit(G, misaligned):
    from fastpm_gb300 import _lib
    n, box, np_ = 32, 64.0, 1001
    rng = numpy.random.RandomState(5)
    off = 1 if misaligned else 0

    def mk(scale, dtype=torch.float32):
        t = torch.from_numpy(rng.normal(scale=scale, size=3 * np_ + off).astype('f4')).cuda().to(dtype)
        return t[off:].view(np_, 3)
    S, P, F = mk(2.0), mk(1.0), mk(0.5)
    Sc, Pc = mk(1e-7, torch.bfloat16), mk(1e-7, torch.bfloat16)   # bfloat16 compensation terms
    q = torch.from_numpy(rng.uniform(-box, 2 * box, size=(np_, 3)).astype('f4')).cuda()
    pm = device_pm(G, n, box, 'tsc')
    st = _lib.stream_ptr()
    a = [x.clone() for x in (S, P, Sc, Pc)]
    b = [torch.empty(3 * np_ + off, dtype=x.dtype, device='cuda')[off:].view(np_, 3) for x in (S, P, Sc, Pc)]
    for x, y in zip(b, (S, P, Sc, Pc)):
        x.copy_(y)
    _lib.call('fpm_kick_drift', _lib.ptr(a[1]), _lib.ptr(a[3]), _lib.ptr(a[0]), _lib.ptr(a[2]), _lib.ptr(F),
              3 * np_, 0.37, 0.21, 1, 0.83, st)
    m0 = torch.empty((n, n, n), dtype=torch.float32, device='cuda')
    pm._paint_sorted(m0, q=q, disp=a[0])
    work, ws = pm._paint_work(np_)
    _lib.call('fpm_kick_drift_bin', _lib.ptr(b[1]), _lib.ptr(b[3]), _lib.ptr(b[0]), _lib.ptr(b[2]),
              _lib.ptr(F), np_, 0.37, 0.21, 1, 0.83, n, box, _lib.ptr(q), 0, 0.0, _lib.FPM_WINDOW['tsc'],
              _lib.ptr(work), ws, st)
    m1 = torch.full((n, n, n), float('nan'), dtype=torch.float32, device='cuda')
    pm._paint_sorted(m1, q=q, disp=b[0], counted=True)
    for x, y in zip(a, b):
        assert torch.equal(x, y)
    assert torch.equal(m0, m1)


def test_workspace_status_word_contract(G):
    """The status word at the end of a force workspace is only ever set by the
    kernels: a buffer of garbage reads as a timeout until cleared, a zeroed one
    (what ParticleMesh scratch buffers are) reads clear, and a force run on a
    cleared workspace leaves it clear."""
    from fastpm_gb300 import _lib
    from fastpm_gb300.force import longrange_mesh
    n = 512
    ws = _lib.query('fpm_force_workspace', n)
    junk = torch.full((ws,), 0xFF, dtype=torch.uint8, device='cuda')
    assert _lib.query('fpm_workspace_status', _lib.ptr(junk), n, 0, 1) == 6   # FPM_ERR_TIMEOUT, cleared
    assert _lib.query('fpm_workspace_status', _lib.ptr(junk), n, 0, 0) == 0
    del junk
    pm = device_pm(G, n, float(n))
    assert _lib.query('fpm_workspace_status', _lib.ptr(pm._scratch('force_ws', ws)), n, 0, 0) == 0
    rho = G.RealField(pm, torch.ones((n, n, n), device='cuda'))
    longrange_mesh(rho, 0.125, 0.45)
    torch.cuda.synchronize()
    assert _lib.query('fpm_workspace_status', _lib.ptr(pm._bufs['force_ws']), n, 0, 0) == 0


@pytest.mark.parametrize('n', [512, 1024])
@pytest.mark.parametrize('variant', [(17, 0), (17, 1), (19, 1), (24, 0), (24, 1), (24, 2), (24, 3)])
def test_pipelined_column_passes_are_bit_identical(G, n, variant):
    """The TMA-pipelined y / x / z passes (the x pass with either line plan at
    n = 1024, option 17; the single-buffer passes at two CTAs per SM, option
    19; the two-stage radix-32 plans, option 24) agree with the plain ones
    (they use other line plans, so only to float32 rounding)."""
    from fastpm_gb300 import _lib
    from fastpm_gb300.force import longrange_mesh
    pm = device_pm(G, n, float(n))
    g = torch.Generator(device='cuda').manual_seed(n)
    rho = G.RealField(pm, 1 + 0.2 * torch.randn((n, n, n), generator=g, device='cuda'))
    old = [_lib.query('fpm_get_option', k) for k in (11, 13, 17, 19, 24)]
    try:
        _lib.call('fpm_set_option', 11, 0)
        _lib.call('fpm_set_option', 13, 0)
        _lib.call('fpm_set_option', 19, 0)
        f0, d0 = longrange_mesh(rho, 0.125, 0.45)
        _lib.call('fpm_set_option', 11, 1)
        _lib.call('fpm_set_option', 13, 1)
        _lib.call('fpm_set_option', variant[0], variant[1])
        f1, d1 = longrange_mesh(rho, 0.125, 0.45)
        # without the delta_k copy in the x pass
        f2, _ = longrange_mesh(rho, 0.125, 0.45, want_delta_k=False)
        torch.cuda.synchronize()
        assert _lib.query('fpm_workspace_status', _lib.ptr(pm._bufs['force_ws']), n, 0, 1) == 0
    finally:
        _lib.call('fpm_set_option', 11, old[0])
        _lib.call('fpm_set_option', 13, old[1])
        _lib.call('fpm_set_option', 17, old[2])
        _lib.call('fpm_set_option', 19, old[3])
        _lib.call('fpm_set_option', 24, old[4])
    for d in range(3):
        assert rel_l2(tonp(f2[d]), tonp(f0[d])) < 5e-6
    for d in range(3):
        assert rel_l2(tonp(f1[d]), tonp(f0[d])) < 5e-6
    assert rel_l2(tonp(d1.value), tonp(d0.value)) < 2e-6
