"""Oracle self-checks that need no reference run."""
import numpy
from numpy.testing import assert_allclose, assert_array_equal

from oracle import pmesh_np, fastpm_np


def test_philox_known_answer():
    # Random123 known-answer vector for philox4x32_10, counter 0, key 0
    out = pmesh_np.philox4x32_10(0, 0, 0, 0, 0, 0)
    assert [int(x) for x in out] == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]


def test_whitenoise_hermitian_and_variance():
    n = 32
    v = pmesh_np.whitenoise([n] * 3, 7)
    real = numpy.fft.irfftn(v, s=(n, n, n), axes=(0, 1, 2))
    back = numpy.fft.rfftn(real)
    assert_allclose(back, v, atol=1e-12)   # Hermitian => lossless round trip
    assert abs(numpy.mean(abs(v[1:, 1:, 1:-1]) ** 2) - 1) < 0.05
    assert v[0, 0, 0] == 0
    u = pmesh_np.whitenoise([n] * 3, 7, unitary=True)
    assert_allclose(abs(u[1:, 1:, 1:-1]), 1.0)


def test_c2r_r2c_identity():
    """fastpm/tests/test_kernel.py:7-13 on the oracle mesh."""
    pm = pmesh_np.ParticleMesh(BoxSize=128., Nmesh=[8, 8, 8])
    data = pm.generate_whitenoise(type='real', seed=333)
    for d in range(3):
        g1 = data.r2c().apply(fastpm_np.gradient(d))
        assert_allclose(g1.c2r().r2c(), g1, atol=1e-9)


def test_paint_conserves_mass_and_readout_is_transpose():
    rng = numpy.random.RandomState(1)
    pos = rng.uniform(-10, 30, size=(500, 3))
    for res in ('cic', 'tsc'):
        m = pmesh_np.paint(pos, [8] * 3, [20.0] * 3, res)
        assert abs(m.sum() - 500) < 1e-9
        f = rng.normal(size=(8, 8, 8))
        # <paint(delta_p), f> == <delta_p, readout(f)>
        lhs = (m * f).sum()
        rhs = pmesh_np.readout(f, pos, [20.0] * 3, res).sum()
        assert abs(lhs - rhs) < 1e-9 * abs(lhs)


def test_cell_keys_lattice_simple():
    key, frac = pmesh_np.cell_keys_lattice(numpy.zeros((8, 3)), 2, 0.0, 4, 4.0, 'cic')
    # lattice (i, j, k) at 2 * (i, j, k) cells
    assert_array_equal(key, [0, 2, 8, 10, 32, 34, 40, 42])
    assert (frac == 0).all()
