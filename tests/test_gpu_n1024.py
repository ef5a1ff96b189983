"""The FFTs and the force mesh at n = 1024 (the benchmarked mesh) against an
independent float64 reference: torch.fft (cuFFT) in complex128 on the same
float32 input, with the pmesh normalisation (r2c carries 1/N) and the
laplace x order-1 gradient transfer of fastpm/force/kernels.py:3-24 applied
in float64.  The comparator lives in the test only (tests/f64_device.py).

Bars (float32 engine, 1024-point transforms): relative L2 error <= 2e-6 for
r2c / c2r and delta_k, <= 1e-5 for the forces (float32 rounding of a
potential whose Fourier weights span 1/k^2 over six decades).
"""
import numpy
import pytest
import torch

from tests import f64_device as F
from tests.helpers import tonp

pytestmark = pytest.mark.gpu

N = 1024


def rel(a, b):
    return float(torch.linalg.norm((a - b).reshape(-1)) / torch.linalg.norm(b.reshape(-1)))


@pytest.fixture(scope='module')
def field():
    import fastpm_gb300 as G
    pm = G.ParticleMesh(BoxSize=float(N), Nmesh=[N] * 3, resampler='tsc')
    g = torch.Generator(device='cuda').manual_seed(1024)
    rho = 1 + 0.3 * torch.randn((N, N, N), generator=g, device='cuda')
    yield G, pm, rho
    torch.cuda.empty_cache()


def test_r2c_c2r_n1024_vs_float64(field):
    G, pm, rho = field
    ck = G.RealField(pm, rho).r2c()
    ref = F.r2c(rho.double())
    nz = N // 2 + 1
    assert rel(ck.value.to(torch.complex128), ref) < 2e-6
    del ref
    back = ck.c2r()
    assert rel(back.value.double(), rho.double()) < 2e-6
    # c2r of the engine's own spectrum against the float64 inverse of it
    ref_r = F.c2r(ck.value.to(torch.complex128), N)
    assert rel(back.value.double(), ref_r) < 2e-6
    assert ck.value.shape[-1] == nz


@pytest.mark.parametrize('packed,plan2', [(True, 3), (False, 3), (True, 0), (True, 1), (True, 2)])
def test_force_mesh_n1024_vs_float64(field, packed, plan2):
    """fpm_force_mesh_packed (stencil into the float4 mesh, the default path)
    and fpm_force_mesh (three meshes): delta_k, the three force components and
    (packed) the density channel against the float64 transfer.  plan2 (option
    24): the y / x pipelines with the two-stage radix-32 line plan, with the
    exchanges in two areas (1) or in the padded work area alone (2), the y
    passes alone (3, the default) or neither (0)."""
    from fastpm_gb300 import _lib
    old24 = _lib.query('fpm_get_option', 24)
    _lib.call('fpm_set_option', 24, plan2)
    try:
        _check_force_mesh_n1024(field, packed)
    finally:
        _lib.call('fpm_set_option', 24, old24)


def _check_force_mesh_n1024(field, packed):
    from fastpm_gb300 import _lib
    from fastpm_gb300.force import longrange_mesh
    G, pm, rho = field
    nbar, factor, box = 0.125, 1.5 * 0.3089, float(N)
    if packed:
        ws = _lib.query('fpm_force_workspace', N)
        work = pm._scratch('force_ws', ws)
        out = torch.empty((N, N, N, 4), dtype=torch.float32, device='cuda')
        dk = G.ComplexField(pm, empty=True)
        _lib.call('fpm_force_mesh_packed', _lib.ptr(rho), N, box, 1.0 / nbar, factor, _lib.ptr(out),
                  _lib.ptr(dk.data), _lib.ptr(work), ws, _lib.stream_ptr())
        torch.cuda.synchronize()
        comps = [out[..., d] for d in range(3)]
        assert rel(out[..., 3].double(), rho.double() / nbar) < 1e-7
    else:
        fmesh, dk = longrange_mesh(G.RealField(pm, rho), nbar, factor=factor)
        comps = [fmesh[d] for d in range(3)]
    torch.cuda.synchronize()
    assert _lib.query('fpm_workspace_status', _lib.ptr(pm._bufs['force_ws']), N, 0, 1) == 0
    ref_dk = F.r2c(rho.double() / nbar)
    assert rel(dk.value.to(torch.complex128), ref_dk) < 2e-6
    pot = F.laplace_inplace(ref_dk, N, box)
    for d in range(3):
        ref = F.c2r(pot * F.gradient_mult(d, N, box, pot.device), N) * factor
        assert rel(comps[d].double(), ref) < 1e-5, d
        del ref
