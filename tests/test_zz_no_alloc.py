"""The allocation-free force entry point against the workspace one.

fpm_force_mesh_static serves callers that cannot allocate device memory where
they need a force (a fixed device-memory budget, or no tolerance for
cudaMalloc's implicit synchronisation).  It must give the same force meshes
and delta_k as fpm_force_mesh, on consecutive calls that share its scratch.
This file is collected last so that a failure here does not hide others.
"""
import numpy
import pytest
import torch

from tests.helpers import rel_l2, tonp

pytestmark = pytest.mark.gpu


def _force(lib_call, n, rho, box, static, ws=None):
    from fastpm_gb300 import _lib
    f = torch.empty((3, n, n, n), dtype=torch.float32, device='cuda')
    zp = _lib.query('fpm_complex_row', n)
    dk = torch.zeros((n, n, zp, 2), dtype=torch.float32, device='cuda')
    args = [_lib.ptr(rho), n, box, 1.0 / 0.125, 0.45, _lib.ptr(f[0]), _lib.ptr(f[1]), _lib.ptr(f[2]),
            _lib.ptr(dk)]
    if static:
        _lib.call('fpm_force_mesh_static', *args, _lib.stream_ptr())
    else:
        _lib.call('fpm_force_mesh', *args, _lib.ptr(ws), ws.numel(), _lib.stream_ptr())
    torch.cuda.synchronize()
    return f, dk[:, :, : n // 2 + 1]


@pytest.mark.parametrize('n', [64, 128])
def test_static_force_matches_workspace_force(n):
    from fastpm_gb300 import _lib
    box = 2.0 * n
    ws = torch.empty(_lib.query('fpm_force_workspace', n), dtype=torch.uint8, device='cuda')
    for seed in (1, 2):   # two calls in a row share the static scratch
        g = torch.Generator(device='cuda').manual_seed(seed)
        rho = 1 + 0.2 * torch.randn((n, n, n), generator=g, device='cuda')
        fs, dks = _force(None, n, rho, box, static=True)
        fw, dkw = _force(None, n, rho, box, static=False, ws=ws)
        for d in range(3):
            assert rel_l2(tonp(fs[d]), tonp(fw[d])) < 5e-6
        assert rel_l2(tonp(dks), tonp(dkw)) < 2e-6


def test_static_force_allocates_nothing():
    """After a first call, further calls leave the device's free memory unchanged."""
    from fastpm_gb300 import _lib
    n = 128
    rho = torch.ones((n, n, n), device='cuda')
    f = torch.empty((3, n, n, n), dtype=torch.float32, device='cuda')
    args = [_lib.ptr(rho), n, 256.0, 1.0, 0.45, _lib.ptr(f[0]), _lib.ptr(f[1]), _lib.ptr(f[2]), None,
            _lib.stream_ptr()]
    _lib.call('fpm_force_mesh_static', *args)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(5):
        _lib.call('fpm_force_mesh_static', *args)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_static_force_rejects_large_mesh():
    from fastpm_gb300 import _lib
    lib = _lib.load()
    buf = torch.empty(16, device='cuda')
    p = _lib.ptr(buf)
    assert lib.fpm_force_mesh_static(p, 256, 256.0, 1.0, 1.0, p, p, p, None, None) == 5  # FPM_ERR_LIMIT
