"""ctypes binding of libfastpm_gb300.so (the C ABI in include/fastpm_gb300.h).

The library is built in place by csrc/build.py.  There is no fallback: if the
shared library is missing, or a call is made without a CUDA device, the call
raises.
"""
import ctypes
import os
import threading

import torch

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, 'libfastpm_gb300.so')

FPM_WINDOW = {'cic': 1, 'tsc': 2}

_c = ctypes
_vp, _i, _ll, _d, _f, _u64 = _c.c_void_p, _c.c_int, _c.c_longlong, _c.c_double, _c.c_float, _c.c_ulonglong
_pp = _c.POINTER(_c.c_void_p)

# name -> (restype, argtypes); the declarations of include/fastpm_gb300.h
SIGNATURES = {
    'fpm_abi_version': (_i, []),
    'fpm_strerror': (_c.c_char_p, [_i]),
    'fpm_fft_supported': (_i, [_i]),
    'fpm_complex_row': (_i, [_i]),
    'fpm_device_init': (_i, []),
    'fpm_set_option': (_i, [_i, _i]),
    'fpm_get_option': (_i, [_i]),
    'fpm_paint': (_i, [_vp, _i, _d, _vp, _vp, _ll, _i, _d, _i, _f, _vp]),
    'fpm_paint_sorted_workspace': (_ll, [_i, _ll]),
    'fpm_paint_sorted': (_i, [_vp, _i, _d, _vp, _vp, _ll, _i, _d, _i, _f, _vp, _ll, _vp]),
    'fpm_paint_sorted_batch_workspace': (_ll, [_i, _ll, _i]),
    'fpm_paint_sorted_batch': (_i, [_vp, _ll, _i, _d, _vp, _ll, _ll, _i, _d, _i, _f, _i, _vp, _vp, _ll, _vp]),
    'fpm_force_mesh_batch_packed': (_i, [_vp, _ll, _i, _d, _d, _vp, _vp, _ll, _vp, _ll, _i, _vp, _vp]),
    'fpm_readout_packed_batch': (_i, [_vp, _ll, _i, _d, _vp, _ll, _ll, _i, _d, _i, _vp, _ll, _vp, _ll, _i, _vp, _vp]),
    'fpm_readout_packed_sorted': (_i, [_vp, _i, _d, _vp, _vp, _ll, _i, _d, _i, _vp, _vp, _i, _vp, _ll, _vp]),
    'fpm_readout_blocked_sorted': (_i, [_vp, _i, _d, _vp, _vp, _ll, _i, _d, _i, _vp, _vp, _i, _vp, _ll, _vp]),
    'fpm_paint_brick_edge': (_i, [_i]),
    'fpm_force_readout_sorted': (_i, [_vp, _i, _d, _d, _d, _vp, _vp, _ll, _vp, _vp, _ll, _i, _d, _i, _vp, _vp, _i, _vp, _ll, _vp]),
    'fpm_kick_drift_bin': (_i, [_vp, _vp, _vp, _vp, _vp, _ll, _d, _d, _i, _d, _i, _d, _vp, _i, _d, _i, _vp, _ll, _vp]),
    'fpm_paint_sorted_counted': (_i, [_vp, _i, _d, _vp, _vp, _ll, _i, _d, _i, _f, _vp, _ll, _vp]),
    'fpm_paint_sorted_add': (_i, [_vp, _i, _d, _vp, _vp, _ll, _i, _d, _i, _f, _vp, _ll, _vp]),
    'fpm_force_mesh_packed_transfer': (_i, [_vp, _i, _d, _d, _d, _vp, _ll, _vp, _vp, _vp, _ll, _vp]),
    'fpm_readout': (_i, [_pp, _i, _i, _d, _vp, _vp, _ll, _i, _d, _i, _pp,
                         _c.POINTER(_i), _c.POINTER(_f), _vp]),
    'fpm_r2c': (_i, [_vp, _vp, _i, _f, _vp]),
    'fpm_c2r_workspace': (_ll, [_i]),
    'fpm_c2r': (_i, [_vp, _vp, _i, _f, _vp, _vp]),
    'fpm_force_workspace': (_ll, [_i]),
    'fpm_force_mesh': (_i, [_vp, _i, _d, _d, _d, _vp, _vp, _vp, _vp, _vp, _ll, _vp]),
    'fpm_force_mesh_packed': (_i, [_vp, _i, _d, _d, _d, _vp, _vp, _vp, _ll, _vp]),
    'fpm_force_mesh_blocked': (_i, [_vp, _i, _d, _d, _d, _vp, _vp, _vp, _ll, _vp]),
    'fpm_readout_packed': (_i, [_vp, _i, _d, _vp, _vp, _ll, _i, _d, _i, _vp, _vp, _vp]),
    'fpm_lpt_workspace': (_ll, [_i]),
    'fpm_lpt1_mesh': (_i, [_vp, _i, _d, _vp, _vp, _vp, _vp, _ll, _vp]),
    'fpm_lpt2_source': (_i, [_vp, _i, _d, _vp, _vp, _ll, _vp]),
    'fpm_workspace_status': (_i, [_vp, _i, _i, _i]),
    'fpm_force_mesh_static': (_i, [_vp, _i, _d, _d, _d, _vp, _vp, _vp, _vp, _vp]),
    'fpm_whitenoise': (_i, [_vp, _i, _u64, _i, _d, _vp]),
    'fpm_apply_isotropic': (_i, [_vp, _i, _vp, _ll, _vp]),
    'fpm_kick': (_i, [_vp, _vp, _vp, _ll, _d, _vp]),
    'fpm_drift': (_i, [_vp, _vp, _vp, _ll, _d, _vp]),
    'fpm_kick_drift': (_i, [_vp, _vp, _vp, _vp, _vp, _ll, _d, _d, _i, _d, _vp]),
    'fpm_cell_keys': (_i, [_vp, _vp, _i, _d, _vp, _vp, _ll, _i, _d, _i, _vp]),
    'fpm_power_accumulate': (_i, [_vp, _vp, _i, _d, _vp, _vp, _vp, _vp]),
    'fpm_paint_batch': (_i, [_vp, _ll, _i, _d, _vp, _ll, _ll, _i, _d, _i, _f, _i, _vp, _vp]),
    'fpm_readout_batch': (_i, [_pp, _ll, _i, _i, _d, _vp, _ll, _ll, _i, _d, _i, _pp,
                               _c.POINTER(_i), _ll, _c.POINTER(_f), _i, _vp, _vp]),
    'fpm_force_batch_workspace': (_ll, [_i, _i]),
    'fpm_force_mesh_batch': (_i, [_vp, _ll, _i, _d, _d, _vp, _vp, _vp, _vp, _ll, _vp, _ll, _i, _vp, _vp]),
    'fpm_kick_drift_batch': (_i, [_vp, _vp, _vp, _vp, _vp, _ll, _ll, _vp, _i, _vp]),
    'fpm_paint_values': (_i, [_pp, _i, _i, _d, _vp, _vp, _ll, _i, _d, _i, _pp, _c.POINTER(_i), _f, _vp]),
    'fpm_readout_vjp': (_i, [_pp, _i, _i, _d, _vp, _vp, _ll, _i, _d, _i, _pp, _c.POINTER(_i),
                             _c.POINTER(_f), _vp, _i, _vp]),
    'fpm_kspace_combine': (_i, [_pp, _i, _c.POINTER(_i), _c.POINTER(_i), _vp, _i, _d, _d, _vp]),
    'fpm_dot': (_i, [_vp, _vp, _ll, _vp, _vp]),
    'fpm_launch_count': (_ll, []),
    'fpm_trace_enable': (_i, [_i]),
    'fpm_trace_summary': (_i, [_c.c_char_p, _ll]),
}

_lock = threading.Lock()
_lib = None


class FastPMError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, name, code, msg):
        RuntimeError.__init__(self, '%s failed with status %d: %s' % (name, code, msg))
        self.code = code


def load():
    """Load the shared library (no GPU needed to load it)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIBPATH):
                raise RuntimeError('libfastpm_gb300.so is not built (%s); run '
                                   '`python fastpm-python_gb300/csrc/build.py`' % LIBPATH)
            lib = ctypes.CDLL(LIBPATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError('fastpm_gb300 needs a CUDA GPU: the particle-mesh kernels have no '
                           'CPU implementation')


def call(name, *args):
    lib = load()
    rc = getattr(lib, name)(*args)
    if rc != 0:
        raise FastPMError(name, rc, lib.fpm_strerror(rc).decode())
    return rc


def query(name, *args):
    return getattr(load(), name)(*args)


def ptr(t):
    """Device pointer of a CUDA tensor (or None)."""
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError('expected a CUDA tensor')
    return ctypes.c_void_p(t.data_ptr())


def stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def workspace_status(work, n, kind, clear=1):
    """fpm_workspace_status of a force (kind 0) or LPT (kind 1) workspace
    of mesh size n; the library reads the status word at an offset that follows
    from n, so the buffer must be at least that workspace's size."""
    need = query('fpm_force_workspace' if kind == 0 else 'fpm_lpt_workspace', n)
    have = work.numel() * work.element_size()
    if have < need:
        raise ValueError('workspace of %d bytes is smaller than the n = %d %s workspace (%d bytes)'
                         % (have, n, 'force' if kind == 0 else 'LPT', need))
    return query('fpm_workspace_status', ptr(work), n, kind, clear)


def ptr_array(tensors_or_ptrs):
    arr = (ctypes.c_void_p * len(tensors_or_ptrs))()
    for i, t in enumerate(tensors_or_ptrs):
        arr[i] = t if isinstance(t, int) else t.data_ptr()
    return ctypes.cast(arr, _pp), arr


def launch_count():
    """Kernels launched by libfastpm_gb300 in this process."""
    return int(load().fpm_launch_count())


def trace(on):
    call('fpm_trace_enable', 1 if on else 0)


def trace_summary():
    """{kernel name: (launches, total ms)} of the launches recorded since the last summary."""
    buf = ctypes.create_string_buffer(1 << 16)
    call('fpm_trace_summary', buf, len(buf))
    out = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms = line.split()
        out[name] = (int(cnt), float(ms))
    return out
