"""Device-resident particle mesh: the pmesh.pm subset the FastPM path calls.

``ParticleMesh``, ``RealField`` and ``ComplexField`` keep pmesh's names and
conventions (fastpm/core.py:102,114,183-207; force/lpt.py; force/gravity.py):
r2c carries 1/N (so c2r(r2c(x)) == x, fastpm/tests/test_kernel.py:12-13),
node-centred cells, CIC / TSC windows, wavenumbers k = 2 pi n / L with n in
fftfreq order on the full axes.  Storage is CUDA memory owned by torch:
  RealField.value     float32 [n, n, n]
  ComplexField.data   float32 [n, n, nzp, 2] (padded rows, see the C ABI);
  ComplexField.value  complex64 view [n, n, n//2 + 1] of it.
Every transform, paint and readout runs in libfastpm_gb300 kernels.
"""
import numpy
import torch

from . import _lib


class SelfComm(object):
    """One process, one GPU: the single-rank communicator."""
    rank = 0
    size = 1

    def allreduce(self, x, op=None):
        return x

    def allgather(self, x):
        return [x]

    def bcast(self, x, root=0):
        return x

    def barrier(self):
        pass


class Layout(object):
    """Domain decomposition on one GPU is the identity (core.py:187-189, 203)."""

    def exchange(self, x, pack=True):
        return x

    def gather(self, x, mode='sum', out=None):
        if out is not None:
            out[...] = x
            return out
        return x


def _as_device_f32(pos, device):
    if isinstance(pos, numpy.ndarray):
        pos = torch.from_numpy(pos)
    return pos.to(device=device, dtype=torch.float32).contiguous()


class RealField(object):
    def __init__(self, pm, value=None):
        self.pm = pm
        if value is None:
            value = torch.zeros(tuple(int(n) for n in pm.Nmesh), dtype=torch.float32, device=pm.device)
        self.value = value

    BoxSize = property(lambda self: self.pm.BoxSize)
    Nmesh = property(lambda self: self.pm.Nmesh)
    ndim = property(lambda self: self.pm.ndim)
    shape = property(lambda self: tuple(self.value.shape))
    dtype = property(lambda self: self.value.dtype)
    csize = property(lambda self: self.value.numel())

    def copy(self):
        return RealField(self.pm, self.value.clone())

    def numpy(self):
        return self.value.cpu().numpy()

    def __getitem__(self, idx):
        return self.value[idx]

    def __setitem__(self, idx, v):
        self.value[idx] = v

    def __itruediv__(self, x):
        self.value /= x
        return self

    def __imul__(self, x):
        self.value *= x
        return self

    def r2c(self, out=None):
        """Forward FFT, scaled by 1/N (pmesh RealField.r2c)."""
        c = out if isinstance(out, ComplexField) else ComplexField(self.pm, empty=True)
        n = self.pm.n
        _lib.call('fpm_r2c', _lib.ptr(self.value), _lib.ptr(c.data), n,
                  1.0 / float(n) ** 3, _lib.stream_ptr())
        return c

    def readout(self, pos, out=None, resampler=None, layout=None):
        """Window-weighted value of the mesh at absolute positions pos."""
        resampler = resampler or self.pm.resampler
        q = _as_device_f32(pos, self.pm.device)
        res = torch.empty(q.shape[0], dtype=torch.float32, device=self.pm.device)
        self.pm._readout([self.value], [res], [1], [1.0], q=q, disp=None, resampler=resampler)
        if out is not None:
            out[...] = res
            return out
        return res

    def paint(self, pos, mass=1.0, resampler=None, layout=None, hold=False):
        if not hold:
            self.value.zero_()
        q = _as_device_f32(pos, self.pm.device)
        self.pm._paint(self.value, q=q, disp=None, resampler=resampler or self.pm.resampler,
                       mass=mass)
        return self


class ComplexField(object):
    def __init__(self, pm, data=None, empty=False):
        self.pm = pm
        n, zp = pm.n, pm.zp
        if data is None:
            alloc = torch.empty if empty else torch.zeros
            data = alloc((n, n, zp, 2), dtype=torch.float32, device=pm.device)
        self.data = data

    BoxSize = property(lambda self: self.pm.BoxSize)
    Nmesh = property(lambda self: self.pm.Nmesh)
    ndim = property(lambda self: self.pm.ndim)

    @property
    def value(self):
        return torch.view_as_complex(self.data)[:, :, : self.pm.n // 2 + 1]

    @property
    def shape(self):
        return tuple(self.value.shape)

    def copy(self):
        return ComplexField(self.pm, self.data.clone())

    def numpy(self):
        return self.value.cpu().numpy()

    def __getitem__(self, idx):
        return self.value[idx]

    def __setitem__(self, idx, v):
        self.value[idx] = v

    def c2r(self, out=None):
        """Inverse FFT, unscaled (pmesh ComplexField.c2r); the input is kept."""
        r = out if isinstance(out, RealField) else RealField(self.pm, torch.empty(
            (self.pm.n,) * 3, dtype=torch.float32, device=self.pm.device))
        work = self.pm._scratch('c2r', _lib.query('fpm_c2r_workspace', self.pm.n))
        _lib.call('fpm_c2r', _lib.ptr(self.data), _lib.ptr(r.value), self.pm.n, 1.0,
                  _lib.ptr(work), _lib.stream_ptr())
        return r

    @property
    def i(self):
        return self.pm.ic

    def apply(self, func, kind='wavenumber', out=None):
        """out = func(k, v) with k the broadcastable wavenumber tensors (device)."""
        v = self.value
        r = func(self.pm.k, _KView(v, self.pm))
        dst = self if out is Ellipsis else (out if isinstance(out, ComplexField)
                                            else ComplexField(self.pm, empty=True))
        dst.value[...] = r
        return dst


class _KView(object):
    """The `v` argument of pmesh kernels: the complex values plus .i/.Nmesh/.BoxSize."""

    def __init__(self, v, pm):
        self.v = v
        self.i = pm.ic
        self.Nmesh = pm.Nmesh
        self.BoxSize = pm.BoxSize

    def __mul__(self, x):
        return self.v * x

    __rmul__ = __mul__

    def __truediv__(self, x):
        return self.v / x


class ParticleMesh(object):
    """Cubic periodic mesh on one CUDA device (pmesh.pm.ParticleMesh subset)."""

    def __init__(self, Nmesh, BoxSize=1.0, comm=None, np=None, dtype='f4', plan_method=None,
                 resampler='cic', device=None):
        Nmesh = numpy.array(Nmesh, dtype='i8').ravel()
        if Nmesh.size == 1:
            Nmesh = numpy.repeat(Nmesh, 3)
        if len(Nmesh) != 3 or len(set(Nmesh.tolist())) != 1:
            raise ValueError('only cubic 3-d meshes are supported, got Nmesh=%s' % (Nmesh,))
        BoxSize = numpy.broadcast_to(numpy.asarray(BoxSize, dtype='f8'), (3,)).copy()
        if len(set(BoxSize.tolist())) != 1:
            raise ValueError('only cubic boxes are supported, got BoxSize=%s' % (BoxSize,))
        if resampler not in _lib.FPM_WINDOW:
            raise ValueError("resampler must be 'cic' or 'tsc'")
        self.Nmesh = Nmesh
        self.BoxSize = BoxSize
        self.ndim = 3
        self.n = int(Nmesh[0])
        self.L = float(BoxSize[0])
        self.dtype = numpy.dtype(dtype)
        self.comm = comm if comm is not None else SelfComm()
        self.resampler = resampler
        self.device = torch.device(device) if device is not None else torch.device('cuda')
        row = _lib.query('fpm_complex_row', self.n)
        if row <= 0:
            raise ValueError('Nmesh=%d is not a supported FFT size' % self.n)
        self.zp = int(row)
        self._bufs = {}
        self._k = None

    # -- wavenumbers (device tensors, for ComplexField.apply) -------------------
    @property
    def k(self):
        if self._k is None:
            n, kf = self.n, 2 * numpy.pi / self.L
            full = torch.fft.fftfreq(n, 1.0 / n, device=self.device, dtype=torch.float64) * kf
            half = torch.arange(n // 2 + 1, device=self.device, dtype=torch.float64) * kf
            self._k = [full.view(-1, 1, 1).float(), full.view(1, -1, 1).float(),
                       half.view(1, 1, -1).float()]
        return self._k

    @property
    def ic(self):
        n = self.n
        return [torch.arange(n, device=self.device).view(-1, 1, 1),
                torch.arange(n, device=self.device).view(1, -1, 1),
                torch.arange(n // 2 + 1, device=self.device).view(1, 1, -1)]

    def _scratch(self, key, nbytes):
        """A device scratch buffer of at least nbytes, kept per key.  New buffers
        start zeroed: the force / LPT workspaces end with the status word the
        pipelined kernels set on a timed-out wait, which must start clear."""
        buf = self._bufs.get(key)
        if buf is None or buf.numel() < nbytes:
            buf = torch.zeros(int(nbytes), dtype=torch.uint8, device=self.device)
            self._bufs[key] = buf
        return buf

    # -- fields ---------------------------------------------------------------
    def create(self, type=None, mode=None, value=None, base=None):
        kind = type or mode or 'real'
        if kind == 'real':
            f = RealField(self)
        elif kind == 'complex':
            f = ComplexField(self)
        else:
            raise ValueError("type must be 'real' or 'complex'")
        if value is not None:
            f.value[...] = torch.as_tensor(value).to(f.value.device)
        return f

    def complex_from(self, array):
        """ComplexField from a host or device [n, n, n//2+1] complex array."""
        c = ComplexField(self)
        c.value[...] = torch.as_tensor(numpy.asarray(array) if not torch.is_tensor(array) else array) \
            .to(device=self.device, dtype=torch.complex64)
        return c

    def decompose(self, pos, smoothing=None, transform=None):
        return Layout()

    def generate_uniform_particle_grid(self, shift=0.5, dtype='f8', return_id=False):
        """One particle per mesh node in C order at (i + shift) L / n, on the device.

        The returned tensor remembers it is this lattice, so the solver keeps
        positions as lattice index + float32 displacement and never reads it.
        """
        n, L = self.n, self.L
        tdt = torch.float64 if numpy.dtype(dtype) == numpy.dtype('f8') else torch.float32
        i = torch.arange(n, device=self.device, dtype=torch.float64)
        g = torch.stack(torch.meshgrid(i, i, i, indexing='ij'), dim=-1).reshape(-1, 3)
        pos = ((g + shift) * (L / n)).to(tdt)
        pos._fpm_lattice = (n, float(shift), L)
        if return_id:
            return pos, torch.arange(n ** 3, device=self.device, dtype=torch.int64)
        return pos

    def generate_whitenoise(self, seed, unitary=False, mean=0, type='complex'):
        c = ComplexField(self)
        _lib.call('fpm_whitenoise', _lib.ptr(c.data), self.n, int(seed) & 0xFFFFFFFFFFFFFFFF,
                  int(bool(unitary)), float(mean), _lib.stream_ptr())
        if type == 'complex':
            return c
        if type == 'real':
            return c.c2r()
        raise ValueError("type must be 'real' or 'complex'")

    def paint(self, pos, mass=1.0, resampler=None, transform=None, hold=False, gradient=None,
              layout=None, out=None):
        real = out if out is not None else RealField(self)
        return real.paint(pos, mass=mass, resampler=resampler, hold=hold)

    # -- kernels on (lattice + displacement) or explicit positions -------------
    def _geom(self, q, disp, lattice):
        if lattice is not None:
            nc, shift = lattice
            np_ = nc ** 3
            return None, np_, nc, shift
        return _lib.ptr(q), q.shape[0], 0, 0.0

    def _paint(self, mesh, q=None, disp=None, lattice=None, resampler=None, mass=1.0):
        qp, np_, nc, shift = self._geom(q, disp, lattice)
        _lib.call('fpm_paint', _lib.ptr(mesh), self.n, self.L, _lib.ptr(disp), qp, np_, nc,
                  shift, _lib.FPM_WINDOW[resampler or self.resampler], float(mass),
                  _lib.stream_ptr())

    def _paint_work(self, np_):
        ws = _lib.query('fpm_paint_sorted_workspace', self.n, np_)
        if ws < 0:
            raise _lib.FastPMError('fpm_paint_sorted_workspace', -ws, 'mesh size not a multiple of 4')
        return self._scratch('paint_ws', ws), ws

    def _paint_sorted(self, mesh, q=None, disp=None, lattice=None, resampler=None, mass=1.0,
                      counted=False, add=False):
        """Cell-sorted paint that OVERWRITES `mesh` (fpm_paint_sorted), or adds
        to it (add=True, fpm_paint_sorted_add); counted: the brick counts of
        these positions are already in the paint workspace (fpm_kick_drift_bin)."""
        qp, np_, nc, shift = self._geom(q, disp, lattice)
        work, ws = self._paint_work(np_)
        name = 'fpm_paint_sorted_add' if add else 'fpm_paint_sorted_counted' if counted else 'fpm_paint_sorted'
        _lib.call(name, _lib.ptr(mesh), self.n,
                  self.L, _lib.ptr(disp), qp, np_, nc, shift,
                  _lib.FPM_WINDOW[resampler or self.resampler], float(mass), _lib.ptr(work), ws,
                  _lib.stream_ptr())
        # the particle lists stay valid for a readout at the same positions
        return dict(work=work, bytes=ws, brick=_lib.query('fpm_paint_brick_edge', self.n))

    def _readout(self, meshes, outs, strides, scales, q=None, disp=None, lattice=None,
                 resampler=None):
        qp, np_, nc, shift = self._geom(q, disp, lattice)
        import ctypes
        m_arr, _keep1 = _lib.ptr_array(meshes)
        o_arr, _keep2 = _lib.ptr_array(outs)
        s_arr = (ctypes.c_int * len(strides))(*strides)
        f_arr = (ctypes.c_float * len(scales))(*scales)
        _lib.call('fpm_readout', m_arr, len(meshes), self.n, self.L, _lib.ptr(disp), qp, np_, nc,
                  shift, _lib.FPM_WINDOW[resampler or self.resampler], o_arr, s_arr, f_arr,
                  _lib.stream_ptr())
