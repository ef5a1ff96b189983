"""numpy restatement of the ``pmesh`` subset used by the FastPM hot path.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py).  Module name and API mirror
``pmesh.pm`` so that the reference's own ``fastpm/core.py`` and
``fastpm/force/*.py`` can be imported unmodified on top of it (the golden
fixture generator injects this module as ``pmesh.pm``).

Call sites in the reference that fix the semantics restated here:
  core.py:102        ParticleMesh(Nmesh=, BoxSize=, dtype=, comm=, resampler=)
  core.py:114        pm.generate_whitenoise(seed, type='complex', unitary=)
  core.py:117-118    ComplexField.apply(lambda k, v: ...), v.BoxSize
  core.py:183-193    Nmesh.prod(), decompose(X, smoothing), Layout.exchange, pm.paint
  core.py:203-207    RealField.readout, Layout.gather, RealField.r2c(out=Ellipsis)
  force/lpt.py:8-22  basepm.create('complex'), decompose/exchange/readout(resampler='cic')
  force/lpt.py:27-64 create('real'), .ndim, .value, c2r(out=Ellipsis), r2c
  force/kernels.py   v.i[dir], v.Nmesh[dir], v.BoxSize[dir], wavenumbers k
  tests/test_kernel.py:12-13  c2r().r2c() is the identity => r2c carries 1/N.

Wavenumbers: full axes use fftfreq order (index n >= N/2 maps to n - N), the
last (compressed) axis runs 0..N/2; k = 2 pi n / L.

Windows (node-centred cells, cell i sits at x = i L / N, periodic):
  cic  support 2: i0 = floor(x),       weights (1 - f, f),                f = x - i0
  tsc  support 3: i0 = floor(x + 1/2), weights (1/2 (1/2 - d)^2, 3/4 - d^2,
                                                 1/2 (1/2 + d)^2) on i0-1..i0+1, d = x - i0
"""
import numpy

try:  # scipy's pocketfft is the same algorithm as numpy.fft, with threads
    import scipy.fft as _fft
    _FFT_KW = dict(workers=-1)
except ImportError:  # pragma: no cover
    import numpy.fft as _fft
    _FFT_KW = {}


class _SelfComm(object):
    """Single-rank stand-in for the mpi4py communicator (pm.comm)."""
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
    """Identity domain decomposition: one rank owns every particle."""

    def exchange(self, x, pack=True):
        return x

    def gather(self, x, mode='sum', out=None):
        if out is not None:
            out[...] = x
            return out
        return x


class _Field(numpy.ndarray):
    """ndarray subclass carrying its ParticleMesh (pmesh Field stand-in)."""

    def __array_finalize__(self, obj):
        self.pm = getattr(obj, 'pm', None)

    @property
    def value(self):
        return self.view(numpy.ndarray)

    @property
    def BoxSize(self):
        return self.pm.BoxSize

    @property
    def Nmesh(self):
        return self.pm.Nmesh

    @property
    def ndim(self):  # noqa: D401  (pmesh fields report the mesh dimension)
        return len(self.pm.Nmesh)

    @property
    def csize(self):
        return int(numpy.prod(self.shape))

    def copy(self, order='C'):
        out = numpy.ndarray.copy(self, order)
        out.pm = self.pm
        return out


class RealField(_Field):
    def r2c(self, out=None):
        """Forward transform with the 1/N normalisation pmesh uses."""
        c = _fft.rfftn(self.value, **_FFT_KW) / float(numpy.prod(self.pm.Nmesh))
        return self.pm._complex(c)

    def readout(self, pos, out=None, resampler=None, layout=None, hold=False):
        resampler = resampler or self.pm.resampler
        v = readout(self.value, pos, self.pm.BoxSize, resampler)
        if out is not None:
            out[...] = v
            return out
        return v

    def paint(self, pos, mass=1.0, resampler=None, layout=None, hold=False):
        resampler = resampler or self.pm.resampler
        if not hold:
            self[...] = 0
        self.value[...] += paint(pos, self.pm.Nmesh, self.pm.BoxSize, resampler,
                                 mass=mass, dtype=self.dtype)
        return self

    def apply(self, func, kind='relative', out=None):
        x = [xi for xi in self.pm.x]
        v = self.view(type(self))
        v.pm = self.pm
        r = numpy.asarray(func(x, v))
        return self.pm._assign(self, r, out, RealField)


class ComplexField(_Field):
    @property
    def i(self):
        return self.pm.ic

    def c2r(self, out=None):
        """Inverse transform, unnormalised (c2r(r2c(x)) == x)."""
        r = _fft.irfftn(self.value, s=tuple(self.pm.Nmesh), **_FFT_KW) \
            * float(numpy.prod(self.pm.Nmesh))
        return self.pm._real(r)

    def apply(self, func, kind='wavenumber', out=None):
        v = self.view(type(self))
        v.pm = self.pm
        r = numpy.asarray(func(self.pm.k, v))
        return self.pm._assign(self, r, out, ComplexField)


class ParticleMesh(object):
    """pmesh.pm.ParticleMesh stand-in (single rank, cubic or box meshes)."""

    def __init__(self, Nmesh, BoxSize=1.0, comm=None, np=None, dtype='f8',
                 plan_method='estimate', resampler='cic'):
        Nmesh = numpy.array(Nmesh, dtype='i8').ravel()
        if Nmesh.size == 1:
            Nmesh = numpy.repeat(Nmesh, 3)
        self.Nmesh = Nmesh
        self.ndim = len(Nmesh)
        self.BoxSize = numpy.empty(self.ndim, dtype='f8')
        self.BoxSize[...] = BoxSize
        self.dtype = numpy.dtype(dtype)
        self.comm = comm if comm is not None else _SelfComm()
        self.resampler = resampler
        self.domain = None

        k, ic, x = [], [], []
        for d in range(self.ndim):
            N = int(Nmesh[d])
            shape = [1] * self.ndim
            if d == self.ndim - 1:
                n = numpy.arange(N // 2 + 1)
            else:
                n = numpy.fft.fftfreq(N, 1.0 / N)
            shape[d] = len(n)
            kd = (2 * numpy.pi / self.BoxSize[d] * n).reshape(shape)
            k.append(kd)
            ic.append(numpy.arange(len(n)).reshape(shape))
            shape = [1] * self.ndim
            shape[d] = N
            x.append((numpy.arange(N) * (self.BoxSize[d] / N)).reshape(shape))
        self.k = k
        self.ic = ic
        self.x = x

    # -- field construction ------------------------------------------------
    @property
    def cdtype(self):
        return numpy.dtype('c16') if self.dtype == numpy.dtype('f8') else numpy.dtype('c8')

    def _real(self, a):
        r = numpy.asarray(a, dtype=self.dtype).view(RealField)
        r.pm = self
        return r

    def _complex(self, a):
        c = numpy.asarray(a, dtype=self.cdtype).view(ComplexField)
        c.pm = self
        return c

    def _assign(self, src, r, out, cls):
        if out is Ellipsis:
            out = src
        if out is None:
            out = numpy.empty_like(src.value).view(cls)
            out.pm = self
        out.value[...] = r
        return out

    def create(self, type=None, mode=None, value=None, base=None):
        kind = type or mode or 'real'
        if kind == 'real':
            f = self._real(numpy.zeros(tuple(self.Nmesh)))
        elif kind == 'complex':
            shape = tuple(self.Nmesh[:-1]) + (int(self.Nmesh[-1]) // 2 + 1,)
            f = self._complex(numpy.zeros(shape))
        else:
            raise ValueError("type must be 'real' or 'complex'")
        if value is not None:
            f.value[...] = value
        return f

    # -- particles ---------------------------------------------------------
    def generate_uniform_particle_grid(self, shift=0.5, dtype='f8', return_id=False):
        """One particle per mesh node, C order (last axis fastest), at (i + shift) L / N."""
        idx = numpy.indices(tuple(self.Nmesh)).reshape(self.ndim, -1).T
        pos = ((idx + shift) * (self.BoxSize / self.Nmesh)).astype(dtype)
        if return_id:
            return pos, numpy.arange(len(pos), dtype='i8')
        return pos

    def decompose(self, pos, smoothing=None, transform=None):
        return Layout()

    def paint(self, pos, mass=1.0, resampler=None, transform=None, hold=False,
              gradient=None, layout=None, out=None):
        real = self.create('real') if out is None else out
        return real.paint(pos, mass=mass, resampler=resampler, hold=hold)

    def generate_whitenoise(self, seed, unitary=False, mean=0, type='complex'):
        """Whitenoise modes from the project's Philox stream (see whitenoise())."""
        c = self._complex(whitenoise(self.Nmesh, seed, unitary=unitary, mean=mean))
        if type == 'complex':
            return c
        elif type == 'real':
            return c.c2r()
        raise ValueError("type must be 'real' or 'complex'")


# ---------------------------------------------------------------------------
# windows
# ---------------------------------------------------------------------------
def _window(x, resampler):
    """Per-axis cell offsets and weights for cell-unit coordinates x (float64)."""
    if resampler == 'cic':
        i0 = numpy.floor(x)
        f = x - i0
        return i0.astype('i8'), [0, 1], [1.0 - f, f]
    elif resampler == 'tsc':
        i0 = numpy.floor(x + 0.5)
        d = x - i0
        return i0.astype('i8'), [-1, 0, 1], [0.5 * (0.5 - d) ** 2, 0.75 - d ** 2,
                                             0.5 * (0.5 + d) ** 2]
    raise ValueError("resampler must be 'cic' or 'tsc', got %r" % (resampler,))


def _iter_window(pos, Nmesh, BoxSize, resampler, chunk=1 << 20):
    Nmesh = numpy.asarray(Nmesh, dtype='i8')
    scale = Nmesh / numpy.asarray(BoxSize, dtype='f8')
    for start in range(0, len(pos), chunk):
        x = numpy.asarray(pos[start:start + chunk], dtype='f8') * scale
        i0x, offs, wx = _window(x[:, 0], resampler)
        i0y, _, wy = _window(x[:, 1], resampler)
        i0z, _, wz = _window(x[:, 2], resampler)
        for a, oa in enumerate(offs):
            ix = (i0x + oa) % Nmesh[0]
            for b, ob in enumerate(offs):
                iy = (i0y + ob) % Nmesh[1]
                wab = wx[a] * wy[b]
                base = (ix * Nmesh[1] + iy) * Nmesh[2]
                for c, oc in enumerate(offs):
                    iz = (i0z + oc) % Nmesh[2]
                    yield start, base + iz, wab * wz[c]


def paint(pos, Nmesh, BoxSize, resampler, mass=1.0, dtype='f8'):
    """Mass assignment of particles at pos onto a periodic mesh (float64 sums)."""
    Nmesh = numpy.asarray(Nmesh, dtype='i8')
    size = int(numpy.prod(Nmesh))
    out = numpy.zeros(size, dtype='f8')
    mass = numpy.asarray(mass, dtype='f8')
    for start, idx, w in _iter_window(pos, Nmesh, BoxSize, resampler):
        if mass.ndim:
            w = w * mass[start:start + len(w)]
        else:
            w = w * mass
        out += numpy.bincount(idx, weights=w, minlength=size)
    return out.reshape(tuple(Nmesh)).astype(dtype)


def readout(mesh, pos, BoxSize, resampler):
    """Window-weighted gather of mesh values at pos (float64 sums)."""
    mesh = numpy.asarray(mesh)
    flat = mesh.reshape(-1)
    out = numpy.zeros(len(pos), dtype='f8')
    for start, idx, w in _iter_window(pos, mesh.shape, BoxSize, resampler):
        out[start:start + len(w)] += w * flat[idx]
    return out.astype(numpy.asarray(pos).dtype if numpy.asarray(pos).dtype.kind == 'f' else 'f8')


def cell_keys_lattice(disp, nc, shift, nmesh, boxsize, resampler):
    """Integer cell index of each particle's window anchor, as the device computes it.

    Positions are the lattice point (i + shift) L / Nc plus a float32
    displacement.  In mesh-cell units, with B = Nmesh / Nc (an integer), the
    device rounds only the product s = f32(disp) * f32(Nmesh / L) (float32,
    round to nearest) and takes the anchor of the EXACT sum with the shift:
        x   = shift * B + s                      (exact: float64 here)
        a   = floor(x)            (cic)   or   floor(x + 1/2)   (tsc)
        i0  = i * B + a                          (integer)
        key = ((i0x mod N) * N + (i0y mod N)) * N + (i0z mod N)
    An integral shift * B is added to the cell as an integer; otherwise the
    device uses f32(shift * B) and recovers the rounding error of the sum
    (TwoSum), restated here in float32.  Returns (key int64 [Np], frac
    float32 [Np, 3]) with frac = x - a rounded once to float32.  With N / L a
    power of two, s is exact and x equals the reference's float64
    (Q + S) N / L - i B.
    """
    nc, nmesh = int(nc), int(nmesh)
    B = nmesh // nc
    assert B * nc == nmesh
    disp = numpy.asarray(disp, dtype='f4').reshape(-1, 3)
    np_ = len(disp)
    pid = numpy.arange(np_, dtype='i8')
    lat = numpy.stack([pid // (nc * nc), (pid // nc) % nc, pid % nc], axis=1)
    sbd = shift * B
    sbi = int(sbd) if sbd == numpy.floor(sbd) else 0
    a = numpy.float32(0.0 if sbi or sbd == 0 else sbd)
    scale = numpy.float32(nmesh / float(boxsize))
    b = (disp * scale).astype('f4')             # float32 product, round to nearest
    # anchor of the exact sum a + b: TwoSum (t + e == a + b exactly, float32)
    t = (a + b).astype('f4')
    bv = (t - a).astype('f4')
    av = (t - bv).astype('f4')
    e = ((a - av).astype('f4') + (b - bv).astype('f4')).astype('f4')
    fl = numpy.floor(t)
    fl = numpy.where((t == fl) & (e < 0), fl - 1, fl).astype('f4')
    dt = (t - fl).astype('f4')                  # exact
    if resampler == 'tsc':
        up = (dt > 0.5) | ((dt == 0.5) & (e >= 0))
        fl = numpy.where(up, fl + 1, fl).astype('f4')
        dt = (t - fl).astype('f4')
    frac = (dt + e).astype('f4')
    fl = fl.astype('i8') + sbi
    i0 = lat * B + fl.astype('i8')
    i0 %= nmesh
    key = (i0[:, 0] * nmesh + i0[:, 1]) * nmesh + i0[:, 2]
    return key, frac


# ---------------------------------------------------------------------------
# whitenoise: Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11) per mode
# ---------------------------------------------------------------------------
_M0 = numpy.uint64(0xD2511F53)
_M1 = numpy.uint64(0xCD9E8D57)
_W0 = numpy.uint32(0x9E3779B9)
_W1 = numpy.uint32(0xBB67AE85)
_LO = numpy.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Vectorised Philox4x32 with 10 rounds; all arguments uint32 arrays/scalars."""
    c0, c1, c2, c3 = (numpy.asarray(c, dtype='u4') for c in (c0, c1, c2, c3))
    k0 = numpy.uint32(k0)
    k1 = numpy.uint32(k1)
    for r in range(10):
        if r > 0:
            k0 = numpy.uint32((int(k0) + int(_W0)) & 0xFFFFFFFF)
            k1 = numpy.uint32((int(k1) + int(_W1)) & 0xFFFFFFFF)
        p0 = _M0 * c0.astype('u8')
        p1 = _M1 * c2.astype('u8')
        hi0 = (p0 >> numpy.uint64(32)).astype('u4')
        lo0 = (p0 & _LO).astype('u4')
        hi1 = (p1 >> numpy.uint64(32)).astype('u4')
        lo1 = (p1 & _LO).astype('u4')
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
    return c0, c1, c2, c3


def _u53(a, b):
    """Uniform double in (0, 1) from two uint32 words (53 random bits, centred)."""
    a = (a >> numpy.uint32(5)).astype('f8')
    b = (b >> numpy.uint32(6)).astype('f8')
    return (a * 67108864.0 + b + 0.5) * (1.0 / 9007199254740992.0)


def whitenoise(Nmesh, seed, unitary=False, mean=0.0):
    """Complex whitenoise on the r2c half mesh [N0][N1][N2/2+1], <|v|^2> = 1.

    Mode (i, j, l) draws Philox4x32-10 with counter (lin_lo, lin_hi, 0, 0),
    lin = (i N1 + j)(N2/2+1) + l, and key (seed_lo, seed_hi); two 53-bit
    uniforms u1, u2 give v = sqrt(-ln u1) exp(2 pi i u2) (|v| = 1 if unitary).
    On the self-conjugate planes l = 0 and l = N2/2 the mode equals the
    conjugate of its mirror (-i, -j); the member with the smaller (i N1 + j)
    draws.  Self-mirrored modes are real: sqrt(-2 ln u1) cos(2 pi u2) (or its
    sign if unitary).  The k = 0 mode is set to `mean`.
    """
    N0, N1, N2 = (int(n) for n in Nmesh)
    Nz = N2 // 2 + 1
    seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    k0, k1 = seed & 0xFFFFFFFF, seed >> 32
    i = numpy.arange(N0).reshape(-1, 1, 1)
    j = numpy.arange(N1).reshape(1, -1, 1)
    l = numpy.arange(Nz).reshape(1, 1, -1)

    def draw(ii, jj, ll):
        lin = ((ii * N1 + jj) * Nz + ll).astype('u8')
        lo = (lin & _LO).astype('u4')
        hi = (lin >> numpy.uint64(32)).astype('u4')
        z = numpy.zeros_like(lo)
        r0, r1, r2, r3 = philox4x32_10(lo, hi, z, z, k0, k1)
        return _u53(r0, r1), _u53(r2, r3)

    ii, jj, ll = numpy.broadcast_arrays(i, j, l)
    u1, u2 = draw(ii, jj, ll)
    phase = 2 * numpy.pi * u2
    if unitary:
        v = numpy.cos(phase) + 1j * numpy.sin(phase)
    else:
        amp = numpy.sqrt(-numpy.log(u1))
        v = amp * numpy.cos(phase) + 1j * (amp * numpy.sin(phase))

    # self-conjugate planes l = 0 and l = N2/2 (the latter only for even N2)
    planes = [0] + ([N2 // 2] if N2 % 2 == 0 else [])
    mi = (-numpy.arange(N0)) % N0
    mj = (-numpy.arange(N1)) % N1
    lin2 = numpy.arange(N0).reshape(-1, 1) * N1 + numpy.arange(N1).reshape(1, -1)
    mlin2 = mi.reshape(-1, 1) * N1 + mj.reshape(1, -1)
    for p in planes:
        vp = v[:, :, p]
        selfc = lin2 == mlin2
        mirror = lin2 > mlin2
        # mirrored members take the conjugate of the drawing member
        vp_m = numpy.conj(vp[mi][:, mj])
        vp = numpy.where(mirror, vp_m, vp)
        # self-mirrored members are real
        a, b = u1[:, :, p], u2[:, :, p]
        c = numpy.cos(2 * numpy.pi * b)
        if unitary:
            real = numpy.where(c >= 0, 1.0, -1.0)
        else:
            real = numpy.sqrt(-2 * numpy.log(a)) * c
        vp = numpy.where(selfc, real + 0j, vp)
        v[:, :, p] = vp
    v[0, 0, 0] = mean
    return v
