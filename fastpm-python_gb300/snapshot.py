"""Snapshot files in the column layout of the reference's StateVector.save.

fastpm/core.py:65-89 writes, through the third-party ``bigfile`` package, one
directory per snapshot holding a ``Header`` block of attributes (Om0, Tcmb0,
Neff, [m_nu,] Ob0, Ode0, Time, h, RSDFactor and the caller's extra attrs) and
three column blocks ``1/Position``, ``1/Velocity`` and ``1/Density``.
``bigfile`` is not installed here, so this module writes that layout itself,
following bigfile's published on-disk conventions: a block is a directory with

  header    text: ``DTYPE: <f8`` / ``NMEMB: 3`` / ``NFILE: 1`` and, per data
            file, ``000000: <rows> : <checksum> : <checksum>`` (the sysv
            checksum of the file's bytes)
  attr-v2   text, one attribute per line: ``<name> <dtype> <nmemb> <hex bytes>``
  000000    the rows, raw little-endian, C order

Columns are streamed from the device in chunks, so a 512^3-particle snapshot
needs a host buffer of one chunk only.  ``read`` loads a snapshot back (the
round trip is what the tests check; bigfile's own reader is absent here).
"""
import os

import numpy

CHUNK_ROWS = 1 << 22


def _sysv_sum(data, s=0):
    """Running byte sum for the sysv checksum (finished by _sysv_finish)."""
    return (s + int(numpy.frombuffer(data, dtype=numpy.uint8).sum(dtype=numpy.uint64))) & 0xFFFFFFFF


def _sysv_finish(s):
    r = (s & 0xFFFF) + (s >> 16)
    return (r & 0xFFFF) + (r >> 16)


def _dtype_str(dt):
    dt = numpy.dtype(dt)
    return dt.newbyteorder('<').str if dt.byteorder != '|' else dt.str


def _write_attrs(path, attrs):
    with open(os.path.join(path, 'attr-v2'), 'w') as f:
        for key in sorted(attrs):
            v = numpy.atleast_1d(numpy.asarray(attrs[key]))
            if v.dtype.kind in 'US':
                v = numpy.frombuffer(str(attrs[key]).encode(), dtype='S1')
            v = v.astype(v.dtype.newbyteorder('<'))
            f.write('%s %s %d %s\n' % (key, _dtype_str(v.dtype), v.size, v.tobytes().hex().upper()))


def _read_attrs(path):
    out = {}
    fn = os.path.join(path, 'attr-v2')
    if not os.path.exists(fn):
        return out
    with open(fn) as f:
        for line in f:
            parts = line.split()
            if len(parts) < 3:
                continue
            name, dt, nmemb = parts[0], parts[1], int(parts[2])
            raw = bytes.fromhex(parts[3]) if len(parts) > 3 else b''
            v = numpy.frombuffer(raw, dtype=numpy.dtype(dt))
            if v.dtype.kind == 'S':
                out[name] = b''.join(v.tolist()).decode()
            else:
                out[name] = v[0] if nmemb == 1 else v.copy()
    return out


def _write_block_header(path, dtype, nmemb, files):
    with open(os.path.join(path, 'header'), 'w') as f:
        f.write('DTYPE: %s\nNMEMB: %d\nNFILE: %d\n' % (_dtype_str(dtype), nmemb, len(files)))
        for i, (rows, ck) in enumerate(files):
            f.write('%06X: %d : %u : %u\n' % (i, rows, ck, ck))


def write_attrs_block(root, name, attrs):
    path = os.path.join(root, name)
    os.makedirs(path, exist_ok=True)
    _write_block_header(path, 'f8', 1, [])
    _write_attrs(path, attrs)


def write_column(root, name, array, dtype=None):
    """Column block `name` from a [rows] or [rows, nmemb] array (numpy or a
    torch tensor, on the device or the host), written in row chunks."""
    path = os.path.join(root, name)
    os.makedirs(path, exist_ok=True)
    rows = int(array.shape[0])
    nmemb = 1 if len(array.shape) == 1 else int(array.shape[1])
    dt = numpy.dtype(dtype) if dtype is not None else None
    s = 0
    with open(os.path.join(path, '000000'), 'wb') as f:
        for start in range(0, max(rows, 1), CHUNK_ROWS):
            part = array[start:start + CHUNK_ROWS]
            if hasattr(part, 'detach'):
                part = part.detach().cpu().numpy()
            part = numpy.ascontiguousarray(part, dtype=dt if dt is not None else part.dtype)
            dt = part.dtype
            part = part.astype(dt.newbyteorder('<'), copy=False)
            b = part.tobytes()
            s = _sysv_sum(b, s)
            f.write(b)
    _write_block_header(path, dt if dt is not None else 'f8', nmemb, [(rows, _sysv_finish(s))])
    _write_attrs(path, {})


def read_column(root, name):
    path = os.path.join(root, name)
    with open(os.path.join(path, 'header')) as f:
        lines = f.read().splitlines()
    meta = dict(l.split(': ', 1) for l in lines[:3])
    dt = numpy.dtype(meta['DTYPE'])
    nmemb = int(meta['NMEMB'])
    parts = []
    for i, line in enumerate(lines[3:3 + int(meta['NFILE'])]):
        rows, ck, _ = (int(x) for x in line.split(':', 1)[1].split(':'))
        raw = open(os.path.join(path, '%06X' % i), 'rb').read()
        if _sysv_finish(_sysv_sum(raw)) != ck:
            raise IOError('checksum mismatch in %s/%06X' % (path, i))
        a = numpy.frombuffer(raw, dtype=dt)
        parts.append(a.reshape(rows, nmemb) if nmemb > 1 else a)
    return numpy.concatenate(parts) if parts else numpy.empty((0, nmemb), dtype=dt)


def header_attrs(cosmology, a, H0=100.0, attrs={}):
    """The Header block's attributes as fastpm/core.py:70-83 sets them."""
    out = {}
    keylist = ['Om0', 'Tcmb0', 'Neff', 'Ob0', 'Ode0']
    if getattr(cosmology, 'm_nu', None) is not None:
        keylist.insert(3, 'm_nu')
    for key in keylist:
        out[key] = getattr(cosmology, key)
    out['Time'] = a
    out['h'] = cosmology.H0 / H0
    out['RSDFactor'] = 1.0 / (H0 * a * cosmology.efunc(1.0 / a - 1))
    for key in attrs:
        try:   # best effort, as the reference: values an attribute cannot hold are skipped
            if numpy.asarray(attrs[key]).dtype.kind in 'OV':
                raise TypeError(key)
            out[key] = attrs[key]
        except Exception:
            pass
    return out


def save_state(state, filename, attrs={}):
    """StateVector.save (core.py:65-89): Header attributes, then X = S + Q,
    V = P H0 / a_P and RHO as 1/Position, 1/Velocity, 1/Density, in the dtype
    of the positions Q (the reference's arrays share Q's dtype)."""
    a = state.a['S']
    os.makedirs(filename, exist_ok=True)
    write_attrs_block(filename, 'Header', header_attrs(state.cosmology, a, state.H0, attrs))
    dt = numpy.dtype(str(state.Q.dtype).replace('torch.', ''))
    vfac = state.H0 / state.a['P']
    n = len(state.Q)
    write_column(filename, '1/Position',
                 _Rows(lambda i, j: state.S[i:j].to(state.Q.dtype) + state.Q[i:j], n, 3), dt)
    write_column(filename, '1/Velocity', _Rows(lambda i, j: state.P[i:j].to(state.Q.dtype) * vfac, n, 3), dt)
    write_column(filename, '1/Density', state.RHO, dt)


class _Rows(object):
    """Array-like view that forms rows [i, j) on demand (slicing only)."""

    def __init__(self, fn, n, nmemb):
        self.fn = fn
        self.shape = (n, nmemb)

    def __getitem__(self, sl):
        i, j, _ = sl.indices(self.shape[0])
        return self.fn(i, j)


def read(filename):
    """(header attributes, {'Position', 'Velocity', 'Density'}) of a snapshot."""
    header = _read_attrs(os.path.join(filename, 'Header'))
    cols = {k: read_column(filename, '1/' + k) for k in ('Position', 'Velocity', 'Density')
            if os.path.isdir(os.path.join(filename, '1', k))}
    return header, cols
