"""StateVector.save's snapshot layout (fastpm/core.py:65-89) on the CPU: the
Header attributes, the three columns, and a write -> read round trip."""
import os

import numpy
import pytest
import torch


class _State(object):
    """The attributes StateVector.save reads (CPU tensors stand in for the
    device ones: the writer moves rows to the host in chunks either way)."""

    def __init__(self, n, cosmology, seed=0):
        g = torch.Generator().manual_seed(seed)
        self.Q = torch.rand((n, 3), generator=g, dtype=torch.float64) * 100
        self.S = torch.randn((n, 3), generator=g).float()
        self.P = torch.randn((n, 3), generator=g).float()
        self.RHO = torch.rand((n,), generator=g).float()
        self.a = dict(S=0.5, P=0.45, F=0.5)
        self.H0 = 100.
        self.cosmology = cosmology


@pytest.mark.parametrize('n', [0, 1000, 5000])
def test_snapshot_round_trip(tmp_path, n, monkeypatch):
    import fastpm_gb300 as G
    from fastpm_gb300 import snapshot
    monkeypatch.setattr(snapshot, 'CHUNK_ROWS', 777)      # several chunks per column
    st = _State(n, G.Planck15)
    path = str(tmp_path / 'snap')
    snapshot.save_state(st, path, attrs=dict(seed=42, note='run-1', bad=object()))
    header, cols = snapshot.read(path)
    X = (st.S.double() + st.Q).numpy()
    V = (st.P.double() * (100. / 0.45)).numpy()
    assert cols['Position'].dtype == numpy.float64 and cols['Position'].shape == (n, 3)
    numpy.testing.assert_array_equal(cols['Position'], X)
    numpy.testing.assert_array_equal(cols['Velocity'], V)
    numpy.testing.assert_array_equal(cols['Density'], st.RHO.double().numpy())
    # header attributes as core.py:70-83 sets them
    c = G.Planck15
    for key in ('Om0', 'Tcmb0', 'Neff', 'Ob0', 'Ode0'):
        assert header[key] == getattr(c, key)
    assert header['Time'] == 0.5
    assert header['h'] == c.H0 / 100.
    assert header['RSDFactor'] == 1.0 / (100. * 0.5 * c.efunc(1.0 / 0.5 - 1))
    assert header['seed'] == 42 and header['note'] == 'run-1'
    assert 'bad' not in header                              # best effort, as the reference
    assert sorted(os.listdir(path)) == ['1', 'Header']
    assert sorted(os.listdir(os.path.join(path, '1'))) == ['Density', 'Position', 'Velocity']
    with open(os.path.join(path, '1', 'Position', 'header')) as f:
        lines = f.read().splitlines()
    assert lines[:3] == ['DTYPE: <f8', 'NMEMB: 3', 'NFILE: 1']
    assert lines[3].startswith('000000: %d : ' % n)


def test_snapshot_checksum_detects_corruption(tmp_path):
    import fastpm_gb300 as G
    from fastpm_gb300 import snapshot
    st = _State(100, G.Planck15, seed=1)
    path = str(tmp_path / 'snap')
    snapshot.save_state(st, path)
    fn = os.path.join(path, '1', 'Velocity', '000000')
    raw = bytearray(open(fn, 'rb').read())
    raw[17] ^= 0x40
    open(fn, 'wb').write(bytes(raw))
    with pytest.raises(IOError):
        snapshot.read(path)
