"""Host logic of the autotuner (no GPU): candidate lists and the per-shape
result cache (in memory and in the JSON file named by FASTPM_GB300_TUNE_CACHE)."""
import json


def test_paint_candidates():
    from fastpm_gb300 import autotune
    c = autotune.paint_candidates(1024, 2)
    assert dict(paint='sorted', paint_brick=16) in c and dict(paint='sorted', paint_brick=8) in c
    assert dict(paint='tiled', tile_el=0) in c
    # the tiled paint's default lattice brick (16 / B, at least 4) is not listed twice
    assert dict(paint='tiled', tile_el=8) not in c and dict(paint='tiled', tile_el=4) in c
    # brick edges that do not divide the mesh, lattice bricks that do not divide the lattice
    c = autotune.paint_candidates(24, 1)
    assert dict(paint='sorted', paint_brick=16) not in c and dict(paint='sorted', paint_brick=8) in c
    assert all(e.get('tile_el', 0) in (0, 4, 8) and 24 % max(e.get('tile_el', 1), 1) == 0
               for e in c if e['paint'] == 'tiled')
    assert autotune.describe(dict(paint='tiled', tile_el=4)) == 'paint=tiled,tile_el=4'


def test_cache_round_trip(tmp_path, monkeypatch):
    from fastpm_gb300 import autotune
    path = tmp_path / 'tune.json'
    monkeypatch.setenv('FASTPM_GB300_TUNE_CACHE', str(path))
    monkeypatch.setattr(autotune, '_cache', {})
    key = 'paint|GB300|64,2'
    assert autotune.lookup(key) is None
    autotune.store(key, dict(paint='sorted', paint_brick=16))
    assert json.loads(path.read_text())[key] == dict(paint='sorted', paint_brick=16)
    # a new process (empty memory cache) finds it in the file
    monkeypatch.setattr(autotune, '_cache', {})
    assert autotune.lookup(key) == dict(paint='sorted', paint_brick=16)
    # a second key keeps the first
    autotune.store('force|GB300|64,2', dict(force='packed'))
    data = json.loads(path.read_text())
    assert set(data) == {key, 'force|GB300|64,2'}


def test_cache_tolerates_a_damaged_file(tmp_path, monkeypatch):
    from fastpm_gb300 import autotune
    path = tmp_path / 'tune.json'
    path.write_text('{not json')
    monkeypatch.setenv('FASTPM_GB300_TUNE_CACHE', str(path))
    monkeypatch.setattr(autotune, '_cache', {})
    assert autotune.lookup('paint|GB300|64,2') is None
    autotune.store('paint|GB300|64,2', dict(paint='tiled', tile_el=0))
    assert json.loads(path.read_text()) == {'paint|GB300|64,2': dict(paint='tiled', tile_el=0)}
