"""Scene snapshots (nans_projekat_gb300/snapshot.py): the file round-trips every field bit for
bit (CPU), and a world saved mid-run and loaded into a new world continues exactly like the
uninterrupted one (GPU)."""
import json

import numpy as np
import pytest

from helpers import canon, same_fields, STATE_FIELDS, PAIR_FIELDS
from nans_projekat_gb300 import scenes, snapshot


def _same_scene(a, b):
    for f in a.cubes.dtype.names:
        assert canon(a.cubes[f]) == canon(b.cubes[f]), f
    for f in a.spheres.dtype.names:
        assert canon(a.spheres[f]) == canon(b.spheres[f]), f
    for f in a.floor.dtype.names:
        assert canon(a.floor[f]) == canon(b.floor[f]), f
    assert canon(a.scale_array()) == canon(b.scale_array())
    assert (a.hull_npts is None) == (b.hull_npts is None)
    if a.hull_npts is not None:
        assert np.array_equal(a.hull_npts, b.hull_npts)
        assert canon(np.asarray(a.hull_pts, np.float32)) == canon(b.hull_pts)
    assert np.float32(a.constants.cr) == np.float32(b.constants.cr)
    assert np.float32(a.constants.cf) == np.float32(b.constants.cf)
    assert a.constants.iterations == b.constants.iterations
    assert np.float32(a.constants.dt) == np.float32(b.constants.dt)
    assert a.rebuild_models == b.rebuild_models and a.name == b.name


@pytest.mark.parametrize("kind", ["stack", "mixed", "demo"])
def test_round_trip(tmp_path, kind):
    if kind == "stack":
        batch = scenes.stack_batch(40, seed=12, lo=4, hi=64)
    elif kind == "mixed":
        batch = scenes.mixed_batch(20, seed=13, lo=8, hi=40)
    else:
        batch = [scenes.demo_scene()]
    p = tmp_path / "s.nans"
    snapshot.save(str(p), batch, meta={"seed": 12, "generator": kind})
    back, meta = snapshot.load(str(p))
    assert meta == {"seed": 12, "generator": kind}
    assert len(back) == len(batch)
    for a, b in zip(batch, back):
        _same_scene(a, b)
    h = snapshot.read_header(str(p))
    assert h["version"] == 1 and h["scenes"] == len(batch)
    for d in h["arrays"]:
        assert d["offset"] % 64 == 0
    raw = p.read_bytes()
    assert raw[:8] == b"NANSSNAP"
    hlen = int(np.frombuffer(raw[12:20], np.uint64)[0])
    assert json.loads(raw[20:20 + hlen].decode())["arrays"] == h["arrays"]


def test_rejects_other_files(tmp_path):
    p = tmp_path / "x.bin"
    p.write_bytes(b"NOTASNAP" + bytes(64))
    with pytest.raises(ValueError):
        snapshot.load(str(p))


@pytest.mark.gpu
def test_saved_world_continues_exactly(nl_world, tmp_path):
    lib = nl_world
    batch = scenes.stack_batch(48, seed=14, lo=4, hi=96)
    dt = np.float32(1 / 60)
    a = lib.World()
    a.upload_batch(batch)
    a.batch_step(dt, 30, graph_steps=10)
    p = tmp_path / "mid.nans"
    snapshot.save(str(p), snapshot.from_world(a), meta={"steps": 30})
    loaded, meta = snapshot.load(str(p))
    assert meta["steps"] == 30
    b = lib.World()
    b.upload_batch(loaded)
    a.batch_step(dt, 20, graph_steps=10)
    b.batch_step(dt, 20, graph_steps=10)
    ca, sa, _ = a.download()
    cb, sb, _ = b.download()
    assert same_fields(ca, cb, STATE_FIELDS)[0]
    assert same_fields(sa, sb, STATE_FIELDS)[0]
    for i in range(len(batch)):
        assert same_fields(a.pairs(i), b.pairs(i), PAIR_FIELDS)[0], i
    a.close()
    b.close()


@pytest.fixture(scope="module")
def nl_world():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from nans_projekat_gb300 import lib
    lib.load()
    return lib
