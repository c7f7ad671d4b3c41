"""The fused per-scene step (NANS_WORLD_FUSED_STEP: after the sweep, one launch in which a block
per scene culls, collides and solves) against the reference's fixtures and the oracle, bit for
bit. It runs the staged kernels' device functions in another schedule, so every result must be
the staged step's: the reference's golden cases step by step on the plain path (the large-EPA
cases through the block-wide and the grid-wide tiers), 48 scenes of the benchmark batch for 600
steps against the reference, and batches with spheres and convex hulls against the oracle."""
import json
import os

import numpy as np
import pytest

from helpers import (GOLDEN_CASES, load_golden, step_digest, same_fields, first_difference, STATE_FIELDS,
                     PAIR_FIELDS)
from nans_projekat_gb300 import scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LARGE_EPA_CASES = [c for c in GOLDEN_CASES if "bigepa" in c or "emptied" in c]


@pytest.fixture(scope="module")
def nl():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from nans_projekat_gb300 import lib
    lib.load()
    return lib


def _plain_digests_match(nl, case, **flags):
    scene, meta, digests, _ = load_golden(case)
    w = nl.World(fused_step=True, **flags)
    w.upload(scene)
    dt = np.float32(scene.constants.dt)
    for k in range(1, meta["nsteps"] + 1):
        w.step(dt, 1)
        cubes, spheres, _ = w.download()
        if step_digest(cubes, spheres, w.pairs(0)) != digests[k - 1]:
            pytest.fail("%s: step %d of the fused step differs from the reference" % (case, k))
    assert w.status() == 0
    w.close()


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_fused_step_reproduces_reference_golden(nl, case):
    _plain_digests_match(nl, case)


@pytest.mark.parametrize("case", LARGE_EPA_CASES)
def test_fused_step_large_epa_on_the_grid_wide_tier(nl, case):
    _plain_digests_match(nl, case, giant_tier_only=True)


def test_fused_step_many_steps_per_call(nl):
    """One nans_step call of many steps replays one-step graphs of the fused step; the 8-cube
    stack's reference digests at steps 1, 10, 100, 250 and 600."""
    scene, _, digests, _ = load_golden("stack8_seed0")
    dt = np.float32(scene.constants.dt)
    w = nl.World(fused_step=True)
    w.upload(scene)
    done = 0
    for k in (1, 10, 100, 250, 600):
        w.step(dt, k - done)
        done = k
        cubes, spheres, _ = w.download()
        assert step_digest(cubes, spheres, w.pairs(0)) == digests[k - 1], "step %d" % k
    assert w.path_counts() == (599, 1)
    assert w.launches_per_step() == (5, 5)
    w.close()


def test_fused_step_benchmark_scenes_600_steps_match_reference(nl):
    """The 48 scenes of the benchmark batch that the reference stepped 600 steps (47 seeded and
    the largest, 256 bodies), as one batch on the fused step in ten 60-step graphs: bit for bit
    at every 60th step. A scene's result does not depend on the other scenes of its batch."""
    z = np.load(os.path.join(GOLDEN, "stack_batch600.npz"), allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    full = scenes.stack_batch(meta["n_scenes"], seed=meta["seed"])
    picked = meta["scenes"]
    batch = [full[i] for i in picked]
    dt = np.float32(batch[0].constants.dt)
    w = nl.World(fused_step=True)
    w.upload_batch(batch)
    every = meta["every"]
    for call in range(meta["nsteps"] // 60):
        w.batch_step(dt, 60, 60)
        k = 60 * (call + 1)
        state = w.download()
        for j, i in enumerate(picked):
            cubes, spheres, _ = w.scene_state(j, state)
            got = int(step_digest(cubes, spheres, w.pairs(j)), 16)
            assert got == int(z["digests"][j][k // every - 1]), \
                "scene %d (%d bodies) differs from the reference at step %d" % (i, batch[j].n_bodies, k)
    assert w.status() == 0
    w.close()


def _oracle_states(scenes_list, nsteps, dt, threads=8):
    from oracle.portbind import OracleWorld
    w = OracleWorld(scenes_list)
    w.step(dt, nsteps, threads)
    return w


@pytest.mark.parametrize("kind", ["stack256", "mixed64", "spheres_all_pairs"])
def test_fused_step_batches_match_oracle(nl, oracle_lib, kind):
    dt = np.float32(1 / 60)
    flags = {}
    if kind == "stack256":
        batch = scenes.stack_batch(16384, seed=2)[:256]
    elif kind == "mixed64":
        batch = scenes.mixed_batch(64, seed=4)
    else:
        batch = scenes.stack_batch(48, seed=5, lo=4, hi=40)
        flags = {"all_pairs": True}
    w = nl.World(fused_step=True, **flags)
    w.upload_batch(batch)
    w.batch_step(dt, 40, graph_steps=20)
    assert w.status() == 0
    state = w.download()
    o = _oracle_states(batch, 40, dt)
    for i in range(len(batch)):
        cubes, spheres, _ = w.scene_state(i, state)
        assert same_fields(o.state(i)[0], cubes, STATE_FIELDS + ("Vertices",))[0], \
            (i, first_difference(o.state(i)[0], cubes, STATE_FIELDS))
        assert same_fields(o.state(i)[1], spheres, STATE_FIELDS)[0], i
        assert same_fields(o.pairs(i), w.pairs(i), PAIR_FIELDS)[0], i
    # the candidate and contact counts of the last step are the staged step's
    ref = nl.World(**flags)
    ref.upload_batch(batch)
    ref.batch_step(dt, 40, graph_steps=20)
    assert w.counts() == ref.counts()
    ref.close()
    w.close()


def test_fused_step_limits(nl):
    with pytest.raises(nl.NansError) as e:
        nl.World(fused_step=True, warm_start=True)
    assert e.value.code == 1
    w = nl.World(fused_step=True)
    with pytest.raises(nl.NansError) as e:
        w.upload(scenes.random_scene(0))  # 4,608 bodies in one scene
    assert e.value.code == 7
    w.close()
