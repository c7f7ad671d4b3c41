"""GPU parity at the benchmark sizes and horizons, against fixtures made by the reference itself
(tests/golden/make_golden_long.py drives the reference's code/nans.cpp compiled headless).

  * the 16,384-scene stack batch (987,052 bodies), 600 steps on the batched path in ten calls of
    60 steps with a download after each (the first step after the upload runs eagerly, its 59
    followers replay the one-step graph, the other nine calls each replay one 60-step CUDA
    graph): 48 scenes, 47 seeded plus the largest, bit for bit at every 60th step;
  * the single large scene (4,096 boxes + 512 spheres), 300 steps of the plain path
    (nans_step, one call per step and a download after it, as the reference's frame calls its
    step and reads the bodies to draw them): every step, bit for bit.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from helpers import step_digest
from nans_projekat_gb300 import scenes

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _fixture(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)
    return z, json.loads(str(z["meta"]))


def _input_digest(scene):
    h = hashlib.sha256()
    for a in (scene.cubes, scene.spheres, scene.floor, scene.scale_array()):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


@pytest.fixture(scope="module")
def nl():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from nans_projekat_gb300 import lib
    lib.load()
    return lib


def test_full_batch_600_steps_in_graphs_matches_reference(nl):
    z, meta = _fixture("stack_batch600")
    batch = scenes.stack_batch(meta["n_scenes"], seed=meta["seed"])
    picked = meta["scenes"]
    for i, d in zip(picked, meta["inputs"]):
        assert _input_digest(batch[i]) == d, "scene %d: the generator no longer makes the fixture's inputs" % i
    assert max(s.n_bodies for s in batch) == batch[picked[-1]].n_bodies  # the largest scene is in
    dt = np.float32(batch[0].constants.dt)
    w = nl.World()
    w.upload_batch(batch)
    every = meta["every"]
    for call in range(meta["nsteps"] // 60):
        w.batch_step(dt, 60, 60)
        k = 60 * (call + 1)
        state = w.download()
        for j, i in enumerate(picked):
            cubes, spheres, _ = w.scene_state(i, state)
            got = int(step_digest(cubes, spheres, w.pairs(i)), 16)
            want = int(z["digests"][j][k // every - 1])
            assert got == want, "scene %d (%d bodies) differs from the reference at step %d" % (
                i, batch[i].n_bodies, k)
    graph_steps, eager_steps = w.path_counts()
    assert (graph_steps, eager_steps) == (599, 1)
    assert w.status() == 0
    w.close()


def test_large_scene_300_steps_matches_reference(nl):
    z, meta = _fixture("large4608_300")
    sc = scenes.random_scene(meta["seed"])
    assert _input_digest(sc) == meta["input"]
    dt = np.float32(sc.constants.dt)
    w = nl.World()
    w.upload(sc)
    for k in range(1, meta["nsteps"] + 1):
        w.step(dt, 1)
        cubes, spheres, _ = w.download()
        pairs = w.pairs(0)
        assert len(pairs) == int(z["contacts"][k - 1]), "step %d: contact count" % k
        assert int(step_digest(cubes, spheres, pairs), 16) == int(z["digests"][k - 1]), \
            "step %d differs from the reference" % k
    graph_steps, eager_steps = w.path_counts()
    assert (graph_steps, eager_steps) == (meta["nsteps"] - 1, 1)
    w.close()


def test_plain_path_graph_replay_matches_reference(nl):
    """nans_step over many steps in one call: after the first step every step replays a
    one-step CUDA graph, with one host synchronisation per call. The 8-cube stack's reference
    digests at steps 1, 10, 100, 250 and 600."""
    from helpers import load_golden
    scene, meta, digests, _ = load_golden("stack8_seed0")
    dt = np.float32(scene.constants.dt)
    w = nl.World()
    w.upload(scene)
    done = 0
    for k in (1, 10, 100, 250, 600):
        w.step(dt, k - done)
        done = k
        cubes, spheres, _ = w.download()
        assert step_digest(cubes, spheres, w.pairs(0)) == digests[k - 1], "step %d" % k
    graph_steps, eager_steps = w.path_counts()
    assert (graph_steps, eager_steps) == (599, 1)
    w.close()


@pytest.mark.parametrize("config", ["grid_stack_1024x120", "mixed_4096x240"])
def test_differentiated_configurations_at_full_size_match_oracle(nl, oracle_lib, config):
    """The differentiated configurations' forward step at their full size and horizon on the
    batched path: 1,024 4x4x2 stacks for 120 steps, and 4,096 mixed scenes of boxes, spheres and
    convex hulls for 240 steps (hulls have no reference counterpart, so the oracle is the
    checker); 64 scenes sampled with SplitMix64(77), bit for bit at the last step."""
    from oracle.portbind import OracleWorld
    if config == "grid_stack_1024x120":
        batch, nsteps = scenes.grid_stack_batch(1024, seed=3), 120
    else:
        batch, nsteps = scenes.mixed_batch(4096, seed=4), 240
    rng = scenes.SplitMix64(77)
    pick = sorted({int(x) for x in rng.uniform(64, 0, len(batch))})
    dt = np.float32(batch[0].constants.dt)
    w = nl.World()
    w.upload_batch(batch)
    w.batch_step(dt, nsteps, 60)
    assert w.status() == 0
    state = w.download()
    o = OracleWorld([batch[i] for i in pick])
    o.step(dt, nsteps, 16)
    for j, i in enumerate(pick):
        cubes, spheres, _ = w.scene_state(i, state)
        oc, os_, _ = o.state(j)
        assert step_digest(cubes, spheres, w.pairs(i)) == step_digest(oc, os_, o.pairs(j)), \
            "%s: scene %d differs from the oracle at step %d" % (config, i, nsteps)
    w.close()
