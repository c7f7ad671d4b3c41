"""Generates the golden fixtures in tests/golden/ from the reference itself.

The reference physics (code/nans.cpp) is compiled headless from its own sources by
``make -C oracle ref`` (needs the reference checkout); this script drives those builds
through oracle/refbind.py and records, per case:

  inputs     the scene records (cubes, spheres, floor, model scales, constants)
  digests    a 16-hex SHA-256 prefix of every step's body state + contact list
  states     full body records at a few steps
  pairs      the contact lists at the same steps

Usage:  python tests/golden/make_golden.py [stack_bigepa_<scene>]
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from nans_projekat_gb300 import scenes  # noqa: E402
from oracle import refbind  # noqa: E402
from helpers import step_digest  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def run_world(name, scene, nsteps, keep_at, variant):
    w = refbind.RefWorld(scene, variant, rebuild=scene.rebuild_models)
    dt = np.float32(scene.constants.dt)
    digests = []
    saved = {}
    for k in range(1, nsteps + 1):
        w.step(dt, 1)
        cubes, spheres, floor = w.state()
        pairs = w.pairs()
        digests.append(step_digest(cubes, spheres, pairs))
        if k in keep_at:
            saved["cubes_%d" % k] = cubes
            saved["spheres_%d" % k] = spheres
            saved["pairs_%d" % k] = pairs
    save(name, scene, nsteps, digests, saved, variant)


def save(name, scene, nsteps, digests, saved, variant):
    c = scene.constants
    meta = dict(name=name, nsteps=nsteps, variant=variant, cr=float(c.cr), cf=float(c.cf),
                iterations=int(c.iterations), dt=float(np.float32(c.dt)),
                rebuild_models=bool(scene.rebuild_models))
    arrays = dict(in_cubes=scene.cubes, in_spheres=scene.spheres, in_floor=scene.floor,
                  in_scale=scene.scale_array(), digests=np.array(digests), meta=np.array(json.dumps(meta)))
    arrays.update(saved)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), **arrays)
    print("wrote", name, nsteps, "steps")


def run_frames(name, nframes, keep_at):
    """The reference's own SimUpdateAndRender on its Init scene (code/nans.cpp:1550-1729)."""
    f = refbind.RefFrame("ref_pristine")
    dt = np.float32(1.0 / 60.0)
    digests = []
    saved = {}
    for k in range(1, nframes + 1):
        f.run(dt, 1)
        cubes, spheres, floor, pairs = f.state()
        digests.append(step_digest(cubes, spheres, pairs))
        if k in keep_at:
            saved["cubes_%d" % k] = cubes
            saved["spheres_%d" % k] = spheres
            saved["pairs_%d" % k] = pairs
    save(name, scenes.demo_scene(), nframes, digests, saved, "ref_pristine(SimUpdateAndRender)")


def main():
    if not refbind.ref_available("refbig"):
        raise SystemExit("build the reference first: make -C oracle ref")
    run_world("stack8_seed0", scenes.stack_scene(0), 600, {1, 10, 100, 600}, "ref16")
    run_world("stack8_refconst", scenes.stack_scene(1, scenes.Constants.reference_defaults()), 200,
              {1, 200}, "ref_pristine")
    run_frames("demo_frames", 300, {1, 50, 300})
    rng = scenes.SplitMix64(11)
    for n in (5, 12, 40, 90):
        sc = scenes.stack_scene_random(rng, n)
        run_world("stack_random_%d" % n, sc, 120, {1, 120}, "ref16" if n <= 16 else "refbig")
    run_world("random_mixed72", scenes.random_scene(5, n_boxes=60, n_spheres=12, extent=8.0), 100,
              {1, 100}, "refbig")
    run_world("random_dense16", scenes.random_scene(6, n_boxes=12, n_spheres=4, extent=3.0), 200,
              {1, 200}, "ref16")
    # Scenes of the 16,384-scene stack workload (seed 2) that hit the reference's rare EPA paths:
    # an EPA that empties its face list (scenes 6663, 5642) and EPAs whose face list outgrows
    # 128 faces (scenes 3029, 7755, 6880).
    batch = scenes.stack_batch(16384, seed=2)
    for idx in (6663, 5642):
        run_world("stack_emptied_%d" % idx, batch[idx], 20, {20}, "refbig")
    for idx in (3029, 7755, 6880):
        run_world("stack_bigepa_%d" % idx, batch[idx], 30, {30}, "refbig")
    # scene 897 grows an EPA polytope beyond 256 faces (1,150) within 60 steps: it reaches the
    # block-wide tier (and, in worlds that route those to it, the grid-wide tier)
    run_world("stack_bigepa_897", batch[897], 60, {60}, "refbig")


def main_one(name):
    """Regenerates one fixture of the stack workload by its scene index (stack_bigepa_<i>)."""
    batch = scenes.stack_batch(16384, seed=2)
    idx = int(name.rsplit("_", 1)[1])
    run_world(name, batch[idx], 60 if idx == 897 else 30, {60 if idx == 897 else 30}, "refbig")


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main_one(sys.argv[1])
    else:
        main()
