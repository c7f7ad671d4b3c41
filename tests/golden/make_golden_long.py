"""Generates the long-horizon and full-size fixtures in tests/golden/ from the reference itself.

The reference physics (code/nans.cpp) is compiled headless from its own sources by
``make -C oracle ref`` (needs the reference checkout). This script drives the 8,192-slot build
(oracle/_ref/libnans_refbig.so, -O0 as the reference's build script compiles it) through
oracle/refbind.py and records step digests (the 16-hex SHA-256 prefix of tests/helpers.py's
step_digest, stored as uint64) for two workloads:

  stack_batch600   48 scenes of the 16,384-scene benchmark batch (seed 2): 47 drawn with a
                   seeded SplitMix64 plus the batch's largest scene, each stepped 600 steps
                   by the reference; digests at every 10th step
  large4608_300    the single large scene (4,096 boxes + 512 spheres in a 64^3 m box, seed 1),
                   300 steps of the reference's all-pairs step; digests at every step, and the
                   reference's wall time per step on one core

Usage:  python tests/golden/make_golden_long.py [stack_batch600] [large4608_300]
"""
import hashlib
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

OUT = os.path.dirname(os.path.abspath(__file__))
BATCH_SEED = 2
BATCH_SCENES = 16384
BATCH_STEPS = 600
BATCH_EVERY = 10
LARGE_STEPS = 300


def input_digest(scene):
    h = hashlib.sha256()
    for a in (scene.cubes, scene.spheres, scene.floor, scene.scale_array()):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


def batch_sample():
    """47 distinct scene indices drawn with SplitMix64(600), plus the largest scene."""
    from nans_projekat_gb300 import scenes
    batch = scenes.stack_batch(BATCH_SCENES, seed=BATCH_SEED)
    counts = np.array([s.n_bodies for s in batch])
    rng = scenes.SplitMix64(600)
    picked = []
    largest = int(np.argmax(counts))
    while len(picked) < 47:
        i = int(rng.uniform(1, 0, BATCH_SCENES)[0])
        if i not in picked and i != largest:
            picked.append(i)
    return sorted(picked) + [largest], batch


def _run_scene(args):
    idx, nsteps, every = args
    from nans_projekat_gb300 import scenes
    from oracle import refbind
    from helpers import step_digest
    scene = scenes.stack_batch(BATCH_SCENES, seed=BATCH_SEED)[idx]
    w = refbind.RefWorld(scene, "refbig", rebuild=scene.rebuild_models)
    dt = np.float32(scene.constants.dt)
    out = []
    t0 = time.time()
    for k in range(1, nsteps + 1):
        w.step(dt, 1)
        if k % every == 0:
            cubes, spheres, _ = w.state()
            out.append(int(step_digest(cubes, spheres, w.pairs()), 16))
    return idx, out, input_digest(scene), time.time() - t0


def make_batch600():
    picked, batch = batch_sample()
    jobs = [(i, BATCH_STEPS, BATCH_EVERY) for i in picked]
    # the largest scenes first, so that the pool's tail is short
    jobs.sort(key=lambda j: -batch[j[0]].n_bodies)
    res = {}
    ctx = mp.get_context("spawn")
    with ctx.Pool(max(1, (os.cpu_count() or 3) - 2)) as pool:
        for idx, dig, ind, secs in pool.imap_unordered(_run_scene, jobs):
            res[idx] = (dig, ind)
            print("scene %5d (%3d bodies): %.1f s" % (idx, batch[idx].n_bodies, secs), flush=True)
    digests = np.array([res[i][0] for i in picked], np.uint64)
    meta = dict(name="stack_batch600", seed=BATCH_SEED, n_scenes=BATCH_SCENES, nsteps=BATCH_STEPS,
                every=BATCH_EVERY, scenes=picked, bodies=[int(batch[i].n_bodies) for i in picked],
                inputs=[res[i][1] for i in picked], variant="refbig (-O0)")
    np.savez_compressed(os.path.join(OUT, "stack_batch600.npz"), digests=digests, meta=np.array(json.dumps(meta)))
    print("wrote stack_batch600")


def make_large300():
    from nans_projekat_gb300 import scenes
    from oracle import refbind
    from helpers import step_digest
    scene = scenes.random_scene(1)
    w = refbind.RefWorld(scene, "refbig", rebuild=scene.rebuild_models)
    dt = np.float32(scene.constants.dt)
    digests, secs, npairs = [], [], []
    for k in range(1, LARGE_STEPS + 1):
        t0 = time.perf_counter()
        w.step(dt, 1)
        secs.append(time.perf_counter() - t0)
        cubes, spheres, _ = w.state()
        pairs = w.pairs()
        npairs.append(len(pairs))
        digests.append(int(step_digest(cubes, spheres, pairs), 16))
        if k % 10 == 0:
            print("large step %d: %.1f s, %d contacts" % (k, secs[-1], len(pairs)), flush=True)
    meta = dict(name="large4608_300", seed=1, nsteps=LARGE_STEPS, bodies=int(scene.n_bodies),
                input=input_digest(scene), variant="refbig (-O0)",
                ref_seconds_per_step_median=float(np.median(secs)), ref_cpu="one core of the fixture host")
    np.savez_compressed(os.path.join(OUT, "large4608_300.npz"), digests=np.array(digests, np.uint64),
                        contacts=np.array(npairs, np.int32), meta=np.array(json.dumps(meta)))
    print("wrote large4608_300")


def main():
    from oracle import refbind
    if not refbind.ref_available("refbig"):
        raise SystemExit("build the reference first: make -C oracle ref")
    which = sys.argv[1:] or ["stack_batch600", "large4608_300"]
    if "stack_batch600" in which:
        make_batch600()
    if "large4608_300" in which:
        make_large300()


if __name__ == "__main__":
    main()
