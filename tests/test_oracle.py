"""CPU tests of the oracle: the restatement against the golden fixtures (made from the
reference compiled headless), against the live reference build when it is present, and the
properties the device kernels rely on (conservative AABB cull, project sincos)."""
import numpy as np
import pytest

from helpers import (GOLDEN_CASES, load_golden, step_digest, same_fields, first_difference,
                     aabb_margin_boxes, STATE_FIELDS, PAIR_FIELDS)
from nans_projekat_gb300 import scenes


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_port_reproduces_golden(oracle_lib, case):
    from oracle.portbind import OracleWorld
    scene, meta, digests, saved = load_golden(case)
    w = OracleWorld([scene])
    dt = np.float32(meta["dt"])
    for k in range(1, meta["nsteps"] + 1):
        w.step(dt, 1)
        cubes, spheres, _ = w.state()
        pairs = w.pairs()
        d = step_digest(cubes, spheres, pairs)
        if d != digests[k - 1]:
            msg = ""
            if "cubes_%d" % k in saved:
                msg = first_difference(saved["cubes_%d" % k], cubes, STATE_FIELDS)
            pytest.fail("%s: step %d differs from the reference %s" % (case, k, msg))
        if "cubes_%d" % k in saved:
            assert same_fields(saved["cubes_%d" % k], cubes, STATE_FIELDS + ("Vertices",))[0]
            assert same_fields(saved["spheres_%d" % k], spheres, STATE_FIELDS)[0]
            assert same_fields(saved["pairs_%d" % k], pairs, PAIR_FIELDS)[0]


def test_golden_fixtures_are_nontrivial():
    # every case exercises contacts; the random cases exercise spheres and all pair types
    types = set()
    for case in GOLDEN_CASES:
        scene, meta, digests, saved = load_golden(case)
        assert len(set(digests)) > 1
        for k, v in saved.items():
            if k.startswith("pairs_"):
                types |= set(int(t) for t in v["Type"])
    assert types >= {0, 1, 2, 4}


def _ref_or_skip(variant):
    from oracle import refbind
    if not refbind.ref_available(variant):
        pytest.skip("reference build absent (make -C oracle ref needs the reference checkout)")
    return refbind


@pytest.mark.reference
@pytest.mark.parametrize("seed", [21, 22, 23])
def test_port_matches_live_reference(oracle_lib, seed):
    refbind = _ref_or_skip("refbig")
    from oracle.portbind import OracleWorld
    rng = scenes.SplitMix64(seed)
    cases = [scenes.stack_scene_random(rng, int(n)) for n in (7, 33, 70)]
    cases.append(scenes.random_scene(seed, n_boxes=40, n_spheres=10, extent=6.0))
    for sc in cases:
        ref = refbind.RefWorld(sc, "refbig")
        por = OracleWorld([sc])
        dt = np.float32(sc.constants.dt)
        for k in range(80):
            ref.step(dt, 1)
            por.step(dt, 1)
            rc, rs, _ = ref.state()
            pc, ps, _ = por.state()
            assert same_fields(rc, pc, STATE_FIELDS + ("Vertices", "Model"))[0], (sc.name, k)
            assert same_fields(rs, ps, STATE_FIELDS)[0], (sc.name, k)
            assert same_fields(ref.pairs(), por.pairs(), PAIR_FIELDS)[0], (sc.name, k)


@pytest.mark.reference
def test_reference_builds_agree():
    """The literal-rewritten build at its defaults equals the unmodified build, and the
    larger-capacity layout equals the 16-slot layout on scenes that fit."""
    refbind = _ref_or_skip("ref_pristine")
    sc = scenes.stack_scene(3, scenes.Constants.reference_defaults())
    worlds = [refbind.RefWorld(sc, v) for v in ("ref_pristine", "ref16", "refbig", "ref16_O2")]
    dt = np.float32(1 / 60)
    for k in range(150):
        outs = []
        for w in worlds:
            w.step(dt, 1)
            outs.append((w.state(), w.pairs()))
        for (c, s, _), p in outs[1:]:
            assert same_fields(outs[0][0][0], c, STATE_FIELDS + ("Vertices", "Model"))[0]
            assert same_fields(outs[0][1], p, PAIR_FIELDS)[0]


def test_reference_frame_matches_harness_rules(oracle_lib):
    """The demo fixture comes from the reference's own SimUpdateAndRender; the oracle's
    harness rules (model rebuild after each step) reproduce it."""
    from oracle.portbind import OracleWorld
    scene, meta, digests, saved = load_golden("demo_frames")
    assert not scene.rebuild_models
    w = OracleWorld([scene])
    w.step(np.float32(meta["dt"]), 50)
    cubes, spheres, _ = w.state()
    assert same_fields(saved["cubes_50"], cubes, STATE_FIELDS + ("Vertices", "Model"))[0]


def test_sincos_accuracy(oracle_lib):
    from oracle.portbind import sincos
    x = np.concatenate([np.linspace(-100, 100, 20001), np.array([0.0, -0.0, 1e-30, 3.14159265, 1e4])])
    x = x.astype(np.float32)
    s, c = sincos(x)
    xs = x.astype(np.float64)
    ulp = np.spacing(np.float32(1.0)).astype(np.float64)
    assert np.max(np.abs(s - np.sin(xs))) < 4 * ulp
    assert np.max(np.abs(c - np.cos(xs))) < 4 * ulp
    s0, c0 = sincos(np.zeros(1, np.float32))
    assert s0[0] == 0.0 and c0[0] == 1.0


def test_scene_generators_are_seeded():
    a = scenes.stack_batch(20, seed=9)
    b = scenes.stack_batch(20, seed=9)
    for x, y in zip(a, b):
        assert x.cubes.tobytes() == y.cubes.tobytes()
        assert x.spheres.tobytes() == y.spheres.tobytes()
    counts = [s.n_bodies for s in scenes.stack_batch(2000, seed=2)]
    assert 4 <= min(counts) and max(counts) <= 256
    # log-uniform in [4, 256]: the median sits near sqrt(4*256) = 32
    assert 20 < np.median(counts) < 50


def test_fp64_oracle_tracks_fp32(oracle_lib):
    from oracle.portbind import OracleWorld
    sc = scenes.stack_scene(0)
    w32 = OracleWorld([sc])
    w64 = OracleWorld([sc], fp64=True)
    w32.step(np.float32(1 / 60), 5)
    w64.step(np.float32(1 / 60), 5)
    a = w32.state_f64()
    b = w64.state_f64()
    assert np.allclose(a[:, :3], b[:, :3], rtol=1e-4, atol=1e-5)


def _cull_cases(seed):
    rng = scenes.SplitMix64(seed)
    cases = [scenes.stack_scene_random(rng, int(n)) for n in (20, 60, 120)]
    cases.append(scenes.random_scene(seed, n_boxes=80, n_spheres=20, extent=7.0))
    # dense random scenes make the reference eject bodies to huge coordinates and NaN
    cases.append(scenes.random_scene(seed, n_boxes=60, n_spheres=12, extent=8.0))
    return cases


@pytest.mark.parametrize("seed", [31, 32, 5])
def test_reference_contacts_have_overlapping_cull_boxes(oracle_lib, seed):
    """Every pair the reference reports overlaps in the boxes the device cull tests, so culling
    the others cannot drop a contact (many steps and scenes, exploding bodies included)."""
    from oracle.portbind import OracleWorld
    from helpers import aabb_margin_spheres
    dt = np.float32(1 / 60)
    checked = 0
    for sc in _cull_cases(seed):
        w = OracleWorld([sc])
        for k in range(100):
            w.stage(0, dt)
            w.stage(1, dt)
            cubes, spheres, floor = w.state()
            pairs = w.pairs()
            clo, chi = aabb_margin_boxes(cubes["Vertices"])
            flo, fhi = aabb_margin_boxes(floor["Vertices"])
            slo, shi = aabb_margin_spheres(spheres["Position"], spheres["Radius"])
            for p in pairs:
                t, a, b = int(p["Type"]), int(p["IndexA"]), int(p["IndexB"])
                A = (slo[a], shi[a]) if t in (3, 4) else (clo[a], chi[a])
                if t in (2, 4):
                    B = (flo[0], fhi[0])
                elif t in (1, 3):
                    B = (slo[b], shi[b])
                else:
                    B = (clo[b], chi[b])
                assert np.all(A[0] <= B[1]) and np.all(B[0] <= A[1]), (sc.name, k, t, a, b)
                checked += 1
            w.stage(2, dt)
            w.stage(3, dt)
            w.stage(4, dt)
    assert checked > 1000


def test_fp32_step_against_fp64_at_short_horizons(oracle_lib):
    """FP32 (what the GPU computes bit for bit) against an FP64 run of the same method
    (oracle/fp64_error.py): relative position error well inside 1e-4 over the first steps,
    before contacts that switch on in one precision and not the other make the runs diverge."""
    from oracle.fp64_error import errors
    from nans_projekat_gb300 import scenes as sc
    e = errors([sc.stack_scene(0)], [1, 10, 60], threads=1)
    assert e[1][1] < 1e-7 and e[10][1] < 1e-6 and e[60][0] < 1e-5 and e[60][1] < 1e-4
    g = errors(sc.grid_stack_batch(8, seed=3), [1], threads=4)
    assert g[1][1] < 1e-7
