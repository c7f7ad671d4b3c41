"""GPU parity tests: the CUDA step, called through the C ABI, against the oracle and the
golden fixtures made from the reference. Parity is bit-exact (NaN matches NaN) for every
body state, every contact list and every step."""
import numpy as np
import pytest

from helpers import (GOLDEN_CASES, canon, load_golden, step_digest, same_fields, first_difference,
                     STATE_FIELDS, PAIR_FIELDS)
from nans_projekat_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def nl():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from nans_projekat_gb300 import lib
    lib.load()
    return lib


def test_device_sincos_matches_oracle(nl, oracle_lib):
    from oracle.portbind import sincos
    rng = np.random.default_rng(0)
    x = np.concatenate([np.linspace(-720, 720, 100001), rng.uniform(-1e5, 1e5, 100000),
                        np.array([0.0, -0.0, 1e-38, np.inf, -np.inf, np.nan])]).astype(np.float32)
    s_h, c_h = sincos(x)
    s_d, c_d = nl.device_sincos(x)
    fin = np.isfinite(x)
    assert s_h[fin].tobytes() == s_d[fin].tobytes()
    assert c_h[fin].tobytes() == c_d[fin].tobytes()
    assert np.all(np.isnan(s_d[~fin])) and np.all(np.isnan(c_d[~fin]))


def _run_plain_digests(nl, scene, nsteps, all_pairs=False, giant_tier_only=False):
    w = nl.World(all_pairs=all_pairs, giant_tier_only=giant_tier_only)
    w.upload(scene)
    dt = np.float32(scene.constants.dt)
    out = []
    for k in range(1, nsteps + 1):
        w.step(dt, 1)
        cubes, spheres, _ = w.download()
        pairs = w.pairs(0)
        out.append((step_digest(cubes, spheres, pairs), cubes, spheres, pairs))
    assert w.status() == 0
    w.close()
    return out


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_plain_step_reproduces_reference_golden(nl, case):
    scene, meta, digests, saved = load_golden(case)
    res = _run_plain_digests(nl, scene, meta["nsteps"])
    for k, (d, cubes, spheres, pairs) in enumerate(res, start=1):
        if d != digests[k - 1]:
            pytest.fail("%s: step %d differs from the reference" % (case, k))
        if "cubes_%d" % k in saved:
            ok, f = same_fields(saved["cubes_%d" % k], cubes, STATE_FIELDS + ("Vertices",))
            assert ok, (f, first_difference(saved["cubes_%d" % k], cubes, STATE_FIELDS))
            assert same_fields(saved["spheres_%d" % k], spheres, STATE_FIELDS)[0]
            assert same_fields(saved["pairs_%d" % k], pairs, PAIR_FIELDS)[0]


LARGE_EPA_CASES = [c for c in GOLDEN_CASES if "bigepa" in c or "emptied" in c]


@pytest.mark.parametrize("case", LARGE_EPA_CASES)
def test_grid_wide_epa_tier_reproduces_reference_golden(nl, case):
    """The same reference fixtures with every EPA beyond the warp tier's 256 faces routed to the
    grid-wide tier (cooperative launch) instead of the per-block tier."""
    scene, meta, digests, _ = load_golden(case)
    res = _run_plain_digests(nl, scene, meta["nsteps"], giant_tier_only=True)
    for k, (d, _, _, _) in enumerate(res, start=1):
        if d != digests[k - 1]:
            pytest.fail("%s: step %d differs from the reference" % (case, k))


def test_grid_wide_epa_tier_in_graphs(nl):
    """The grid-wide tier inside the batched path's CUDA graphs: the large-EPA fixtures as one
    batch, final state and contacts against the reference's digests."""
    cases = [load_golden(c) for c in LARGE_EPA_CASES]
    dt = np.float32(cases[0][0].constants.dt)
    cases = [c for c in cases if np.float32(c[0].constants.dt) == dt and
             c[0].rebuild_models == cases[0][0].rebuild_models]
    n = min(c[1]["nsteps"] for c in cases)
    w = nl.World(giant_tier_only=True)
    w.upload_batch([c[0] for c in cases])
    w.batch_step(dt, n, graph_steps=max(1, n // 3))
    state = w.download()
    for i, (_, _, digests, _) in enumerate(cases):
        cubes, spheres, _ = w.scene_state(i, state)
        assert step_digest(cubes, spheres, w.pairs(i)) == digests[n - 1], LARGE_EPA_CASES[i]
    w.close()


def test_large_scene_cull_equals_all_pairs(nl):
    """One 6,600-body scene (21.8 M pairs, 680,000 mask words): the culled step must give the
    all-pairs result."""
    sc = scenes.random_scene(seed=4, n_boxes=6000, n_spheres=600, extent=150.0)
    dt = np.float32(1 / 60)
    a = nl.World()
    b = nl.World(all_pairs=True)
    a.upload(sc)
    b.upload(sc)
    a.step(dt, 3)
    b.step(dt, 3)
    ca, sa, _ = a.download()
    cb, sb, _ = b.download()
    assert same_fields(ca, cb, STATE_FIELDS)[0]
    assert same_fields(sa, sb, STATE_FIELDS)[0]
    assert same_fields(a.pairs(0), b.pairs(0), PAIR_FIELDS)[0]
    assert len(a.pairs(0)) > 0
    a.close()
    b.close()


def _single_box_scenes(n):
    from nans_projekat_gb300.types import SPHERE_DTYPE
    out = []
    for k in range(n):
        pos = np.array([[0.01 * (k % 5), 0.49 + 0.002 * (k % 3), 0.0]])
        m = np.ones(1)
        cubes = scenes._cubes(pos, None, m, m / 12.0 * 2.0, vel=[[0.3 * ((k % 4) - 1.5), -0.5, 0.0]])
        out.append(scenes.Scene(cubes, np.zeros(0, SPHERE_DTYPE), scenes.ground(20.0), name="box1"))
    return out


def test_one_wave_per_contact_scenes(nl, oracle_lib):
    """Scenes whose every candidate is a contact in a wave of its own (one box on the ground:
    one candidate, one contact, one wave) use all of their solver slots; 512 of them solved side
    by side must still match the oracle."""
    batch = _single_box_scenes(512)
    dt = np.float32(1 / 60)
    n = 30
    o = _oracle_states(batch, n, dt)
    for graph in (False, True):
        w = nl.World()
        w.upload_batch(batch)
        if graph:
            w.batch_step(dt, n, graph_steps=10)
        else:
            w.step(dt, n)
        state = w.download()
        for i in range(len(batch)):
            cubes, _, _ = w.scene_state(i, state)
            assert same_fields(o.state(i)[0], cubes, STATE_FIELDS)[0], (graph, i)
            assert same_fields(o.pairs(i), w.pairs(i), PAIR_FIELDS)[0], (graph, i)
        assert sum(len(w.pairs(i)) for i in range(0, 512, 16)) > 0
        w.close()


def test_warm_start_matches_oracle(nl, oracle_lib):
    """NANS_WORLD_WARM_START against the oracle's warm starting (accumulators carried across
    steps for pairs that stay in contact), bit for bit, on the batched and the plain path; and
    it does change the result."""
    batch = scenes.stack_batch(64, seed=15, lo=4, hi=64)
    dt = np.float32(1 / 60)
    n = 60
    o = _oracle_states(batch, 0, dt)
    o.set_warm(True)
    o.step(dt, n, 8)
    w = nl.World(warm_start=True)
    w.upload_batch(batch)
    w.batch_step(dt, n, graph_steps=20)
    state = w.download()
    for i in range(len(batch)):
        cubes, spheres, _ = w.scene_state(i, state)
        oc, os_, _ = o.state(i)
        assert same_fields(oc, cubes, STATE_FIELDS)[0], (i, first_difference(oc, cubes, STATE_FIELDS))
        assert same_fields(os_, spheres, STATE_FIELDS)[0], i
    p = nl.World(warm_start=True)
    p.upload(batch[3])
    p.step(dt, n)
    assert same_fields(p.download()[0], w.scene_state(3, state)[0], STATE_FIELDS)[0]
    cold = nl.World()
    cold.upload_batch(batch)
    cold.batch_step(dt, n, graph_steps=20)
    assert not same_fields(cold.download()[0], state[0], STATE_FIELDS)[0]
    for x in (w, p, cold):
        x.close()


def test_state_arrays_match_records(nl):
    """nans_world_get_state_arrays returns the records' Position / Angles / V / W in record
    order, and a step after nans_world_set_state_arrays equals a step after the record-based
    nans_world_set_state (Model rebuilt, no external forces) bit for bit."""
    batch = scenes.stack_batch(64, seed=9, lo=4, hi=48)
    dt = np.float32(1 / 60)
    a = nl.World()
    a.upload_batch(batch)
    a.batch_step(dt, 25, graph_steps=10)
    cubes, spheres, _ = a.download()
    P, A, V, W = a.get_state_arrays()
    cat = lambda f: np.concatenate([cubes[f], spheres[f]]).astype(np.float32)
    for got, f in ((P, "Position"), (A, "Angles"), (V, "V"), (W, "W")):
        assert canon(got) == canon(cat(f)), f
    b = nl.World()
    b.upload_batch(batch)
    b.set_state_arrays(P, A, V, W)
    a.set_state(cubes, spheres, keep_model=False)
    a.step(dt, 5)
    b.step(dt, 5)
    ca, sa, _ = a.download()
    cb, sb, _ = b.download()
    assert same_fields(ca, cb, STATE_FIELDS + ("Vertices",))[0]
    assert same_fields(sa, sb, STATE_FIELDS)[0]
    for i in range(len(batch)):
        assert same_fields(a.pairs(i), b.pairs(i), PAIR_FIELDS)[0], i
    a.close()
    b.close()


def test_state_arrays_through_pinned_host_memory(nl):
    """Page-locked host arrays (the end-to-end benchmark's) carry the same values as pageable
    arrays, in both directions."""
    import torch
    batch = scenes.stack_batch(32, seed=10, lo=4, hi=40)
    dt = np.float32(1 / 60)
    w = nl.World()
    w.upload_batch(batch)
    w.batch_step(dt, 12, graph_steps=0)
    n = w.n_bodies

    def pinned():
        return torch.empty(n * 12, dtype=torch.uint8, pin_memory=True).numpy().view(np.float32).reshape(n, 3)

    ref = w.get_state_arrays()
    pin = tuple(pinned() for _ in range(4))
    w.get_state_arrays(out=pin)
    for r, p in zip(ref, pin):
        assert canon(r) == canon(p)
    moved = [p.copy() for p in pin]
    moved[2][:] += np.float32(0.5)
    for p, m in zip(pin, moved):
        p[:] = m
    w.set_state_arrays(*pin)
    back = w.get_state_arrays()
    for m, b in zip(moved, back):
        assert canon(m) == canon(b)
    w.close()


def test_demo_frames_model_and_vertices(nl):
    """The reference frame's records after 300 frames, Model and Vertices included."""
    scene, meta, digests, saved = load_golden("demo_frames")
    w = nl.World()
    w.upload(scene)
    w.step(np.float32(meta["dt"]), 300)
    cubes, spheres, _ = w.download()
    assert same_fields(saved["cubes_300"], cubes, STATE_FIELDS + ("Vertices", "Model"))[0]
    assert same_fields(saved["spheres_300"], spheres, STATE_FIELDS + ("Model",))[0]


@pytest.mark.parametrize("seed", [41, 42])
def test_cull_equals_all_pairs(nl, oracle_lib, seed):
    """The conservative AABB cull yields exactly the reference's all-pairs result."""
    rng = scenes.SplitMix64(seed)
    sc = scenes.stack_scene_random(rng, 64)
    a = _run_plain_digests(nl, sc, 40, all_pairs=False)
    b = _run_plain_digests(nl, sc, 40, all_pairs=True)
    assert [x[0] for x in a] == [x[0] for x in b]


def _oracle_states(scenes_list, nsteps, dt, threads=8):
    from oracle.portbind import OracleWorld
    w = OracleWorld(scenes_list)
    w.step(dt, nsteps, threads)
    return w


def test_batched_graph_path_matches_oracle(nl, oracle_lib):
    batch = scenes.stack_batch(96, seed=5, lo=4, hi=96)
    dt = np.float32(1 / 60)
    nsteps = 50
    w = nl.World()
    w.upload_batch(batch)
    w.batch_step(dt, nsteps, graph_steps=20)  # 1 eager + 2 graphs of 20 + 9 eager
    state = w.download()
    o = _oracle_states(batch, nsteps, dt)
    for i, sc in enumerate(batch):
        cubes, spheres, _ = w.scene_state(i, state)
        oc, os_, _ = o.state(i)
        assert same_fields(oc, cubes, STATE_FIELDS + ("Vertices",))[0], (i, first_difference(oc, cubes, STATE_FIELDS))
        assert same_fields(os_, spheres, STATE_FIELDS)[0], i
        assert same_fields(o.pairs(i), w.pairs(i), PAIR_FIELDS)[0], i
    assert w.status() == 0


def test_autotune_keeps_results(nl, oracle_lib):
    batch = scenes.stack_batch(40, seed=6, lo=8, hi=64)
    dt = np.float32(1 / 60)
    w = nl.World()
    w.upload_batch(batch)
    w.autotune(dt)
    w.batch_step(dt, 30, graph_steps=10)
    state = w.download()
    o = _oracle_states(batch, 30, dt)
    for i in range(len(batch)):
        assert same_fields(o.state(i)[0], w.scene_state(i, state)[0], STATE_FIELDS)[0], i


def test_large_random_scene_matches_oracle(nl, oracle_lib):
    """A scaled-down version of the 4,096-box + 512-sphere scene (same distributions)."""
    sc = scenes.random_scene(1, n_boxes=700, n_spheres=90, extent=16.0)
    dt = np.float32(1 / 60)
    w = nl.World()
    w.upload(sc)
    w.step(dt, 40)
    cubes, spheres, _ = w.download()
    o = _oracle_states([sc], 40, dt)
    oc, os_, _ = o.state(0)
    assert same_fields(oc, cubes, STATE_FIELDS + ("Vertices",))[0], first_difference(oc, cubes, STATE_FIELDS)
    assert same_fields(os_, spheres, STATE_FIELDS)[0]
    assert same_fields(o.pairs(0), w.pairs(0), PAIR_FIELDS)[0]


def test_hull_scenes_match_oracle(nl, oracle_lib):
    """Convex hulls of 8-32 points (a shape the reference lacks) against the oracle's hull
    support map with the same first-maximum rule."""
    batch = scenes.mixed_batch(24, seed=8, lo=8, hi=48)
    dt = np.float32(1 / 60)
    w = nl.World()
    w.upload_batch(batch)
    w.batch_step(dt, 40, graph_steps=10)
    state = w.download()
    o = _oracle_states(batch, 40, dt)
    for i in range(len(batch)):
        cubes, spheres, _ = w.scene_state(i, state)
        oc, os_, _ = o.state(i)
        assert same_fields(oc, cubes, STATE_FIELDS)[0], (i, first_difference(oc, cubes, STATE_FIELDS))
        assert same_fields(os_, spheres, STATE_FIELDS)[0], i


def test_set_state_continues_exactly(nl):
    sc = scenes.stack_scene(0)
    dt = np.float32(1 / 60)
    a = nl.World()
    a.upload(sc)
    a.step(dt, 30)
    ca, sa, _ = a.download()
    b = nl.World()
    b.upload(sc)
    b.step(dt, 10)
    cb, sb, _ = b.download()
    b.set_state(cb, sb, keep_model=True)
    b.step(dt, 20)
    cb, sb, _ = b.download()
    assert same_fields(ca, cb, STATE_FIELDS + ("Vertices", "Model"))[0]
    assert same_fields(sa, sb, STATE_FIELDS)[0]


def test_error_codes(nl):
    sc = scenes.stack_scene(0)
    w = nl.World()
    with pytest.raises(nl.NansError) as e:
        w.step(np.float32(1 / 60), 1)
    assert e.value.code == 6  # not uploaded
    bad = scenes.stack_scene(0)
    bad.cubes["Mass"][2] = np.nan
    with pytest.raises(nl.NansError) as e:
        w.upload(bad)
    assert e.value.code == 3  # NaN input
    bad = scenes.stack_scene(0)
    bad.spheres["Radius"][0] = 0.0
    with pytest.raises(nl.NansError) as e:
        w.upload(bad)
    assert e.value.code == 3
    w.upload(sc)
    for dt in (0.0, -1.0, np.inf, np.nan):
        with pytest.raises(nl.NansError) as e:
            w.step(np.float32(dt), 1)
        assert e.value.code == 1
    with pytest.raises(nl.NansError) as e:
        w.pairs(5)
    assert e.value.code == 1


def test_candidate_capacity(nl, oracle_lib):
    """The plain path grows its candidate buffers; the batched (graph) path reports
    NANS_ERR_CAPACITY instead of dropping pairs."""
    sc = scenes.stack_scene_random(scenes.SplitMix64(3), 80)
    dt = np.float32(1 / 60)
    w = nl.World(max_candidates=4)
    w.upload(sc)
    w.step(dt, 5)
    o = _oracle_states([sc], 5, dt)
    assert same_fields(o.state(0)[0], w.download()[0], STATE_FIELDS)[0]
    w2 = nl.World(max_candidates=4)
    w2.upload_batch([sc])
    with pytest.raises(nl.NansError) as e:
        w2.batch_step(dt, 3, graph_steps=2)
    assert e.value.code == 2


def test_full_size_batch_samples_match_oracle(nl, oracle_lib):
    """16,384 uneven scenes (log-uniform 4..256 bodies) for 20 steps on the GPU; a sample of
    scenes is replayed on the oracle (scenes are independent) and must match bit for bit."""
    batch = scenes.stack_batch(16384, seed=2)
    dt = np.float32(1 / 60)
    w = nl.World()
    w.upload_batch(batch)
    w.batch_step(dt, 20, graph_steps=10)
    assert w.status() == 0
    state = w.download()
    cubes_all, spheres_all, _ = state
    assert np.all(np.isfinite(cubes_all["Position"]))
    rng = np.random.default_rng(1)
    pick = sorted(set(rng.integers(0, len(batch), 48).tolist()) | {int(np.argmax([s.n_bodies for s in batch]))})
    o = _oracle_states([batch[i] for i in pick], 20, dt)
    for j, i in enumerate(pick):
        cubes, spheres, _ = w.scene_state(i, state)
        oc, os_, _ = o.state(j)
        assert same_fields(oc, cubes, STATE_FIELDS)[0], (i, first_difference(oc, cubes, STATE_FIELDS))
        assert same_fields(os_, spheres, STATE_FIELDS)[0], i
        assert same_fields(o.pairs(j), w.pairs(i), PAIR_FIELDS)[0], i


@pytest.mark.parametrize("tuning", [(0, 32, 128, 1, 6, 2), (4, 64, 256, 0, 2, 3), (2, 32, 64, 1, 12, 1),
                                    (0, 32, 128, 0, 1, 3)])
def test_results_do_not_depend_on_launch_parameters(nl, oracle_lib, tuning):
    """The GJK blocks per SM, the solver's threads per scene (both passes), its late-pass blocks
    per SM, the warp-tier EPA's blocks per SM and the cull method (tiles or one lane per pair)
    change the schedule, never the result: 256 workload scenes for 40 steps against the oracle,
    bit for bit."""
    batch = scenes.stack_batch(16384, seed=2)[:256]
    dt = np.float32(1 / 60)
    w = nl.World()
    w.upload_batch(batch)
    w.set_tuning(*tuning)
    w.batch_step(dt, 40, graph_steps=20)
    assert w.status() == 0
    t = w.tuning()
    assert (t["gjk_blocks_per_sm"], t["solve_threads"], t["solve_threads_late"], t["cull_tiles"],
            t["solve_late_blocks_per_sm"], t["warp_epa_blocks_per_sm"]) == tuning
    state = w.download()
    o = _oracle_states(batch, 40, dt)
    for i in range(len(batch)):
        cubes, spheres, _ = w.scene_state(i, state)
        oc, os_, _ = o.state(i)
        assert same_fields(oc, cubes, STATE_FIELDS)[0], (i, first_difference(oc, cubes, STATE_FIELDS))
        assert same_fields(os_, spheres, STATE_FIELDS)[0], i
        assert same_fields(o.pairs(i), w.pairs(i), PAIR_FIELDS)[0], i
    w.close()


def test_autotuner_times_every_candidate(nl):
    batch = scenes.stack_batch(16384, seed=2)[:512]
    w = nl.World()
    w.upload_batch(batch)
    w.step(np.float32(1 / 60), 2)
    w.autotune(np.float32(1 / 60))
    t = w.tuning()
    assert t["candidates_timed"] == 12 and t["us_per_step"] > 0
    assert t["gjk_blocks_per_sm"] in (0, 4) and t["solve_threads"] in (32, 64)
    w.close()


def test_giant_tier_barrier_timeout_is_reported(nl, oracle_lib):
    """The grid-wide EPA tier's barrier waits are bounded. With NANS_WORLD_TEST_BARRIER_TIMEOUT a
    barrier waits for one arrival more than the grid has (an arrival that never comes) and gives
    up after 4,096 polls: the step must return NANS_ERR_EPA_CAPACITY with the timeout bit set,
    and the GPU must keep answering (a following world steps bit-exactly against the oracle)."""
    raised = 0
    for case in LARGE_EPA_CASES:
        scene, meta, _, _ = load_golden(case)
        dt = np.float32(scene.constants.dt)
        probe = nl.World(giant_tier_only=True)
        probe.upload(scene)
        probe.step(dt, meta["nsteps"])
        ran = probe.epa_stats()["giant_tier"]
        probe.close()
        if case == "stack_bigepa_897":
            assert ran >= 1  # its 1,150-face EPA leaves the warp tier
        if ran == 0:
            continue
        w = nl.World(giant_tier_only=True, barrier_timeout_test=True)
        w.upload(scene)
        with pytest.raises(nl.NansError) as e:
            for _ in range(meta["nsteps"]):
                w.step(dt, 1)
        assert e.value.code == 5 and "timed out" in str(e.value)
        assert w.status() & (1 << 5)
        w.close()
        raised += 1
    assert raised >= 1
    sc = scenes.stack_scene(0)
    w = nl.World()
    w.upload(sc)
    w.step(np.float32(1 / 60), 30)
    o = _oracle_states([sc], 30, np.float32(1 / 60))
    assert same_fields(o.state(0)[0], w.download()[0], STATE_FIELDS)[0]
    w.close()


def test_warp_per_pair_gjk_matches_oracle(nl, oracle_lib):
    """GJK with one warp per candidate pair (NANS_WORLD_GJK_WARP: supports evaluated across the
    lanes, first-maximum shuffle reductions) gives the one-thread-per-pair result: 256 workload
    scenes for 40 steps against the oracle, bit for bit, with a convex-hull batch as well."""
    dt = np.float32(1 / 60)
    for batch in (scenes.stack_batch(16384, seed=2)[:256], scenes.mixed_batch(64, seed=4)):
        w = nl.World(gjk_warp=True)
        w.upload_batch(batch)
        w.batch_step(dt, 40, graph_steps=20)
        assert w.status() == 0
        state = w.download()
        o = _oracle_states(batch, 40, dt)
        for i in range(len(batch)):
            cubes, spheres, _ = w.scene_state(i, state)
            assert same_fields(o.state(i)[0], cubes, STATE_FIELDS)[0], (i, first_difference(o.state(i)[0], cubes,
                                                                                             STATE_FIELDS))
            assert same_fields(o.state(i)[1], spheres, STATE_FIELDS)[0], i
            assert same_fields(o.pairs(i), w.pairs(i), PAIR_FIELDS)[0], i
        w.close()
