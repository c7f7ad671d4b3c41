"""Hand-built known-answer cases of the detect stage: a sphere, boxes and a convex hull resting
on the ground, overlapping and separated box pairs, a hull against a box, a box-sphere pair
whose EPA outgrows the per-thread polytope, and the symmetric poses in which the reference's
GJK reports nothing.

Each case holds its physical answer (contact type, normal, depth = |PointA - PointB|, contact
points) where the reference gives one. The reference's GJK resets its search direction to
normalize(PB - PA) on every call and has its own line case (code/nans.cpp:539-769), so poses
with tied supports (a box straight above the origin, axis-aligned boxes in line, two spheres)
end without a contact, and a sphere inside a box runs EPA to its 64-iteration cap
(code/nans.cpp:804, 903); those answers are the reference's own, pinned against the reference
built from source.

CPU: the oracle gives the physical answers; the reference build (when present) gives the
oracle's contacts bit for bit. GPU: the plain path gives the oracle's contacts bit for bit, and
the box-sphere stress case leaves the per-thread EPA tier."""
import numpy as np
import pytest

from helpers import canon, same_fields, PAIR_FIELDS, STATE_FIELDS
from nans_projekat_gb300.scenes import Scene, _cubes, _spheres, ground, sphere_moi
from nans_projekat_gb300.types import CC, CS, CF, SF

DT = np.float32(1.0 / 60.0)
NONE = np.zeros((0, 3))


def _boxes(pos, angles=None):
    pos = np.array(pos, np.float64).reshape(-1, 3)
    m = np.ones(len(pos))
    c = _cubes(pos, None, m, m / 12.0 * 2.0)
    if angles is not None:
        c["Angles"] = angles
    return c


def _balls(pos, r=0.5, m=2.0):
    return _spheres(np.array(pos, np.float64).reshape(-1, 3), r, m, sphere_moi(m, r))


def _hull_scene(pos, k, seed, more_boxes=None):
    """A convex hull of k points on a sphere of radius 0.5 (a shape the reference does not have;
    its checker is the oracle), unrotated and unscaled, so its world points are pos + points."""
    from nans_projekat_gb300 import scenes
    pts = scenes.hull_points(scenes.SplitMix64(seed), k).astype(np.float32)
    hull = _boxes([pos])
    hull["MOI"] = np.float32(0.4 * 0.25)
    cubes = hull if more_boxes is None else np.concatenate([hull, more_boxes])
    npts = np.zeros(len(cubes), np.int32)
    npts[0] = k
    return Scene(cubes, _balls(NONE), ground(20.0), cube_scale=np.ones((len(cubes), 3), np.float32),
                 hull_npts=npts, hull_pts=pts)


def _hull_world_points(sc):
    return sc.cubes["Position"][0].astype(np.float64) + sc.hull_pts.astype(np.float64)


def cases():
    """name -> (scene, expected contact types in list order)."""
    g = ground(20.0)  # top face at y = 0
    return {
        "sphere_on_ground": (Scene(_boxes(NONE), _balls([0.13, 0.47, -0.21]), g), [SF]),
        "box_on_ground": (Scene(_boxes([0.1, 0.48, 0.2]), _balls(NONE), g), [CF]),
        "tilted_box_on_ground": (Scene(_boxes([0.1, 0.55, 0.2], [[7.0, 3.0, 11.0]]), _balls(NONE), g), [CF]),
        "boxes_overlapping": (Scene(_boxes([[0.0, 5.0, 0.0], [0.9, 5.3, 0.2]]), _balls(NONE), g), [CC]),
        "boxes_rotated": (Scene(_boxes([[0.0, 5.0, 0.0], [0.85, 5.2, 0.1]], [[0, 0, 0], [10.0, 20.0, 30.0]]),
                                _balls(NONE), g), [CC]),
        "boxes_separated": (Scene(_boxes([[0.0, 5.0, 0.0], [1.5, 5.3, 0.2]]), _balls(NONE), g), []),
        "box_sphere": (Scene(_boxes([0.0, 5.0, 0.0], [[5.0, 15.0, 25.0]]), _balls([0.8, 5.3, 0.1]), g), [CS]),
        "box_sphere_epa_stress": (Scene(_boxes([0.0, 5.0, 0.0], [[79.64529, 11.156005, 28.8532]]),
                                        _balls([-0.77295178, 5.4026804, 0.16208237], r=0.4682042), g), [CS]),
        # convex hulls (no reference counterpart)
        "hull_on_ground": (_hull_scene([0.1, 0.40, 0.2], 24, 5), [CF]),
        "hull_above_ground": (_hull_scene([0.1, 0.45, 0.2], 24, 5), []),
        "hull_box": (_hull_scene([0.0, 5.0, 0.0], 24, 6, _boxes([[0.8, 5.2, 0.1]])), [CC]),
        # the reference's answers for symmetric poses: no contact
        "sphere_above_origin": (Scene(_boxes(NONE), _balls([0.0, 0.49, 0.0]), g), []),
        "boxes_in_line": (Scene(_boxes([[0.0, 5.0, 0.0], [0.9, 5.0, 0.0]]), _balls(NONE), g), []),
        "boxes_touching": (Scene(_boxes([[0.0, 5.0, 0.0], [1.0, 5.0, 0.0]]), _balls(NONE), g), []),
        "spheres_overlapping": (Scene(_boxes(NONE), _balls([[0.0, 5.0, 0.0], [0.7, 5.3, 0.2]]), g), []),
        "sphere_inside_box": (Scene(_boxes([0.0, 5.0, 0.0]), _balls([0.2, 5.1, 0.1]), g), []),
    }


def _box_frame(verts):
    """Centre, unit axes and half-extents of a box from its 8 world vertices in the reference's
    order (+++, ++-, -++, -+-, +-+, +--, --+, ---; code/nans.cpp:379-395)."""
    v = verts.astype(np.float64)
    centre = v.mean(0)
    edges = [v[0] - v[2], v[0] - v[4], v[0] - v[1]]  # x, y, z
    axes = [e / np.linalg.norm(e) for e in edges]
    half = [np.linalg.norm(e) / 2.0 for e in edges]
    return centre, axes, half


def _box_point_distance(verts, p):
    centre, axes, half = _box_frame(verts)
    local = np.array([np.dot(p - centre, a) for a in axes])
    return np.linalg.norm(local - np.clip(local, -np.array(half), np.array(half)))


def _oracle_detect(sc):
    from oracle.portbind import OracleWorld
    o = OracleWorld([sc])
    o.stage(0, DT)  # IntegrateForces: world vertices from the Model
    o.stage(1, DT)  # DetectCollisions
    return o.state(0), o.pairs(0)


@pytest.mark.parametrize("name", sorted(cases()))
def test_known_answer_on_the_oracle(oracle_lib, name):
    sc, types = cases()[name]
    (cubes, spheres, _), pairs = _oracle_detect(sc)
    assert [int(t) for t in pairs["Type"]] == types
    for p in pairs:
        depth = float(np.linalg.norm(p["PointA"].astype(np.float64) - p["PointB"]))
        n = p["N"].astype(np.float64)
        assert abs(np.linalg.norm(n) - 1.0) < 1e-5
        if p["Type"] in (CF, SF):
            # the ground's top face: normal +y, PointB on the face, PointA the deepest point
            assert np.allclose(n, (0.0, 1.0, 0.0), atol=1e-6)
            assert abs(float(p["PointB"][1])) < 1e-5
            if p["Type"] == SF:
                s = spheres[p["IndexA"]]
                lowest = s["Position"].astype(np.float64) - (0.0, float(s["Radius"]), 0.0)
                assert np.allclose(p["PointA"], lowest, atol=1e-4)
            elif sc.hull_npts is not None:
                pts = _hull_world_points(sc)
                lowest = pts[np.argmin(pts[:, 1])]
                assert np.allclose(p["PointA"], lowest, atol=1e-4)
            else:
                # a point of the box at the height of its lowest vertex (a face when level)
                v = cubes[p["IndexA"]]["Vertices"]
                lowest = v[np.argmin(v[:, 1])].astype(np.float64)
                assert abs(float(p["PointA"][1]) - lowest[1]) < 1e-4
                assert _box_point_distance(v, p["PointA"].astype(np.float64)) < 1e-4
            assert abs(depth + lowest[1]) < 1e-4
        elif p["Type"] == CS:
            s = spheres[p["IndexB"]]
            d = _box_point_distance(cubes[p["IndexA"]]["Vertices"], s["Position"].astype(np.float64))
            assert abs(depth - (float(s["Radius"]) - d)) < 1e-3  # EPA tolerance
        elif name == "hull_box":
            # the hull's furthest point along +x against the box's face x = 0.3
            reach = _hull_world_points(sc)[:, 0].max()
            assert np.allclose(n, (-1.0, 0.0, 0.0), atol=1e-6)
            assert abs(p["PointB"][0] - 0.3) < 1e-5 and abs(depth - (reach - 0.3)) < 1e-4
        elif name == "boxes_overlapping":
            # faces x = 0.5 of box 0 and x = 0.4 of box 1: 0.1 deep along x, normal towards box 0
            assert np.allclose(n, (-1.0, 0.0, 0.0), atol=1e-6)
            assert abs(depth - 0.1) < 1e-5 and abs(p["PointA"][0] - 0.5) < 1e-5 and abs(p["PointB"][0] - 0.4) < 1e-5
        else:
            assert p["Type"] == CC and depth > 0.0


def test_epa_stress_case_outgrows_the_per_thread_polytope(oracle_lib):
    from oracle import portbind
    portbind.stats_enable(True)
    try:
        portbind.epa_stats(reset=True)
        _oracle_detect(cases()["box_sphere_epa_stress"][0])
        st = portbind.epa_stats(reset=True)
    finally:
        portbind.stats_enable(False)
    assert st["max_faces"] > 20 and st["max_iter"] > 30  # the per-thread EPA holds 20 faces


@pytest.mark.reference
@pytest.mark.parametrize("name", sorted(cases()))
def test_known_answer_matches_the_reference(oracle_lib, name):
    from oracle import refbind
    if not refbind.ref_available("refbig"):
        pytest.skip("reference build absent (make -C oracle ref needs the reference checkout)")
    from oracle.portbind import OracleWorld
    sc, _ = cases()[name]
    if sc.hull_npts is not None:
        pytest.skip("the reference has no convex hulls")
    o = OracleWorld([sc])
    r = refbind.RefWorld(sc)
    for _ in range(3):
        o.step(DT, 1)
        r.step(DT, 1)
        assert o.pairs(0).tobytes() == r.pairs().tobytes()
        (oc, os_, _), (rc, rs, _) = o.state(0), r.state()
        for f in ("Position", "Angles", "V", "W"):
            assert canon(oc[f]) == canon(rc[f]) and canon(os_[f]) == canon(rs[f]), f


@pytest.fixture(scope="module")
def nl():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from nans_projekat_gb300 import lib
    lib.load()
    return lib


@pytest.mark.gpu
def test_known_answers_on_the_gpu(nl, oracle_lib):
    from oracle.portbind import OracleWorld
    for name, (sc, types) in sorted(cases().items()):
        w = nl.World()
        w.upload(sc)
        o = OracleWorld([sc])
        for k in range(3):
            w.step(DT, 1)
            o.step(DT, 1)
            got, ref = w.pairs(0), o.pairs(0)
            assert same_fields(ref, got, PAIR_FIELDS)[0], (name, k)
            cubes, spheres, _ = w.download()
            oc, os_, _ = o.state(0)
            assert same_fields(oc, cubes, STATE_FIELDS)[0] and same_fields(os_, spheres, STATE_FIELDS)[0], (name, k)
            if k == 0:
                assert [int(t) for t in got["Type"]] == types, name
        if name == "box_sphere_epa_stress":
            st = w.epa_stats()  # the EPA left the per-thread polytope (20 faces)
            assert st["warp_tier"] + st["slow_epas"] >= 1
        w.close()
