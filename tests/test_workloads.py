"""The seeded synthetic workloads (nans_projekat_gb300/scenes.py) have the shapes, sizes and
value distributions of the configurations they stand in for (the reference has no benchmark
suite; its demo scene is code/nans.cpp:1598-1678). Pure CPU."""
import numpy as np
import pytest

from nans_projekat_gb300 import scenes


@pytest.fixture(scope="module")
def stack16384():
    return scenes.stack_batch(16384, seed=2)


def test_stack_benchmark_workload(stack16384):
    """16,384 stack scenes, body counts log-uniform in [4, 256] (987,052 bodies with seed 2),
    boxes with half-extents in [0.25, 0.75] and one sphere projectile at 5-25 m/s each."""
    counts = np.array([s.n_bodies for s in stack16384])
    assert len(counts) == 16384 and counts.sum() == 987052
    assert counts.min() == 4 and counts.max() == 256
    # log-uniform: E[n] = (257 - 4) / ln(257 / 4) ~ 60.8, median ~ sqrt(4 * 257) ~ 32
    assert 57.0 < counts.mean() < 64.0 and 28 <= np.median(counts) <= 36
    lo = np.log(counts)
    hist = np.histogram(lo, bins=4, range=(np.log(4), np.log(257)))[0]
    assert hist.min() > 0.8 * hist.mean()
    for s in stack16384[::97]:
        assert len(s.spheres) == 1
        half = s.cube_scale / 2.0
        assert half.min() >= 0.25 and half.max() <= 0.75
        speed = float(np.linalg.norm(s.spheres["V"][0]))
        assert 5.0 <= speed <= 25.0
        assert np.allclose(s.cubes["Mass"], s.cube_scale.astype(np.float64).prod(axis=1), rtol=1e-6)


def test_large_single_scene_workload():
    """4,096 boxes (half-extents U[0.25, 1]^3) and 512 spheres (r U[0.25, 1]) in a 64^3 box
    above the ground, densities U[0.5, 2], v ~ N(0, 2), w ~ N(0, 1)."""
    sc = scenes.random_scene()
    assert len(sc.cubes) == 4096 and len(sc.spheres) == 512
    half = sc.cube_scale.astype(np.float64) / 2.0
    assert half.min() >= 0.25 and half.max() <= 1.0
    r = sc.spheres["Radius"].astype(np.float64)
    assert r.min() >= 0.25 and r.max() <= 1.0
    for rec in (sc.cubes, sc.spheres):
        p = rec["Position"]
        assert np.abs(p[:, [0, 2]]).max() <= 32.0 and p[:, 1].min() >= 1.0 and p[:, 1].max() <= 65.0
    dens = sc.cubes["Mass"].astype(np.float64) / (2.0 * half).prod(axis=1)
    assert dens.min() >= 0.5 - 1e-5 and dens.max() <= 2.0 + 1e-5
    v = sc.cubes["V"].astype(np.float64).ravel()
    assert abs(v.mean()) < 0.1 and 1.9 < v.std() < 2.1
    w = sc.cubes["W"].astype(np.float64).ravel()
    assert abs(w.mean()) < 0.05 and 0.95 < w.std() < 1.05


def test_differentiable_workload():
    """1,024 scenes of a jittered 4x4x2 stack of unit cubes plus one 20 m/s sphere (33 bodies)."""
    batch = scenes.grid_stack_batch(1024, seed=3)
    assert len(batch) == 1024 and all(s.n_bodies == 33 for s in batch)
    s = batch[7]
    assert len(s.cubes) == 32 and np.allclose(s.spheres["V"][0], (20.0, 0.0, 0.0))
    y = s.cubes["Position"][:, 1].astype(np.float64)
    layer = np.where(y < 1.0, 0.5, 1.5)
    assert (layer == 0.5).sum() == 16 and np.abs(y - layer).max() <= 0.01 + 1e-6


def test_mixed_hull_workload():
    """Scenes of 8-128 bodies: boxes, spheres and convex hulls of 8-32 points on r = 0.5."""
    batch = scenes.mixed_batch(256, seed=4)
    counts = np.array([s.n_bodies for s in batch])
    assert counts.min() >= 8 and counts.max() <= 128
    kinds = np.zeros(3)
    for s in batch:
        npts = s.hull_npts
        hulls = npts[npts > 0]
        assert ((hulls >= 8) & (hulls <= 32)).all()
        assert len(s.hull_pts) == hulls.sum()
        if len(s.hull_pts):
            assert np.allclose(np.linalg.norm(s.hull_pts.astype(np.float64), axis=1), 0.5, atol=1e-6)
        kinds += (int((npts == 0).sum()), len(hulls), len(s.spheres))
    frac = kinds / kinds.sum()
    # kinds drawn as spheres 25 %, hulls 35 %, boxes 40 %
    assert abs(frac[0] - 0.40) < 0.03 and abs(frac[1] - 0.35) < 0.03 and abs(frac[2] - 0.25) < 0.03


def test_reference_stack_and_demo_scenes():
    """The 2x2x2 stack of unit cubes (jitter within 0.01) with a 20 m/s sphere, and the
    reference's Init scene: 4 cubes with cube 3 at scale (0.5, 1, 0.5), a 0.25 m sphere and the
    100-wide floor of mass 1e5 (code/nans.cpp:1598-1678)."""
    sc = scenes.stack_scene(0)
    assert len(sc.cubes) == 8 and len(sc.spheres) == 1
    grid = np.array([[x, y, z] for y in (0.5, 1.5) for x in (-0.5, 0.5) for z in (-0.5, 0.5)])
    assert np.abs(sc.cubes["Position"] - grid).max() <= 0.01 + 1e-6
    assert np.allclose(sc.spheres["V"][0], (20.0, 0.0, 0.0))
    demo = scenes.demo_scene()
    assert len(demo.cubes) == 4 and len(demo.spheres) == 1 and not demo.rebuild_models
    assert np.allclose(demo.cube_scale[3], (0.5, 1.0, 0.5))
    assert float(demo.spheres["Radius"][0]) == 0.25
    assert float(demo.floor["Size"][0]) == 100.0 and float(demo.floor["Mass"][0]) == 100000.0
