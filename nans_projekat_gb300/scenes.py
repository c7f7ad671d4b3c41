"""Seeded synthetic scenes for the physics step.

The reference builds one hard-coded demo scene in ``Init`` (code/nans.cpp:1550-1717). The
workloads here are seeded generators instead, one per benchmark configuration:

* ``stack_scene``    -- 8 unit cubes in a 2x2x2 stack on a 20x1x20 ground, jittered by
                        U(+-0.01) m, plus a sphere (r 0.5, m 2) launched at 20 m/s at it.
* ``random_scene``   -- 4,096 boxes (half-extents U[0.25,1]^3) + 512 spheres (r U[0.25,1])
                        at uniform positions in a 64^3 m box above the ground, densities
                        U[0.5,2], v ~ N(0,2) m/s, w ~ N(0,1) rad/s.
* ``stack_batch``    -- independent scenes with log-uniform body counts in [4,256]: a
                        seeded stack of boxes (half-extents U[0.25,0.75]) plus one sphere
                        projectile with speed U[5,25] m/s.
* ``grid_stack_batch``-- scenes of a 4x4x2 stack of unit cubes + one sphere (the stack scene
                        scaled up), used by the differentiable step.
* ``mixed_batch``    -- scenes with U[8,128] bodies mixing boxes, spheres and convex hulls
                        of 8-32 seeded points on a sphere of radius 0.5.
* ``demo_scene``     -- the reference's own Init scene (code/nans.cpp:1598-1678).

All randomness comes from an in-repo SplitMix64 generator; the seed is part of the scene.
Moments of inertia follow the reference's scalar form: m/12 * 2 * s^2 for a cube of edge s
(code/nans.cpp:1609-1610), generalised to the mean principal moment m/12 * 2/3 * (sx^2 +
sy^2 + sz^2) for a box, and 2/5 m r^2 for a sphere (code/nans.cpp:1663-1664).
"""
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .types import CUBE_DTYPE, SPHERE_DTYPE, IDENTITY16

GOLDEN = np.uint64(0x9E3779B97F4A7C15)


class SplitMix64:
    """SplitMix64 (Steele, Lea, Flood 2014), vectorised with numpy uint64 wrap-around."""

    def __init__(self, seed):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)

    def u64(self, n):
        with np.errstate(over="ignore"):
            idx = np.arange(1, n + 1, dtype=np.uint64)
            z = self.state + idx * GOLDEN
            self.state = self.state + np.uint64(n) * GOLDEN
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        return z

    def uniform(self, n, lo=0.0, hi=1.0):
        u = (self.u64(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + (hi - lo) * u

    def normal(self, n, mean=0.0, std=1.0):
        m = (n + 1) // 2
        u1 = self.uniform(m)
        u2 = self.uniform(m)
        r = np.sqrt(-2.0 * np.log1p(-u1))
        z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])[:n]
        return mean + std * z


@dataclass
class Constants:
    """Solver constants. The reference keeps them as literals; ``reference_defaults``
    reproduces code/nans.cpp:1154 (Cr=0.1), :1159 (Cf=0.1) and :1176 (70 iterations)."""
    cr: float = 0.2
    cf: float = 0.5
    iterations: int = 10
    dt: float = 1.0 / 60.0

    @staticmethod
    def reference_defaults(dt=1.0 / 60.0):
        return Constants(cr=np.float32(0.1).item(), cf=0.1, iterations=70, dt=dt)


@dataclass
class Scene:
    cubes: np.ndarray                       # CUBE_DTYPE records (boxes and hulls)
    spheres: np.ndarray                     # SPHERE_DTYPE records
    floor: np.ndarray                       # 1 CUBE_DTYPE record (static ground box)
    cube_scale: Optional[np.ndarray] = None  # (ncubes, 3) model scale; None = Size
    hull_npts: Optional[np.ndarray] = None   # (ncubes,) local point count, 0 = unit cube
    hull_pts: Optional[np.ndarray] = None    # (sum npts, 3) local points
    constants: Constants = field(default_factory=Constants)
    rebuild_models: bool = True              # build Model from Position/Angles/scale first
    name: str = ""

    @property
    def n_bodies(self):
        return len(self.cubes) + len(self.spheres)

    def scale_array(self):
        if self.cube_scale is not None:
            return np.ascontiguousarray(self.cube_scale, np.float32)
        s = self.cubes["Size"].astype(np.float32)
        return np.ascontiguousarray(np.stack([s, s, s], axis=1))


def _cubes(pos, scale, mass, moi, vel=None, w=None, size=None):
    n = len(pos)
    c = np.zeros(n, CUBE_DTYPE)
    c["Model"] = IDENTITY16
    c["Position"] = pos
    if vel is not None:
        c["V"] = vel
    if w is not None:
        c["W"] = w
    c["Size"] = 1.0 if size is None else size
    c["Mass"] = mass
    c["MOI"] = moi
    return c


def _spheres(pos, radius, mass, moi, vel=None, w=None):
    n = len(pos)
    s = np.zeros(n, SPHERE_DTYPE)
    s["Model"] = IDENTITY16
    s["Position"] = pos
    if vel is not None:
        s["V"] = vel
    if w is not None:
        s["W"] = w
    s["Radius"] = radius
    s["Mass"] = mass
    s["MOI"] = moi
    return s


def ground(size=20.0, top=0.0, mass=100000.0):
    """Static ground box of Size x 1 x Size (model scale (Size, 1, Size), code/nans.cpp:1878)
    with its top face at y = top. Mass and the MOI formula follow code/nans.cpp:1675-1678."""
    f = np.zeros(1, CUBE_DTYPE)
    f["Model"] = IDENTITY16
    f["Position"] = (0.0, top - 0.5, 0.0)
    f["Size"] = size
    f["Mass"] = mass
    f["MOI"] = np.float32(mass / 12.0) * np.float32(2.0 * size * size)
    return f


def box_moi(mass, scale):
    s2 = (scale.astype(np.float64) ** 2).sum(axis=-1)
    return (mass / 12.0) * (2.0 / 3.0) * s2


def sphere_moi(mass, r):
    return 0.4 * mass * r * r


def stack_scene(seed=0, constants=None):
    """8 unit cubes in a 2x2x2 stack on a 20x1x20 ground plus a 20 m/s sphere."""
    rng = SplitMix64(seed)
    base = np.array([[x, y, z] for y in (0.5, 1.5) for x in (-0.5, 0.5) for z in (-0.5, 0.5)],
                    np.float64)
    pos = base + rng.uniform(24, -0.01, 0.01).reshape(8, 3)
    mass = np.ones(8)
    cubes = _cubes(pos, None, mass, mass / 12.0 * 2.0)
    sp = _spheres([[-6.0, 1.0, 0.0]], 0.5, 2.0, sphere_moi(2.0, 0.5), vel=[[20.0, 0.0, 0.0]])
    return Scene(cubes, sp, ground(20.0), constants=constants or Constants(), name="stack8")


def random_scene(seed=1, n_boxes=4096, n_spheres=512, extent=64.0, constants=None):
    """Boxes and spheres at uniform positions in an extent^3 box above a static ground."""
    rng = SplitMix64(seed)
    h = rng.uniform(3 * n_boxes, 0.25, 1.0).reshape(n_boxes, 3)
    scale = 2.0 * h
    pos = np.stack([rng.uniform(n_boxes, -extent / 2, extent / 2),
                    rng.uniform(n_boxes, 1.0, 1.0 + extent),
                    rng.uniform(n_boxes, -extent / 2, extent / 2)], axis=1)
    dens = rng.uniform(n_boxes, 0.5, 2.0)
    mass = dens * scale.prod(axis=1)
    vel = rng.normal(3 * n_boxes, 0.0, 2.0).reshape(n_boxes, 3)
    w = rng.normal(3 * n_boxes, 0.0, 1.0).reshape(n_boxes, 3)
    cubes = _cubes(pos, scale, mass, box_moi(mass, scale), vel, w)
    r = rng.uniform(n_spheres, 0.25, 1.0)
    spos = np.stack([rng.uniform(n_spheres, -extent / 2, extent / 2),
                     rng.uniform(n_spheres, 1.0, 1.0 + extent),
                     rng.uniform(n_spheres, -extent / 2, extent / 2)], axis=1)
    sdens = rng.uniform(n_spheres, 0.5, 2.0)
    smass = sdens * (4.0 / 3.0) * np.pi * r ** 3
    svel = rng.normal(3 * n_spheres, 0.0, 2.0).reshape(n_spheres, 3)
    sw = rng.normal(3 * n_spheres, 0.0, 1.0).reshape(n_spheres, 3)
    spheres = _spheres(spos, r, smass, sphere_moi(smass, r), svel, sw)
    return Scene(cubes, spheres, ground(extent + 8.0), cube_scale=scale.astype(np.float32),
                 constants=constants or Constants(), name="random%d" % (n_boxes + n_spheres))


def _stack_positions(rng, n_boxes, half):
    """Columns of boxes on a square footprint; each box rests on the one below it."""
    cols = max(1, int(np.ceil(np.sqrt(n_boxes / max(1.0, np.cbrt(n_boxes))))))
    pitch = 2.0 * 0.75 + 0.1
    pos = np.zeros((n_boxes, 3))
    top = np.zeros(cols * cols)
    for i in range(n_boxes):
        c = i % (cols * cols)
        cx, cz = c % cols, c // cols
        pos[i, 0] = (cx - (cols - 1) / 2.0) * pitch
        pos[i, 2] = (cz - (cols - 1) / 2.0) * pitch
        pos[i, 1] = top[c] + half[i, 1] + 0.002
        top[c] = pos[i, 1] + half[i, 1]
    pos[:, 0] += rng.uniform(n_boxes, -0.01, 0.01)
    pos[:, 2] += rng.uniform(n_boxes, -0.01, 0.01)
    return pos, cols * pitch, top.max()


def stack_scene_random(rng, n_bodies, constants=None, half_lo=0.25, half_hi=0.75):
    nb = max(1, n_bodies - 1)
    half = rng.uniform(3 * nb, half_lo, half_hi).reshape(nb, 3)
    scale = 2.0 * half
    pos, width, height = _stack_positions(rng, nb, half)
    mass = scale.prod(axis=1)  # density 1
    cubes = _cubes(pos, scale, mass, box_moi(mass, scale))
    speed = rng.uniform(1, 5.0, 25.0)[0]
    start = np.array([-(width / 2.0 + 4.0), 0.5 + rng.uniform(1, 0.0, max(0.0, height - 0.5))[0], 0.0])
    aim = np.array([0.0, 0.5 * height, 0.0])
    d = aim - start
    d /= np.linalg.norm(d)
    sp = _spheres([start], 0.5, 2.0, sphere_moi(2.0, 0.5), vel=[speed * d])
    return Scene(cubes, sp, ground(max(20.0, width + 12.0)), cube_scale=scale.astype(np.float32),
                 constants=constants or Constants(), name="stack%d" % n_bodies)


def stack_batch(n_scenes=16384, seed=2, lo=4, hi=256, constants=None):
    """Independent stack scenes whose body counts are log-uniform in [lo, hi]."""
    rng = SplitMix64(seed)
    counts = np.floor(np.exp(rng.uniform(n_scenes, np.log(lo), np.log(hi + 1)))).astype(int)
    counts = np.clip(counts, lo, hi)
    return [stack_scene_random(rng, int(n), constants) for n in counts]


def grid_stack_batch(n_scenes=1024, seed=3, constants=None):
    """Scenes of a 4x4x2 stack of unit cubes (jittered) plus one 20 m/s sphere."""
    rng = SplitMix64(seed)
    out = []
    base = np.array([[x, y, z] for y in (0.5, 1.5) for x in (-1.5, -0.5, 0.5, 1.5)
                     for z in (-1.5, -0.5, 0.5, 1.5)], np.float64)
    for _ in range(n_scenes):
        pos = base + rng.uniform(base.size, -0.01, 0.01).reshape(base.shape)
        m = np.ones(len(pos))
        cubes = _cubes(pos, None, m, m / 12.0 * 2.0)
        sp = _spheres([[-8.0, 1.0, 0.0]], 0.5, 2.0, sphere_moi(2.0, 0.5), vel=[[20.0, 0.0, 0.0]])
        out.append(Scene(cubes, sp, ground(20.0), constants=constants or Constants(), name="grid33"))
    return out


def hull_points(rng, k, radius=0.5):
    """k seeded points on a sphere of the given radius (a convex hull's local points)."""
    z = rng.uniform(k, -1.0, 1.0)
    phi = rng.uniform(k, 0.0, 2.0 * np.pi)
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    return radius * np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def mixed_scene(rng, n_bodies, constants=None):
    kinds = rng.uniform(n_bodies)
    n_sph = int((kinds < 0.25).sum())
    n_hull = int(((kinds >= 0.25) & (kinds < 0.6)).sum())
    n_box = n_bodies - n_sph - n_hull
    nc = n_box + n_hull
    half = np.ones((nc, 3)) * 0.5
    half[:n_box] = rng.uniform(3 * n_box, 0.25, 0.75).reshape(n_box, 3)
    pos, width, height = _stack_positions(rng, nc, half)
    scale = 2.0 * half
    scale[n_box:] = 1.0
    mass = scale.prod(axis=1)
    npts = np.zeros(nc, np.int32)
    pts = []
    for i in range(n_box, nc):
        k = int(rng.uniform(1, 8, 33)[0])
        npts[i] = k
        pts.append(hull_points(rng, k))
    moi = box_moi(mass, scale)
    moi[n_box:] = 0.4 * mass[n_box:] * 0.25
    cubes = _cubes(pos, scale, mass, moi)
    sr = rng.uniform(n_sph, 0.25, 0.5)
    spos = np.stack([rng.uniform(n_sph, -width / 2, width / 2), height + 1.0 + 1.2 * np.arange(n_sph),
                     rng.uniform(n_sph, -width / 2, width / 2)], axis=1)
    smass = (4.0 / 3.0) * np.pi * sr ** 3
    spheres = _spheres(spos, sr, smass, sphere_moi(smass, sr))
    return Scene(cubes, spheres, ground(max(20.0, width + 12.0)), cube_scale=scale.astype(np.float32),
                 hull_npts=npts, hull_pts=(np.concatenate(pts).astype(np.float32) if pts else
                                           np.zeros((0, 3), np.float32)),
                 constants=constants or Constants(), name="mixed%d" % n_bodies)


def mixed_batch(n_scenes=4096, seed=4, lo=8, hi=128, constants=None):
    rng = SplitMix64(seed)
    counts = np.floor(rng.uniform(n_scenes, lo, hi + 1)).astype(int)
    return [mixed_scene(rng, int(n), constants) for n in counts]


def demo_scene():
    """The reference's Init scene (code/nans.cpp:1598-1678): 4 unit cubes, 1 sphere and a
    100-wide floor, every Model the identity (so the first step sees unit cubes at the origin,
    as the reference does)."""
    pos = np.array([[2.0, 3.5, 2.0], [2.0, 1.0, 2.0], [2.0, 4.5, 2.0], [1.0, 1.0, 1.0]])
    m = np.ones(4, np.float32)
    moi = (m / np.float32(12.0)) * (np.float32(2.0) * np.float32(1.0) * np.float32(1.0))
    cubes = _cubes(pos, None, m, moi)
    sp = _spheres([[0.1, 1.1, 1.1]], 0.25, 2.0,
                  np.float32(2.0 / 5.0) * np.float32(2.0) * np.float32(0.25 ** 2))
    fl = np.zeros(1, CUBE_DTYPE)
    fl["Model"] = IDENTITY16
    fl["Position"] = (1.2, -0.5, 1.0)
    fl["Size"] = 100.0
    fl["Mass"] = 100000.0
    fl["MOI"] = np.float32(100000.0 / 12.0) * np.float32(2.0 * 100.0 * 100.0)
    sc = np.ones((4, 3), np.float32)
    sc[3] = (0.5, 1.0, 0.5)
    return Scene(cubes, sp, fl, cube_scale=sc, constants=Constants.reference_defaults(),
                 rebuild_models=False, name="demo")
