"""Headless renderer: one scene's picture from the step's world vertices (the reference draws the
same bodies with OpenGL, code/nans.cpp:1853-2025). Checks the silhouette of a box against its
projected vertices, the ground and sphere passes, determinism and argument errors."""
import numpy as np
import pytest

from nans_projekat_gb300 import scenes

pytestmark = pytest.mark.gpu

BACKGROUND = (0x1c, 0x20, 0x28)
GROUND = ((0x70, 0x75, 0x7a), (0x8a, 0x90, 0x96))


@pytest.fixture(scope="module")
def nl():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from nans_projekat_gb300 import lib
    lib.load()
    return lib


def _is(img, rgb):
    return np.all(img == np.array(rgb, np.uint8), axis=-1)


def _camera(eye, target, fov, width, height):
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd /= np.linalg.norm(fwd)
    right = np.cross(fwd, [0.0, 1.0, 0.0])
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd)
    focal = 0.5 * height / np.tan(np.radians(0.5 * fov))
    return eye, fwd, right, up, focal


def _project(cam, width, height, p):
    eye, fwd, right, up, focal = cam
    d = p - eye
    z = d @ fwd
    return np.stack([0.5 * width + focal * (d @ right) / z, 0.5 * height - focal * (d @ up) / z], axis=-1)


def _one_box_scene():
    cubes = scenes._cubes(np.array([[0.0, 0.5, 0.0]]), None, np.ones(1), np.ones(1) / 6.0)
    return scenes.Scene(cubes, np.zeros(0, scenes.SPHERE_DTYPE), scenes.ground(20.0), name="one box")


def test_box_silhouette_matches_projected_vertices(nl):
    from scipy.spatial import ConvexHull
    w = nl.World()
    w.upload(_one_box_scene())
    w.step(np.float32(1.0 / 60.0), 1)
    W, H, fov = 200, 150, 45.0
    eye, target = (3.0, 2.5, 4.0), (0.0, 0.5, 0.0)
    img = w.render(0, eye, target, fov, W, H)
    cubes, _, _ = w.download()
    w.close()
    assert img.shape == (H, W, 3) and img.dtype == np.uint8
    corners = _project(_camera(eye, target, fov, W, H), W, H, cubes["Vertices"][0].astype(np.float64))
    eq = ConvexHull(corners).equations  # a.x + b.y + c <= 0 inside
    ys, xs = np.mgrid[0:H, 0:W]
    pix = np.stack([xs + 0.5, ys + 0.5], axis=-1).reshape(-1, 2)
    sd = (pix @ eq[:, :2].T + eq[:, 2]).max(axis=1).reshape(H, W)  # signed distance to the hull (px)
    box = ~_is(img, BACKGROUND) & ~_is(img, GROUND[0]) & ~_is(img, GROUND[1])
    inside, outside = sd < -1.0, sd > 1.0
    assert inside.sum() > 500
    assert box[inside].all(), "pixels inside the projected box not drawn as the box"
    assert not box[outside].any(), "box colour outside the projected box"
    # the ground fills the lower part of the frame around the box, the sky the top rows
    assert (_is(img, GROUND[0]) | _is(img, GROUND[1]))[outside & (ys > 0.8 * H)].all()
    assert _is(img, BACKGROUND)[:3].all()


def test_sphere_and_determinism(nl):
    sc = scenes.stack_scene(0)
    w = nl.World()
    w.upload(sc)
    w.step(np.float32(sc.constants.dt), 2)
    _, spheres, _ = w.download()
    c = spheres["Position"][0].astype(np.float64)
    eye = tuple(c + np.array([0.0, 0.0, 3.0]))
    a = w.render(0, eye, tuple(c), 40.0, 120, 90)
    b = w.render(0, eye, tuple(c), 40.0, 120, 90)
    assert np.array_equal(a, b)
    r = float(spheres["Radius"][0])
    focal = 0.5 * 90 / np.tan(np.radians(20.0))
    rad_px = focal * r / 3.0
    ys, xs = np.mgrid[0:90, 0:120]
    d = np.hypot(xs + 0.5 - 60.0, ys + 0.5 - 45.0)
    body = ~_is(a, BACKGROUND) & ~_is(a, GROUND[0]) & ~_is(a, GROUND[1])
    assert body[d < rad_px - 1.5].all(), "sphere disc not drawn"
    # looking straight up from above the scene: nothing but background
    top = w.render(0, (0.0, 50.0, 0.0), (0.0, 60.0, 0.01), 30.0, 64, 48)
    assert _is(top, BACKGROUND).all()
    w.close()


def test_render_argument_errors(nl):
    w = nl.World()
    w.upload(scenes.stack_scene(0))
    with pytest.raises(nl.NansError):
        w.render(1)
    with pytest.raises(nl.NansError):
        w.render(0, width=0, height=10)
    with pytest.raises(nl.NansError):
        w.render(0, fov=180.0)
    w.close()

