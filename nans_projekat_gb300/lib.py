"""ctypes binding of the C ABI (include/nans_gb300.h) and a small host-side World class that
mirrors the reference's step interface: bodies go in as the reference's own records
(cube / sphere, code/nans.h:303-336), the step runs on the GPU, and bodies and the contact
list (contact_pair, code/nans.h:338-372) come back in the same layouts.

There is no CPU fallback: importing works without a GPU, but every call needs the CUDA
library and a device, and raises if either is missing.
"""
import ctypes
import os

import numpy as np

from .types import CUBE_DTYPE, SPHERE_DTYPE, PAIR_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libnans_gb300.so")

NANS_OK = 0
ERRORS = {
    1: "NANS_ERR_INVALID_ARGUMENT",
    2: "NANS_ERR_CAPACITY",
    3: "NANS_ERR_NAN_INPUT",
    4: "NANS_ERR_CUDA",
    5: "NANS_ERR_EPA_CAPACITY",
    6: "NANS_ERR_NOT_UPLOADED",
    7: "NANS_ERR_SCENE_TOO_LARGE",
    8: "NANS_ERR_NO_TAPE",
}
UPLOAD_KEEP_MODEL = 1
WORLD_ALL_PAIRS = 1
WORLD_STRICT_EPA = 2
WORLD_TEST_GIANT_TIER = 4
WORLD_WARM_START = 8
WORLD_TEST_BARRIER_TIMEOUT = 16
WORLD_GJK_WARP = 32
WORLD_FUSED_STEP = 64

# Every symbol include/nans_gb300.h declares.
EXPORTS = (
    "nans_world_create", "nans_world_destroy", "nans_world_upload", "nans_batch_upload", "nans_step",
    "nans_batch_step", "nans_batch_autotune", "nans_world_download", "nans_world_set_state",
    "nans_get_pairs", "nans_world_status", "nans_world_counts", "nans_world_stream",
    "nans_launches_per_step", "nans_device_sincos", "nans_last_error", "nans_profile_steps", "nans_profile_timeline",
    "nans_world_epa_stats", "nans_solve_contacts_static", "nans_diff_forward", "nans_diff_backward",
    "nans_diff_tape_info", "nans_world_set_state_arrays", "nans_world_get_state_arrays", "nans_render_scene",
    "nans_world_path_counts", "nans_world_tuning", "nans_world_set_tuning", "nans_batch_prepare",
)


class NansError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (ERRORS.get(code, str(code)), msg))
        self.code = code


class WorldDesc(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("flags", ctypes.c_uint32), ("max_candidates", ctypes.c_uint32)]


class StepParams(ctypes.Structure):
    _fields_ = [("cr", ctypes.c_float), ("cf", ctypes.c_float), ("iterations", ctypes.c_int32)]


class DiffGrads(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("dl_position", "dl_angles", "dl_velocity", "dl_omega", "position0",
                                              "angles0", "velocity0", "omega0", "mass", "restitution",
                                              "friction")]


_LIB = None
_P = ctypes.c_void_p
_U = ctypes.c_uint32
_F = ctypes.c_float


def load(path=LIB_PATH):
    """Loads the CUDA library (building it first if it is absent and nvcc is present)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(path)
    L.nans_last_error.restype = ctypes.c_char_p
    L.nans_world_create.argtypes = [ctypes.POINTER(WorldDesc), ctypes.POINTER(_P)]
    L.nans_world_destroy.argtypes = [_P]
    L.nans_world_upload.argtypes = [_P, _P, _U, _P, _U, _P, _P, _U]
    L.nans_batch_upload.argtypes = [_P, _U, _P, _P, _P, _P, _P, _P, _P, _P, _P, _U]
    L.nans_step.argtypes = [_P, ctypes.POINTER(StepParams), _F, _U]
    L.nans_batch_step.argtypes = [_P, _F, _U, _U]
    L.nans_batch_autotune.argtypes = [_P, _F]
    L.nans_batch_prepare.argtypes = [_P, _F, _U]
    L.nans_world_download.argtypes = [_P, _P, _P, _P]
    L.nans_world_set_state.argtypes = [_P, _P, _P, _U]
    L.nans_get_pairs.argtypes = [_P, _U, _P, _U, ctypes.POINTER(_U)]
    L.nans_world_status.argtypes = [_P, ctypes.POINTER(_U)]
    L.nans_world_counts.argtypes = [_P, ctypes.POINTER(_U), ctypes.POINTER(_U)]
    L.nans_world_stream.argtypes = [_P]
    L.nans_world_stream.restype = _P
    L.nans_launches_per_step.argtypes = [_P, ctypes.POINTER(_U), ctypes.POINTER(_U)]
    L.nans_world_path_counts.argtypes = [_P, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    L.nans_world_tuning.argtypes = [_P, _P]
    L.nans_world_set_tuning.argtypes = [_P, _P]
    L.nans_device_sincos.argtypes = [_P, _P, _P, _U]
    L.nans_profile_steps.argtypes = [_P, _F, _U, _P]
    L.nans_profile_timeline.argtypes = [_P, _F, _U, _P]
    L.nans_world_epa_stats.argtypes = [_P, _P, ctypes.c_int]
    L.nans_world_set_state_arrays.argtypes = [_P, _P, _P, _P, _P]
    L.nans_render_scene.argtypes = [_P, _U, _P, _P, _F, _U, _U, _P]
    L.nans_world_get_state_arrays.argtypes = [_P, _P, _P, _P, _P]
    L.nans_diff_forward.argtypes = [_P, ctypes.POINTER(StepParams), _F, _U]
    L.nans_diff_backward.argtypes = [_P, ctypes.POINTER(DiffGrads)]
    L.nans_diff_tape_info.argtypes = [_P, ctypes.POINTER(_U), ctypes.POINTER(ctypes.c_uint64)]
    L.nans_solve_contacts_static.argtypes = [_U, _U, _P, _P, _P, _P, _P, _P, _P, _U, _F, _F, ctypes.c_int32,
                                             _F, _P]
    _LIB = L
    return L


def _check(rc):
    if rc != NANS_OK:
        raise NansError(rc, load().nans_last_error().decode())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def device_sincos(x):
    x = np.ascontiguousarray(x, np.float32)
    s = np.zeros_like(x)
    c = np.zeros_like(x)
    _check(load().nans_device_sincos(_ptr(x), _ptr(s), _ptr(c), len(x)))
    return s, c


class World:
    """A set of independent scenes on one GPU.

    upload(scene)          one scene (the plain drop-in for one reference sdl_state)
    upload_batch(scenes)   many scenes (the batched form)
    step(dt, n, params)    the plain path: stage-by-stage launches, synchronised
    batch_step(dt, n, g)   the batched path: persistent kernels replayed from a CUDA graph
    fused_step=True        one detect-and-solve launch per step, a block per scene, in place of
                           the staged kernels (same results; scenes of at most 1,024 bodies)
    """

    def __init__(self, device=0, all_pairs=False, max_candidates=0, strict_epa=False, giant_tier_only=False,
                 warm_start=False, barrier_timeout_test=False, gjk_warp=False, fused_step=False):
        self.lib = load()
        flags = (WORLD_ALL_PAIRS if all_pairs else 0) | (WORLD_STRICT_EPA if strict_epa else 0) | \
            (WORLD_TEST_GIANT_TIER if giant_tier_only else 0) | (WORLD_WARM_START if warm_start else 0) | \
            (WORLD_TEST_BARRIER_TIMEOUT if barrier_timeout_test else 0) | (WORLD_GJK_WARP if gjk_warp else 0) | \
            (WORLD_FUSED_STEP if fused_step else 0)
        d = WorldDesc(device, flags, max_candidates)
        h = _P()
        _check(self.lib.nans_world_create(ctypes.byref(d), ctypes.byref(h)))
        self.h = h
        self.scenes = []
        self._counts = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.nans_world_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    # -- upload -------------------------------------------------------------------------
    def upload(self, scene):
        self.upload_batch([scene])

    def upload_batch(self, scenes):
        scenes = list(scenes)
        self.scenes = scenes
        ncs = np.array([len(s.cubes) for s in scenes], np.uint32)
        nss = np.array([len(s.spheres) for s in scenes], np.uint32)
        cubes = np.ascontiguousarray(np.concatenate([s.cubes for s in scenes])) if ncs.sum() else \
            np.zeros(0, CUBE_DTYPE)
        spheres = np.ascontiguousarray(np.concatenate([s.spheres for s in scenes])) if nss.sum() else \
            np.zeros(0, SPHERE_DTYPE)
        floors = np.ascontiguousarray(np.concatenate([s.floor for s in scenes]))
        scale = np.ascontiguousarray(np.concatenate([s.scale_array() for s in scenes]) if ncs.sum() else
                                     np.zeros((0, 3), np.float32), np.float32)
        has_hull = any(s.hull_npts is not None for s in scenes)
        npts = pts = None
        if has_hull:
            npts = np.ascontiguousarray(np.concatenate(
                [s.hull_npts if s.hull_npts is not None else np.zeros(len(s.cubes), np.int32)
                 for s in scenes]).astype(np.int32))
            pl = [s.hull_pts for s in scenes if s.hull_pts is not None and len(s.hull_pts)]
            pts = np.ascontiguousarray(np.concatenate(pl).astype(np.float32)) if pl else np.zeros((1, 3), np.float32)
        params = (StepParams * len(scenes))()
        for i, s in enumerate(scenes):
            params[i].cr = s.constants.cr
            params[i].cf = s.constants.cf
            params[i].iterations = s.constants.iterations
        keep = all(not s.rebuild_models for s in scenes)
        if not keep and any(not s.rebuild_models for s in scenes):
            raise ValueError("all scenes of a batch must agree on rebuild_models")
        self._keep = (cubes, spheres, floors, scale, npts, pts, ncs, nss, params)
        _check(self.lib.nans_batch_upload(
            self.h, len(scenes), _ptr(ncs), _ptr(nss), _ptr(cubes), _ptr(spheres), _ptr(floors), _ptr(scale),
            _ptr(npts), _ptr(pts), ctypes.cast(params, _P), UPLOAD_KEEP_MODEL if keep else 0))
        self._ncubes = int(ncs.sum())
        self._nspheres = int(nss.sum())
        self._cube_off = np.concatenate([[0], np.cumsum(ncs)]).astype(np.int64)
        self._sphere_off = np.concatenate([[0], np.cumsum(nss)]).astype(np.int64)

    # -- stepping ----------------------------------------------------------------------
    def step(self, dt, n=1, params=None):
        p = None
        if params is not None:
            p = ctypes.byref(StepParams(params.cr, params.cf, params.iterations))
        _check(self.lib.nans_step(self.h, p, dt, n))

    def batch_step(self, dt, n=1, graph_steps=60):
        _check(self.lib.nans_batch_step(self.h, dt, n, graph_steps))

    def prepare(self, dt, graph_steps=60):
        """Captures the graph the next batch_step(dt, n, graph_steps) replays first."""
        _check(self.lib.nans_batch_prepare(self.h, dt, graph_steps))

    def autotune(self, dt):
        _check(self.lib.nans_batch_autotune(self.h, dt))

    # -- readback ----------------------------------------------------------------------
    def download(self):
        """(cubes, spheres, floors) for all scenes, concatenated in upload order."""
        cubes = np.zeros(self._ncubes, CUBE_DTYPE)
        spheres = np.zeros(self._nspheres, SPHERE_DTYPE)
        floors = np.zeros(len(self.scenes), CUBE_DTYPE)
        _check(self.lib.nans_world_download(self.h, _ptr(cubes), _ptr(spheres), _ptr(floors)))
        return cubes, spheres, floors

    def scene_state(self, i, state=None):
        cubes, spheres, floors = self.download() if state is None else state
        return (cubes[self._cube_off[i]:self._cube_off[i + 1]],
                spheres[self._sphere_off[i]:self._sphere_off[i + 1]], floors[i:i + 1])

    def set_state(self, cubes, spheres, keep_model=False):
        _check(self.lib.nans_world_set_state(self.h, _ptr(np.ascontiguousarray(cubes)),
                                             _ptr(np.ascontiguousarray(spheres)),
                                             UPLOAD_KEEP_MODEL if keep_model else 0))

    def set_state_arrays(self, position=None, angles=None, velocity=None, omega=None):
        """Dynamic state from (n_bodies, 3) float32 arrays in record order (None = keep)."""
        arrs = []
        for a in (position, angles, velocity, omega):
            if a is not None:
                a = np.ascontiguousarray(a, np.float32)
                if a.shape != (self.n_bodies, 3):
                    raise ValueError("state arrays must have shape (%d, 3)" % self.n_bodies)
            arrs.append(a)
        self._state_keep = arrs
        _check(self.lib.nans_world_set_state_arrays(self.h, *[_ptr(a) for a in arrs]))

    def get_state_arrays(self, out=None):
        """(position, angles, velocity, omega) as (n_bodies, 3) float32 arrays in record order;
        `out` may supply the four arrays (e.g. in pinned memory)."""
        if out is None:
            out = tuple(np.zeros((self.n_bodies, 3), np.float32) for _ in range(4))
        _check(self.lib.nans_world_get_state_arrays(self.h, *[_ptr(a) for a in out]))
        return out

    def render(self, scene=0, eye=(6.0, 4.0, 8.0), target=(0.0, 0.5, 0.0), fov=45.0, width=640, height=480):
        """(height, width, 3) uint8 picture of one scene (headless CUDA rasteriser)."""
        img = np.zeros((height, width, 3), np.uint8)
        e = np.asarray(eye, np.float32)
        t = np.asarray(target, np.float32)
        _check(self.lib.nans_render_scene(self.h, scene, _ptr(e), _ptr(t), fov, width, height, _ptr(img)))
        return img

    def pairs(self, scene=0):
        cnt = _U()
        _check(self.lib.nans_get_pairs(self.h, scene, None, 0, ctypes.byref(cnt)))
        out = np.zeros(cnt.value, PAIR_DTYPE)
        if cnt.value:
            _check(self.lib.nans_get_pairs(self.h, scene, _ptr(out), cnt.value, ctypes.byref(cnt)))
        return out

    def status(self):
        s = _U()
        _check(self.lib.nans_world_status(self.h, ctypes.byref(s)))
        return s.value

    def counts(self):
        a, b = _U(), _U()
        _check(self.lib.nans_world_counts(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def launches_per_step(self):
        a, b = _U(), _U()
        _check(self.lib.nans_launches_per_step(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def tuning(self):
        """The launch parameters in use (nans_batch_autotune's choice, or the defaults)."""
        out = np.zeros(8, np.int32)
        _check(self.lib.nans_world_tuning(self.h, _ptr(out)))
        return {"gjk_blocks_per_sm": int(out[0]), "solve_threads": int(out[1]), "solve_threads_late": int(out[2]),
                "cull_tiles": int(out[3]), "solve_late_blocks_per_sm": int(out[4]), "warp_epa_blocks_per_sm": int(out[5]),
                "candidates_timed": int(out[6]), "us_per_step": int(out[7])}

    def set_tuning(self, gjk_blocks_per_sm, solve_threads, solve_threads_late, cull_tiles=1, solve_late_blocks_per_sm=6,
                   warp_epa_blocks_per_sm=2):
        a = np.array([gjk_blocks_per_sm, solve_threads, solve_threads_late, cull_tiles, solve_late_blocks_per_sm,
                      warp_epa_blocks_per_sm], np.int32)
        _check(self.lib.nans_world_set_tuning(self.h, _ptr(a)))

    def path_counts(self):
        """(steps replayed from CUDA graphs, steps launched eagerly) since the last upload."""
        g, e = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self.lib.nans_world_path_counts(self.h, ctypes.byref(g), ctypes.byref(e)))
        return g.value, e.value

    def profile(self, dt, n):
        """Device milliseconds per stage summed over n steps: sweep, cull, narrowphase
        (GJK + per-thread EPA), warp-tier EPA, large-polytope EPA, solver."""
        ms = np.zeros(6, np.float32)
        _check(self.lib.nans_profile_steps(self.h, dt, n, _ptr(ms)))
        return ms

    def timeline(self, dt, n):
        """Mean milliseconds from a step's start to the end of each stage over n eager steps
        with the stream overlap: sweep, cull, GJK + per-thread EPA, warp tier, large tiers
        (second stream), solve pass 0, solve pass 1 (the step's end)."""
        ms = np.zeros(7, np.float32)
        _check(self.lib.nans_profile_timeline(self.h, dt, n, _ptr(ms)))
        return ms / max(1, n)

    def epa_stats(self, reset=False):
        out = np.zeros(8, np.uint32)
        _check(self.lib.nans_world_epa_stats(self.h, _ptr(out), 1 if reset else 0))
        return dict(max_faces=int(out[0]), max_edges=int(out[1]), slow_epas=int(out[2]),
                    overflow_candidate=int(out[3]) - 1, overflow_scene=int(out[4]) - 1,
                    overflows=int(out[5]), warp_tier=int(out[6]), giant_tier=int(out[7]))

    # -- differentiable rollout -------------------------------------------------------
    def diff_forward(self, dt, n, params=None):
        """n plain steps that also record the adjoint's tape (same results as step)."""
        p = None
        if params is not None:
            p = ctypes.byref(StepParams(params.cr, params.cf, params.iterations))
        _check(self.lib.nans_diff_forward(self.h, p, dt, n))

    def diff_backward(self, dl_position=None, dl_angles=None, dl_velocity=None, dl_omega=None):
        """Gradients of a loss of the final state with respect to the initial state, the
        masses and the solver constants of the last diff_forward. Per-body arrays are
        (n_bodies, 3) in record order (all cubes, then all spheres); returns a dict with
        position0, angles0, velocity0, omega0 (n_bodies, 3), mass (n_bodies,), restitution
        and friction (n_scenes,)."""
        nb, ns = self.n_bodies, len(self.scenes)

        def inp(a):
            if a is None:
                return None
            a = np.ascontiguousarray(a, np.float32)
            if a.shape != (nb, 3):
                raise ValueError("gradient input must have shape (%d, 3)" % nb)
            return a
        ins = [inp(a) for a in (dl_position, dl_angles, dl_velocity, dl_omega)]
        out = dict(position0=np.zeros((nb, 3), np.float32), angles0=np.zeros((nb, 3), np.float32),
                   velocity0=np.zeros((nb, 3), np.float32), omega0=np.zeros((nb, 3), np.float32),
                   mass=np.zeros(nb, np.float32), restitution=np.zeros(ns, np.float32),
                   friction=np.zeros(ns, np.float32))
        g = DiffGrads(*([_ptr(a) for a in ins] + [_ptr(out[k]) for k in ("position0", "angles0", "velocity0",
                                                                        "omega0", "mass", "restitution",
                                                                        "friction")]))
        _check(self.lib.nans_diff_backward(self.h, ctypes.byref(g)))
        return out

    def diff_tape_info(self):
        n, b = _U(), ctypes.c_uint64()
        _check(self.lib.nans_diff_tape_info(self.h, ctypes.byref(n), ctypes.byref(b)))
        return n.value, b.value

    @property
    def n_bodies(self):
        return self._ncubes + self._nspheres

    @property
    def stream(self):
        return self.lib.nans_world_stream(self.h)


def save_ppm(path, img):
    """Writes a (height, width, 3) uint8 image as binary PPM."""
    h, w = img.shape[:2]
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(img, np.uint8).tobytes())


def solve_contacts_static(nbodies, ncubes, d_position, d_mass, d_moi, d_velocity, d_angular_velocity, floor,
                          d_pairs, npairs, cr, cf, iterations, dt, stream=None):
    """Allocation-free contact solve on caller-owned device buffers (raw device addresses)."""
    floor = np.ascontiguousarray(floor, np.float32)
    _check(load().nans_solve_contacts_static(nbodies, ncubes, d_position, d_mass, d_moi, d_velocity,
                                             d_angular_velocity, _ptr(floor), d_pairs, npairs, cr, cf,
                                             iterations, dt, stream))
