"""Test infrastructure: ctypes binding of the oracle restatement (oracle/port/nans_oracle.cpp,
built by ``make -C oracle port`` into oracle/_build/libnans_oracle.so).

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may use this
module, and only as the checker.
"""
import ctypes
import os
import subprocess

import numpy as np

from nans_projekat_gb300.types import CUBE_DTYPE, SPHERE_DTYPE, PAIR_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libnans_oracle.so")

_P = ctypes.c_void_p
_U = ctypes.c_uint32
_F = ctypes.c_float
_I = ctypes.c_int

_LIB = None


def build():
    subprocess.check_call(["make", "-s", "-C", HERE, "port"])


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.nanso_create.argtypes = [_I]
        L.nanso_create.restype = _P
        L.nanso_destroy.argtypes = [_P]
        L.nanso_num_scenes.argtypes = [_P]
        L.nanso_num_scenes.restype = _I
        L.nanso_add_scene.argtypes = [_P, _P, _U, _P, _U, _P, _P, _P, _P, _P, _F, _F, _I, _I]
        L.nanso_add_scene.restype = _I
        L.nanso_step.argtypes = [_P, _F, _I, _I]
        L.nanso_stage.argtypes = [_P, _I, _F, _I]
        L.nanso_step_range.argtypes = [_P, _I, _I, _F, _I, _I]
        L.nanso_store.argtypes = [_P, _I, _P, _P, _P]
        L.nanso_state_f64.argtypes = [_P, _I, _P]
        L.nanso_set_warm.argtypes = [_P, _I]
        L.nanso_pairs.argtypes = [_P, _I, _P, _U]
        L.nanso_pairs.restype = _U
        L.nanso_set_constants.argtypes = [_P, _I, _F, _F, _I]
        L.nanso_set_replay.argtypes = [_P, _I, _I, _P, _P, _P, _P]
        L.nanso_sincosf.argtypes = [_P, _P, _P, _I]
        L.nanso_epa_stats.argtypes = [_P, _I]
        L.nanso_stats_enable.argtypes = [_I]
        _LIB = L
    return _LIB


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class OracleWorld:
    """A set of independent scenes stepped by the oracle (FP32 or FP64)."""

    def __init__(self, scenes, fp64=False):
        self.lib = lib()
        self.fp64 = bool(fp64)
        self.h = self.lib.nanso_create(1 if fp64 else 0)
        self.scenes = list(scenes)
        self._keep = []
        for sc in self.scenes:
            cubes = np.ascontiguousarray(sc.cubes)
            spheres = np.ascontiguousarray(sc.spheres)
            floor = np.ascontiguousarray(sc.floor)
            scale = None if sc.cube_scale is None else np.ascontiguousarray(sc.cube_scale, np.float32)
            npts = None if sc.hull_npts is None else np.ascontiguousarray(sc.hull_npts, np.int32)
            pts = None if sc.hull_pts is None else np.ascontiguousarray(sc.hull_pts, np.float32)
            c = sc.constants
            self.lib.nanso_add_scene(self.h, _ptr(cubes), len(cubes), _ptr(spheres), len(spheres),
                                     _ptr(floor), _ptr(scale), None, _ptr(npts), _ptr(pts),
                                     c.cr, c.cf, c.iterations, 1 if sc.rebuild_models else 0)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.nanso_destroy(self.h)
            self.h = None

    def set_warm(self, on=True):
        """Warm starting: accumulators carried across steps for pairs that stay in contact."""
        self.lib.nanso_set_warm(self.h, 1 if on else 0)

    def step(self, dt, n=1, threads=1):
        self.lib.nanso_step(self.h, dt, n, threads)

    def stage(self, st, dt, threads=1):
        self.lib.nanso_stage(self.h, st, dt, threads)

    def step_range(self, lo, hi, dt, n=1, threads=1):
        self.lib.nanso_step_range(self.h, lo, hi, dt, n, threads)

    def state(self, i=0):
        sc = self.scenes[i]
        cubes = np.zeros(len(sc.cubes), CUBE_DTYPE)
        spheres = np.zeros(len(sc.spheres), SPHERE_DTYPE)
        floor = np.zeros(1, CUBE_DTYPE)
        self.lib.nanso_store(self.h, i, _ptr(cubes), _ptr(spheres), _ptr(floor))
        return cubes, spheres, floor

    def state_f64(self, i=0):
        """(n_bodies, 12) array: P, V, Angles, W for cubes then spheres."""
        n = self.scenes[i].n_bodies
        out = np.zeros((n, 12), np.float64)
        self.lib.nanso_state_f64(self.h, i, _ptr(out))
        return out

    def hold_contacts(self, i, steps):
        """Holds scene i's contacts for its next len(steps) steps: steps[k] = (positions of the
        scene's dynamic bodies at step k's solve, the floor's position, the contact records of
        step k), as recorded from another run. The detect stage then replays them and the solve
        takes lever arms and depth from the recorded positions: the rollout with its contact set
        and contact geometry held fixed. An empty list turns it off."""
        nc = len(self.scenes[i].cubes)
        counts = np.array([len(p) for _, _, p in steps], np.int32)
        pairs = np.concatenate([p for _, _, p in steps]) if len(steps) else np.zeros(0, PAIR_DTYPE)
        pos_a = np.zeros((len(pairs), 3), np.float32)
        pos_b = np.zeros((len(pairs), 3), np.float32)
        q = 0
        for pos, floor_pos, prs in steps:
            for r in prs:
                t = int(r["Type"])
                a = int(r["IndexA"]) + (nc if t in (3, 4) else 0)           # SS, SF: A is a sphere
                pos_a[q] = pos[a]
                if t in (2, 4):                                              # CF, SF: B is the floor
                    pos_b[q] = floor_pos
                else:
                    pos_b[q] = pos[int(r["IndexB"]) + (nc if t in (1, 3) else 0)]  # CS, SS: B a sphere
                q += 1
        pairs = np.ascontiguousarray(pairs)
        self.lib.nanso_set_replay(self.h, i, len(steps), _ptr(counts), _ptr(pairs), _ptr(pos_a), _ptr(pos_b))

    def pairs(self, i=0):
        n = self.lib.nanso_pairs(self.h, i, None, 0)
        out = np.zeros(n, PAIR_DTYPE)
        if n:
            self.lib.nanso_pairs(self.h, i, _ptr(out), n)
        return out


def sincos(x):
    x = np.ascontiguousarray(x, np.float32)
    s = np.zeros_like(x)
    c = np.zeros_like(x)
    lib().nanso_sincosf(_ptr(x), _ptr(s), _ptr(c), len(x))
    return s, c


def stats_enable(on=True):
    lib().nanso_stats_enable(1 if on else 0)


def epa_stats(reset=True):
    """EPA / GJK statistics collected while stats_enable(True) is on."""
    out = np.zeros(94, np.int64)
    lib().nanso_epa_stats(_ptr(out), 1 if reset else 0)
    return dict(max_faces=int(out[0]), max_edges=int(out[1]), max_iter=int(out[2]), calls=int(out[3]),
                over128=int(out[4]), over256=int(out[5]), over1024=int(out[6]), over4096=int(out[7]), over128_nan_face0=int(out[8]), emptied=int(out[9]), over1024_contact=int(out[10]),
                epa_iter_hist=[int(x) for x in out[11:16]], gjk_evolves=int(out[16]), gjk_runs=int(out[17]),
                tiny_fit=[int(x) for x in out[18:22]], faces_hist=[int(x) for x in out[22:86]],
                gjk_hist=[int(x) for x in out[86:94]])
