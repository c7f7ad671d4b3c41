"""Test infrastructure: ctypes binding of the reference physics compiled headless
(oracle/_ref/libnans_ref*.so, built by ``make -C oracle ref`` from the reference sources).

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may use this
module, and only as the checker. The libraries exist only where the reference checkout
was present when they were built.
"""
import ctypes
import os

import numpy as np

from nans_projekat_gb300.types import CUBE_DTYPE, SPHERE_DTYPE, PAIR_DTYPE

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
VARIANTS = ("ref16", "refbig", "ref_pristine", "ref16_O2", "refbig_O2")


def ref_path(variant="refbig"):
    return os.path.join(REF_DIR, "libnans_%s.so" % variant)


def ref_available(variant="refbig"):
    return os.path.exists(ref_path(variant))


_P = ctypes.c_void_p
_U = ctypes.c_uint32
_F = ctypes.c_float
_I = ctypes.c_int


def _load(variant):
    lib = ctypes.CDLL(ref_path(variant))
    lib.nansref_create.restype = _P
    lib.nansref_destroy.argtypes = [_P]
    lib.nansref_capacity.restype = _I
    lib.nansref_sizeof_cube.restype = _I
    lib.nansref_sizeof_sphere.restype = _I
    lib.nansref_sizeof_pair.restype = _I
    lib.nansref_set_constants.argtypes = [_F, _F, _I]
    lib.nansref_load.argtypes = [_P, _P, _U, _P, _U, _P, _P, _P]
    lib.nansref_load.restype = _I
    lib.nansref_store.argtypes = [_P, _P, _P, _P]
    lib.nansref_rebuild.argtypes = [_P]
    lib.nansref_stage.argtypes = [_P, _I, _F]
    lib.nansref_step.argtypes = [_P, _F, _I]
    lib.nansref_pairs.argtypes = [_P, _P, _U]
    lib.nansref_pairs.restype = _U
    lib.nansref_frame_create.restype = _P
    lib.nansref_frame_destroy.argtypes = [_P]
    lib.nansref_frame_run.argtypes = [_P, _F, _I]
    lib.nansref_frame_state.argtypes = [_P, _P, _P, _P, _P, _P, _P, _U, _P]
    assert lib.nansref_sizeof_cube() == CUBE_DTYPE.itemsize
    assert lib.nansref_sizeof_sphere() == SPHERE_DTYPE.itemsize
    assert lib.nansref_sizeof_pair() == PAIR_DTYPE.itemsize
    return lib


_LIBS = {}


def lib(variant="refbig"):
    if variant not in _LIBS:
        _LIBS[variant] = _load(variant)
    return _LIBS[variant]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class RefWorld:
    """One reference scene driven through the reference's own static physics functions."""

    def __init__(self, scene, variant="refbig", cr=None, cf=None, iters=None, rebuild=True):
        self.lib = lib(variant)
        self.variant = variant
        self.scene = scene
        self.h = self.lib.nansref_create()
        c = scene.constants
        self.lib.nansref_set_constants(
            c.cr if cr is None else cr, c.cf if cf is None else cf,
            c.iterations if iters is None else iters)
        self.cubes = np.ascontiguousarray(scene.cubes.copy())
        self.spheres = np.ascontiguousarray(scene.spheres.copy())
        self.floor = np.ascontiguousarray(scene.floor.copy())
        scale = None if scene.cube_scale is None else np.ascontiguousarray(scene.cube_scale, np.float32)
        rc = self.lib.nansref_load(self.h, _ptr(self.cubes), len(self.cubes), _ptr(self.spheres),
                                   len(self.spheres), _ptr(self.floor), _ptr(scale), None)
        if rc != 0:
            raise ValueError("scene exceeds the reference build's capacity (%d)"
                             % self.lib.nansref_capacity())
        if rebuild:
            self.lib.nansref_rebuild(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.nansref_destroy(self.h)
            self.h = None

    def set_constants(self, cr, cf, iters):
        self.lib.nansref_set_constants(cr, cf, iters)

    def step(self, dt, n=1):
        self.lib.nansref_set_constants(*self._consts())
        self.lib.nansref_step(self.h, dt, n)

    def stage(self, stage, dt):
        self.lib.nansref_set_constants(*self._consts())
        self.lib.nansref_stage(self.h, stage, dt)

    def _consts(self):
        c = self.scene.constants
        return (c.cr, c.cf, c.iterations)

    def state(self):
        cubes = np.zeros(len(self.scene.cubes), CUBE_DTYPE)
        spheres = np.zeros(len(self.scene.spheres), SPHERE_DTYPE)
        floor = np.zeros(1, CUBE_DTYPE)
        self.lib.nansref_store(self.h, _ptr(cubes), _ptr(spheres), _ptr(floor))
        return cubes, spheres, floor

    def pairs(self):
        n = self.lib.nansref_pairs(self.h, None, 0)
        out = np.zeros(n, PAIR_DTYPE)
        if n:
            self.lib.nansref_pairs(self.h, _ptr(out), n)
        return out


class RefFrame:
    """The reference's own SimUpdateAndRender (code/nans.cpp:1719), headless."""

    def __init__(self, variant="ref_pristine"):
        self.lib = lib(variant)
        self.h = self.lib.nansref_frame_create()

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.nansref_frame_destroy(self.h)
            self.h = None

    def run(self, dt, nframes=1):
        self.lib.nansref_frame_run(self.h, dt, nframes)

    def state(self, pair_cap=4096):
        nc, ns, npairs = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        cap = self.lib.nansref_capacity()
        cubes = np.zeros(cap, CUBE_DTYPE)
        spheres = np.zeros(cap, SPHERE_DTYPE)
        floor = np.zeros(1, CUBE_DTYPE)
        pairs = np.zeros(pair_cap, PAIR_DTYPE)
        self.lib.nansref_frame_state(self.h, ctypes.byref(nc), ctypes.byref(ns), _ptr(cubes),
                                     _ptr(spheres), _ptr(floor), _ptr(pairs), pair_cap,
                                     ctypes.byref(npairs))
        return (cubes[:nc.value].copy(), spheres[:ns.value].copy(), floor.copy(),
                pairs[:min(npairs.value, pair_cap)].copy())
