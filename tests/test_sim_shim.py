"""The headless SimUpdateAndRender (libnans_sim.so, include/nans_sim.h): the reference's frame
entry point over the GPU step. CPU tests check the exported symbols and the platform struct
layouts; the GPU test drives 300 frames with no input and compares every frame's bodies and
contact list with the reference's own SimUpdateAndRender (tests/golden/demo_frames.npz)."""
import ctypes
import os

import numpy as np
import pytest

from helpers import load_golden, step_digest
from nans_projekat_gb300 import build
from nans_projekat_gb300.types import CUBE_DTYPE, SPHERE_DTYPE, PAIR_DTYPE

CAMERA = np.dtype([("FOV", "<f4"), ("Pitch", "<f4"), ("Yaw", "<f4"), ("Speed", "<f4"), ("Position", "<f4", 3),
                   ("Target", "<f4", 3), ("Direction", "<f4", 3), ("Up", "<f4", 3), ("Front", "<f4", 3),
                   ("Right", "<f4", 3)])
STATE = np.dtype([("Cubes", CUBE_DTYPE, 16), ("Spheres", SPHERE_DTYPE, 16), ("Floor", CUBE_DTYPE),
                  ("Camera", CAMERA), ("CubeCount", "<u4"), ("SphereCount", "<u4"), ("PairCount", "<u4"),
                  ("Pairs", PAIR_DTYPE, 1024), ("Frames", "<u8"), ("LastStatus", "<i4"), ("World", "<u8")],
                 align=True)


class Memory(ctypes.Structure):  # struct memory (code/nans.h:227-235)
    _fields_ = [("PermanentStorage", ctypes.c_void_p), ("PermanentStorageSize", ctypes.c_uint64),
                ("TransientStorage", ctypes.c_void_p), ("TransientStorageSize", ctypes.c_uint64),
                ("IsInitialized", ctypes.c_int32)]


class Input(ctypes.Structure):  # struct sdl_input (code/nans.h:120-165)
    _fields_ = [("Buttons", ctypes.c_int32 * 26), ("Sensitivity", ctypes.c_float), ("XRel", ctypes.c_int32),
                ("YRel", ctypes.c_int32), ("X", ctypes.c_int32), ("Y", ctypes.c_int32)]


@pytest.fixture(scope="module")
def sim():
    build.build()
    L = ctypes.CDLL(build.SIM_PATH)
    L.SimUpdateAndRender.argtypes = [ctypes.POINTER(Memory), ctypes.POINTER(Input), ctypes.c_void_p, ctypes.c_float]
    L.nans_sim_state_bytes.restype = ctypes.c_uint64
    return L


def test_layouts(sim):
    assert ctypes.sizeof(Memory) == 40      # two pointers, two uint64, bool32, padding
    assert ctypes.sizeof(Input) == 13 * 8 + 20
    assert sim.nans_sim_state_bytes() == STATE.itemsize


def _run(sim, frames, dt, press=None):
    buf = np.zeros(STATE.itemsize, np.uint8)
    mem = Memory(buf.ctypes.data, buf.nbytes, None, 0, 0)
    inp = Input()
    inp.Sensitivity = 0.1
    out = []
    for k in range(frames):
        for i in range(26):
            inp.Buttons[i] = 0
        if press is not None and k in press:
            inp.Buttons[2 * press[k] + 1] = 1
        sim.SimUpdateAndRender(ctypes.byref(mem), ctypes.byref(inp), None, ctypes.c_float(dt))
        st = buf.view(STATE)[0]
        out.append(st.copy())
    return out, mem


@pytest.mark.gpu
def test_frames_match_reference_frame_function(sim):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required")
    scene, meta, digests, saved = load_golden("demo_frames")
    states, mem = _run(sim, meta["nsteps"], np.float32(meta["dt"]))
    assert mem.IsInitialized == 1
    for k, st in enumerate(states, start=1):
        assert st["LastStatus"] == 0 and st["Frames"] == k
        cubes = st["Cubes"][:st["CubeCount"]]
        spheres = st["Spheres"][:st["SphereCount"]]
        pairs = st["Pairs"][:st["PairCount"]]
        if step_digest(cubes, spheres, pairs) != digests[k - 1]:
            pytest.fail("frame %d differs from the reference's SimUpdateAndRender" % k)


@pytest.mark.gpu
def test_shoot_input_launches_the_sphere(sim):
    """ShootSphere (code/nans.cpp:105-112): the sphere restarts at the camera and is pushed
    along the camera's front (-z at start) by SHOOT_FORCE for one step."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required")
    states, _ = _run(sim, 3, np.float32(1 / 60), press={1: 4})
    sp = states[1]["Spheres"][0]
    assert states[1]["LastStatus"] == 0
    assert sp["V"][2] < -10.0 and abs(sp["V"][0]) < 1e-3
    assert abs(sp["Position"][0] - 0.0) < 1e-3 and sp["Position"][2] < 3.0
