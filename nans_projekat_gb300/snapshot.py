"""Scene snapshots: a batch of scenes (bodies, shapes, ground, solver constants) in one file,
structure-of-arrays binary with a JSON header.

The reference builds its one scene in code (Init, code/nans.cpp:1550-1717) and has no file
format; a snapshot replaces that step for reproducible inputs and fixtures, and stores a world's
state between runs (a saved state continues bit for bit: every field the step reads is kept,
including each body's Model matrix).

Layout (little-endian):
    bytes 0-7     magic  b"NANSSNAP"
    bytes 8-11    uint32 format version (1)
    bytes 12-19   uint64 header length H
    bytes 20-     UTF-8 JSON header of H bytes, then zero padding to a 64-byte boundary
    then          the arrays, each starting on a 64-byte boundary

The header holds "scenes", "cubes", "spheres", "hull_points", "rebuild_models", free-form
"meta" (a seed, a generator name, a step count ...) and "arrays": for every array its name,
dtype ("f4", "i4", "u4"), shape, byte offset from the start of the file and byte length.
Per-body arrays are in record order: the cubes of every scene in scene order, then the spheres.
"""
import json

import numpy as np

from .scenes import Scene, Constants
from .types import CUBE_DTYPE, SPHERE_DTYPE

MAGIC = b"NANSSNAP"
VERSION = 1
ALIGN = 64

# name -> (record field or None, dtype, per-row shape)
_CUBE_FIELDS = [("Model", "model", (16,)), ("Vertices", "vertices", (8, 3)), ("Position", "position", (3,)),
                ("V", "velocity", (3,)), ("Forces", "force", (3,)), ("Angles", "angles", (3,)),
                ("W", "omega", (3,)), ("Torque", "torque", (3,)), ("Size", "size", ()), ("Mass", "mass", ()),
                ("MOI", "moi", ())]
_SPHERE_FIELDS = [("Model", "model", (16,)), ("Position", "position", (3,)), ("V", "velocity", (3,)),
                  ("Forces", "force", (3,)), ("Angles", "angles", (3,)), ("W", "omega", (3,)),
                  ("Torque", "torque", (3,)), ("Radius", "radius", ()), ("Mass", "mass", ()), ("MOI", "moi", ())]


def _pad(n):
    return (-n) % ALIGN


def save(path, scenes, meta=None):
    """Writes the scenes to `path`."""
    scenes = list(scenes)
    if not scenes:
        raise ValueError("no scenes")
    rebuild = scenes[0].rebuild_models
    if any(s.rebuild_models != rebuild for s in scenes):
        raise ValueError("all scenes of a snapshot must agree on rebuild_models")
    cubes = np.concatenate([s.cubes for s in scenes]) if sum(len(s.cubes) for s in scenes) else \
        np.zeros(0, CUBE_DTYPE)
    spheres = np.concatenate([s.spheres for s in scenes]) if sum(len(s.spheres) for s in scenes) else \
        np.zeros(0, SPHERE_DTYPE)
    floors = np.concatenate([s.floor for s in scenes])
    arrays = {
        "scene_cubes": np.array([len(s.cubes) for s in scenes], np.uint32),
        "scene_spheres": np.array([len(s.spheres) for s in scenes], np.uint32),
        "restitution": np.array([s.constants.cr for s in scenes], np.float32),
        "friction": np.array([s.constants.cf for s in scenes], np.float32),
        "iterations": np.array([s.constants.iterations for s in scenes], np.int32),
        "dt": np.array([s.constants.dt for s in scenes], np.float32),
        "cube_scale": np.concatenate([s.scale_array() for s in scenes]).astype(np.float32).reshape(-1, 3),
        "hull_npts": np.concatenate([s.hull_npts if s.hull_npts is not None else np.zeros(len(s.cubes), np.int32)
                                     for s in scenes]).astype(np.int32),
        "hull_pts": (np.concatenate([s.hull_pts for s in scenes if s.hull_pts is not None and len(s.hull_pts)])
                     .astype(np.float32).reshape(-1, 3)
                     if any(s.hull_pts is not None and len(s.hull_pts) for s in scenes)
                     else np.zeros((0, 3), np.float32)),
    }
    for rec, prefix, fields in ((cubes, "cube_", _CUBE_FIELDS), (spheres, "sphere_", _SPHERE_FIELDS),
                                (floors, "floor_", _CUBE_FIELDS)):
        for f, name, shape in fields:
            arrays[prefix + name] = np.ascontiguousarray(rec[f], np.float32).reshape((len(rec),) + shape)
    header = {"format": "nans snapshot", "version": VERSION, "scenes": len(scenes), "cubes": int(len(cubes)),
              "spheres": int(len(spheres)), "hull_points": int(len(arrays["hull_pts"])),
              "rebuild_models": bool(rebuild), "names": [s.name for s in scenes], "meta": meta or {},
              "arrays": []}
    # offsets depend on the header length: lay out with a provisional header, then fix
    names = list(arrays)
    for _ in range(3):
        hbytes = json.dumps(header).encode()
        pos = 20 + len(hbytes)
        pos += _pad(pos)
        header["arrays"] = []
        for n in names:
            a = arrays[n]
            header["arrays"].append({"name": n, "dtype": a.dtype.str[1:], "shape": list(a.shape), "offset": pos,
                                     "bytes": int(a.nbytes)})
            pos += a.nbytes + _pad(a.nbytes)
    hbytes = json.dumps(header).encode()
    assert 20 + len(hbytes) <= header["arrays"][0]["offset"]
    with open(path, "wb") as f:
        f.write(MAGIC)
        f.write(np.uint32(VERSION).tobytes())
        f.write(np.uint64(len(hbytes)).tobytes())
        f.write(hbytes)
        for n, d in zip(names, header["arrays"]):
            f.write(b"\0" * (d["offset"] - f.tell()))
            f.write(np.ascontiguousarray(arrays[n]).tobytes())
    return header


def read_header(path):
    with open(path, "rb") as f:
        head = f.read(20)
        if head[:8] != MAGIC:
            raise ValueError("%s: not a nans snapshot" % path)
        version = int(np.frombuffer(head[8:12], np.uint32)[0])
        if version != VERSION:
            raise ValueError("%s: snapshot version %d, expected %d" % (path, version, VERSION))
        hlen = int(np.frombuffer(head[12:20], np.uint64)[0])
        return json.loads(f.read(hlen).decode())


def load(path):
    """Reads the scenes back (a list of Scene), with the header's meta."""
    header = read_header(path)
    raw = np.fromfile(path, np.uint8)
    arrays = {}
    for d in header["arrays"]:
        a = raw[d["offset"]:d["offset"] + d["bytes"]].view(np.dtype("<" + d["dtype"]))
        arrays[d["name"]] = a.reshape(d["shape"])
    nc_all, ns_all = header["cubes"], header["spheres"]
    cubes = np.zeros(nc_all, CUBE_DTYPE)
    spheres = np.zeros(ns_all, SPHERE_DTYPE)
    floors = np.zeros(header["scenes"], CUBE_DTYPE)
    for rec, prefix, fields in ((cubes, "cube_", _CUBE_FIELDS), (spheres, "sphere_", _SPHERE_FIELDS),
                                (floors, "floor_", _CUBE_FIELDS)):
        for f, name, shape in fields:
            rec[f] = arrays[prefix + name].reshape((len(rec),) + shape)
    snc = arrays["scene_cubes"].astype(np.int64)
    sns = arrays["scene_spheres"].astype(np.int64)
    npts = arrays["hull_npts"]
    out = []
    co = so = ho = 0
    for i in range(header["scenes"]):
        c = cubes[co:co + snc[i]].copy()
        s = spheres[so:so + sns[i]].copy()
        hn = npts[co:co + snc[i]].copy()
        k = int(hn.sum())
        hp = arrays["hull_pts"][ho:ho + k].copy()
        hull = bool(hn.any())
        out.append(Scene(c, s, floors[i:i + 1].copy(), cube_scale=arrays["cube_scale"][co:co + snc[i]].copy(),
                         hull_npts=hn if hull else None, hull_pts=hp if hull else None,
                         constants=Constants(cr=float(arrays["restitution"][i]), cf=float(arrays["friction"][i]),
                                             iterations=int(arrays["iterations"][i]), dt=float(arrays["dt"][i])),
                         rebuild_models=header["rebuild_models"], name=header["names"][i]))
        co += snc[i]
        so += sns[i]
        ho += k
    return out, header["meta"]


def from_world(world):
    """The world's current state as scenes (shapes and constants from its upload), continuing
    bit for bit when uploaded again: Model matrices are kept and the first step uses them."""
    cubes, spheres, floors = world.download()
    out = []
    for i, sc in enumerate(world.scenes):
        c, s, f = world.scene_state(i, (cubes, spheres, floors))
        s2 = Scene(c.copy(), s.copy(), f.copy(), cube_scale=sc.scale_array(), hull_npts=sc.hull_npts,
                   hull_pts=sc.hull_pts, constants=sc.constants, rebuild_models=False, name=sc.name)
        out.append(s2)
    return out
