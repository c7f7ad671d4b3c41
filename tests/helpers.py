"""Shared helpers for the tests: canonical state/pair bytes and field-wise comparison."""
import hashlib

import numpy as np

STATE_FIELDS = ("Position", "V", "Angles", "W")
PAIR_FIELDS = ("Type", "IndexA", "IndexB", "PointA", "PointB", "N")


def canon(x):
    """Array bytes with every NaN replaced by one quiet NaN. IEEE 754 leaves the sign and
    payload of a NaN result unspecified (x86 SSE, aarch64 and the GPU differ), so parity is
    bit-exact for every other value and NaN-for-NaN here."""
    a = np.array(x, copy=True)
    if a.dtype == np.float32:
        a = a.view(np.uint32)
        nan = (a & 0x7F800000) == 0x7F800000
        nan &= (a & 0x007FFFFF) != 0
        a[nan] = 0x7FC00000
    return np.ascontiguousarray(a).tobytes()


def state_bytes(cubes, spheres):
    parts = []
    for f in STATE_FIELDS:
        parts.append(canon(np.asarray(cubes[f], np.float32)))
        parts.append(canon(np.asarray(spheres[f], np.float32)))
    return b"".join(parts)


def pair_bytes(pairs):
    return b"".join(canon(np.asarray(pairs[f])) for f in PAIR_FIELDS)


def step_digest(cubes, spheres, pairs):
    h = hashlib.sha256()
    h.update(state_bytes(cubes, spheres))
    h.update(pair_bytes(pairs))
    return h.hexdigest()[:16]


def same_fields(a, b, fields):
    """Bit-exact equality of the named fields (NaN matches NaN, see canon)."""
    for f in fields:
        x = np.asarray(a[f])
        y = np.asarray(b[f])
        if x.shape != y.shape or canon(x) != canon(y):
            return False, f
    return True, None


def first_difference(a, b, fields):
    for f in fields:
        x = np.asarray(a[f]).reshape(len(a), -1)
        y = np.asarray(b[f]).reshape(len(b), -1)
        if x.shape != y.shape:
            return "%s: shape %s vs %s" % (f, x.shape, y.shape)
        xb = np.frombuffer(canon(x), np.uint32 if x.dtype == np.float32 else x.dtype).reshape(x.shape)
        yb = np.frombuffer(canon(y), np.uint32 if y.dtype == np.float32 else y.dtype).reshape(y.shape)
        bad = np.nonzero(xb != yb)
        if len(bad[0]):
            i, j = bad[0][0], bad[1][0]
            return "%s[%d][%d]: %r vs %r" % (f, i, j, x[i, j], y[i, j])
    return None


GOLDEN_CASES = ("stack8_seed0", "stack8_refconst", "demo_frames", "stack_random_5", "stack_random_12",
                "stack_random_40", "stack_random_90", "random_mixed72", "random_dense16",
                "stack_emptied_6663", "stack_emptied_5642", "stack_bigepa_3029", "stack_bigepa_7755",
                "stack_bigepa_6880", "stack_bigepa_897")


def load_golden(name):
    """Returns (scene, meta, digests, saved) for a fixture written by golden/make_golden.py."""
    import json
    import os

    from nans_projekat_gb300.scenes import Scene, Constants

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name + ".npz")
    z = np.load(path, allow_pickle=False)
    meta = json.loads(str(z["meta"]))
    consts = Constants(cr=meta["cr"], cf=meta["cf"], iterations=meta["iterations"], dt=meta["dt"])
    scene = Scene(z["in_cubes"], z["in_spheres"], z["in_floor"], cube_scale=z["in_scale"],
                  constants=consts, rebuild_models=meta["rebuild_models"], name=name)
    saved = {k: z[k] for k in z.files if k.split("_")[0] in ("cubes", "spheres", "pairs")}
    return scene, meta, [str(d) for d in z["digests"]], saved


def _inflate(lo, hi, finite):
    mag = np.maximum(np.abs(lo), np.abs(hi)).max(axis=-1)
    m = (np.float32(1e-4) * mag + np.float32(1e-5)).astype(np.float32)
    lo = (lo - m[..., None]).astype(np.float32)
    hi = (hi + m[..., None]).astype(np.float32)
    unbounded = ~finite | ~(mag <= np.float32(1e6))
    lo[unbounded] = -np.inf
    hi[unbounded] = np.inf
    return lo, hi


def aabb_margin_boxes(vertices):
    """Cull boxes of hulls exactly as the device sweep computes them (float32)."""
    v = np.asarray(vertices, np.float32)
    finite = np.isfinite(v).all(axis=(-1, -2))
    fv = np.where(np.isfinite(v), v, np.float32(0))
    lo = fv.min(axis=-2)
    hi = fv.max(axis=-2)
    lo = np.where(np.isnan(lo), np.float32(0), lo).astype(np.float32)
    hi = np.where(np.isnan(hi), np.float32(0), hi).astype(np.float32)
    return _inflate(lo, hi, finite)


def aabb_margin_spheres(position, radius):
    p = np.asarray(position, np.float32)
    r = np.asarray(radius, np.float32)[:, None]
    with np.errstate(invalid="ignore", over="ignore"):
        lo = (p - r).astype(np.float32)
        hi = (p + r).astype(np.float32)
        finite = np.isfinite(lo).all(axis=-1) & np.isfinite(hi).all(axis=-1)
    return _inflate(np.where(np.isfinite(lo), lo, 0).astype(np.float32),
                    np.where(np.isfinite(hi), hi, 0).astype(np.float32), finite)
