"""Central finite differences of the FP64 oracle on the differentiated configuration: 4x4x2 stacks
of unit boxes plus one sphere launched at 20 m/s (scenes.grid_stack_batch, seed 3), loss = the
squared distance of the sphere's final position to a seeded target point; parameters = the
sphere's initial velocity (3), every body's mass (33; the moment of inertia scales with it) and
the restitution (1).

Two FP64 references:
  * the oracle's step itself (GJK/EPA run on every perturbed state);
  * the same step with each step's contact set and contact geometry held at the values of the
    unperturbed FP32 run (OracleWorld.hold_contacts) -- the model the GPU adjoint differentiates.

Test infrastructure only: it drives the oracle, which only tests use.
"""
import numpy as np

from nans_projekat_gb300 import diff, scenes
from nans_projekat_gb300.scenes import Constants

DT = np.float32(1.0 / 60.0)
H = 1e-3
N_PARAMS = 3 + 1 + 33
LAYOUT_SEED = 3
N_BATCH = 1024


def c3_scenes(k=8, seed=33):
    """k scenes of the 1,024-scene configuration, drawn with SplitMix64(seed), and one target
    point per scene (uniform over the stack's extent: x, z in [-2, 2] m, y in [0.5, 2] m)."""
    batch = scenes.grid_stack_batch(N_BATCH, seed=LAYOUT_SEED)
    rng = scenes.SplitMix64(seed)
    idx = []
    while len(idx) < k:
        i = int(rng.uniform(1, 0, N_BATCH)[0])
        if i not in idx:
            idx.append(i)
    targets = np.stack([rng.uniform(k, -2.0, 2.0), rng.uniform(k, 0.5, 2.0), rng.uniform(k, -2.0, 2.0)], axis=1)
    return [batch[i] for i in idx], targets, idx


def state_scene(sc, nsteps):
    """The scene's state after nsteps steps of the FP32 oracle, as a scene (records of that state;
    the Model is rebuilt from Position and Angles, as every step does)."""
    from oracle.portbind import OracleWorld
    o = OracleWorld([sc])
    if nsteps:
        o.step(DT, nsteps)
    c, s, _ = o.state(0)
    out = diff.with_state([sc])[0]
    out.cubes = c.copy()
    out.spheres = s.copy()
    return out


def first_impact(sc, limit=120):
    """First step whose contact list has a box-sphere pair."""
    from oracle.portbind import OracleWorld
    o = OracleWorld([sc])
    for k in range(1, limit + 1):
        o.step(DT, 1)
        if np.any(o.pairs(0)["Type"] == 1):
            return k
    return None


def perturbed(sc, p, h):
    """(scene with parameter p moved by h, the parameter's value as stored in float32).
    p = ("V", component) of the sphere, ("cr",) or ("m", body) in record order."""
    s2 = diff.with_state([sc])[0]
    if p[0] == "V":
        s2.spheres = s2.spheres.copy()
        s2.spheres["V"][0, p[1]] += np.float32(h)
        return s2, float(s2.spheres["V"][0, p[1]])
    if p[0] == "cr":
        k = s2.constants
        s2.constants = Constants(cr=np.float32(float(k.cr) + h), cf=k.cf, iterations=k.iterations, dt=k.dt)
        return s2, float(s2.constants.cr)
    nc = len(s2.cubes)
    i = p[1]
    recs = (s2.cubes if i < nc else s2.spheres).copy()
    j = i if i < nc else i - nc
    m0 = float(recs["Mass"][j])
    recs["Mass"][j] = np.float32(m0 + h)
    recs["MOI"][j] = np.float32(float(recs["MOI"][j]) * float(recs["Mass"][j]) / m0)
    if i < nc:
        s2.cubes = recs
    else:
        s2.spheres = recs
    return s2, float(recs["Mass"][j])


def params(sc):
    return [("V", c) for c in range(3)] + [("cr",)] + [("m", i) for i in range(sc.n_bodies)]


def fd(sc, target, nsteps, held=None, h=H, threads=16):
    """Central differences of the loss for every parameter (order of params()), and for each
    parameter whether both perturbed runs ended their steps with the unperturbed run's contact
    lists (same pairs in the same order). held = the recorded steps (diff_replay.record_contacts)
    to hold the contacts to, or None for the oracle's full step."""
    from oracle.portbind import OracleWorld
    runs, xs = [], []
    for p in params(sc):
        for sgn in (1, -1):
            s2, x = perturbed(sc, p, sgn * h)
            runs.append(s2)
            xs.append(x)
    o = OracleWorld(runs, fp64=True)
    if held is not None:
        for i in range(len(runs)):
            o.hold_contacts(i, held)
    same = np.ones(len(runs), bool)
    ref = None
    if held is None:
        r = OracleWorld([sc], fp64=True)
        ref = []
        for _ in range(nsteps):
            r.step(DT, 1)
            ref.append(_pair_key(r.pairs(0)))
        for k in range(nsteps):
            o.step(DT, 1, threads)
            for i in range(len(runs)):
                same[i] &= _pair_key(o.pairs(i)) == ref[k]
    else:
        o.step(DT, nsteps, threads)
    loss = np.array([((o.state_f64(i)[-1, 0:3] - target) ** 2).sum() for i in range(len(runs))])
    g = (loss[0::2] - loss[1::2]) / (np.array(xs[0::2]) - np.array(xs[1::2]))
    return g, same[0::2] & same[1::2]


def _pair_key(p):
    return np.ascontiguousarray(p[["Type", "IndexA", "IndexB"]]).tobytes()


def loss_weights(world_or_positions, scenes_list, targets):
    """dL/d(final position) in record order (cubes of all scenes, then spheres): 2 (P - target)
    on each scene's sphere, zero elsewhere."""
    P = np.asarray(world_or_positions, np.float64)
    g = np.zeros_like(P)
    nc = sum(len(s.cubes) for s in scenes_list)
    for k in range(len(scenes_list)):
        g[nc + k] = 2.0 * (P[nc + k] - targets[k])
    return g.astype(np.float32)


def gpu_gradients(nl, scenes_list, targets, nsteps):
    """The GPU adjoint's gradients of every scene's loss, per scene in params() order."""
    w = nl.World()
    w.upload_batch(scenes_list)
    w.diff_forward(DT, nsteps)
    cubes, spheres, _ = w.download()
    P = np.concatenate([cubes["Position"], spheres["Position"]])
    g = w.diff_backward(dl_position=loss_weights(P, scenes_list, targets))
    w.close()
    nc = sum(len(s.cubes) for s in scenes_list)
    out = []
    co = 0
    for k, s in enumerate(scenes_list):
        n = len(s.cubes)
        masses = np.concatenate([g["mass"][co:co + n], g["mass"][nc + k:nc + k + 1]])
        out.append(np.concatenate([g["velocity0"][nc + k], [g["restitution"][k]], masses]).astype(np.float64))
        co += n
    return out
