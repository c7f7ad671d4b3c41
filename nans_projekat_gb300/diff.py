"""Differentiable rollouts on the GPU for PyTorch.

`rollout` runs `nsteps` plain steps of a batch of scenes through nans_diff_forward and returns
the final state as tensors; its backward calls nans_diff_backward, which runs the adjoint of
the whole rollout in one kernel. The gradient is that of the rollout with each step's contact
set and contact geometry held at their forward values (the C header describes the model), so
it is the gradient an optimiser wants for small parameter changes that keep the contacts.

Arrays are in record order: the cubes of all scenes in upload order, then the spheres.
Masses change the moment of inertia in proportion (the shape is fixed). The world holds one
tape: run backward before the next forward on the same world.

With `checkpoint_every=k` the forward keeps no tape: it runs plain steps and saves the state
(Position, Angles, V, W: 48 bytes per body) at the start of every k-step segment. The backward
then walks the segments last to first; for each it restores the saved state, re-runs the
segment with a tape and runs the adjoint, whose gradients with respect to the segment's
initial state are the incoming gradients of the segment before it. The tape held at any time
is one segment's, so rollouts whose whole tape would not fit in device memory (the tape keeps
every candidate pair of every step) run at the cost of a second forward. Restoring a state
continues the trajectory bit for bit (the Model is rebuilt from Position and Angles at every
step), so the gradients are those of the single-tape backward up to the order in which the
per-segment mass and solver-constant terms are summed. After such a backward the world holds
the state at the end of the first segment.
"""
import copy

import numpy as np
import torch

from .scenes import Constants


def _split(scenes):
    nc = [len(s.cubes) for s in scenes]
    ns = [len(s.spheres) for s in scenes]
    return nc, ns


def _cat(scenes, field):
    return np.concatenate([s.cubes[field] for s in scenes] + [s.spheres[field] for s in scenes])


def initial_state(scenes):
    """(position, angles, velocity, omega, mass, restitution, friction) of the scenes as float32
    tensors in record order."""
    f = lambda a: torch.tensor(np.asarray(a, np.float32))
    return (f(_cat(scenes, "Position")), f(_cat(scenes, "Angles")), f(_cat(scenes, "V")), f(_cat(scenes, "W")),
            f(_cat(scenes, "Mass")), f([s.constants.cr for s in scenes]), f([s.constants.cf for s in scenes]))


def with_state(scenes, position=None, angles=None, velocity=None, omega=None, mass=None, restitution=None,
               friction=None):
    """Copies of the scenes with the given record-order values written into their records."""
    nc, ns = _split(scenes)
    tc = sum(nc)
    out = []
    co = so = 0
    for i, s in enumerate(scenes):
        s2 = copy.copy(s)
        s2.cubes = s.cubes.copy()
        s2.spheres = s.spheres.copy()
        for recs, lo, n in ((s2.cubes, co, nc[i]), (s2.spheres, tc + so, ns[i])):
            sl = slice(lo, lo + n)
            for name, val in (("Position", position), ("Angles", angles), ("V", velocity), ("W", omega)):
                if val is not None:
                    recs[name] = np.asarray(val[sl], np.float32)
            if mass is not None:
                m = np.asarray(mass[sl], np.float64)
                recs["MOI"] = (recs["MOI"].astype(np.float64) * m / recs["Mass"].astype(np.float64)).astype(np.float32)
                recs["Mass"] = m.astype(np.float32)
        c = s.constants
        cr = c.cr if restitution is None else float(restitution[i])
        cf = c.cf if friction is None else float(friction[i])
        s2.constants = Constants(cr=np.float32(cr), cf=np.float32(cf), iterations=c.iterations, dt=c.dt)
        out.append(s2)
        co += nc[i]
        so += ns[i]
    return out


def final_state(world):
    """(position, angles, velocity, omega) after the last step, float32 arrays in record order."""
    cubes, spheres, _ = world.download()
    cat = lambda f: np.concatenate([cubes[f], spheres[f]]).astype(np.float32)
    return cat("Position"), cat("Angles"), cat("V"), cat("W")


def _start(world, scenes, position0, angles0, velocity0, omega0, mass, restitution, friction, upload=None):
    """Puts the initial state into the world: a full upload when the masses or the solver
    constants changed since the last rollout on this world, else the four state arrays only
    (`upload` forces the choice). Returns whether it uploaded: an upload also applies the
    records' external forces on the first step and, for scenes that keep their Model, the
    uploaded Model, which the state arrays do not carry."""
    key = (tuple(id(s) for s in scenes), mass.tobytes(), restitution.tobytes(), friction.tobytes())
    if upload is None:
        upload = getattr(world, "_diff_key", None) != key
    if upload:
        world.upload_batch(with_state(scenes, position0, angles0, velocity0, omega0, mass, restitution, friction))
        world._diff_key = key
    else:
        world.set_state_arrays(position0, angles0, velocity0, omega0)
    return upload


def segments(nsteps, checkpoint_every):
    """Step counts of the rollout's segments: k-step segments and a shorter last one."""
    if not checkpoint_every or checkpoint_every >= nsteps:
        return [nsteps]
    k = int(checkpoint_every)
    if k < 1:
        raise ValueError("checkpoint_every must be a positive number of steps")
    return [k] * (nsteps // k) + ([nsteps % k] if nsteps % k else [])


def _backward_segments(world, dt, restart, grads):
    """Gradients of a checkpointed rollout: each segment, last to first, is restored, re-run
    with a tape and differentiated; its initial-state gradients feed the segment before it and
    its mass and solver-constant gradients are summed."""
    scenes, args, uploaded, starts, segs = restart
    g_state = list(grads)
    total = None
    for k in range(len(segs) - 1, -1, -1):
        if k == 0:
            _start(world, scenes, *args, upload=uploaded)
        else:
            world.set_state_arrays(*starts[k - 1])
        world.diff_forward(dt, segs[k])
        g = world.diff_backward(*g_state)
        g_state = [g["position0"], g["angles0"], g["velocity0"], g["omega0"]]
        if total is None:
            total = {q: g[q].copy() for q in ("mass", "restitution", "friction")}
        else:
            for q in total:
                total[q] += g[q]
    out = dict(position0=g_state[0], angles0=g_state[1], velocity0=g_state[2], omega0=g_state[3])
    out.update(total)
    return out


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, world, scenes, dt, nsteps, checkpoint_every, position0, angles0, velocity0, omega0, mass,
                restitution, friction):
        host = lambda t: np.ascontiguousarray(t.detach().to("cpu", torch.float32).numpy())
        args = tuple(host(t) for t in (position0, angles0, velocity0, omega0, mass, restitution, friction))
        uploaded = _start(world, scenes, *args)
        segs = segments(nsteps, checkpoint_every)
        ctx.restart = None
        if len(segs) == 1:
            world.diff_forward(dt, nsteps)
        else:
            starts = []
            for k, n in enumerate(segs):
                if k:
                    starts.append(world.get_state_arrays())
                world.step(dt, n)
            ctx.restart = (scenes, args, uploaded, starts, segs)
        ctx.world = world
        ctx.dt = dt
        ctx.device = velocity0.device
        return tuple(torch.from_numpy(a).to(velocity0.device) for a in final_state(world))

    @staticmethod
    def backward(ctx, g_pos, g_ang, g_vel, g_omg):
        host = lambda t: None if t is None else t.detach().to("cpu", torch.float32).contiguous().numpy()
        grads = (host(g_pos), host(g_ang), host(g_vel), host(g_omg))
        if ctx.restart is None:
            g = ctx.world.diff_backward(*grads)
        else:
            g = _backward_segments(ctx.world, ctx.dt, ctx.restart, grads)
        dev = lambda k: torch.from_numpy(g[k]).to(ctx.device)
        return (None, None, None, None, None, dev("position0"), dev("angles0"), dev("velocity0"), dev("omega0"),
                dev("mass"), dev("restitution"), dev("friction"))


def rollout(world, scenes, dt, nsteps, position0, angles0, velocity0, omega0, mass, restitution, friction,
            checkpoint_every=None):
    """Final (position, angles, velocity, omega) after nsteps steps from the given initial
    state; differentiable with respect to every tensor argument. `checkpoint_every` = k keeps
    one k-step segment's tape at a time instead of the whole rollout's."""
    return _Rollout.apply(world, list(scenes), float(dt), int(nsteps), checkpoint_every, position0, angles0,
                          velocity0, omega0, mass, restitution, friction)
