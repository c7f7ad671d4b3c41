"""Differentiable rollouts on the GPU for PyTorch.

`rollout` runs `nsteps` plain steps of a batch of scenes through nans_diff_forward and returns
the final state as tensors; its backward calls nans_diff_backward, which runs the adjoint of
the whole rollout in one kernel. The gradient is that of the rollout with each step's contact
set and contact geometry held at their forward values (the C header describes the model), so
it is the gradient an optimiser wants for small parameter changes that keep the contacts.

Arrays are in record order: the cubes of all scenes in upload order, then the spheres.
Masses change the moment of inertia in proportion (the shape is fixed). The world holds one
tape: run backward before the next forward on the same world.
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


def _start(world, scenes, position0, angles0, velocity0, omega0, mass, restitution, friction):
    """Puts the initial state into the world: a full upload when the masses or the solver
    constants changed since the last rollout on this world, else the four state arrays only."""
    key = (tuple(id(s) for s in scenes), mass.tobytes(), restitution.tobytes(), friction.tobytes())
    if getattr(world, "_diff_key", None) != key:
        world.upload_batch(with_state(scenes, position0, angles0, velocity0, omega0, mass, restitution, friction))
        world._diff_key = key
    else:
        world.set_state_arrays(position0, angles0, velocity0, omega0)


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, world, scenes, dt, nsteps, position0, angles0, velocity0, omega0, mass, restitution, friction):
        host = lambda t: np.ascontiguousarray(t.detach().to("cpu", torch.float32).numpy())
        _start(world, scenes, host(position0), host(angles0), host(velocity0), host(omega0), host(mass),
               host(restitution), host(friction))
        world.diff_forward(dt, nsteps)
        ctx.world = world
        ctx.device = velocity0.device
        return tuple(torch.from_numpy(a).to(velocity0.device) for a in final_state(world))

    @staticmethod
    def backward(ctx, g_pos, g_ang, g_vel, g_omg):
        host = lambda t: None if t is None else t.detach().to("cpu", torch.float32).contiguous().numpy()
        g = ctx.world.diff_backward(host(g_pos), host(g_ang), host(g_vel), host(g_omg))
        dev = lambda k: torch.from_numpy(g[k]).to(ctx.device)
        return (None, None, None, None, dev("position0"), dev("angles0"), dev("velocity0"), dev("omega0"),
                dev("mass"), dev("restitution"), dev("friction"))


def rollout(world, scenes, dt, nsteps, position0, angles0, velocity0, omega0, mass, restitution, friction):
    """Final (position, angles, velocity, omega) after nsteps steps from the given initial
    state; differentiable with respect to every tensor argument."""
    return _Rollout.apply(world, list(scenes), float(dt), int(nsteps), position0, angles0, velocity0, omega0,
                          mass, restitution, friction)
