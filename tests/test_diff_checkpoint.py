"""Checkpointed differentiable rollouts (nans_projekat_gb300/diff.py, `checkpoint_every`).

CPU: the segment bookkeeping runs against a fake world that keeps the C ABI's contract (FP32
state, a tape per diff_forward, gradients of the last tape's initial state, external forces
applied on the first step after an upload only) with a small nonlinear step, so that a segment
restored from the wrong state or in the wrong order changes the gradients. The fake's own
adjoint is checked against torch autograd of the same step.
GPU: on contact scenes the checkpointed rollout gives the single-tape rollout's final state bit
for bit and its gradients up to the summation order of the per-segment terms."""
import numpy as np
import pytest
import torch

from nans_projekat_gb300 import diff, scenes
from nans_projekat_gb300.types import CUBE_DTYPE, SPHERE_DTYPE

DT = np.float32(1.0 / 60.0)
G = np.array([0.0, 9.81, 0.0])
K_DRAG, K_SPIN, K_POS = 0.3, 0.1, 0.5


def fake_step(P, A, V, W, m, cr, cf, F, kick, dt, xp=np):
    """One step of the fake world's dynamics (float64); `xp` is numpy or torch."""
    u = V + (dt * F / m[:, None] if kick else 0.0)
    V2 = u - dt * K_DRAG / m[:, None] * u * xp.abs(u) - dt * cr[:, None] * xp.asarray(G) - dt * K_POS * xp.sin(P)
    W2 = W * (1.0 - dt * cf[:, None]) - dt * K_SPIN * W * xp.abs(W)
    return P + dt * V2, A + dt * W2, V2, W2


class FakeWorld:
    def __init__(self):
        self.scenes = []
        self.tape = None
        self.uploads = 0

    @property
    def n_bodies(self):
        return len(self.m)

    def upload_batch(self, scs):
        self.scenes = list(scs)
        recs = [s.cubes for s in scs] + [s.spheres for s in scs]
        cat = lambda f: np.concatenate([r[f] for r in recs]).astype(np.float32)
        self.state = [cat("Position"), cat("Angles"), cat("V"), cat("W")]
        self.m = cat("Mass").astype(np.float64)
        self.F = cat("Forces").astype(np.float64)
        self.ncubes = sum(len(s.cubes) for s in scs)
        self.scene_of = np.concatenate([np.full(len(s.cubes), i) for i, s in enumerate(scs)] +
                                       [np.full(len(s.spheres), i) for i, s in enumerate(scs)])
        self.cr = np.array([float(s.constants.cr) for s in scs])
        self.cf = np.array([float(s.constants.cf) for s in scs])
        self.kick = True
        self.tape = None
        self.uploads += 1

    def set_state_arrays(self, P, A, V, W):
        self.state = [np.array(x, np.float32) for x in (P, A, V, W)]
        self.kick = False
        self.tape = None

    def get_state_arrays(self):
        return tuple(x.copy() for x in self.state)

    def _advance(self, dt, tape):
        s64 = [x.astype(np.float64) for x in self.state]
        if tape is not None:
            tape.append((s64, self.kick))
        out = fake_step(*s64, self.m, self.cr[self.scene_of], self.cf[self.scene_of], self.F, self.kick, float(dt))
        self.state = [x.astype(np.float32) for x in out]
        self.kick = False

    def step(self, dt, n):
        self.tape = None
        for _ in range(n):
            self._advance(dt, None)

    def diff_forward(self, dt, n):
        self.tape, self.tape_dt = [], float(dt)
        for _ in range(n):
            self._advance(dt, self.tape)

    def diff_backward(self, gP=None, gA=None, gV=None, gW=None):
        assert self.tape is not None, "no tape"
        z = np.zeros((self.n_bodies, 3))
        gP, gA, gV, gW = [z.copy() if g is None else np.asarray(g, np.float64) for g in (gP, gA, gV, gW)]
        dt, m = self.tape_dt, self.m
        cr, cf = self.cr[self.scene_of], self.cf[self.scene_of]
        g_m = np.zeros(self.n_bodies)
        g_cr = np.zeros(len(self.scenes))
        g_cf = np.zeros(len(self.scenes))
        for (P, A, V, W), kick in reversed(self.tape):
            u = V + (dt * self.F / m[:, None] if kick else 0.0)
            gv2 = gV + dt * gP
            gw2 = gW + dt * gA
            gu = gv2 * (1.0 - 2.0 * dt * K_DRAG / m[:, None] * np.abs(u))
            g_m += (gv2 * dt * K_DRAG / m[:, None] ** 2 * u * np.abs(u)).sum(1)
            if kick:
                g_m += (gu * -dt * self.F / m[:, None] ** 2).sum(1)
            np.add.at(g_cr, self.scene_of, (gv2 * -dt * G).sum(1))
            np.add.at(g_cf, self.scene_of, (gw2 * -dt * W).sum(1))
            gP = gP + gv2 * (-dt * K_POS * np.cos(P))
            gV = gu
            gW = gw2 * ((1.0 - dt * cf[:, None]) - 2.0 * dt * K_SPIN * np.abs(W))
        f32 = lambda x: x.astype(np.float32)
        return dict(position0=f32(gP), angles0=f32(gA), velocity0=f32(gV), omega0=f32(gW), mass=f32(g_m),
                    restitution=f32(g_cr), friction=f32(g_cf))

    def download(self):
        c = np.zeros(self.ncubes, CUBE_DTYPE)
        s = np.zeros(self.n_bodies - self.ncubes, SPHERE_DTYPE)
        for f, x in zip(("Position", "Angles", "V", "W"), self.state):
            c[f] = x[:self.ncubes]
            s[f] = x[self.ncubes:]
        return c, s, None


def _batch():
    batch = scenes.grid_stack_batch(3, seed=5)
    rng = np.random.default_rng(2)
    for s in batch:
        for r in (s.cubes, s.spheres):
            r["Forces"] = rng.normal(size=(len(r), 3)).astype(np.float32)
            r["W"] = rng.normal(size=(len(r), 3)).astype(np.float32)
    return batch


def _grads(world, batch, nsteps, every, wts, params=None):
    P0, A0, V0, W0, m, cr, cf = params if params is not None else diff.initial_state(batch)
    ins = [t.clone().requires_grad_(True) for t in (P0, A0, V0, W0, m, cr, cf)]
    out = diff.rollout(world, batch, DT, nsteps, *ins, checkpoint_every=every)
    loss = sum((torch.from_numpy(w.astype(np.float32)) * o).sum() for w, o in zip(wts, out))
    return [o.detach().numpy() for o in out], [g.numpy() for g in torch.autograd.grad(loss, ins)]


def _assert_close(a, b, rtol, what):
    scale = max(np.abs(b).max(), 1e-30)
    assert np.abs(np.asarray(a, np.float64) - b).max() <= rtol * scale, what


def test_segments():
    assert diff.segments(30, None) == [30] and diff.segments(30, 0) == [30] and diff.segments(30, 40) == [30]
    assert diff.segments(30, 7) == [7, 7, 7, 7, 2] and diff.segments(30, 10) == [10, 10, 10]
    with pytest.raises(ValueError):
        diff.segments(30, -2)


def test_fake_adjoint_matches_autograd():
    batch = _batch()
    w = FakeWorld()
    w.upload_batch(batch)
    n = w.n_bodies
    wts = [np.random.default_rng(q).normal(size=(n, 3)) for q in range(4)]
    init = [torch.tensor(x.astype(np.float64), requires_grad=True) for x in w.get_state_arrays()]
    m = torch.tensor(w.m, requires_grad=True)
    cr = torch.tensor(w.cr, requires_grad=True)
    cf = torch.tensor(w.cf, requires_grad=True)
    sc = torch.tensor(w.scene_of)
    F = torch.tensor(w.F)
    st = init
    for k in range(12):
        st = fake_step(*st, m, cr[sc], cf[sc], F, k == 0, float(DT), xp=torch)
    loss = sum((torch.tensor(wt) * x).sum() for wt, x in zip(wts, st))
    ref = torch.autograd.grad(loss, init + [m, cr, cf])
    w.diff_forward(DT, 12)
    got = w.diff_backward(*wts)
    for key, r in zip(("position0", "angles0", "velocity0", "omega0", "mass", "restitution", "friction"), ref):
        assert np.abs(r.numpy()).max() > 0.0, key
        _assert_close(got[key], r.numpy(), 1e-6, key)


@pytest.mark.parametrize("every", [1, 4, 7, 29])
def test_checkpointed_equals_single_tape_on_the_fake(every):
    batch = _batch()
    nsteps = 30
    wts = [np.random.default_rng(10 + q).normal(size=(sum(s.n_bodies for s in batch), 3)) for q in range(4)]
    a, b = FakeWorld(), FakeWorld()
    for rep in range(2):  # the first rollout uploads (forces on its first step), the second sets the state
        out_a, g_a = _grads(a, batch, nsteps, None, wts)
        out_b, g_b = _grads(b, batch, nsteps, every, wts)
        for x, y in zip(out_a, out_b):
            assert np.array_equal(x, y)
        for k, (x, y) in enumerate(zip(g_b, g_a)):
            _assert_close(x, y, 1e-6, "rep %d input %d" % (rep, k))
    assert a.uploads == 1 and b.uploads == 2  # the checkpointed backward re-uploaded once


def test_checkpointed_backward_restores_the_segment_starts():
    """Dropping the restore of one segment (its re-run continues from the wrong state) changes
    the gradients: the check above is sensitive to the bookkeeping."""
    batch = _batch()
    n = sum(s.n_bodies for s in batch)
    wts = [np.random.default_rng(20 + q).normal(size=(n, 3)) for q in range(4)]
    _, g_ref = _grads(FakeWorld(), batch, 24, None, wts)

    class Forgetful(FakeWorld):
        calls = 0

        def set_state_arrays(self, *a):
            Forgetful.calls += 1
            if Forgetful.calls != 2:
                super().set_state_arrays(*a)

    _, g_bad = _grads(Forgetful(), batch, 24, 6, wts)
    assert any(np.abs(x - y).max() > 1e-3 * max(np.abs(y).max(), 1e-30) for x, y in zip(g_bad, g_ref))


@pytest.fixture(scope="module")
def nl():
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from nans_projekat_gb300 import lib
    lib.load()
    return lib


@pytest.mark.gpu
def test_checkpointed_rollout_on_the_gpu(nl):
    batch = scenes.grid_stack_batch(16, seed=3)
    n = sum(s.n_bodies for s in batch)
    wts = [np.random.default_rng(30 + q).normal(size=(n, 3)) for q in range(4)]
    a, b = nl.World(), nl.World()
    out_a, g_a = _grads(a, batch, 40, None, wts)
    out_b, g_b = _grads(b, batch, 40, 9, wts)
    for x, y in zip(out_a, out_b):
        assert x.tobytes() == y.tobytes()
    # state gradients pass between segments unchanged; the mass and solver-constant terms are
    # summed per segment, in another order than the single tape's accumulation
    for k, (x, y) in enumerate(zip(g_b, g_a)):
        _assert_close(x, y, 1e-4 if k < 4 else 1e-3, "input %d" % k)
    a.close()
    b.close()
