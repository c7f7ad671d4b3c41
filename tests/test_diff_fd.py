"""The contact adjoint on the differentiated configuration (4x4x2 box stacks plus a 20 m/s sphere;
loss = squared distance of the sphere's final position to a seeded target) against central finite
differences (h = 1e-3) of the FP64 oracle, for the sphere's initial velocity (3), all 33 masses and
the restitution.

The adjoint differentiates the rollout with each step's contact set and contact geometry (normal,
contact points, depth) held at their forward values. Two checks follow from that:

  * one step of the oracle's full step: a step's contacts are found from the positions and angles
    at its start, which none of the parameters move, so over one step the held-contact model IS
    the step and the adjoint must equal the full step's finite differences. Checked from the state
    before the sphere's first impact on the stack, five steps into the impact, and at steps 60 and
    119, on eight scenes;
  * the whole 120-step rollout of the FP64 oracle with the contacts held (the oracle replays the
    FP32 run's contact lists and geometry): the adjoint must equal its finite differences.

Beyond one step the full step's derivative also carries the contacts' dependence on the moving
bodies (the Baumgarte depth term, -0.3/dt * depth, code/nans.cpp:1152, moves with the positions),
which the held-contact model leaves out by construction; oracle/fd_horizon.py reports that gap.
"""
import numpy as np
import pytest

from fd_c3 import DT, H, c3_scenes, first_impact, state_scene, fd, gpu_gradients, params

GRAD_RTOL = 1e-3


def _record(sc, n):
    from diff_replay import record_contacts
    return record_contacts(sc, n, DT)


# ---- CPU: the held-contact oracle ------------------------------------------------------

def test_held_contacts_reproduce_the_fp32_run(oracle_lib):
    """Holding a run's own contacts changes nothing: the FP32 oracle with the recorded contact
    lists and geometry replays the run bit for bit."""
    from oracle.portbind import OracleWorld
    (sc,), _, _ = c3_scenes(1)
    steps = _record(sc, 40)
    a = OracleWorld([sc])
    a.step(DT, 40)
    b = OracleWorld([sc])
    b.hold_contacts(0, steps)
    b.step(DT, 40)
    for x, y in zip(a.state(0)[:2], b.state(0)[:2]):
        for f in ("Position", "V", "Angles", "W"):
            assert x[f].tobytes() == y[f].tobytes(), f


def test_held_contacts_fp64_match_the_torch_replay(oracle_lib):
    """Two independent restatements of the held-contact model agree: the FP64 oracle with held
    contacts and the FP64 torch replay (tests/diff_replay.py) end in the same state."""
    from diff_replay import replay, _v
    from oracle.portbind import OracleWorld
    (sc,), _, _ = c3_scenes(1)
    steps = _record(sc, 60)
    o = OracleWorld([sc], fp64=True)
    o.hold_contacts(0, steps)
    o.step(DT, 60)
    st = o.state_f64(0)
    cat = lambda f: _v(np.concatenate([sc.cubes[f], sc.spheres[f]]))
    P, A, V, W = replay(sc, steps, float(DT), cat("Position"), cat("Angles"), cat("V"), cat("W"), cat("Mass"),
                        float(np.float32(sc.constants.cr)), float(np.float32(sc.constants.cf)))
    assert np.allclose(st[:, 0:3], P.numpy(), rtol=1e-11, atol=1e-11)
    assert np.allclose(st[:, 3:6], V.numpy(), rtol=1e-11, atol=1e-11)


def test_one_step_held_model_is_the_full_step(oracle_lib):
    """Over one step the finite differences of the full FP64 step and of the held-contact step
    agree (and every perturbed run keeps the contact list): the model is exact there."""
    (sc0,), targets, _ = c3_scenes(1)
    k = first_impact(sc0)
    assert k is not None
    sc = state_scene(sc0, k - 1)
    g_full, same = fd(sc, targets[0], 1)
    g_held, _ = fd(sc, targets[0], 1, held=_record(sc, 1))
    assert same.all()
    scale = np.abs(g_full).max()
    assert np.abs(g_full - g_held).max() <= 1e-6 * scale
    assert abs(g_full[3]) > 1e-3 * scale  # restitution moves the sphere at its impact


# ---- GPU ---------------------------------------------------------------------------------

@pytest.fixture(scope="module")
def nl():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from nans_projekat_gb300 import lib
    lib.load()
    return lib


def _check(got, ref, what):
    """Per group (velocity, restitution, masses): |g - fd| <= 1e-3 * max|fd| of the group."""
    errs = {}
    for name, sl in (("velocity", slice(0, 3)), ("restitution", slice(3, 4)), ("mass", slice(4, None))):
        scale = max(np.abs(ref[sl]).max(), 1e-12)
        err = np.abs(got[sl] - ref[sl]).max() / scale
        errs[name] = err
        assert err <= GRAD_RTOL, "%s %s: relative error %.3g (scale %.3g)" % (what, name, err, scale)
    return errs


@pytest.mark.gpu
def test_c3_adjoint_one_step_matches_fd_of_fp64_step(nl, oracle_lib):
    scs, targets, idx = c3_scenes(8)
    checked_cr = 0
    for j, sc0 in enumerate(scs):
        k = first_impact(sc0)
        assert k is not None, "scene %d: the sphere never reaches the stack" % idx[j]
        for start in (k - 1, k + 4, 60, 119):
            sc = state_scene(sc0, start)
            ref, same = fd(sc, targets[j], 1)
            assert same.all(), "scene %d step %d: a perturbed run changed the contact list" % (idx[j], start)
            got = gpu_gradients(nl, [sc], targets[j:j + 1], 1)[0]
            _check(got, ref, "scene %d from step %d" % (idx[j], start))
            checked_cr += abs(ref[3]) > 1e-3 * np.abs(ref).max()
    assert checked_cr >= 8  # the restitution gradient is nonzero (and matched) in many of the states


@pytest.mark.gpu
def test_c3_adjoint_full_rollout_matches_fd_of_fp64_held_step(nl, oracle_lib):
    """120 steps (the configuration's horizon) from the initial state. A parameter whose central
    difference changes between h and h/4 by more than 1e-4 of its group's scale has a clamp of
    the solver switching inside [-h, h]; such parameters are counted, not compared, and must be
    few."""
    scs, targets, idx = c3_scenes(8)
    n = 120
    got = gpu_gradients(nl, scs, targets, n)
    kinks = total = 0
    for j, sc in enumerate(scs):
        held = _record(sc, n)
        ref, _ = fd(sc, targets[j], n, held=held)
        ref4, _ = fd(sc, targets[j], n, held=held, h=H / 4)
        smooth = np.ones(len(ref), bool)
        for sl in (slice(0, 3), slice(3, 4), slice(4, None)):
            scale = max(np.abs(ref4[sl]).max(), 1e-12)
            smooth[sl] = np.abs(ref[sl] - ref4[sl]) <= 1e-4 * scale
        kinks += int((~smooth).sum())
        total += len(ref)
        g = got[j]
        for name, sl in (("velocity", slice(0, 3)), ("restitution", slice(3, 4)), ("mass", slice(4, None))):
            scale = max(np.abs(ref4[sl]).max(), 1e-12)
            m = smooth[sl]
            err = np.abs(g[sl][m] - ref[sl][m]).max() / scale if m.any() else 0.0
            assert err <= GRAD_RTOL, "scene %d %s: relative error %.3g" % (idx[j], name, err)
        assert abs(ref[3]) > 0.0
    assert kinks <= total // 10, "%d of %d parameters at a clamp switch" % (kinks, total)
    assert len(params(scs[0])) == 37
