"""Differentiable rollout: nans_diff_forward / nans_diff_backward and the torch harness.

CPU tests check the two references the GPU gradients are compared with: the FP64 replay of a
rollout with fixed contacts (tests/diff_replay.py) against the oracle's trajectory, and the
closed forms the adjoint is built on (the accumulate/clamp loop and RK4) against the loop and
the oracle. GPU tests compare the adjoint, called through the C ABI, with the replay's autograd
gradients (contact scenes), with central finite differences of the FP64 oracle (free flight,
where the fixed-contact model is the full model), and check that the taped forward is the
plain step bit for bit."""
import numpy as np
import pytest

from helpers import canon
from nans_projekat_gb300 import scenes

DT = np.float32(1.0 / 60.0)

# Gradient tolerance: |g_gpu - g_ref| <= GRAD_RTOL * max|g_ref| per array (FP32 adjoint
# against an FP64 reference).
GRAD_RTOL = 1e-3


def _weights(n, seed):
    rng = np.random.default_rng(seed)
    return [rng.normal(size=(n, 3)) for _ in range(4)]


def _free_flight_scene():
    """A box and a sphere well above the ground for the whole rollout (no contacts)."""
    sc = scenes.stack_scene(0)
    sc.cubes = sc.cubes[:1].copy()
    sc.cubes["Position"] = (0.3, 30.0, -0.2)
    sc.cubes["V"] = (1.0, 2.0, -0.5)
    sc.cubes["W"] = (0.3, -0.7, 1.1)
    sc.cubes["Mass"] = 1.5
    sc.cubes["MOI"] = np.float32(1.5 / 12.0 * 2.0)
    sc.spheres = sc.spheres.copy()
    sc.spheres["Position"] = (-4.0, 25.0, 1.0)
    sc.spheres["V"] = (3.0, 1.0, 0.5)
    sc.spheres["W"] = (-0.4, 0.2, 0.9)
    sc.name = "free_flight"
    return sc


# ---- CPU: the references ---------------------------------------------------------------

def test_replay_follows_oracle_trajectory(oracle_lib):
    """The FP64 replay with the oracle's contacts reproduces the oracle's FP32 trajectory to
    FP32 rounding, so it restates the step the GPU runs."""
    from diff_replay import record_contacts, replay, _v
    from oracle.portbind import OracleWorld
    sc = scenes.stack_scene(0)
    steps = record_contacts(sc, 25, DT)
    assert sum(len(s[2]) for s in steps) > 100
    cat = lambda f: _v(np.concatenate([sc.cubes[f], sc.spheres[f]]))
    P, A, V, W = replay(sc, steps, float(DT), cat("Position"), cat("Angles"), cat("V"), cat("W"), cat("Mass"),
                        float(np.float32(sc.constants.cr)), float(np.float32(sc.constants.cf)))
    o = OracleWorld([sc])
    o.step(DT, 25)
    c, s, _ = o.state(0)
    ref = lambda f: np.concatenate([c[f], s[f]]).astype(np.float64)
    for got, f in ((P, "Position"), (V, "V"), (A, "Angles"), (W, "W")):
        scale = max(1.0, np.abs(ref(f)).max())
        assert np.abs(got.numpy() - ref(f)).max() <= 1e-5 * scale, f


def test_solver_loop_closed_form():
    """The reference's accumulate/clamp loop on constants (code/nans.cpp:1176-1227) applies
    dn = max(Ln, 0) and dt = clamp(Lt, -mu Ln, mu Ln) with mu = sqrt(2) Cf: the closed form the
    adjoint differentiates (FP64, random constants, 1 to 70 iterations)."""
    rng = np.random.default_rng(1)
    for _ in range(2000):
        ln, lt1, lt2 = rng.normal(size=3) * 10.0 ** rng.uniform(-3, 2)
        cf = rng.uniform(0.0, 1.0)
        iters = int(rng.integers(1, 71))
        sn = st1 = st2 = 0.0
        for _ in range(iters):
            old = sn
            sn = max(sn + ln, 0.0)
            dn = sn - old
            b = np.sqrt(2.0) * cf * sn
            old = st1
            st1 = min(max(st1 + lt1, -b), b)
            dt1 = st1 - old
            old = st2
            st2 = min(max(st2 + lt2, -b), b)
            dt2 = st2 - old
        mu = np.sqrt(2.0) * cf
        bn = mu * max(ln, 0.0)
        tol = 1e-12 * iters * (abs(ln) + abs(lt1) + abs(lt2) + 1.0)
        assert abs(dn - max(ln, 0.0)) <= tol
        assert abs(dt1 - min(max(lt1, -bn), bn)) <= tol
        assert abs(dt2 - min(max(lt2, -bn), bn)) <= tol


def test_rk4_closed_form_matches_oracle(oracle_lib):
    """RK4 on dv/dt = g - (1.5/m) v is V+ = P(z) V + h Q(z) g with z = -1.5 h/m (and
    W+ = P(zw) W): the FP64 oracle's free flight follows the polynomials."""
    from oracle.portbind import OracleWorld
    sc = _free_flight_scene()
    n = 30
    o = OracleWorld([sc], fp64=True)
    o.step(DT, n)
    st = o.state_f64(0)
    h = float(DT)
    g = np.array([0.0, -9.81, 0.0])
    for i, rec in enumerate([sc.cubes[0], sc.spheres[0]]):
        z = -1.5 * h / float(rec["Mass"])
        zw = -1.5 * h / float(rec["MOI"])
        P = lambda x: 1 + x + x * x / 2 + x ** 3 / 6 + x ** 4 / 24
        Q = lambda x: 1 + x / 2 + x * x / 6 + x ** 3 / 24
        v = rec["V"].astype(np.float64)
        w = rec["W"].astype(np.float64)
        p = rec["Position"].astype(np.float64)
        for _ in range(n):
            v = P(z) * v + h * Q(z) * g
            w = P(zw) * w
            p = p + h * v
        assert np.allclose(st[i, 0:3], p, rtol=1e-12, atol=1e-10)
        assert np.allclose(st[i, 3:6], v, rtol=1e-12, atol=1e-12)
        assert np.allclose(st[i, 9:12], w, rtol=1e-12, atol=1e-12)


# ---- GPU ---------------------------------------------------------------------------------

@pytest.fixture(scope="module")
def nl():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    from nans_projekat_gb300 import lib
    lib.load()
    return lib


def _close(got, ref, what):
    ref = np.asarray(ref, np.float64)
    got = np.asarray(got, np.float64)
    scale = max(np.abs(ref).max(), 1e-30)
    err = np.abs(got - ref).max()
    assert err <= GRAD_RTOL * scale, "%s: max error %.3g vs scale %.3g" % (what, err, scale)


@pytest.mark.gpu
def test_taped_forward_is_the_plain_step(nl):
    sc = scenes.stack_scene_random(scenes.SplitMix64(11), 40)
    a = nl.World()
    a.upload(sc)
    a.step(DT, 60)
    b = nl.World()
    b.upload(sc)
    b.diff_forward(DT, 60)
    ca, sa, _ = a.download()
    cb, sb, _ = b.download()
    for f in ("Position", "V", "Angles", "W"):
        assert canon(ca[f]) == canon(cb[f]), f
        assert canon(sa[f]) == canon(sb[f]), f
    steps, nbytes = b.diff_tape_info()
    assert steps == 60 and nbytes > 60 * 32 * sc.n_bodies
    a.close()
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case,nsteps", [("stack8", 40), ("stack_random_12", 60), ("stack_random_40", 30),
                                         ("grid33", 20)])
def test_adjoint_matches_fixed_contact_replay(nl, oracle_lib, case, nsteps):
    from diff_replay import record_contacts, replay_gradients
    if case == "stack8":
        sc = scenes.stack_scene(0)
    elif case == "grid33":
        sc = scenes.grid_stack_batch(1, seed=3)[0]
    else:
        sc = scenes.stack_scene_random(scenes.SplitMix64(int(case.rsplit("_", 1)[1])), int(case.rsplit("_", 1)[1]))
    steps = record_contacts(sc, nsteps, DT)
    assert sum(len(s[2]) for s in steps) > 0
    wts = _weights(sc.n_bodies, 7)
    ref, _ = replay_gradients(sc, steps, float(DT), wts)
    w = nl.World()
    w.upload(sc)
    w.diff_forward(DT, nsteps)
    got = w.diff_backward(*[x.astype(np.float32) for x in wts])
    for k in ("position0", "angles0", "velocity0", "omega0", "mass", "restitution", "friction"):
        _close(got[k], ref[k], "%s %s" % (case, k))
    again = w.diff_backward(*[x.astype(np.float32) for x in wts])
    assert all(np.array_equal(got[k], again[k]) for k in got)
    w.close()


@pytest.mark.gpu
def test_adjoint_matches_oracle_fd_in_free_flight(nl, oracle_lib):
    """Without contacts the fixed-contact model is the whole step: the adjoint must match
    central differences (h = 1e-3) of the FP64 oracle for V0, W0 and the masses."""
    from oracle.portbind import OracleWorld
    sc = _free_flight_scene()
    n = 30
    wts = _weights(sc.n_bodies, 3)

    def loss(s):
        o = OracleWorld([s], fp64=True)
        o.step(DT, n)
        st = o.state_f64(0)
        return sum((wt * st[:, 3 * q:3 * q + 3]).sum() for q, wt in enumerate((wts[0], wts[2], wts[1], wts[3])))

    w = nl.World()
    w.upload(sc)
    w.diff_forward(DT, n)
    got = w.diff_backward(*[x.astype(np.float32) for x in wts])
    recs = [("cubes", 0), ("spheres", 0)]
    fd_v, fd_w, fd_m = np.zeros((2, 3)), np.zeros((2, 3)), np.zeros(2)
    for b, (kind, i) in enumerate(recs):
        for field, out in (("V", fd_v), ("W", fd_w)):
            for c in range(3):
                vals = []
                for sgn in (1, -1):
                    s2 = _free_flight_scene()
                    getattr(s2, kind)[field][i, c] += np.float32(sgn * 1e-3)
                    vals.append((loss(s2), float(getattr(s2, kind)[field][i, c])))
                out[b, c] = (vals[0][0] - vals[1][0]) / (vals[0][1] - vals[1][1])
        vals = []
        for sgn in (1, -1):
            s2 = _free_flight_scene()
            r = getattr(s2, kind)
            m0 = float(r["Mass"][i])
            r["Mass"][i] = np.float32(m0 + sgn * 1e-3)
            r["MOI"][i] = np.float32(float(r["MOI"][i]) * float(r["Mass"][i]) / m0)
            vals.append((loss(s2), float(r["Mass"][i])))
        fd_m[b] = (vals[0][0] - vals[1][0]) / (vals[0][1] - vals[1][1])
    _close(got["velocity0"], fd_v, "velocity0")
    _close(got["omega0"], fd_w, "omega0")
    _close(got["mass"], fd_m, "mass")
    _close(got["position0"], wts[0], "position0")
    _close(got["angles0"], wts[1], "angles0")
    w.close()


@pytest.mark.gpu
def test_backward_needs_a_current_tape(nl):
    sc = scenes.stack_scene(0)
    w = nl.World()
    w.upload(sc)
    with pytest.raises(nl.NansError) as e:
        w.diff_backward(np.ones((sc.n_bodies, 3), np.float32))
    assert e.value.code == 8
    w.diff_forward(DT, 5)
    w.diff_backward(np.ones((sc.n_bodies, 3), np.float32))
    w.step(DT, 1)
    with pytest.raises(nl.NansError) as e:
        w.diff_backward(np.ones((sc.n_bodies, 3), np.float32))
    assert e.value.code == 8
    w.close()


@pytest.mark.gpu
def test_torch_rollout_gradients_and_fit(nl):
    """The autograd harness returns the C ABI's gradients, and gradient descent on a sphere's
    initial velocity through it moves the sphere's final position to a target (free flight)."""
    import torch
    from nans_projekat_gb300 import diff
    sc = _free_flight_scene()
    w = nl.World()
    P0, A0, V0, W0, m, cr, cf = diff.initial_state([sc])
    V0.requires_grad_(True)
    m.requires_grad_(True)
    target = torch.tensor([0.0, 20.0, 0.0])
    losses = []
    for it in range(40):
        P, A, V, W = diff.rollout(w, [sc], DT, 30, P0, A0, V0, W0, m, cr, cf)
        loss = ((P[1] - target) ** 2).sum()
        losses.append(float(loss.detach()))
        gV, gm = torch.autograd.grad(loss, [V0, m])
        if it == 0:
            ref = w.diff_backward(dl_position=(2.0 * (P.detach() - target) * torch.tensor([[0.0], [1.0]])).numpy())
            assert np.allclose(gV.numpy(), ref["velocity0"]) and np.allclose(gm.numpy(), ref["mass"])
        with torch.no_grad():
            V0 -= 0.5 * gV
    assert losses[-1] < 1e-3 * losses[0]
    w.close()
