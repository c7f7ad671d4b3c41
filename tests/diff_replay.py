"""FP64 replay of a rollout with its contacts held fixed, differentiated by torch autograd.

This is the model the GPU adjoint differentiates, restated independently: each step runs
RK4 (code/nans.cpp:50-78), then the reference's sequential-impulse loop (Constraint,
code/nans.cpp:1020-1329) over that step's contact list in list order, with the accumulate /
clamp iterations written out as the reference runs them (not the closed form the adjoint
uses), then P += dt V (code/nans.cpp:1331-1349). Contact lists, contact points and the
positions that define the lever arms come from the oracle's FP32 trajectory, which the GPU step
reproduces bit for bit, and stay fixed while the state and the parameters carry gradients.

Test infrastructure only: it reads the oracle, which only tests use.
"""
import numpy as np
import torch

from nans_projekat_gb300.types import PAIR_DTYPE  # noqa: F401  (pair records come from the oracle)

T_CC, T_CS, T_CF, T_SS, T_SF = 0, 1, 2, 3, 4


def record_contacts(scene, nsteps, dt):
    """Per step k (1-based): (positions of the dynamic bodies and the floor at the step's
    solve, the step's contact list) from the FP32 oracle."""
    from oracle.portbind import OracleWorld
    o = OracleWorld([scene])
    steps = []
    for _ in range(nsteps):
        cubes, spheres, floor = o.state(0)
        pos = np.concatenate([cubes["Position"], spheres["Position"]]).astype(np.float64)
        o.step(np.float32(dt), 1)
        steps.append((pos, np.asarray(floor["Position"][0], np.float64), o.pairs(0).copy()))
    return steps


def _v(x):
    return torch.as_tensor(np.asarray(x, np.float64), dtype=torch.float64)


def _cross(a, b):
    return torch.stack([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]])


def _dot(a, b):
    return (a * b).sum()


def _rk4(y0, f, dt):
    k1 = dt * f(y0)
    k2 = dt * f(y0 + k1 / 2.0)
    k3 = dt * f(y0 + k2 / 2.0)
    k4 = dt * f(y0 + k3)
    return y0 + (((k1 + 2.0 * k2) + 2.0 * k3) + k4) / 6.0


def replay(scene, steps, dt, P0, A0, V0, W0, mass, cr, cf):
    """Final (P, A, V, W) as float64 tensors; inputs are float64 tensors in body order (the
    scene's cubes, then its spheres); mass (n,), cr and cf scalars."""
    nc = len(scene.cubes)
    n = nc + len(scene.spheres)
    moi0 = _v(np.concatenate([scene.cubes["MOI"], scene.spheres["MOI"]]))
    m0 = _v(np.concatenate([scene.cubes["Mass"], scene.spheres["Mass"]]))
    moi = moi0 * mass / m0
    invm = [1.0 / mass[i] for i in range(n)]
    invi = [1.0 / moi[i] for i in range(n)]
    fm = float(scene.floor["Mass"][0])
    fmoi = float(scene.floor["MOI"][0])
    iters = int(scene.constants.iterations)
    grav = _v([0.0, -9.81, 0.0])
    V = [V0[i] for i in range(n)]
    W = [W0[i] for i in range(n)]
    P = [P0[i] for i in range(n)]
    A = [A0[i] for i in range(n)]
    zero = _v([0.0, 0.0, 0.0])
    for pos, floor_pos, pairs in steps:
        for i in range(n):
            V[i] = _rk4(V[i], lambda v, i=i: invm[i] * (mass[i] * grav) - invm[i] * (1.5 * v), dt)
            W[i] = _rk4(W[i], lambda w, i=i: -invi[i] * (1.5 * w), dt)
        for p in pairs:
            t = int(p["Type"])
            a = int(p["IndexA"]) + (nc if t in (T_SS, T_SF) else 0)
            floor = t in (T_CF, T_SF)
            b = None if floor else int(p["IndexB"]) + (nc if t in (T_CS, T_SS) else 0)
            pa = pos[a]
            pb = floor_pos if floor else pos[b]
            nn = np.asarray(p["N"], np.float64)
            if not np.any(nn):
                nn = pb - pa
            nn = nn / np.linalg.norm(nn)
            r1 = np.asarray(p["PointA"], np.float64) - pa
            r2 = np.asarray(p["PointB"], np.float64) - pb
            t1 = np.array([nn[1], -nn[0], 0.0]) if nn[0] >= 0.57735 else np.array([0.0, nn[2], -nn[1]])
            t2 = np.cross(nn, t1)
            depth = np.dot((pa + r1) - (pb + r2), nn)
            N, T1, T2 = _v(nn), _v(t1), _v(t2)
            rn1, rn2 = _v(np.cross(r1, nn)), _v(np.cross(r2, nn))
            r1t1, r2t1 = _v(np.cross(r1, t1)), _v(np.cross(r2, t1))
            r1t2, r2t2 = _v(np.cross(r1, t2)), _v(np.cross(r2, t2))
            im1, ii1 = invm[a], invi[a]
            im2, ii2 = (1.0 / fm, 1.0 / fmoi) if floor else (invm[b], invi[b])
            jn = 1.0 / ((im1 + im2) + (ii1 * _dot(rn1, rn1) - ii2 * _dot(rn2, rn2)))
            jt1 = 1.0 / ((im1 + im2) + (ii1 * _dot(r1t1, r1t1) - ii2 * _dot(r2t1, r2t1)))
            jt2 = 1.0 / ((im1 + im2) + (ii1 * _dot(r1t2, r1t2) - ii2 * _dot(r2t2, r2t2)))
            bias0 = -0.3 / dt * depth
            V1, W1 = V[a], W[a]
            V2, W2 = (zero, zero) if floor else (V[b], W[b])
            jdvn = _dot(((V1 + _cross(W1, N)) - V2) - _cross(W2, N), N)
            jdvt1 = _dot(((V1 + _cross(W1, T1)) - V2) - _cross(W2, T1), T1)
            jdvt2 = _dot(((V1 + _cross(W1, T2)) - V2) - _cross(W2, T2), T2)
            bias = bias0 + cr * jdvn
            sn = st1 = st2 = torch.zeros((), dtype=torch.float64)
            dn = dt1 = dt2 = torch.zeros((), dtype=torch.float64)
            for _ in range(iters):
                old = sn
                sn = torch.clamp(sn + (-jdvn + bias) * jn, min=0.0)
                dn = sn - old
                bound = np.sqrt(2.0) * cf * sn
                old = st1
                st1 = torch.minimum(torch.maximum(st1 + (-jdvt1) * jt1, -bound), bound)
                dt1 = st1 - old
                old = st2
                st2 = torch.minimum(torch.maximum(st2 + (-jdvt2) * jt2, -bound), bound)
                dt2 = st2 - old
            V[a] = V1 + im1 * (dn * N + dt1 * T1 + dt2 * T2)
            W[a] = W1 + ii1 * (dn * rn1 + dt1 * r1t1 + dt2 * r1t2)
            if not floor:
                V[b] = V2 - im2 * (dn * N + dt1 * T1 + dt2 * T2)
                W[b] = W2 - ii2 * (dn * rn2 + dt1 * r2t1 + dt2 * r2t2)
        for i in range(n):
            P[i] = P[i] + dt * V[i]
            A[i] = A[i] + dt * W[i]
    return torch.stack(P), torch.stack(A), torch.stack(V), torch.stack(W)


def replay_gradients(scene, steps, dt, weights):
    """Gradients of L = sum(wP*P_N + wA*A_N + wV*V_N + wW*W_N) of the replay with respect to the
    initial state, masses, Cr and Cf (float64 numpy arrays)."""
    cat = lambda f: np.concatenate([scene.cubes[f], scene.spheres[f]]).astype(np.float64)
    leaves = [_v(cat("Position")), _v(cat("Angles")), _v(cat("V")), _v(cat("W")), _v(cat("Mass")),
              _v(np.float32(scene.constants.cr)), _v(np.float32(scene.constants.cf))]
    for x in leaves:
        x.requires_grad_(True)
    out = replay(scene, steps, dt, *leaves)
    loss = sum((_v(wt) * o).sum() for wt, o in zip(weights, out))
    grads = torch.autograd.grad(loss, leaves, allow_unused=True)
    names = ("position0", "angles0", "velocity0", "omega0", "mass", "restitution", "friction")
    return {k: (np.zeros(tuple(x.shape)) if g is None else g.detach().numpy()) for k, g, x in
            zip(names, grads, leaves)}, [o.detach().numpy() for o in out]
