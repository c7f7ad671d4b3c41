"""GPU test of nans_solve_contacts_static, the allocation-free solve for callers that must not
allocate GPU memory after start-up (a host that owns all memory, as the reference's platform
layer does, or an engine with a fixed memory pool).

It is called through the C ABI on device buffers the test owns and must give the same
velocities, bit for bit, as the solve inside the existing nans_step entry point, on two
calls in a row (the second call reuses the library's static scratch array), and the second call
must leave the device's free memory unchanged.
This file is named so that pytest collects it last.
"""
import numpy as np
import pytest

from helpers import canon

pytestmark = pytest.mark.gpu

DT = np.float32(1.0 / 60.0)
PRE_STEPS = 29  # the solve compared is the one of step 30, when the stacks are in contact


def _scene_cases():
    from nans_projekat_gb300 import scenes
    return [scenes.stack_scene(0), scenes.stack_scene_random(scenes.SplitMix64(7), 40)]


def _world_reference(lib, sc):
    """Step PRE_STEPS + 1 of the existing entry point: its contacts and solved velocities."""
    w = lib.World()
    w.upload(sc)
    w.step(DT, PRE_STEPS)
    w.step(DT, 1)
    pairs = w.pairs(0)
    cubes, spheres, _ = w.download()
    w.close()
    return pairs, np.concatenate([cubes["V"], spheres["V"]]), np.concatenate([cubes["W"], spheres["W"]])


def _solve_inputs(sc):
    """Body state at solve time: velocities after IntegrateForces, positions before
    IntegrateVelocities (stage 0 of the oracle, which matches the device sweep bit for bit)."""
    from oracle.portbind import OracleWorld
    o = OracleWorld([sc])
    o.step(DT, PRE_STEPS)
    o.stage(0, DT)
    cubes, spheres, _ = o.state(0)
    cat = lambda f: np.ascontiguousarray(np.concatenate([cubes[f], spheres[f]]), np.float32)
    return cat("Position"), cat("V"), cat("W"), cat("Mass"), cat("MOI")


def test_static_solve_matches_world_step(oracle_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required")
    from nans_projekat_gb300 import lib
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    calls = 0
    for sc in _scene_cases():  # two calls in a row
        pairs, v_ref, w_ref = _world_reference(lib, sc)
        assert len(pairs) > 0
        pos, vel, omg, mass, moi = _solve_inputs(sc)
        t_pos = torch.from_numpy(pos).to(dev)
        t_vel = torch.from_numpy(vel).to(dev)
        t_omg = torch.from_numpy(omg).to(dev)
        t_mass = torch.from_numpy(mass).to(dev)
        t_moi = torch.from_numpy(moi).to(dev)
        t_pairs = torch.from_numpy(np.frombuffer(pairs.tobytes(), np.uint8).copy()).to(dev)
        f = sc.floor[0]
        floor = np.concatenate([f["Position"], f["V"], f["W"], [f["Mass"], f["MOI"]]]).astype(np.float32)
        c = sc.constants
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info(dev)[0]
        lib.solve_contacts_static(len(pos), len(sc.cubes), t_pos.data_ptr(), t_mass.data_ptr(), t_moi.data_ptr(),
                                  t_vel.data_ptr(), t_omg.data_ptr(), floor, t_pairs.data_ptr(), len(pairs),
                                  c.cr, c.cf, c.iterations, DT, None)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info(dev)[0]
        calls += 1
        if calls == 2:
            # the first call may load the kernel's module (lazy loading takes device memory once);
            # the second must not change the device's free memory at all
            assert free_after == free_before, (free_before, free_after)
        got_v = t_vel.cpu().numpy()
        got_w = t_omg.cpu().numpy()
        assert canon(got_v) == canon(v_ref.astype(np.float32)), sc.name
        assert canon(got_w) == canon(w_ref.astype(np.float32)), sc.name
    assert calls == 2


def test_static_solve_rejects_same_body_contacts():
    """A cube-cube contact naming one body on both sides is skipped and reported: the sequential
    solve interleaves both sides' updates on that body, which a per-side solve cannot reproduce."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required")
    from nans_projekat_gb300 import lib
    from nans_projekat_gb300.types import PAIR_DTYPE
    dev = torch.device("cuda", 0)
    pos = torch.zeros(6, device=dev)
    vel = torch.ones(6, device=dev)
    omg = torch.zeros(6, device=dev)
    mass = torch.ones(2, device=dev)
    moi = torch.ones(2, device=dev)
    pair = np.zeros(1, PAIR_DTYPE)
    pair["Type"] = 0  # cube-cube
    pair["IndexA"] = 1
    pair["IndexB"] = 1
    pair["N"] = (0.0, 1.0, 0.0)
    t_pair = torch.from_numpy(np.frombuffer(pair.tobytes(), np.uint8).copy()).to(dev)
    floor = np.zeros(11, np.float32)
    floor[9] = floor[10] = 1.0
    with pytest.raises(lib.NansError) as e:
        lib.solve_contacts_static(2, 2, pos.data_ptr(), mass.data_ptr(), moi.data_ptr(), vel.data_ptr(),
                                  omg.data_ptr(), floor, t_pair.data_ptr(), 1, 0.2, 0.5, 10, DT, None)
    assert e.value.code == 1 and "same body" in str(e.value)
    assert torch.equal(vel, torch.ones(6, device=dev))


def test_static_solve_rejects_oversized_requests():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required")
    from nans_projekat_gb300 import lib
    floor = np.zeros(11, np.float32)
    floor[9] = floor[10] = 1.0
    with pytest.raises(lib.NansError) as e:
        lib.solve_contacts_static(16385, 16385, 1, 1, 1, 1, 1, floor, 1, 1, 0.2, 0.5, 10, DT, None)
    assert e.value.code == 1 and "16384" in str(e.value)
    with pytest.raises(lib.NansError) as e:
        lib.solve_contacts_static(10, 10, 1, 1, 1, 1, 1, floor, 1, 16385, 0.2, 0.5, 10, DT, None)
    assert e.value.code == 1 and "16384" in str(e.value)
