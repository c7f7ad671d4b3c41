"""Benchmark of the physics step: body-steps/s on one GB300.

Workload (default): 16,384 independent scenes whose body counts are log-uniform in [4, 256]
(seeded stacks of boxes with half-extents U[0.25, 0.75] on a ground box plus one sphere
projectile at U[5, 25] m/s), FP32, dt = 1/60, 10 impulse iterations, restitution 0.2,
friction 0.5; the batched path replays CUDA graphs of min(60, K) steps (captured after the
warm-up steps, so the timed region is graph replays only). A step is one full physics step over
every scene. value = dynamic body-steps / device time of the timed steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank steps its own shard of 16,384 scenes (weak scaling, no
collective on the data path); the timed region is bracketed by barriers and the slowest
rank's time is used.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "body-steps/s"
UNIT = "body-steps/s"
DT = np.float32(1.0 / 60.0)
FUSED_MAX_BODIES = 1024           # NANS_WORLD_FUSED_STEP: bodies per scene, at most
ALG_BYTES_SWEEP_BODY = 68 + 72     # read P,A,V,W,m,I,extents; write P,A,V,W,AABB
ALG_BYTES_SWEEP_BOX_VERTS = 96     # world vertices written for the narrowphase
# per body-step with the world vertices kept in registers: read P,A,V,W,F,T (72 B), m, I (8 B),
# half-extents (12 B); write P,A,V,W (48 B), AABB (24 B)
ALG_BYTES_SWEEP_164 = 92 + 72
ALG_BYTES_NARROW_CAND = 12 + 4 + 2 * (16 + 16) + 2 * 96  # pair, flag, 2 shapes, 2 vertex sets
ALG_BYTES_NARROW_HIT = 36          # contact points and normal


def _jsonable(o):
    if isinstance(o, (np.floating,)):
        return float(o)
    if isinstance(o, (np.integer,)):
        return int(o)
    raise TypeError(type(o).__name__)


def _strict(o):
    """Strict JSON: a non-finite float (never a headline figure) becomes its string form."""
    if isinstance(o, dict):
        return {k: _strict(v) for k, v in o.items()}
    if isinstance(o, (list, tuple)):
        return [_strict(v) for v in o]
    if isinstance(o, (float, np.floating)) and not np.isfinite(o):
        return str(float(o))
    return o


def emit(line):
    print(json.dumps(_strict(line), default=_jsonable, allow_nan=False))


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=600)
    p.add_argument("--warmup", type=int, default=60)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--scenes", type=int, default=16384)
    p.add_argument("--graph-steps", type=int, default=60)
    p.add_argument("--e2e-steps", type=int, default=60)
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-autotune", action="store_true")
    p.add_argument("--no-secondary", action="store_true",
                   help="skip the plain-path and single-large-scene measurements")
    p.add_argument("--fit-full", action="store_true",
                   help="only the gradient fit at full size (4,096 mixed scenes x 240 steps x 50 Adam steps "
                        "fitting per-scene masses) with checkpointed rollouts; prints its own JSON line")
    p.add_argument("--checkpoint-every", type=int, default=20,
                   help="steps per rollout segment for --fit-full")
    p.add_argument("--single", choices=["stack8", "random4608"],
                   help="only the single-scene drop-in line of that scene (nans_step per step, staged and, "
                        "where the scene allows it, fused); prints its own JSON line")
    p.add_argument("--single-steps", type=int, default=600, help="GPU steps of each --single timing")
    return p.parse_args()


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws <= 1:
        return None, 0, 1
    import torch
    import torch.distributed as dist
    backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dist.init_process_group(backend)
    return dist, rank, ws


def max_over_ranks(dist, value, device=None):
    """Maximum of a float over ranks (identity without a process group)."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(dist, value, device=None):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist, device=None):
    if dist is not None:
        if device is not None:
            dist.barrier(device_ids=[device.index])
        else:
            dist.barrier()


def make_workload(n_scenes, rank):
    from nans_projekat_gb300 import scenes
    return scenes.stack_batch(n_scenes, seed=2 + 1000 * rank)


class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, ValueError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_traffic(kernel):
    """DRAM bytes per launch of a kernel from the committed ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f).get(kernel)
    return None


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------------------
# CPU baseline: the oracle's restatement of the reference step (or the reference itself
# compiled headless, where that build is present), all host threads, bounded sample.
# ---------------------------------------------------------------------------------------
def cpu_reference_impl():
    from oracle import refbind
    try:
        if refbind.ref_available("refbig"):
            refbind.lib("refbig")
            return "reference"
    except OSError:
        pass
    return "port"


def cpu_sample_rate(scenes_list, seconds, threads, kind):
    """body-steps/s of the CPU implementation on a bounded sample of scenes."""
    stride = max(1, len(scenes_list) // 512)
    sample = scenes_list[::stride]
    bodies = sum(s.n_bodies for s in sample)
    if kind == "reference":
        from concurrent.futures import ThreadPoolExecutor
        from oracle.refbind import RefWorld
        worlds = [RefWorld(s, "refbig") for s in sample]
        pool = ThreadPoolExecutor(threads)

        def run(n):
            list(pool.map(lambda w: w.step(DT, n), worlds))
    else:
        from oracle.portbind import OracleWorld
        ow = OracleWorld(sample)

        def run(n):
            ow.step(DT, n, threads)
    t0 = time.perf_counter()
    run(1)
    t1 = time.perf_counter() - t0
    n = max(1, min(3000, int(seconds / max(t1, 1e-6))))
    t0 = time.perf_counter()
    run(n)
    t = time.perf_counter() - t0
    return {"value": bodies * n / t, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": "%d of the workload's scenes (every %dth, %d bodies) x %d steps, %.1f s" % (
                len(sample), stride, bodies, n, t)}


def run_reference_arm(args):
    """--impl reference: the CPU implementation of the step, all host threads, each timed
    step a bounded sample of the workload."""
    dist, rank, ws = dist_init()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    kind = cpu_reference_impl()
    batch = make_workload(args.scenes, 0)
    # sample sized so one step takes ~0.1 s
    probe = cpu_sample_rate(batch, 0.5, threads, kind)
    per_step_bodies = max(64, int(probe["value"] * 0.1))
    stride = max(1, int(sum(s.n_bodies for s in batch) / per_step_bodies))
    sample = batch[::stride]
    bodies = sum(s.n_bodies for s in sample)
    if kind == "reference":
        from concurrent.futures import ThreadPoolExecutor
        from oracle.refbind import RefWorld
        worlds = [RefWorld(s, "refbig") for s in sample]
        pool = ThreadPoolExecutor(threads)

        def step():
            list(pool.map(lambda w: w.step(DT, 1), worlds))
    else:
        from oracle.portbind import OracleWorld
        ow = OracleWorld(sample)

        def step():
            ow.step(DT, 1, threads)
    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    t = time.perf_counter() - t0
    value = bodies * args.steps / t
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": "stack_batch%d" % args.scenes, "scenes": args.scenes, "dt": float(DT),
                   "iterations": 10, "sample_scenes_per_step": len(sample), "sample_bodies": bodies},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": "%d scenes (every %dth) per step, %d bodies" % (len(sample), stride, bodies)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    emit(line)


def single_scene_line(lib, device, scene, name, gpu_steps, cpu_steps):
    """One scene on the plain drop-in path: GPU microseconds per step (one nans_step call per
    step, as the reference's frame calls its step; with and without reading the bodies back
    after each step), next to the reference step on one host core: the oracle's restatement
    (-O2), and where the reference compiled from source is present (oracle/_ref), the
    reference itself at -O0 as its build script compiles it and at -O2."""
    import torch
    dt = np.float32(scene.constants.dt)

    def timed(fused):
        w = lib.World(device=device, fused_step=fused)
        w.upload(scene)
        w.step(dt, 2)
        w.download()
        w.step(dt, 1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(gpu_steps):
            w.step(dt, 1)
        t_call = (time.perf_counter() - t0) / gpu_steps
        t0 = time.perf_counter()
        for _ in range(gpu_steps):
            w.step(dt, 1)
            w.download()
        t_frame = (time.perf_counter() - t0) / gpu_steps
        t0 = time.perf_counter()
        w.step(dt, gpu_steps)
        t_batch = (time.perf_counter() - t0) / gpu_steps
        graph_steps, eager_steps = w.path_counts()
        w.close()
        return t_call, t_frame, t_batch, graph_steps, eager_steps

    t_call, t_frame, t_batch, graph_steps, eager_steps = timed(False)
    out = {"workload": name, "bodies": int(scene.n_bodies),
           "gpu_us_per_step": 1e6 * t_call, "gpu_us_per_step_with_download": 1e6 * t_frame,
           "gpu_us_per_step_one_call": 1e6 * t_batch,
           "gpu_path": "nans_step; %d of %d steps replayed from one-step CUDA graphs" % (
               graph_steps, graph_steps + eager_steps)}
    if scene.n_bodies <= FUSED_MAX_BODIES:
        t_call, t_frame, t_batch, _, _ = timed(True)
        out["fused_step"] = {"gpu_us_per_step": 1e6 * t_call, "gpu_us_per_step_with_download": 1e6 * t_frame,
                             "gpu_us_per_step_one_call": 1e6 * t_batch,
                             "gpu_path": "nans_step on a NANS_WORLD_FUSED_STEP world (sweep + one detect-and-"
                                         "solve launch + the large-EPA tiers and late solve, in one-step graphs)"}
    from oracle.portbind import OracleWorld
    o = OracleWorld([scene])
    t0 = time.perf_counter()
    o.step(dt, cpu_steps, 1)
    out["cpu_port_O2_us_per_step"] = 1e6 * (time.perf_counter() - t0) / cpu_steps
    out["cpu_steps"] = cpu_steps
    out["cpu_cores"] = 1
    from oracle import refbind
    for variant, key in (("refbig", "cpu_reference_O0_us_per_step"), ("refbig_O2", "cpu_reference_O2_us_per_step")):
        if refbind.ref_available(variant):
            r = refbind.RefWorld(scene, variant, rebuild=scene.rebuild_models)
            n = max(1, cpu_steps // (4 if variant == "refbig" else 1))
            t0 = time.perf_counter()
            r.step(dt, n)
            out[key] = 1e6 * (time.perf_counter() - t0) / n
    if "cpu_reference_O0_us_per_step" not in out:
        out["cpu_reference"] = "reference build absent on this host (no reference checkout): the port stands in"
    out["speedup_vs_cpu_port"] = out["cpu_port_O2_us_per_step"] / out["gpu_us_per_step"]
    return out


def schedule_ab(lib, batch, device, warm=25, n=10):
    """A/B of schedules on identical windows of the workload (each world steps the same scenes to
    the same state, then the per-stage device time of n eager steps is taken with
    nans_profile_steps): the library's defaults (GJK one thread per candidate pair, cube-cube cull
    by 32 x 32 tiles, six late-scene solver blocks per SM) against GJK with one warp per pair (the
    supports evaluated across the lanes), the cull with one lane per pair, two late-scene solver
    blocks per SM, and three warp-tier EPA blocks per SM. Results are the same in all of them."""
    names = ["sweep", "cull", "gjk_and_thread_epa", "warp_epa", "large_epa", "solve"]
    out = {}
    for key, warp, tiles, late, med in (("default", False, 1, None, None), ("gjk_warp_per_pair", True, 1, None, None),
                                        ("cull_lane_per_pair", False, 0, None, None),
                                        ("late_solve_2_blocks_per_sm", False, 1, 2, None),
                                        ("warp_epa_3_blocks_per_sm", False, 1, None, 3)):
        w = lib.World(device=device, gjk_warp=warp)
        w.upload_batch(batch)
        t = w.tuning()
        w.set_tuning(t["gjk_blocks_per_sm"], t["solve_threads"], t["solve_threads_late"], tiles,
                     late or t["solve_late_blocks_per_sm"], med or t["warp_epa_blocks_per_sm"])
        w.batch_step(DT, warm, 1)
        ms = w.profile(DT, n) / n
        out[key] = {nm: float(x) for nm, x in zip(names, ms)}
        w.close()
    out["window"] = "steps %d-%d of the workload, %d eager steps each" % (warm + 1, warm + n, n)
    return out


def fused_ab(lib, batch, device, warm=5, n=20):
    """The staged step (12 kernels, each over the whole world) against the fused step
    (NANS_WORLD_FUSED_STEP: after the sweep, one launch in which a block per scene culls, collides
    and solves) on identical windows: each world steps the same scenes from the upload (the
    results are the same bit for bit), then n steps from one CUDA graph are timed with CUDA
    events. The whole workload and its scenes binned by size."""
    import torch
    bins = (("all", 0, 10 ** 9), ("4-16 bodies", 0, 16), ("17-64 bodies", 17, 64), ("65-256 bodies", 65, 10 ** 9))
    out = {}
    for name, lo, hi in bins:
        sub = [sc for sc in batch if lo <= sc.n_bodies <= hi]
        if not sub:
            continue
        row = {"scenes": len(sub), "bodies": int(sum(sc.n_bodies for sc in sub))}
        for key, fused in (("staged_ms_per_step", False), ("fused_ms_per_step", True)):
            w = lib.World(device=device, fused_step=fused)
            w.upload_batch(sub)
            w.batch_step(DT, warm, 1)
            w.prepare(DT, n)
            torch.cuda.synchronize()
            st = torch.cuda.ExternalStream(w.stream, device=device)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            w.batch_step(DT, n, n)
            e1.record(st)
            torch.cuda.synchronize()
            row[key] = e0.elapsed_time(e1) / n
            assert w.path_counts()[0] >= n
            w.close()
        row["fused_over_staged"] = row["fused_ms_per_step"] / row["staged_ms_per_step"]
        out[name] = row
    out["window"] = "steps %d-%d after the upload, one %d-step CUDA graph each" % (warm + 1, warm + n, n)
    return out


def secondary_measurements(lib, batch, device):
    """Plain path vs batched path on the same scenes, and the single large scene."""
    import torch
    from nans_projekat_gb300 import scenes
    out = {}
    out["schedule_ab"] = schedule_ab(lib, batch, device)
    out["fused_ab"] = fused_ab(lib, batch, device)
    out["c0_plain"] = single_scene_line(lib, device, scenes.stack_scene(0), "stack8: 8 unit cubes + 1 sphere",
                                        600, 600)
    out["c1_plain"] = single_scene_line(lib, device, scenes.random_scene(1),
                                        "random4608: 4,096 boxes + 512 spheres in a 64^3 m box", 60, 3)
    # plain drop-in: one world per scene, stepped with nans_step (stage-by-stage launches and
    # one synchronisation per call), on every 256th scene of the batched workload
    sample = batch[::256]
    worlds = []
    for sc in sample:
        wd = lib.World(device=device)
        wd.upload(sc)
        wd.step(DT, 2)
        worlds.append(wd)
    n = 20
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for wd in worlds:
        wd.step(DT, n)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    bodies = sum(s.n_bodies for s in sample)
    out["plain_path"] = {"value": bodies * n / t, "unit": UNIT, "scenes": len(sample), "steps": n,
                         "sample": "every 256th scene of the workload, one world per scene, nans_step"}
    for wd in worlds:
        wd.close()
    worlds = []
    for sc in sample:
        wd = lib.World(device=device, fused_step=True)
        wd.upload(sc)
        wd.step(DT, 2)
        worlds.append(wd)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for wd in worlds:
        wd.step(DT, n)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    out["plain_path"]["fused_step_value"] = bodies * n / t
    for wd in worlds:
        wd.close()
    # one large scene: 4,096 boxes + 512 spheres in a 64^3 m box, plain path
    big = scenes.random_scene(1)
    wb = lib.World(device=device)
    wb.upload(big)
    wb.step(DT, 3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n = 60
    wb.step(DT, n)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    out["large_scene_plain"] = {"value": big.n_bodies * n / t, "unit": UNIT, "bodies": big.n_bodies,
                                "steps": n, "ms_per_step": 1000.0 * t / n,
                                "workload": "random4608: 4,096 boxes + 512 spheres, 64^3 m box, plain path"}
    wb.close()
    out["differentiable"] = differentiable_measurement(lib, device)
    try:
        out["fit_mixed"] = fit_measurement(lib, device)
    except Exception as e:  # reported, not fatal: the headline does not depend on it
        out["fit_mixed"] = {"unavailable": str(e)[:200]}
    return out


def fit_measurement(lib, device, n_scenes=1024, nsteps=120, iters=20, checkpoint_every=None):
    """Gradient-based fitting through the differentiable rollout on the mixed workload (1,024
    scenes of 8-128 boxes, spheres and convex hulls, 120 steps, 20 Adam steps): the spheres'
    initial velocities are fitted so that their positions after the rollout match those of a
    rollout from perturbed velocities (N(0, 0.2) m/s); spheres flung beyond 10 km drop out of
    the loss. Gradient norm clipped at 10. (A fit of 4,096 scenes x 240 steps x 50 Adam steps
    keeps a tape of every candidate pair of every step; scenes whose bodies the reference's
    solver flings away turn every pair into a candidate, which makes that tape outgrow the
    GPU; `checkpoint_every` keeps one segment's tape at a time, see --fit-full.)"""
    import torch
    from nans_projekat_gb300 import diff, scenes
    batch = scenes.mixed_batch(n_scenes, seed=4)
    w = lib.World(device=device)
    P0, A0, V0, W0, m, cr, cf = diff.initial_state(batch)
    n_cubes = sum(len(s.cubes) for s in batch)
    rng = np.random.default_rng(0)
    noise = np.zeros(V0.shape, np.float32)
    noise[n_cubes:] = rng.normal(0.0, 0.2, (V0.shape[0] - n_cubes, 3))
    with torch.no_grad():
        target = diff.rollout(w, batch, DT, nsteps, P0, A0, V0 + torch.from_numpy(noise), W0, m, cr, cf,
                              checkpoint_every=checkpoint_every)[0]
    # spheres that the reference's solver flings to huge or non-finite coordinates drop out
    keep = torch.isfinite(target).all(dim=1) & (target.abs() < 1e4).all(dim=1)
    keep[:n_cubes] = False
    V = V0.clone().requires_grad_(True)
    opt = torch.optim.Adam([V], lr=0.05)
    losses = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(iters):
        opt.zero_grad()
        P = diff.rollout(w, batch, DT, nsteps, P0, A0, V, W0, m, cr, cf, checkpoint_every=checkpoint_every)[0]
        ok = keep & torch.isfinite(P).all(dim=1) & (P.abs() < 1e4).all(dim=1)
        loss = ((P[ok] - target[ok]) ** 2).sum() / max(1, int(ok.sum()))
        loss.backward()
        torch.nn.utils.clip_grad_norm_([V], 10.0)
        opt.step()
        losses.append(float(loss.detach()))
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    bodies = int(V0.shape[0])
    w.close()
    out = {"workload": "mixed%d: %d scenes of 8-128 boxes, spheres and convex hulls" % (n_scenes, n_scenes),
           "bodies": bodies,
           "steps": nsteps, "adam_steps": iters, "s_per_adam_step": t / iters,
           "forward_backward_value": bodies * nsteps * iters / t, "unit": UNIT,
           "mean_sq_error_first": losses[0], "mean_sq_error_last": losses[-1], "fitted_spheres": int(keep.sum())}
    if checkpoint_every:
        out["checkpoint_every"] = int(checkpoint_every)
    return out


def mass_fit_measurement(lib, device, n_scenes=4096, nsteps=240, iters=50, checkpoint_every=20):
    """The batched + differentiated configuration: 4,096 mixed scenes (8-128 boxes, spheres and
    convex hulls), 240 steps, then Adam steps fitting one mass scale per scene (every body's
    mass and moment of inertia times exp(theta_s)) so that the final positions match a target
    rollout whose scenes have seeded mass scales exp(U[-0.2, 0.2]). Each Adam step is a forward
    rollout and its adjoint in one batched launch sequence (checkpointed every
    `checkpoint_every` steps, one segment's tape on the GPU at a time). Bodies whose target or
    current position is non-finite or beyond 10 km (bodies the reference's solver flings away)
    are left out of the loss."""
    import torch
    from nans_projekat_gb300 import diff, scenes
    batch = scenes.mixed_batch(n_scenes, seed=4)
    w = lib.World(device=device)
    P0, A0, V0, W0, m0, cr, cf = diff.initial_state(batch)
    scene_of = torch.tensor(np.concatenate([np.full(len(s.cubes), i) for i, s in enumerate(batch)] +
                                           [np.full(len(s.spheres), i) for i, s in enumerate(batch)]), dtype=torch.long)
    rng = np.random.default_rng(44)
    theta_true = torch.tensor(rng.uniform(-0.2, 0.2, n_scenes), dtype=torch.float32)
    with torch.no_grad():
        target = diff.rollout(w, batch, DT, nsteps, P0, A0, V0, W0, m0 * torch.exp(theta_true)[scene_of], cr, cf,
                              checkpoint_every=checkpoint_every)[0]
    keep0 = torch.isfinite(target).all(dim=1) & (target.abs() < 1e4).all(dim=1)
    theta = torch.zeros(n_scenes, requires_grad=True)
    opt = torch.optim.Adam([theta], lr=0.02)
    losses, errs = [], []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(iters):
        opt.zero_grad()
        P = diff.rollout(w, batch, DT, nsteps, P0, A0, V0, W0, m0 * torch.exp(theta)[scene_of], cr, cf,
                         checkpoint_every=checkpoint_every)[0]
        ok = keep0 & torch.isfinite(P).all(dim=1) & (P.abs() < 1e4).all(dim=1)
        loss = ((P[ok] - target[ok]) ** 2).sum() / max(1, int(ok.sum()))
        loss.backward()
        with torch.no_grad():
            theta.grad[~torch.isfinite(theta.grad)] = 0.0
        opt.step()
        losses.append(float(loss.detach()))
        errs.append(float((theta.detach() - theta_true).abs().mean()))
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    bodies = int(V0.shape[0])
    w.close()
    return {"workload": "mixed%d: %d scenes of 8-128 boxes, spheres and convex hulls" % (n_scenes, n_scenes),
            "bodies": bodies, "steps": nsteps, "adam_steps": iters, "checkpoint_every": checkpoint_every,
            "fitted": "one mass scale per scene (4,096 parameters), target scales exp(U[-0.2, 0.2])",
            "s_per_adam_step": t / iters, "forward_backward_value": bodies * nsteps * iters / t, "unit": UNIT,
            "loss_first": losses[0], "loss_last": losses[-1], "loss_min": min(losses),
            "mean_abs_log_scale_error_first": errs[0], "mean_abs_log_scale_error_last": errs[-1],
            "bodies_in_loss": int(keep0.sum()), "losses": losses[::5]}


def differentiable_measurement(lib, device):
    """1,024 scenes of a 4x4x2 box stack plus a sphere, 120 steps: the plain forward, the
    taped forward (nans_diff_forward) and the adjoint (nans_diff_backward, host gradient
    arrays in and out), wall clock around the synchronous calls."""
    import torch
    from nans_projekat_gb300 import scenes
    grid = scenes.grid_stack_batch(1024, seed=3)
    n = 120
    wg = lib.World(device=device)
    wg.upload_batch(grid)
    wg.step(DT, 2)

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return 1e3 * (time.perf_counter() - t0), r

    wg.upload_batch(grid)
    t_plain, _ = timed(lambda: wg.step(DT, n))
    wg.upload_batch(grid)
    t_fwd, _ = timed(lambda: wg.diff_forward(DT, n))
    steps, tape_bytes = wg.diff_tape_info()
    rng = np.random.default_rng(0)
    wts = [rng.normal(size=(wg.n_bodies, 3)).astype(np.float32) for _ in range(4)]
    wg.diff_backward(*wts)
    t_bwd = min(timed(lambda: wg.diff_backward(*wts))[0] for _ in range(3))
    bodies = wg.n_bodies
    wg.close()
    return {"workload": "grid33x1024: 1,024 scenes of a 4x4x2 stack of unit boxes + one 20 m/s sphere",
            "bodies": bodies, "steps": n, "plain_forward_ms": t_plain, "taped_forward_ms": t_fwd,
            "backward_ms": t_bwd, "backward_over_forward": t_bwd / t_fwd,
            "tape_bytes": int(tape_bytes), "tape_steps": int(steps),
            "forward_value": bodies * n / (t_fwd / 1e3), "unit": UNIT}


# worlds of the overlapped end-to-end measurement: four quarter batches took 736-745 M body-steps/s
# against 698 M for two halves, 734 M for three and 692 / 675 M for six / eight
E2E_WORLDS = 4


def e2e_overlapped(lib, batch, device, steps, dist):
    """End to end through the C ABI with the scenes split over E2E_WORLDS worlds (one stream
    each), each driven by its own host thread: every step, each world's state arrays go in from
    pinned host memory (H2D), the world steps once (nans_batch_step with a one-step CUDA graph)
    and its state arrays come back (D2H), so that the worlds' copies overlap the others' steps."""
    import torch

    def pinned(shape, dtype):
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        return torch.empty(max(1, n), dtype=torch.uint8, pin_memory=True).numpy()[:n].view(dtype).reshape(shape)

    worlds, states = [], []
    for idx in np.array_split(np.arange(len(batch)), E2E_WORLDS):
        part = [batch[i] for i in idx]
        wd = lib.World(device=device)
        wd.upload_batch(part)
        wd.batch_step(DT, 2, 1)
        st = tuple(pinned((wd.n_bodies, 3), np.float32) for _ in range(4))
        wd.get_state_arrays(out=st)
        worlds.append(wd)
        states.append(st)

    def loop(wd, st, n):
        for _ in range(n):
            wd.lib.nans_world_set_state_arrays(wd.h, *[a.ctypes.data for a in st])
            wd.batch_step(DT, 1, 1)
            wd.lib.nans_world_get_state_arrays(wd.h, *[a.ctypes.data for a in st])

    for wd, st in zip(worlds, states):  # capture the one-step graphs
        loop(wd, st, 2)
    torch.cuda.synchronize()
    barrier(dist, device)
    threads = [threading.Thread(target=loop, args=(wd, st, steps)) for wd, st in zip(worlds, states)]
    t0 = time.perf_counter()
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    t = max_over_ranks(dist, time.perf_counter() - t0, device)
    bodies = sum(wd.n_bodies for wd in worlds)
    nbytes = sum(a.nbytes for st in states for a in st)
    paths = [wd.path_counts() for wd in worlds]
    for wd in worlds:
        wd.close()
    return t, bodies, nbytes, paths


def run_ours(args):
    import torch
    dist, rank, ws = dist_init()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device")
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    from nans_projekat_gb300 import lib
    from nans_projekat_gb300.types import CUBE_DTYPE, SPHERE_DTYPE

    batch = make_workload(args.scenes, rank)
    w = lib.World(device=local)
    w.upload_batch(batch)
    bodies = w.n_bodies
    if not args.no_autotune:
        w.autotune(DT)
    tuning = w.tuning()
    # one CUDA graph covers gsteps steps; with fewer timed steps than that the graph is cut to the
    # timed step count, so that the timed region always replays graphs
    gsteps = max(1, min(args.graph_steps, args.steps))
    # warm-up: W steps, then the capture of the graph the timed steps replay (no step runs)
    w.batch_step(DT, args.warmup, gsteps)
    w.prepare(DT, gsteps)
    warm_steps = args.warmup
    g0, e0_ = w.path_counts()
    stream = torch.cuda.ExternalStream(w.stream, device=device)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier(dist, device)
    torch.cuda.synchronize()
    e0.record(stream)
    w.batch_step(DT, args.steps, gsteps)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(dist, device)
    clocks = sampler.stop()
    g1, e1_ = w.path_counts()
    timed_graph, timed_eager = g1 - g0, e1_ - e0_
    ms = e0.elapsed_time(e1)
    ms_max = max_over_ranks(dist, ms, device)
    total_bodies = sum_over_ranks(dist, float(bodies), device)
    value = total_bodies * args.steps / (ms_max / 1000.0)
    n_cand, n_contacts = w.counts()
    epa = w.epa_stats()

    # per-stage device time from a live event-timed pass over the same world
    prof_steps = 10
    stage_ms = w.profile(DT, prof_steps) / prof_steps
    # the same steps' stage ends with the production overlap of the two streams (the step's
    # critical path): from the step's start to the end of each stage
    ends = w.timeline(DT, prof_steps)
    end_names = ["sweep", "cull", "gjk_and_thread_epa", "warp_epa (stream 2)", "large_epa (stream 2)",
                 "solve_pass0", "solve_pass1 (step end)"]
    names = ["k_sweep", "k_cull (3 kernels)", "k_narrow_tiny", "k_epa_medium", "k_narrow_big (block + giant tiers)", "k_solve"]
    dom = int(np.argmax(stage_ms))
    peak, peak_kind = measured_peaks()
    n_boxes = int(sum(len(s.cubes) for s in batch))
    sweep_bytes = ALG_BYTES_SWEEP_BODY * bodies + ALG_BYTES_SWEEP_BOX_VERTS * n_boxes
    sweep_bytes_164 = ALG_BYTES_SWEEP_164 * bodies
    narrow_bytes = ALG_BYTES_NARROW_CAND * n_cand + ALG_BYTES_NARROW_HIT * n_contacts
    alg = {0: sweep_bytes_164, 2: narrow_bytes, 3: narrow_bytes, 4: narrow_bytes}
    dom_bytes = alg.get(dom, narrow_bytes)
    achieved = dom_bytes / (stage_ms[dom] / 1000.0) / 1e9
    sweep_gbs = sweep_bytes / (stage_ms[0] / 1000.0) / 1e9
    sweep_gbs_164 = sweep_bytes_164 / (stage_ms[0] / 1000.0) / 1e9

    # end to end through the C ABI with pinned host buffers, every step: the whole dynamic
    # state in (Position, Angles, V, W as float[n][3], H2D), one step, the whole state out (D2H)
    def pinned(shape, dtype):
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        return torch.empty(max(1, n), dtype=torch.uint8, pin_memory=True).numpy()[:n].view(dtype).reshape(shape)

    state = tuple(pinned((bodies, 3), np.float32) for _ in range(4))
    w.get_state_arrays(out=state)
    for _ in range(2):  # capture the one-step graph
        w.lib.nans_world_set_state_arrays(w.h, *[a.ctypes.data for a in state])
        w.batch_step(DT, 1, 1)
        w.lib.nans_world_get_state_arrays(w.h, *[a.ctypes.data for a in state])
    barrier(dist, device)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        w.lib.nans_world_set_state_arrays(w.h, *[a.ctypes.data for a in state])
        w.batch_step(DT, 1, 1)
        w.lib.nans_world_get_state_arrays(w.h, *[a.ctypes.data for a in state])
    te2e_serial = max_over_ranks(dist, time.perf_counter() - t0, device)
    state_bytes = sum(a.nbytes for a in state)
    e2e_serial = {"value": total_bodies * args.e2e_steps / te2e_serial, "unit": UNIT,
                  "h2d_bytes_per_step": int(state_bytes), "d2h_bytes_per_step": int(state_bytes),
                  "path": "one world: nans_world_set_state_arrays + nans_batch_step(1, one-step graph) + "
                          "nans_world_get_state_arrays, pinned host, serial"}

    # the same through the reference's record layouts (cube 244 B, sphere 148 B)
    cubes, spheres, floors = w.download()
    pin_c = pinned((len(cubes),), CUBE_DTYPE)
    pin_s = pinned((len(spheres),), SPHERE_DTYPE)
    pin_c[:] = cubes
    pin_s[:] = spheres
    pin_f = np.zeros(len(floors), CUBE_DTYPE)
    barrier(dist, device)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        w.set_state(pin_c, pin_s, keep_model=True)
        w.batch_step(DT, 1, 1)
        w.lib.nans_world_download(w.h, pin_c.ctypes.data, pin_s.ctypes.data, pin_f.ctypes.data)
    trec = max_over_ranks(dist, time.perf_counter() - t0, device)
    e2e_records = {"value": total_bodies * args.e2e_steps / trec, "unit": UNIT,
                   "h2d_bytes_per_step": int(cubes.nbytes + spheres.nbytes),
                   "d2h_bytes_per_step": int(cubes.nbytes + spheres.nbytes + pin_f.nbytes),
                   "path": "nans_world_set_state + nans_batch_step(1, one-step graph) + nans_world_download "
                           "(records), pinned host"}
    launches_batched, _ = w.launches_per_step()
    w.close()  # the overlapped e2e and the secondary measurements build worlds of their own

    te2e, e2e_bodies, e2e_bytes, e2e_paths = e2e_overlapped(lib, batch, local, args.e2e_steps, dist)
    e2e_value = sum_over_ranks(dist, float(e2e_bodies), device) * args.e2e_steps / te2e

    secondary = None
    if rank == 0 and not args.no_secondary:
        secondary = secondary_measurements(lib, batch, local)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_sample_rate(batch, args.cpu_seconds, os.cpu_count() or 1, cpu_reference_impl())

    if rank == 0:
        path = "batched: %d steps from CUDA graphs of %d steps, %d eager" % (timed_graph, gsteps, timed_eager)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {
                "workload": "stack_batch%d" % args.scenes, "scenes_per_gpu": args.scenes,
                "bodies_per_gpu": bodies, "body_counts": "log-uniform [4, 256]", "dt": float(DT),
                "iterations": 10, "restitution": 0.2, "friction": 0.5, "graph_steps": gsteps,
                "path": path, "timed_graph_steps": timed_graph, "timed_eager_steps": timed_eager,
                "tuning": tuning,
                "warmup_steps_run": warm_steps,
                "l2": "working set larger than L2 (%.0f MB of state, vertices and candidates)"
                      % ((bodies * 64 + n_boxes * 96 + n_cand * 60) / 1e6),
                "candidates_per_step": n_cand, "contacts_per_step": n_contacts,
                "large_epa": {"slow_path_epas": epa["slow_epas"], "max_faces": epa["max_faces"],
                              "max_horizon_edges": epa["max_edges"], "beyond_capacity": epa["overflows"],
                              "warp_tier_epas": epa["warp_tier"], "giant_tier_epas": epa["giant_tier"]},
            },
            "roofline": {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak,
                         "unit": "GB/s", "frac": achieved / peak, "traffic": measured_traffic(names[dom]),
                         "peak_source": peak_kind + " hbm_gbs",
                         "bytes_per_launch": dom_bytes,
                         "stage_ms": {n: float(x) for n, x in zip(names, stage_ms)},
                         "stage_end_ms": {n: float(x) for n, x in zip(end_names, ends)},
                         "sweep": {"basis_164B_per_body": {"achieved": sweep_gbs_164, "frac": sweep_gbs_164 / peak,
                                                           "bytes_per_launch": sweep_bytes_164},
                                   "basis_with_vertices": {"achieved": sweep_gbs, "frac": sweep_gbs / peak,
                                                           "bytes_per_launch": sweep_bytes},
                                   "traffic": measured_traffic("k_sweep")}},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(e2e_bytes),
                    "d2h_bytes_per_step": int(e2e_bytes),
                    "path": "%d worlds of 1/%d of the scenes each, one host thread each: "
                            "nans_world_set_state_arrays + nans_batch_step(1, one-step graph) + "
                            "nans_world_get_state_arrays per step, pinned host, each world's copies "
                            "overlapping the others' steps" % (E2E_WORLDS, E2E_WORLDS),
                    "graph_and_eager_steps_per_world": e2e_paths,
                    "serial": e2e_serial, "records": e2e_records},
            "gpu_launches": int(launches_batched * args.steps),
            "secondary": secondary,
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        emit(line)
    if dist is not None:
        dist.destroy_process_group()


def run_fit_full(args):
    """The differentiable configuration at full size: 4,096 mixed scenes, 240 steps, 50 Adam
    steps, rollouts checkpointed every --checkpoint-every steps (one segment's tape on the GPU at
    a time). Time-consuming; not part of the default run."""
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device")
    torch.cuda.set_device(0)
    from nans_projekat_gb300 import lib
    r = mass_fit_measurement(lib, 0, n_scenes=4096, nsteps=240, iters=50, checkpoint_every=args.checkpoint_every)
    emit({"metric": "body-steps/s (taped forward + adjoint, Adam fit of per-scene masses)",
          "value": r["forward_backward_value"], "unit": UNIT, "n_gpus": 1, "higher_is_better": True, "dtype": "f32",
          "data": "synthetic (seeded)",
          "config": {"workload": r["workload"], "bodies": r["bodies"], "steps": r["steps"],
                     "adam_steps": r["adam_steps"], "checkpoint_every": args.checkpoint_every},
          "fit": r})


def run_single(args):
    """The single-scene drop-in line alone (also a small target for a profiler's launch list)."""
    import torch
    from nans_projekat_gb300 import lib, scenes
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device")
    lib.load()
    if args.single == "stack8":
        sc, name, cpu_steps = scenes.stack_scene(0), "stack8: 8 unit cubes + 1 sphere", 600
    else:
        sc, name, cpu_steps = scenes.random_scene(1), "random4608: 4,096 boxes + 512 spheres in a 64^3 m box", 3
    line = single_scene_line(lib, 0, sc, name, args.single_steps, cpu_steps)
    emit({"metric": "single-scene step latency", "unit": "us/step", "higher_is_better": False,
          "value": line["gpu_us_per_step"], "n_gpus": 1, "data": "synthetic", "config": {"workload": name},
          "single": line})


def main():
    args = parse()
    if args.impl == "reference":
        run_reference_arm(args)
    elif args.fit_full:
        run_fit_full(args)
    elif args.single:
        run_single(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
