"""CPU test of bench.py's multi-rank plumbing with gloo and two ranks: every rank steps its own
scene shard, the timed region uses the slowest rank, totals are summed."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    dist, r, n = bench.dist_init()
    assert (r, n) == (rank, ws)
    bench.barrier(dist)
    slowest = bench.max_over_ranks(dist, float(10 + rank))
    total = bench.sum_over_ranks(dist, float(100 * (rank + 1)))
    shard = bench.make_workload(8, rank)
    q.put((rank, slowest, total, shard[0].cubes["Position"].tobytes()))
    dist.destroy_process_group()


def test_two_rank_gloo_aggregation():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert [r[1] for r in res] == [11.0, 11.0]        # max over ranks
    assert [r[2] for r in res] == [300.0, 300.0]      # sum over ranks
    assert res[0][3] != res[1][3]                     # independent shards per rank


def test_bench_line_is_strict_json(capsys):
    """The bench line never carries NaN or Infinity tokens (a non-finite secondary figure is
    written as a string), and numpy scalars serialise as numbers."""
    import json
    import sys
    import numpy as np
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    bench.emit({"value": np.float32(1.5), "n": np.int64(3),
                "secondary": {"loss": float("inf"), "x": [float("nan"), 2.0]}})
    line = capsys.readouterr().out.strip()
    d = json.loads(line, parse_constant=lambda c: (_ for _ in ()).throw(ValueError(c)))
    assert d["value"] == 1.5 and d["n"] == 3
    assert d["secondary"]["loss"] == "inf" and d["secondary"]["x"][0] == "nan"


def test_traffic_figures_cover_the_reported_kernels():
    """Every kernel name the bench's roofline can report has a measured DRAM figure."""
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    for k in ("k_narrow_tiny", "k_sweep", "k_cull_mask", "k_solve"):
        v = bench.measured_traffic(k)
        assert v is not None and v > 0, k


def test_reference_arm_under_torchrun_prints_one_line():
    """`bench.py --impl reference` launched as two ranks: rank 0 alone times the CPU step and
    prints one JSON line, the other rank exits 0 without work."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    env["CUDA_VISIBLE_DEVICES"] = ""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "2", "--warmup", "1", "--scenes", "512"]
    r = subprocess.run(cmd, cwd=root, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["e2e"]["h2d_bytes_per_step"] == 0
