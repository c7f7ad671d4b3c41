"""Test infrastructure: error of the FP32 step (the CUDA library reproduces the FP32 oracle bit
for bit) against an FP64 run of the same method, for every benchmark configuration.

Error of a body = |P32 - P64| / (|P64| + 1 m), over the dynamic bodies; reported as median and
max at several step counts. The step is chaotic (contacts switch on and off), so the error at
long horizons is a property of the method, not of the implementation.

Usage:  python oracle/fp64_error.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from nans_projekat_gb300 import scenes  # noqa: E402
from oracle.portbind import OracleWorld  # noqa: E402

DT = np.float32(1.0 / 60.0)


def errors(scene_list, checkpoints, threads=8):
    w32 = OracleWorld(scene_list)
    w64 = OracleWorld(scene_list, fp64=True)
    out = {}
    done = 0
    for cp in checkpoints:
        w32.step(DT, cp - done, threads)
        w64.step(DT, cp - done, threads)
        done = cp
        e = []
        for i in range(len(scene_list)):
            a = w32.state_f64(i)[:, :3]
            b = w64.state_f64(i)[:, :3]
            with np.errstate(invalid="ignore"):
                e.append(np.linalg.norm(a - b, axis=1) / (np.linalg.norm(b, axis=1) + 1.0))
        e = np.concatenate(e)
        e = e[np.isfinite(e)]
        out[cp] = (float(np.median(e)), float(np.max(e)))
    return out


def table():
    rows = []
    rows.append(("C0 stack8 (8 cubes + sphere)", errors([scenes.stack_scene(0)], [1, 10, 60, 600])))
    rows.append(("C1 random4608 (4,096 boxes + 512 spheres)", errors([scenes.random_scene(1)], [1, 5, 20])))
    rows.append(("C2 stack_batch (64 of 16,384 scenes)",
                 errors(scenes.stack_batch(16384, seed=2)[::256], [1, 10, 60, 600])))
    rows.append(("C3 grid33 (64 of 1,024 scenes)",
                 errors(scenes.grid_stack_batch(1024, seed=3)[::16], [1, 10, 120])))
    rows.append(("C4 mixed (64 of 4,096 scenes)", errors(scenes.mixed_batch(4096, seed=4)[::64], [1, 10, 240])))
    return rows


if __name__ == "__main__":
    for name, e in table():
        print(name)
        for k, (med, mx) in e.items():
            print("  step %4d  median %.3e  max %.3e" % (k, med, mx))
