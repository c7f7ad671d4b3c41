"""Report: how far the held-contact model (the one the GPU adjoint differentiates) is from the full
FP64 step, by horizon, on the differentiated configuration.

For each of the eight scenes of tests/fd_c3.py, from the state one step before the sphere's first
impact on the stack, and for horizons T = 1, 2, 3, 5, 10, 20 steps: the central differences
(h = 1e-3) of the full FP64 oracle step and of the FP64 step with the contacts held, per parameter
group (the sphere's initial velocity, the restitution, the 33 masses), as the relative gap
max |FD_full - FD_held| / max |FD_full|, and the share of perturbed runs that kept the unperturbed
run's contact lists at every step. The GPU adjoint equals FD_held (tests/test_diff_fd.py), so the
gap is the adjoint's model error against the full step.

Usage:  python tests/fd_horizon.py        (CPU only, about a minute)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, HERE)

from fd_c3 import DT, c3_scenes, first_impact, state_scene, fd  # noqa: E402
from diff_replay import record_contacts  # noqa: E402

HORIZONS = (1, 2, 3, 5, 10, 20)
GROUPS = (("velocity", slice(0, 3)), ("restitution", slice(3, 4)), ("mass", slice(4, None)))


def main():
    scs, targets, idx = c3_scenes(8)
    rows = {T: {g: [] for g, _ in GROUPS} for T in HORIZONS}
    kept = {T: [] for T in HORIZONS}
    for j, sc0 in enumerate(scs):
        k = first_impact(sc0)
        sc = state_scene(sc0, k - 1)
        for T in HORIZONS:
            full, same = fd(sc, targets[j], T)
            held, _ = fd(sc, targets[j], T, held=record_contacts(sc, T, DT))
            for g, sl in GROUPS:
                rows[T][g].append(np.abs(full[sl] - held[sl]).max() / max(np.abs(full[sl]).max(), 1e-30))
            kept[T].append(same.mean())
        print("scene %d (impact at step %d) done" % (idx[j], k), flush=True)
    print("| horizon (steps from the step before impact) | velocity gap (median / max) | restitution gap | "
          "mass gap | perturbed runs that kept every contact list |")
    print("|---|---|---|---|---|")
    for T in HORIZONS:
        cells = ["%.1e / %.1e" % (np.median(rows[T][g]), np.max(rows[T][g])) for g, _ in GROUPS]
        print("| %d | %s | %s | %s | %.0f %% |" % (T, cells[0], cells[1], cells[2], 100 * np.mean(kept[T])))


if __name__ == "__main__":
    main()
