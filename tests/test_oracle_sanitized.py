"""The oracle restatement under AddressSanitizer and UndefinedBehaviorSanitizer (CPU).

The oracle is the checker of every GPU parity test, so it must itself be free of memory errors
and undefined behaviour on the inputs the tests use, including the reference's own corner
cases: the EPA that empties its face list (the reference then reads a stale face), EPAs that
grow to hundreds of faces, bodies flung to huge or non-finite coordinates, FP64 and warm-started
runs. `make -C oracle port-san` builds the sanitized library; a child process loads it with the
ASan runtime preloaded, steps the golden cases (checking each step's digest against the
reference's) and the known-answer scenes, and any sanitizer report ends it with a non-zero
status.

The same runner also checks the restatement built with -funsigned-char: the GPU machine is an Arm
machine, where plain char is unsigned, and the oracle is the checker there."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SAN_LIB = os.path.join(ROOT, "oracle", "_build", "libnans_oracle_san.so")


def _asan_runtime():
    try:
        path = subprocess.run(["gcc", "-print-file-name=libasan.so"], capture_output=True, text=True,
                              check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return None
    return path if os.path.isabs(path) and os.path.exists(path) else None


def test_oracle_is_clean_under_sanitizers():
    rt = _asan_runtime()
    if rt is None:
        pytest.skip("no AddressSanitizer runtime for this compiler")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port-san"], check=True)
    env = dict(os.environ, LD_PRELOAD=rt, ASAN_OPTIONS="detect_leaks=0:abort_on_error=0:exitcode=23",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1:exitcode=24")
    r = subprocess.run([sys.executable, os.path.abspath(__file__)], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0 and "oracle run ok" in r.stdout, (r.stdout[-2000:] + r.stderr[-4000:])


def test_oracle_is_bit_exact_with_unsigned_char(tmp_path):
    import shutil
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    lib = str(tmp_path / "libnans_oracle_uchar.so")
    subprocess.run([cxx, "-O2", "-funsigned-char", "-ffp-contract=off", "-fno-fast-math", "-std=c++17", "-fPIC",
                    "-shared", "-pthread", "-I", os.path.join(ROOT, "oracle", "port"),
                    "-I", os.path.join(ROOT, "oracle", "shim", "glm"),
                    os.path.join(ROOT, "oracle", "port", "nans_oracle.cpp"), "-o", lib], check=True)
    env = dict(os.environ, NANS_ORACLE_LIB=lib)
    r = subprocess.run([sys.executable, os.path.abspath(__file__)], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0 and "oracle run ok" in r.stdout, (r.stdout[-2000:] + r.stderr[-4000:])


def _child():
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    from oracle import portbind
    portbind.LIB_PATH = os.environ.get("NANS_ORACLE_LIB", SAN_LIB)
    from helpers import GOLDEN_CASES, load_golden, step_digest
    import test_known_answers
    from nans_projekat_gb300 import scenes
    for case in GOLDEN_CASES:
        scene, meta, digests, _ = load_golden(case)
        w = portbind.OracleWorld([scene])
        dt = np.float32(meta["dt"])
        for k in range(1, min(meta["nsteps"], 200) + 1):
            w.step(dt, 1)
            cubes, spheres, _ = w.state()
            assert step_digest(cubes, spheres, w.pairs()) == digests[k - 1], (case, k)
    for sc, _ in test_known_answers.cases().values():
        portbind.OracleWorld([sc]).step(test_known_answers.DT, 30)
    dt = np.float32(1 / 60)
    portbind.OracleWorld(scenes.mixed_batch(16, seed=4), fp64=True).step(dt, 20, threads=4)
    w = portbind.OracleWorld(scenes.mixed_batch(16, seed=4))
    w.set_warm(True)
    w.step(dt, 20, threads=4)
    print("oracle run ok")


if __name__ == "__main__":
    _child()
