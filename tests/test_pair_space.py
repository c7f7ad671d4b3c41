"""CPU check of the cull's pair-space index arithmetic: tests/pair_space_check.cpp compiles
the kernels' own decode header (nans_projekat_gb300/csrc/nans_pairs.cuh) for the host and
compares it with a brute-force walk of the reference's pair order (code/nans.cpp:1355-1535)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_pair_decode_matches_the_reference_order(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "pair_space_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "nans_projekat_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "pair_space_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    ok, decodes, afters, rows = r.stdout.split()
    assert ok == "ok" and int(decodes) > 500_000 and int(afters) > int(decodes) and int(rows) > 200_000
