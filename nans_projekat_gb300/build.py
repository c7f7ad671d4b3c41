"""Builds the CUDA library nans_projekat_gb300/_lib/libnans_gb300.so for sm_103a.

Every translation unit is compiled in parallel with nvcc, then linked into one shared
library with the CUDA runtime linked statically. The physics kernels must reproduce IEEE
single precision exactly, so the build pins: no FMA contraction (-fmad=false), IEEE
division and square root, no flush-to-zero.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB_PATH = os.path.join(OUT_DIR, "libnans_gb300.so")
SIM_PATH = os.path.join(OUT_DIR, "libnans_sim.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-std=c++17", "-lineinfo",
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
    "-I", CSRC, "-I", INCLUDE,
]

SOURCES = ["k_sweep.cu", "k_cull.cu", "k_narrow.cu", "k_epa_large.cu", "k_solve.cu", "k_adjoint.cu", "k_render.cu",
           "api.cu", "noalloc.cu"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "nans_gb300.h"))
    files.append(os.path.join(INCLUDE, "nans_sim.h"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date():
    if not os.path.exists(LIB_PATH) or not os.path.exists(SIM_PATH):
        return False
    t = os.path.getmtime(LIB_PATH)
    return all(os.path.getmtime(f) <= t for f in _deps())


def build(force=False, verbose=False, extra_flags=()):
    if not force and up_to_date():
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    nv = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [nv] + NVCC_FLAGS + list(extra_flags) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        return obj, r.stderr

    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        for obj, err in ex.map(compile_one, SOURCES):
            objs.append(obj)
            if verbose and err:
                sys.stderr.write(err)
    tmp = LIB_PATH + ".tmp"
    cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB_PATH)
    build_sim()
    return LIB_PATH


def build_sim():
    """libnans_sim.so: the headless SimUpdateAndRender (host C++ over libnans_gb300.so)."""
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        raise RuntimeError("g++ not found")
    tmp = SIM_PATH + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", INCLUDE,
           os.path.join(CSRC, "sim_shim.cpp"), "-L", OUT_DIR, "-lnans_gb300", "-Wl,-rpath,$ORIGIN", "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("sim shim build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, SIM_PATH)
    return SIM_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv,
          extra_flags=["-Xptxas", "-v"] if "--ptxas" in sys.argv else ())
    print(LIB_PATH)
