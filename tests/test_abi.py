"""CPU tests of the C ABI library: it builds for sm_103a, loads, and exports every entry
point that include/nans_gb300.h declares. No compute call is made here."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "nans_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void\s*\*|const char\s*\*|void)\s*(nans_\w+)\s*\(", text, re.M)))


def test_header_declares_the_abi():
    names = declared_functions()
    assert "nans_step" in names and "nans_world_create" in names and "nans_get_pairs" in names
    assert len(names) >= 15


def test_library_builds_and_exports_every_declared_symbol():
    from nans_projekat_gb300 import build, lib
    path = build.build()
    assert os.path.exists(path)
    L = ctypes.CDLL(path)
    for name in declared_functions():
        assert hasattr(L, name), name
    assert set(lib.EXPORTS) == set(declared_functions())


def test_record_layouts_match_header():
    from nans_projekat_gb300.types import CUBE_DTYPE, SPHERE_DTYPE, PAIR_DTYPE
    text = open(HEADER).read()
    assert "244 bytes" in text and CUBE_DTYPE.itemsize == 244
    assert "148 bytes" in text and SPHERE_DTYPE.itemsize == 148
    assert "96 bytes" in text and PAIR_DTYPE.itemsize == 96


def test_python_constants_match_header():
    """The Python mirror's flag and error values are the header's #defines (NANS_WORLD_*,
    NANS_UPLOAD_*, NANS_ERR_*), every one of them."""
    from nans_projekat_gb300 import lib
    text = open(HEADER).read()
    defines = {m.group(1): int(m.group(2)) for m in re.finditer(r"^#define (NANS_\w+) (\d+)u?\b", text, re.M)}
    flags = {k: v for k, v in defines.items() if k.startswith(("NANS_WORLD_", "NANS_UPLOAD_"))}
    assert "NANS_WORLD_FUSED_STEP" in flags and len(flags) >= 8
    for name, value in flags.items():
        assert getattr(lib, name[len("NANS_"):]) == value, name
    errors = {k: v for k, v in defines.items() if k.startswith("NANS_ERR_")}
    assert errors and {v: k for k, v in errors.items()} == lib.ERRORS
    assert defines["NANS_OK"] == lib.NANS_OK


def test_last_error_is_empty_string_initially():
    from nans_projekat_gb300 import lib
    L = lib.load()
    assert isinstance(L.nans_last_error(), bytes)


def test_save_ppm(tmp_path):
    import numpy as np
    from nans_projekat_gb300 import lib
    img = np.arange(2 * 3 * 3, dtype=np.uint8).reshape(2, 3, 3)
    p = tmp_path / "a.ppm"
    lib.save_ppm(str(p), img)
    raw = p.read_bytes()
    assert raw.startswith(b"P6\n3 2\n255\n") and raw[-18:] == img.tobytes()


def test_no_silent_fallback_without_a_device():
    """Without a GPU every compute entry point raises: there is no CPU path to fall back to."""
    import numpy as np
    import torch
    from nans_projekat_gb300 import lib
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(lib.NansError) as e:
        lib.World()
    assert e.value.code == 4  # NANS_ERR_CUDA
    with pytest.raises(lib.NansError):
        lib.device_sincos(np.zeros(4, np.float32))


@pytest.mark.parametrize("header", ["nans_gb300.h", "nans_sim.h"])
def test_headers_compile_as_c_and_cpp(header):
    """The C ABI headers are plain C99 (what cgo / FFI binders parse) and valid C++."""
    import shutil
    import subprocess
    path = os.path.join(ROOT, "include", header)
    for cc, lang, std in (("gcc", "c", "-std=c99"), ("g++", "c++", "-std=c++17")):
        if shutil.which(cc) is None:
            pytest.skip("no %s" % cc)
        subprocess.run([cc, "-x", lang, std, "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only", path],
                       check=True)


def test_plain_c_consumer_links_and_reports_status(tmp_path):
    """tests/abi_consumer.c, a C99 program in the reference's record layouts, links against the
    library and gets a status from every call: NANS_ERR_CUDA from nans_world_create without a
    GPU (with the output pointer left NULL), NANS_OK through a 30-step run with one."""
    import shutil
    import subprocess
    import torch
    from nans_projekat_gb300 import build
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    lib_path = build.build()
    lib_dir = os.path.dirname(lib_path)
    exe = str(tmp_path / "abi_consumer")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "abi_consumer.c"), "-L", lib_dir, "-lnans_gb300",
                    "-Wl,-rpath," + lib_dir, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.splitlines()
    if torch.cuda.is_available():
        assert lines[0] == "create 0" and lines[1].startswith("step 0 ")
    else:
        assert lines[0] == "create 4" and lines[1].startswith("last_error create:")
