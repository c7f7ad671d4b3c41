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
