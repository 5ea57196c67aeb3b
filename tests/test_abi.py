"""CPU-only checks of the C-ABI boundary: the library builds, loads without a
GPU and exports every entry point include/slg.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "slg.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"\b(slg_[a-z_0-9]+)\s*\(", txt)
    return sorted(set(names))


def test_header_and_binding_agree():
    from softlight_gb300.api import exported_symbols
    assert set(header_functions()) == set(exported_symbols("slg_", gpu=True))


def test_library_builds_and_exports_every_symbol():
    import softlight_gb300 as sg
    path = sg.build()
    assert os.path.exists(path)
    lib = ctypes.CDLL(path)  # loads without a GPU: no CUDA call happens at load time
    missing = [n for n in header_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_open_library_binds_signatures():
    import softlight_gb300 as sg
    from softlight_gb300.api import open_library
    lib = open_library(sg.build(), "slg_", gpu=True)
    assert lib.slg_create_shader.restype is ctypes.c_size_t


def test_missing_library_fails_loudly(tmp_path):
    from softlight_gb300.api import open_library
    with pytest.raises(OSError):
        open_library(str(tmp_path / "nope.so"), "slg_", gpu=True)


def test_oracle_exports_same_api():
    import oracle
    lib = ctypes.CDLL(oracle.build_oracle())
    from softlight_gb300.api import exported_symbols
    missing = [n for n in exported_symbols("slo_", gpu=False) if not hasattr(lib, n)]
    assert not missing, missing
