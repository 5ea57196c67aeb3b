"""The C++ SL_Context-shaped facade (include/slg_context.hpp): compiles and
links a C++ caller against libslg.so here (no GPU needed), and on a GPU runs it
and compares its image with the CPU oracle's rendering of the same scene."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_cpp(tmp_path, name="draw_test"):
    import softlight_gb300 as sg
    lib = sg.build()
    exe = str(tmp_path / name)
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", name + ".cpp"), "-o", exe,
           "-L", os.path.dirname(lib), "-lslg", f"-Wl,-rpath,{os.path.dirname(lib)}"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def test_cpp_facade_compiles_and_links(tmp_path):
    assert os.path.exists(build_cpp(tmp_path))
    assert os.path.exists(build_cpp(tmp_path, "scene_test"))


@pytest.mark.gpu
def test_cpp_scene_graph_facade(tmp_path):
    """SL_SceneGraph-shaped calls from C++: exact model matrices of a
    two-level graph and a drawn draw list."""
    exe = build_cpp(tmp_path, "scene_test")
    res = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, (res.returncode, res.stdout, res.stderr)


@pytest.mark.gpu
def test_cpp_facade_renders_like_oracle(tmp_path, oracle_mod):
    exe = build_cpp(tmp_path)
    out = str(tmp_path / "img.rgba")
    res = subprocess.run([exe, out], capture_output=True, text=True, timeout=120)
    assert res.returncode == 0, res.stderr
    img = np.fromfile(out, dtype=np.uint8).reshape(480, 640, 4)
    import edge_scenes as E
    o = oracle_mod.Context()
    s = E.flat_triangle(o)
    s.render()
    assert np.array_equal(img, s.read_color())
    assert (img[..., 0] == 255).sum() > 100000
