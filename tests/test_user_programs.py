"""Caller-defined shader programs (include/slg_shader.cuh): tests/cpp/
user_programs.cu writes an alpha-test program, a fragment-coordinate program
and a three-binding vertex program the way SoftLight's test shaders are
written, over slg::VertexParam / slg::FragmentParam. It is compiled here into
its own shared library (no GPU needed); on a GPU its table is registered with
slg_register_programs and its images must equal those of the built-in
programs with the same arithmetic bit for bit (which the golden fixtures pin
to the reference), in both raster configurations and every primitive kind."""
import ctypes
import os
import subprocess
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from softlight_gb300 import api as A
from softlight_gb300 import scenes as S

import edge_scenes as E
from parity import compare_scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "user_programs.cu")
OUT = os.path.join(ROOT, "tests", "cpp", "_build")
LIB = os.path.join(OUT, "libslg_user_programs.so")

CUTOUT, FRAG_COORD, SPLIT_VS = 256, 257, 258
PROGRAMS = [(CUTOUT, 36, A.PROGRAM_DISCARDS), (FRAG_COORD, 36, A.PROGRAM_DISCARDS | A.PROGRAM_WRITES_DEPTH),
            (SPLIT_VS, 12, 0)]


def build_user_programs():
    """Compiles the four parts of user_programs.cu in parallel with the
    library's flags and links them; returns the shared library's path."""
    from softlight_gb300.buildlib import NVCC_FLAGS, nvcc
    deps = [SRC] + [os.path.join(ROOT, "include", f) for f in os.listdir(os.path.join(ROOT, "include"))]
    deps += [os.path.join(ROOT, "softlight_gb300", "csrc", f) for f in os.listdir(os.path.join(ROOT, "softlight_gb300", "csrc"))]
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps):
        return LIB
    os.makedirs(OUT, exist_ok=True)

    def part(k):
        obj = os.path.join(OUT, f"user_programs_{k}.o")
        cmd = [nvcc(), *NVCC_FLAGS, "-I", os.path.join(ROOT, "include"), f"-DSLG_USER_PART={k}", "-c", SRC, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        assert res.returncode == 0, res.stderr
        return obj

    with ThreadPoolExecutor(max_workers=4) as ex:
        objs = list(ex.map(part, range(4)))
    tmp = LIB + ".tmp"
    res = subprocess.run([nvcc(), "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *objs, "-o", tmp, "-lcudart"],
                         capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    os.replace(tmp, LIB)
    return LIB


def table_address():
    lib = ctypes.CDLL(build_user_programs())
    fn = lib.slg_test_user_programs
    fn.restype = ctypes.c_void_p
    return lib, fn()


def test_user_programs_compile_and_export_their_table():
    path = build_user_programs()
    lib = ctypes.CDLL(path)   # loads without a GPU: the table is built on first call, no CUDA call
    assert hasattr(lib, "slg_test_user_programs")


@pytest.fixture()
def ctxs(gpu_lib, oracle_mod):
    g = gpu_lib.Context()
    o = oracle_mod.Context()
    keep, ops = table_address()
    g.register_programs(ops, PROGRAMS)
    g._keep.append(keep)
    yield g, o
    g.close()
    o.close()


def with_program(scene, vs, fs):
    """Replaces the scene's shader by one with the given program ids and the
    same state and uniform block."""
    mesh, n, _ = scene.draws[0]
    ubo = scene.frame_ubos[-1][0]
    sh = scene.ctx.create_shader(A.VertexShader(2, A.CULL_OFF, vs), A.FragmentShader(2, 1, scene.blend_mode, scene.depth_test,
                                                                                      scene.depth_mask, fs), ubo)
    scene.draws[0] = (mesh, n, sh)


def program_scene(ctx, program, **kw):
    s = E.program_soup(ctx, program, **kw)
    s.blend_mode = kw.get("blend", A.BLEND_OFF)
    s.depth_test = kw.get("depth_test", A.DEPTH_TEST_LESS_THAN)
    s.depth_mask = kw.get("depth_mask", A.DEPTH_MASK_ON)
    return s


@pytest.mark.gpu
@pytest.mark.parametrize("prim", ["tri", "wire", "line", "point"])
@pytest.mark.parametrize("mode", [0, 1])
def test_user_cutout_equals_builtin(ctxs, prim, mode):
    g, o = ctxs
    g.set_raster_mode(mode)
    kw = dict(prim=prim, seed=71, num_tris=600 if prim != "point" else 2000, width=160, height=120)
    su = program_scene(g, A.PROGRAM_VCOLOR_TEX_CUTOUT, **kw)
    with_program(su, CUTOUT, CUTOUT)
    so = program_scene(o, A.PROGRAM_VCOLOR_TEX_CUTOUT, **kw)
    su.render()
    so.render()
    g.finish()
    compare_scenes(su, so, f"user cutout {prim}")
    assert (su.read_depth() < 1.0).sum() > 1000


@pytest.mark.gpu
@pytest.mark.parametrize("prim", ["tri", "wire", "line", "point"])
def test_user_frag_coord_equals_builtin(ctxs, prim):
    g, o = ctxs
    kw = dict(prim=prim, seed=72, num_tris=600 if prim != "point" else 2000, width=160, height=120,
              color_type=A.COLOR_RGBA_FLOAT)
    su = program_scene(g, A.PROGRAM_FRAG_COORD, **kw)
    with_program(su, CUTOUT, FRAG_COORD)
    so = program_scene(o, A.PROGRAM_FRAG_COORD, **kw)
    su.render()
    so.render()
    g.finish()
    compare_scenes(su, so, f"user frag coord {prim}")


@pytest.mark.gpu
def test_user_vertex_program_reads_three_bindings(ctxs):
    """SL_VertexArray::offset(bindId, vertId) over three bindings of one
    interleaved buffer: the same image as the one-binding program."""
    g, o = ctxs
    kw = dict(seed=73, num_tris=500, width=128, height=96)
    su = program_scene(g, A.PROGRAM_VCOLOR_TEX_CUTOUT, **kw)
    vao = su.draws[0][0].vaoId
    g.vao_set_binding(vao, 1, 12, 36, 4, A.VERTEX_DATA_FLOAT)
    g.vao_set_binding(vao, 2, 28, 36, 2, A.VERTEX_DATA_FLOAT)
    with_program(su, SPLIT_VS, CUTOUT)
    so = program_scene(o, A.PROGRAM_VCOLOR_TEX_CUTOUT, **kw)
    su.render()
    so.render()
    g.finish()
    compare_scenes(su, so, "three bindings")
    # a binding that reaches past the buffer is rejected before any launch
    g.vao_set_binding(vao, 2, 36 * 1500, 36, 2, A.VERTEX_DATA_FLOAT)
    with pytest.raises(A.SLError, match="binding 2"):
        su.render()


@pytest.mark.gpu
def test_undeclared_discard_is_reported(gpu_lib):
    """A program registered without SLG_PROGRAM_DISCARDS takes the
    order-free raster; when it discards there, slg_finish says so."""
    g = gpu_lib.Context()
    keep, ops = table_address()
    g.register_programs(ops, [(CUTOUT, 36, 0)])
    s = program_scene(g, A.PROGRAM_VCOLOR_TEX_CUTOUT, seed=74, num_tris=400, width=96, height=80)
    with_program(s, CUTOUT, CUTOUT)
    s.render()
    with pytest.raises(A.SLError, match="SLG_PROGRAM_DISCARDS"):
        g.finish()
    g.finish()
    g.close()


@pytest.mark.gpu
def test_registration_checks(gpu_lib):
    g = gpu_lib.Context()
    keep, ops = table_address()
    with pytest.raises(A.SLError, match="SLG_PROGRAM_USER_FIRST"):
        g.register_programs(ops, [(7, 36, 0)])
    with pytest.raises(A.SLError, match="listed twice"):
        g.register_programs(ops, [(300, 36, 0), (300, 36, 0)])
    g.register_programs(ops, [(300, 36, 0)])
    with pytest.raises(A.SLError, match="already registered"):
        g.register_programs(ops, [(300, 36, 0)])
    # a table compiled against other headers is refused
    raw = (ctypes.c_uint32 * 2).from_address(ops)
    fake = (ctypes.c_uint8 * 64)()
    ctypes.memmove(fake, ops, 40)
    ctypes.cast(fake, ctypes.POINTER(ctypes.c_uint32))[1] = raw[1] + 8
    with pytest.raises(A.SLError, match="another version"):
        g.register_programs(ctypes.addressof(fake), [(301, 36, 0)])
    # a shader pairing programs of two sets, or unknown ids, is refused
    ubo = g.create_ubo()
    with pytest.raises(A.SLError, match="different program sets"):
        g.create_shader(A.VertexShader(2, A.CULL_OFF, 300), A.FragmentShader(2, 1, 0, 1, 1, A.PROGRAM_FLAT_COLOR), ubo)
    with pytest.raises(A.SLError, match="unknown shader program"):
        g.create_shader(A.VertexShader(2, A.CULL_OFF, 999), A.FragmentShader(2, 1, 0, 1, 1, 999), ubo)
    g.close()
