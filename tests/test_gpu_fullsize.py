"""GPU parity at the full benchmark sizes: the frames bench.py times, rendered
through the C ABI with the launch configuration the benchmark uses, against
the CPU oracle (all host cores; its multi-threaded mode reproduces the
one-thread result, tests/test_golden.py) on the same seeded inputs.

  instanced scene   1920x1080, 1024 instances of the 64x32 sphere (4.19 M
                    triangles), Blinn-Phong, 1024^2 texture: the autotuner's
                    pick and the 8x8 tiles / 64-thread vertex block it
                    usually picks
  triangle soup     1920x1080, 2 M triangles, 30 % back-facing, 10 % clipped
                    at the near plane, alpha blended (ordered raster)
  batched draws     3840x2160, 256 meshes of 12..65k triangles with their own
                    512^2 textures: one batched launch replayed from a CUDA
                    graph, and the same frame as one launch per draw

Bar: depth bit-exact (coverage and depth-test outcomes), RGBA8 colour within
1 LSB per channel (tests/parity.py)."""
import os

import pytest

from softlight_gb300 import api as A
from softlight_gb300 import scenes as S

from parity import compare_scenes

pytestmark = pytest.mark.gpu


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


@pytest.fixture()
def ctxs(gpu_lib, oracle_mod):
    g = gpu_lib.Context()
    o = oracle_mod.Context(num_threads=host_cores())
    yield g, o
    g.close()
    o.close()


def covered(scene):
    return int((scene.read_depth() < scene.clear_depth).sum())


def test_instanced_1080p_autotuned(ctxs):
    g, o = ctxs
    sg, so = S.build_c2(g), S.build_c2(o)
    cmds = [A.DrawCmd(m, n, sh) for (m, n, sh) in sg.draws]
    tw, th, vb = g.autotune(cmds, sg.fbo, sg.clear_color, sg.clear_depth)
    sg.render()
    so.render()
    g.finish()
    compare_scenes(sg, so, f"instanced 1080p, tile {tw}x{th}, vertex block {vb}")
    assert covered(sg) > 300000


@pytest.mark.parametrize("tile,vblock", [((8, 8), 64), ((16, 16), 128)])
def test_instanced_1080p_fixed_config(ctxs, tile, vblock):
    g, o = ctxs
    g.set_tile_size(*tile)
    g.set_vertex_block(vblock)
    sg, so = S.build_c2(g), S.build_c2(o)
    for _ in range(2):     # a second frame over the first one's scratch
        sg.render()
    so.render()
    g.finish()
    compare_scenes(sg, so, f"instanced 1080p, tile {tile}, vertex block {vblock}")


def test_soup_2m_blended_1080p(ctxs):
    g, o = ctxs
    sg, so = S.build_c3(g), S.build_c3(o)
    cmds = [A.DrawCmd(m, n, sh) for (m, n, sh) in sg.draws]
    tw, th, vb = g.autotune(cmds, sg.fbo, sg.clear_color, sg.clear_depth)
    sg.render()
    so.render()
    g.finish()
    compare_scenes(sg, so, f"2M soup 1080p, tile {tw}x{th}, vertex block {vb}")
    assert covered(sg) > 1500000


def test_batched_256_draws_2160p(ctxs):
    g, o = ctxs
    sg, so = S.build_c4(g), S.build_c4(o)
    assert sg.batched
    cmds = [A.DrawCmd(m, n, sh) for (m, n, sh) in sg.draws]
    tw, th, vb = g.autotune(cmds, sg.fbo, sg.clear_color, sg.clear_depth)
    g.set_batch_graphs(True)
    so.render()
    for _ in range(2):     # capture, then replay the graph
        sg.render()
    g.finish()
    compare_scenes(sg, so, f"256 draws 2160p batched graph, tile {tw}x{th}, vertex block {vb}")
    assert covered(sg) > 1000000
    sg.batched = False     # the same frame, one launch per draw
    sg.render()
    g.finish()
    compare_scenes(sg, so, "256 draws 2160p, one launch per draw")
