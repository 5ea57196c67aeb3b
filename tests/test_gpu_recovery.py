"""Overflow recovery. Scratch buffers are sized from what earlier launches
needed; with slg_set_scratch_caps a context starts them small, so launches
overflow the tile-entry buffer, the clipped-triangle record region or the
shared-memory tile sort. The device skips the overflowed launch and the work
queued after it; at the next synchronisation point the host grows the buffer
and replays the recorded operations (draws, clears, blits, uniform-block
writes) from that launch on. The frames must equal the oracle's, as if the
buffers had been large enough (depth bit-exact, colour within 1 LSB)."""
import numpy as np
import pytest

from softlight_gb300 import api as A
from softlight_gb300 import scenes as S

import edge_scenes as E
from parity import compare_scenes, compare_colors

pytestmark = pytest.mark.gpu


@pytest.fixture()
def ctxs(gpu_lib, oracle_mod):
    g = gpu_lib.Context()
    o = oracle_mod.Context()
    yield g, o
    g.close()
    o.close()


CAPS = {
    "entries": dict(entries=3000),
    "clip_records": dict(clip_records=8),
    "sort_keys": dict(sort_keys=16),
    "all": dict(entries=3000, clip_records=8, sort_keys=16),
}


@pytest.mark.parametrize("caps", sorted(CAPS))
@pytest.mark.parametrize("blend", [A.BLEND_OFF, A.BLEND_ALPHA])
@pytest.mark.parametrize("mode", [2, 3])
def test_overflowed_launch_is_replayed(ctxs, caps, blend, mode):
    """mode 2: opaque launches on tiles (tile entries can overflow); mode 3:
    untiled (only the clipped-record region can)."""
    g, o = ctxs
    g.set_raster_mode(mode)
    kw = dict(num_tris=3000, width=200, height=150, seed=111, blend=blend, cull=A.CULL_OFF)
    sg, so = E.random_soup(g, **kw), E.random_soup(o, **kw)
    sg.render()
    g.finish()
    g.set_scratch_caps(**CAPS[caps])
    sg.render()
    so.render()
    g.finish()
    compare_scenes(sg, so, f"recovered ({caps}, blend {blend})")
    # the grown buffers serve the next frame directly
    sg.render()
    g.finish()
    compare_scenes(sg, so, f"after recovery ({caps}, blend {blend})")


def test_sequence_after_overflow_is_replayed_in_order(ctxs):
    """Overflowing draw, a uniform block re-written, two more draws and a
    blit of the attachment, all before the next synchronisation point:
    the replay restores the block for the first draw and re-applies the
    write for the later ones."""
    g, o = ctxs
    results = []
    for ctx in (g, o):
        s = E.random_soup(ctx, num_tris=2500, width=160, height=120, seed=112, blend=A.BLEND_ALPHA, cull=A.CULL_OFF)
        s.render()
        ctx.finish()
        mesh, _, shader = s.draws[0]
        ubo = s.frame_ubos[-1][0]
        verts, proj = S.soup_triangles(2500, 160, 120, seed=112)
        moved = S.col_major(S.translate((0.3, -0.2, 0.0)) @ proj).tobytes() + s.frame_ubos[-1][1][64:]
        other = ctx.create_texture()
        ctx.texture_init(other, A.COLOR_RGBA_8U, 80, 60, 1)
        if ctx is g:
            g.set_scratch_caps(entries=2000, clip_records=8, sort_keys=16)
        ctx.clear_framebuffer(s.fbo, 0, s.clear_color, s.clear_depth)
        ctx.draw(mesh, shader, s.fbo)              # overflows on the GPU
        ctx.ubo_assign(ubo, moved)
        ctx.draw(mesh, shader, s.fbo)
        ctx.blit(other, s.color_tex)
        ctx.draw(mesh, shader, s.fbo)
        ctx.finish()
        results.append((s.read_color(), s.read_depth(), ctx.texture_read(other, (60, 80, 4), np.uint8)))
    (cg, dg, bg), (co, do, bo) = results
    assert np.array_equal(dg.view(np.uint32), do.view(np.uint32)), "depth differs after the replay"
    compare_colors(cg, co, "colour after the replay")
    compare_colors(bg, bo, "blit after the replay")


def test_batch_graph_overflow_is_replayed(ctxs):
    g, o = ctxs
    sg, so = S.build_c4(g, num_draws=12, width=400, height=240, tex_size=64), S.build_c4(o, num_draws=12, width=400, height=240,
                                                                                     tex_size=64)
    g.set_batch_graphs(True)
    sg.render()
    g.finish()
    g.set_scratch_caps(entries=4000, clip_records=8, sort_keys=16)
    for _ in range(2):
        sg.render()
    so.render()
    g.finish()
    compare_scenes(sg, so, "batched graph after recovery")


def test_scene_graph_overflow_is_reported(gpu_lib, oracle_mod):
    """The scene graph's draw list is written on the device, so its launch
    is not replayed: the overflow is reported at finish with the buffers
    grown, and the next frame renders in full (the scene animates: frame 3
    is compared with the oracle's frame 3). Its opaque launches run on
    tiles here (raster mode 2), so a small tile-entry cap overflows."""
    g = gpu_lib.Context()
    g.set_raster_mode(2)
    o = oracle_mod.Context()
    s = S.build_scene_graph(g, width=160, height=120, groups=3, per_group=3)
    so = S.build_scene_graph(o, width=160, height=120, groups=3, per_group=3)
    s.render()
    g.finish()
    g.set_scratch_caps(entries=64)
    s.render()
    with pytest.raises(A.SLError, match="scene-graph"):
        g.finish()
    s.render()
    g.finish()
    for _ in range(3):
        so.render()
    compare_scenes(s, so, "scene graph after a reported overflow")
    assert np.array_equal(s.read_models().view(np.uint32), so.read_models().view(np.uint32))
    g.close()
    o.close()
