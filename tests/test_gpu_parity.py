"""GPU parity tests: the CUDA draw path (through the C ABI) against the CPU
oracle on identical seeded inputs. Coverage and depth must be bit-exact,
colour within 1 LSB (RGBA8) or 1e-5 relative (float)."""
import numpy as np
import pytest

from softlight_gb300 import api as A
from softlight_gb300 import scenes as S

import edge_scenes as E
from parity import compare_scenes, render_both

pytestmark = pytest.mark.gpu


@pytest.fixture()
def ctxs(gpu_lib, oracle_mod):
    g = gpu_lib.Context()
    o = oracle_mod.Context()
    yield g, o
    g.close()
    o.close()


def test_c1_sphere_exact(ctxs):
    g, o = ctxs
    sg, so = render_both(S.build_c1, g, o)
    assert compare_scenes(sg, so, "c1") == 0
    assert (sg.read_depth() < 1.0).sum() > 50000


@pytest.mark.parametrize("mode", [0, 1, 2, 3])
def test_raster_modes_agree(ctxs, mode):
    """The default plan (mode 0: order-free on tiles until the autotuner
    picks otherwise), the ordered replay (1), the order-free resolve on
    tiles (2) and untiled (3) all match."""
    g, o = ctxs
    g.set_raster_mode(mode)
    sg, so = render_both(S.build_c2, g, o, num_instances=24, width=320, height=200, tex_size=128)
    assert compare_scenes(sg, so, f"c2 mode {mode}") == 0
    sg, so = render_both(E.multi_draw, g, o)
    compare_scenes(sg, so, f"multi mode {mode}")


@pytest.mark.parametrize("depth_test", [1, 2, 3, 4, 5, 0])
@pytest.mark.parametrize("depth_mask", [0, 1])
@pytest.mark.parametrize("mode", [2, 3])
def test_order_free_depth_rules(ctxs, depth_test, depth_mask, mode):
    """Opaque draws take the order-free path (on tiles in mode 2, untiled in
    mode 3); every depth rule it accepts must reproduce the sequential
    result, ties included."""
    g, o = ctxs
    g.set_raster_mode(mode)
    sg, so = render_both(E.random_soup, g, o, depth_test=depth_test, depth_mask=depth_mask, clear_depth=0.5,
                         frames=2, num_tris=500)
    compare_scenes(sg, so, f"free depth {depth_test}/{depth_mask}")
    sg, so = render_both(E.big_triangles, g, o)
    compare_scenes(sg, so, "free big")


def test_c1_two_frames_and_rerender(ctxs):
    g, o = ctxs
    sg, so = render_both(S.build_c1, g, o, frames=3)
    assert compare_scenes(sg, so, "c1x3") == 0


@pytest.mark.parametrize("tile", [(8, 8), (16, 16), (32, 16), (32, 32), (64, 32), (64, 64)])
def test_c1_all_tile_sizes(ctxs, tile):
    g, o = ctxs
    g.set_tile_size(*tile)
    sg, so = render_both(S.build_c1, g, o, width=333, height=211)
    assert compare_scenes(sg, so, f"c1 tile {tile}") == 0


def test_c2_instanced_small(ctxs):
    g, o = ctxs
    sg, so = render_both(S.build_c2, g, o, num_instances=48, width=480, height=270, tex_size=256)
    assert compare_scenes(sg, so, "c2 small") == 0


def test_c3_soup_small_blend_clip(ctxs):
    g, o = ctxs
    sg, so = render_both(S.build_c3, g, o, num_tris=3000, width=320, height=180, tex_size=256)
    assert compare_scenes(sg, so, "c3 small") == 0


def test_c4_batched_small(ctxs):
    g, o = ctxs
    sg, so = render_both(S.build_c4, g, o, num_draws=12, width=400, height=240, tex_size=64)
    assert compare_scenes(sg, so, "c4 small") == 0


@pytest.mark.parametrize("depth_test", range(7))
@pytest.mark.parametrize("depth_mask", [0, 1])
def test_depth_functions(ctxs, depth_test, depth_mask):
    g, o = ctxs
    sg, so = render_both(E.random_soup, g, o, depth_test=depth_test, depth_mask=depth_mask, clear_depth=0.5, frames=2)
    compare_scenes(sg, so, f"depth {depth_test}/{depth_mask}")


@pytest.mark.parametrize("blend", [A.BLEND_ALPHA, A.BLEND_PREMULTIPLED_ALPHA, A.BLEND_ADDITIVE, A.BLEND_SCREEN])
@pytest.mark.parametrize("fmt", [A.COLOR_RGBA_8U, A.COLOR_RGBA_FLOAT])
def test_blend_modes(ctxs, blend, fmt):
    g, o = ctxs
    sg, so = render_both(E.random_soup, g, o, blend=blend, color_type=fmt, num_tris=400)
    compare_scenes(sg, so, f"blend {blend} fmt {fmt}")


@pytest.mark.parametrize("cull", [A.CULL_BACK_FACE, A.CULL_FRONT_FACE, A.CULL_OFF])
def test_cull_modes(ctxs, cull):
    g, o = ctxs
    sg, so = render_both(E.random_soup, g, o, cull=cull)
    compare_scenes(sg, so, f"cull {cull}")


@pytest.mark.parametrize("dtype", [np.uint8, np.uint16, np.uint32])
def test_index_types(ctxs, dtype):
    g, o = ctxs
    sg, so = render_both(E.random_soup, g, o, indexed=dtype, num_tris=80)
    compare_scenes(sg, so, f"index {np.dtype(dtype).name}")


def test_float_target_and_texture(ctxs):
    g, o = ctxs
    sg, so = render_both(E.random_soup, g, o, program=A.PROGRAM_VCOLOR_TEXF, color_type=A.COLOR_RGBA_FLOAT)
    compare_scenes(sg, so, "texf")


def test_c5_differentiable_scene_exact(ctxs):
    """The differentiable-render scene (its framebuffer records a visibility
    map on the GPU) renders exactly like the oracle."""
    g, o = ctxs
    sg, so = render_both(S.build_c5, g, o)
    compare_scenes(sg, so, "c5")
    assert (sg.read_depth() < 1.0).sum() > 100000


def test_big_triangles_and_ties(ctxs):
    g, o = ctxs
    for tile in [(8, 8), (32, 32), (64, 64)]:
        g.set_tile_size(*tile)
        sg, so = render_both(E.big_triangles, g, o)
        assert compare_scenes(sg, so, f"big {tile}") == 0


@pytest.mark.parametrize("batched", [False, True])
def test_multi_draw(ctxs, batched):
    g, o = ctxs
    sg, so = render_both(E.multi_draw, g, o, batched=batched)
    compare_scenes(sg, so, f"multi batched={batched}")


@pytest.mark.parametrize("mode", [0, 3])
@pytest.mark.parametrize("graphs", [False, True])
def test_batched_equals_per_draw(gpu_lib, mode, graphs):
    """One batched launch (replayed from a CUDA graph when enabled) gives the
    frames of one launch per draw, on tiles (mode 0) and untiled (mode 3)."""
    a, b = gpu_lib.Context(), gpu_lib.Context()
    a.set_raster_mode(mode)
    b.set_raster_mode(mode)
    a.set_batch_graphs(graphs)
    sa = S.build_c4(a, num_draws=20, width=320, height=200, tex_size=32, batched=True)
    sb = S.build_c4(b, num_draws=20, width=320, height=200, tex_size=32, batched=False)
    for _ in range(2):
        sa.render()
        sb.render()
        assert np.array_equal(sa.read_color(), sb.read_color())
        assert np.array_equal(sa.read_depth().view(np.uint32), sb.read_depth().view(np.uint32))


def test_flat_triangle_draw_test_scene(ctxs):
    g, o = ctxs
    sg, so = render_both(E.flat_triangle, g, o)
    assert compare_scenes(sg, so, "flat") == 0
    img = sg.read_color()
    assert (img[..., 0] == 255).sum() > 100000


def test_empty_and_degenerate_draws(ctxs):
    g, o = ctxs
    for ctx in (g, o):
        s = S.build_c1(ctx, width=64, height=48)
        s.render()
        mesh = s.draws[0][0]
        empty = A.Mesh(mesh.vaoId, 0, 0, mesh.mode, 0)
        ctx.draw(empty, s.draws[0][2], s.fbo)
        ctx.draw_instanced(mesh, 0, s.draws[0][2], s.fbo)
        ctx.finish()
    # invalid ids are rejected, not executed
    with pytest.raises(A.SLError):
        g.draw(A.Mesh(999, 0, 3, A.RENDER_MODE_TRIANGLES, 0), 0, 0)


@pytest.mark.parametrize("vs_block", [64, 128, 256])
def test_vertex_block_sizes(ctxs, vs_block):
    g, o = ctxs
    g.set_vertex_block(vs_block)
    sg, so = render_both(S.build_c4, g, o, num_draws=8, width=256, height=160, tex_size=32)
    assert compare_scenes(sg, so, f"vs block {vs_block}") == 0


def test_batch_graph_replay_tracks_uniforms(ctxs):
    """Graph replays of a batch pick up uniform-block updates and match the
    oracle frame by frame; a changed draw list is recaptured."""
    import numpy as np
    g, o = ctxs
    g.set_batch_graphs(True)
    sg = S.build_c4(g, num_draws=10, width=256, height=160, tex_size=32)
    so = S.build_c4(o, num_draws=10, width=256, height=160, tex_size=32)
    rng = np.random.default_rng(9)
    for frame in range(4):
        if frame >= 2:
            # move one mesh: rewrite its uniform block on both sides
            ubo, data = sg.frame_ubos[frame]
            arr = np.frombuffer(data, dtype=np.uint8).copy()
            model = arr[64:128].view(np.float32).copy()
            model[12:15] += rng.uniform(-3, 3, 3).astype(np.float32)
            arr[64:128] = model.view(np.uint8)
            g.ubo_assign(ubo, arr.tobytes())
            o.ubo_assign(so.frame_ubos[frame][0], arr.tobytes())
        if frame == 3:
            sg.draws = sg.draws[:-2]
            so.draws = so.draws[:-2]
        sg.render()
        so.render()
        g.finish()
        assert compare_scenes(sg, so, f"graph frame {frame}") == 0


def test_autotune_picks_a_valid_config(ctxs):
    g, o = ctxs
    sg = S.build_c4(g, num_draws=12, width=320, height=200, tex_size=32)
    so = S.build_c4(o, num_draws=12, width=320, height=200, tex_size=32)
    from softlight_gb300 import api as A2
    cmds = [A2.DrawCmd(m, n, s) for (m, n, s) in sg.draws]
    tw, th, vb = g.autotune(cmds, sg.fbo)
    assert (tw, th) in [(8, 8), (16, 16), (32, 16), (32, 32), (64, 32), (64, 64)] and vb in (64, 128, 256)
    sg.render()
    so.render()
    assert compare_scenes(sg, so, "autotuned") == 0


@pytest.mark.parametrize("kw", [
    dict(num_points=200000, width=320, height=240),
    dict(num_points=100000, width=256, height=192, blend=A.BLEND_ALPHA, depth_mask=A.DEPTH_MASK_OFF, seed=52),
    dict(num_points=50000, width=200, height=150, num_instances=3, seed=53),
    dict(num_points=50000, width=200, height=150, depth_test=A.DEPTH_TEST_LESS_EQUAL, indexed=np.uint32, seed=54),
], ids=["less_200k", "blend_100k", "instanced_3x50k", "lequal_indexed"])
def test_points(ctxs, kw):
    """SL_RENDER_MODE_POINTS: order-free (depth rules) and ordered (blending)
    resolution of many points per pixel, against the oracle."""
    g, o = ctxs
    sg, so = render_both(E.random_points, g, o, **kw)
    compare_scenes(sg, so, "points")


@pytest.mark.parametrize("tile", [(8, 8), (64, 64)])
def test_points_all_tiles(ctxs, tile):
    g, o = ctxs
    g.set_tile_size(*tile)
    sg, so = render_both(E.random_points, g, o, num_points=30000, width=300, height=200, seed=55)
    compare_scenes(sg, so, f"points {tile}")


@pytest.mark.parametrize("kw", [
    dict(num_lines=4000, width=320, height=240),
    dict(num_lines=3000, width=256, height=192, persp=True, seed=72),
    dict(num_lines=2000, width=256, height=192, blend=A.BLEND_ALPHA, depth_mask=A.DEPTH_MASK_OFF, seed=73),
    dict(num_lines=1500, width=200, height=150, num_instances=3, odd_end=True, seed=74),
    dict(num_lines=2000, width=200, height=150, depth_test=A.DEPTH_TEST_LESS_EQUAL, indexed=np.uint32, seed=75),
    dict(num_lines=3000, width=1000, height=60, depth_test=A.DEPTH_TEST_NOT_EQUAL, clear_depth=0.5, seed=76),
    dict(num_lines=2000, width=240, height=160, depth_test=A.DEPTH_TEST_GREATER_EQUAL, clear_depth=-1.0,
         color_type=A.COLOR_RGBA_FLOAT, seed=77),
], ids=["less_4k", "persp_clip_cull", "blend_alpha", "instanced_odd_end", "lequal_indexed", "not_equal_1000x60",
        "gequal_float"])
def test_lines(ctxs, kw):
    """SL_RENDER_MODE_LINES: clipping, Bresenham walk, per-pixel depth and
    varyings along the line, order-free and ordered resolution."""
    g, o = ctxs
    sg, so = render_both(E.random_lines, g, o, **kw)
    compare_scenes(sg, so, "lines")
    assert (sg.read_depth() != sg.clear_depth).sum() > 1000 or kw.get("depth_mask") == A.DEPTH_MASK_OFF


@pytest.mark.parametrize("tile", [(8, 8), (32, 16), (64, 64)])
@pytest.mark.parametrize("mode", [0, 1])
def test_lines_all_tiles_and_modes(ctxs, tile, mode):
    """Launches with line draws use 32 x 32 tiles whatever the context's tile
    setting; both raster strategies."""
    g, o = ctxs
    g.set_tile_size(*tile)
    g.set_raster_mode(mode)
    sg, so = render_both(E.line_edges, g, o)
    compare_scenes(sg, so, f"line edges {tile} mode {mode}")
    sg, so = render_both(E.random_lines, g, o, num_lines=2500, width=300, height=200, persp=True, seed=78)
    compare_scenes(sg, so, f"lines {tile} mode {mode}")


def test_line_alias(ctxs):
    """A line whose last pixel (x = W) shares its first pixel's address: both
    are tested against the depth before the line, the later one wins."""
    g, o = ctxs
    sg, so = render_both(E.line_alias, g, o)
    compare_scenes(sg, so, "line alias")
    assert sg.read_depth()[E.LINE_ALIAS_PIXEL] == np.float32(0.5)


@pytest.mark.parametrize("occluded", [True, False])
@pytest.mark.parametrize("batched", [False, True])
@pytest.mark.parametrize("blend", [A.BLEND_OFF, A.BLEND_ALPHA])
def test_line_alias_queue_rule(ctxs, occluded, batched, blend):
    """700 px wide: occluded, fewer than 600 of the line's fragments are
    queued before its last step (tested against the depth before the line);
    open, the queue is written in between (tested after the first write)."""
    g, o = ctxs
    sg, so = render_both(E.line_alias_wide, g, o, occluded=occluded, batched=batched, blend=blend)
    compare_scenes(sg, so, f"wide alias occluded={occluded} batched={batched} blend={blend}")
    assert sg.read_depth()[10, 0] == np.float32(0.5 if occluded else 0.2)


@pytest.mark.parametrize("threads", [1, 3, 7])
def test_clear_extent_and_carry_over(ctxs, threads):
    """SoftLight's clear reaches only the prefix its thread partition covers
    (53 x 37 = 1961 texels, 1961 % 3 == 2: one thread leaves the last texel);
    what the previous frame drew there carries over into the next."""
    g, o = ctxs
    g.num_threads(threads)
    o.num_threads(threads)
    sg, so = render_both(E.random_soup, g, o, width=53, height=37, frames=3, num_tris=400)
    compare_scenes(sg, so, f"clear extent, {threads} threads")


@pytest.mark.parametrize("batched", [False, True])
@pytest.mark.parametrize("blend_lines", [False, True])
def test_mixed_primitives(ctxs, batched, blend_lines):
    """Triangles, lines and points into one frame; batched, one launch holds
    all three record kinds."""
    g, o = ctxs
    sg, so = render_both(E.mixed_prims, g, o, batched=batched, blend_lines=blend_lines)
    compare_scenes(sg, so, f"mixed batched={batched} blend={blend_lines}")


def test_line_draw_rejections(gpu_lib):
    """Line draws whose last line would read past the index buffer, and line
    draws into framebuffers wider than the reference's int16 Bresenham error
    term allows, are rejected before any launch."""
    ctx = gpu_lib.Context()
    s = E.random_lines(ctx, num_lines=10, indexed=np.uint16)
    mesh = s.draws[0][0]
    bad = A.Mesh(mesh.vaoId, 1, 20, A.RENDER_MODE_INDEXED_LINES, 0)   # last line reads element 20
    with pytest.raises(A.SLError):
        ctx.draw(bad, s.draws[0][2], s.fbo)
    wide = E.random_lines(ctx, num_lines=10, width=11000, height=4)
    with pytest.raises(A.SLError):
        ctx.draw(wide.draws[0][0], wide.draws[0][2], wide.fbo)
    ctx.close()


@pytest.mark.parametrize("kw", [
    dict(num_tris=2000, width=320, height=240),
    dict(num_tris=1500, width=320, height=240, depth_test=A.DEPTH_TEST_NOT_EQUAL, clear_depth=0.5, seed=92),
    dict(num_tris=800, width=160, height=120, blend=A.BLEND_ALPHA, seed=93),
    dict(num_tris=800, width=160, height=120, blend=A.BLEND_ADDITIVE, depth_mask=A.DEPTH_MASK_OFF,
         color_type=A.COLOR_RGBA_FLOAT, seed=94),
    dict(num_tris=600, width=200, height=150, cull=A.CULL_OFF, indexed=np.uint32, num_instances=2, seed=95),
], ids=["less_2k", "not_equal", "blend_alpha", "additive_float_mask_off", "indexed_instanced"])
@pytest.mark.parametrize("mode", [0, 1])
def test_wireframe(ctxs, kw, mode):
    """SL_RENDER_MODE_TRI_WIRE: the edge runs of every scan-line, direct
    barycentrics, pixels visited twice on narrow rows (blended twice)."""
    g, o = ctxs
    g.set_raster_mode(mode)
    sg, so = render_both(E.random_soup, g, o, wire=True, **kw)
    compare_scenes(sg, so, f"wire mode {mode}")


def test_wireframe_queue_order_reported(gpu_lib):
    """A blended wireframe triangle that revisits a pixel after 600 queued
    fragments is reported (SLError at finish), not silently drawn with
    another queue flush order; opaque, the same triangle is exact."""
    ctx = gpu_lib.Context()
    s = E.wire_queue(ctx)
    with pytest.raises(A.SLError, match="queue flush order"):
        s.render()
        ctx.finish()
    ctx.close()


def test_wireframe_queue_scene_opaque_exact(ctxs):
    g, o = ctxs
    sg, so = render_both(E.wire_queue, g, o, blend=A.BLEND_OFF)
    compare_scenes(sg, so, "wire queue opaque")


@pytest.mark.parametrize("kw", [
    dict(num_tris=2000, width=320, height=240),
    dict(types=(A.COLOR_RGBA_8U, A.COLOR_RGBA_8U, A.COLOR_RGBA_FLOAT), num_outputs=3, blend=A.BLEND_ALPHA,
         num_tris=1500, width=320, height=240, seed=112),
    dict(types=(A.COLOR_RGBA_FLOAT, A.COLOR_R_FLOAT), num_outputs=2, depth_test=A.DEPTH_TEST_NOT_EQUAL,
         num_tris=1000, width=200, height=150, seed=113),
    dict(num_outputs=2, single_after=True, num_tris=1000, width=200, height=150, seed=114),
    dict(num_outputs=4, single_after=True, batched=True, blend=A.BLEND_SCREEN, num_tris=800, width=200, height=150,
         seed=115),
    dict(prim="wire", blend=A.BLEND_ADDITIVE, num_tris=600, width=160, height=120, seed=116),
    dict(prim="line", num_tris=2000, width=256, height=192, seed=117),
    dict(prim="point", num_tris=4000, width=200, height=150, blend=A.BLEND_PREMULTIPLED_ALPHA, seed=118),
], ids=["four_targets", "three_blend_alpha", "two_not_equal", "two_then_single", "batched_screen", "wire_additive",
        "lines", "points_premultiplied"])
@pytest.mark.parametrize("mode", [0, 1])
def test_multiple_render_targets(ctxs, kw, mode):
    """Up to four colour attachments of mixed formats: output k of the
    G-buffer program into attachment k, blended per attachment."""
    g, o = ctxs
    g.set_raster_mode(mode)
    sg, so = render_both(E.mrt, g, o, **kw)
    compare_scenes(sg, so, f"mrt mode {mode}")


def test_mrt_rejections(gpu_lib):
    """A program writing more outputs than the framebuffer has attachments is
    rejected (the reference would call unset output functions); counts of
    attachments outside 1..4 are rejected as in SL_Framebuffer."""
    ctx = gpu_lib.Context()
    s = E.mrt(ctx, types=(A.COLOR_RGBA_8U, A.COLOR_RGBA_8U), num_outputs=3)
    with pytest.raises(A.SLError):
        ctx.draw(s.draws[0][0], s.draws[0][2], s.fbo)
    with pytest.raises(A.SLError):
        ctx.fbo_reserve_color_buffers(s.fbo, 5)
    with pytest.raises(A.SLError):
        ctx.fbo_reserve_color_buffers(s.fbo, 0)
    ctx.close()


@pytest.mark.parametrize("depth_type", [A.COLOR_R_HALF, A.COLOR_R_DOUBLE])
@pytest.mark.parametrize("depth_test", [A.DEPTH_TEST_LESS_THAN, A.DEPTH_TEST_LESS_EQUAL, A.DEPTH_TEST_GREATER_EQUAL,
                                        A.DEPTH_TEST_EQUAL, A.DEPTH_TEST_NOT_EQUAL])
def test_half_and_double_depth(ctxs, depth_type, depth_test):
    """R_HALF and R_DOUBLE depth attachments: compared as (float)depth,
    written as (depth_type)z; a half depth is re-read rounded after each
    write (ordered raster), a double depth keeps z exactly."""
    g, o = ctxs
    clear = 0.5 if depth_test in (A.DEPTH_TEST_GREATER_EQUAL, A.DEPTH_TEST_EQUAL, A.DEPTH_TEST_NOT_EQUAL) else 1.0
    sg, so = render_both(E.random_soup, g, o, depth_type=depth_type, depth_test=depth_test, clear_depth=clear,
                         num_tris=1500, width=320, height=240, frames=2)
    compare_scenes(sg, so, f"depth type {depth_type} test {depth_test}")


@pytest.mark.parametrize("depth_type", [A.COLOR_R_HALF, A.COLOR_R_DOUBLE])
def test_half_and_double_depth_other_primitives(ctxs, depth_type):
    g, o = ctxs
    for builder, kw in [(E.random_lines, dict(num_lines=2000, width=256, height=192, persp=True, seed=131)),
                        (E.random_soup, dict(wire=True, num_tris=800, width=200, height=150, seed=132)),
                        (E.random_soup, dict(blend=A.BLEND_ADDITIVE, num_tris=800, width=200, height=150, seed=133))]:
        sg, so = render_both(builder, g, o, depth_type=depth_type, **kw)
        compare_scenes(sg, so, f"{builder.__name__} depth type {depth_type}")


@pytest.mark.parametrize("batched", [False, True])
def test_vertex_cache_mixed_launch(ctxs, batched):
    """Batched, the five 16K-triangle sphere draws are served by the vertex
    cache in the same launch as the blended, non-indexed soup (which is not);
    one by one, each draw is below the cache's size threshold."""
    g, o = ctxs
    sg, so = render_both(E.multi_draw, g, o, batched=batched, lon=128, lat=64, width=320, height=240)
    compare_scenes(sg, so, f"cache mix batched={batched}")
    assert (sg.read_depth() < 1.0).sum() > 10000


@pytest.mark.parametrize("types", E.FORMAT_GROUPS, ids=[f"formats_{t[0]}_{t[-1]}" for t in E.FORMAT_GROUPS])
@pytest.mark.parametrize("blend", [A.BLEND_OFF, A.BLEND_ALPHA, A.BLEND_ADDITIVE])
def test_colour_formats(ctxs, types, blend):
    """All 33 colour formats (R / RG / RGB / RGBA of u8, u16, u32, u64, half,
    float, double; the five packed ones), four attachments per launch,
    attachment 0 included: written as color_cast<T, float> (rgba_cast for
    packed texels), blended through the format's read-back."""
    g, o = ctxs
    sg, so = render_both(E.mrt, g, o, types=types, blend=blend, num_tris=1200, width=200, height=150,
                         seed=150 + types[0], clear_color=(0.2, 0.4, 0.6, 0.8))
    compare_scenes(sg, so, f"formats {types} blend {blend}")


@pytest.mark.parametrize("color_type", range(33))
def test_format_edges(ctxs, color_type):
    """Out-of-range and NaN components (their conversions to unsigned follow
    the reference build), per format."""
    g, o = ctxs
    sg, so = render_both(E.format_edges, g, o, color_type=color_type, width=40, height=24)
    compare_scenes(sg, so, f"format edges {color_type}")


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("cull_fov", [None, 30.0])
def test_scene_graph(ctxs, mode, cull_fov):
    """A larger scene graph over five frames in both raster modes: model
    matrices bit for bit, images against the oracle."""
    g, o = ctxs
    g.set_raster_mode(mode)
    sg = S.build_scene_graph(g, width=640, height=480, groups=14, per_group=9, seed=44, cull_fov=cull_fov)
    so = S.build_scene_graph(o, width=640, height=480, groups=14, per_group=9, seed=44, cull_fov=cull_fov)
    for f in range(5):
        sg.render()
        so.render()
        mg, mo = sg.read_models(), so.read_models()
        assert np.array_equal(mg.view(np.uint32), mo.view(np.uint32)), f"frame {f}: model matrices differ"
        compare_scenes(sg, so, f"scene graph frame {f} cull {cull_fov} mode {mode}")


def test_scene_graph_grown_and_redrawn(ctxs):
    """Grows the graph between frames (the draw list is rebuilt), then draws
    over the previous frame without clearing, with the first and then a
    second template shader."""
    g, o = ctxs
    out = []
    for c in (g, o):
        s = S.build_scene_graph(c, groups=4, per_group=4, seed=9)
        s.render()
        c.scene_insert_node(s.scene, A.SCENE_ROOT, [0, 1], A.make_transform((0.0, -1.0, 2.0), (2.0, 2.0, 2.0)))
        s.num_nodes += 1
        s.render(clear=False)
        s.shader = s.add_shader(A.PROGRAM_LAMBERT_TEX, 2, S.lambert_uniforms(np.eye(4), np.eye(4), [0.0, 1.0, 0.0, 0.0],
                                                                           [0.3, 0.2, 0.1, 0.0], 0), cull=A.CULL_OFF)
        s.render(clear=False)
        out.append(s)
    assert np.array_equal(out[0].read_models().view(np.uint32), out[1].read_models().view(np.uint32))
    compare_scenes(out[0], out[1], "scene graph grown and redrawn")


def test_scene_graph_rejections(gpu_lib):
    ctx = gpu_lib.Context()
    s = S.build_scene_graph(ctx, groups=2, per_group=2)
    T = A.make_transform
    with pytest.raises(A.SLError, match="invalid parent"):
        ctx.scene_insert_node(s.scene, 10 ** 6, [], T())
    with pytest.raises(A.SLError, match="invalid submesh"):
        ctx.scene_insert_node(s.scene, A.SCENE_ROOT, [99], T())
    parent = A.SCENE_ROOT
    for _ in range(64):
        parent = ctx.scene_insert_node(s.scene, parent, [], T())
    with pytest.raises(A.SLError, match="at most 64"):
        ctx.scene_insert_node(s.scene, parent, [], T())
    flat = s.add_shader(A.PROGRAM_FLAT_COLOR, 0, S.flat_uniforms(np.eye(4), (1, 1, 1, 1)))
    with pytest.raises(A.SLError, match="LAMBERT_TEX"):
        ctx.scene_draw(s.scene, s.fbo, flat, np.eye(4), np.eye(4))
    ctx.close()


def test_uniform_block_reassigned_between_draws(ctxs):
    """Uniform blocks are uploaded in batches before the next launch: a block
    assigned twice (the second time partially) before a draw, and between
    draws of one frame, must draw what the last assignment holds."""
    g, o = ctxs
    out = []
    for c in (g, o):
        s = S.build_c1(c, width=160, height=120)
        ubo, ub = s.frame_ubos[0]
        s.render()
        moved = bytearray(ub)
        model = np.eye(4, dtype=np.float32)
        model[0, 3] = 0.35
        moved[64:128] = S.col_major(model).tobytes()
        c.ubo_assign(ubo, bytes(moved))
        c.ubo_assign(ubo, bytes(ub[:64]))             # vpMatrix only: the moved model matrix stays
        s.render(clear=False)
        c.ubo_assign(ubo, bytes(ub))
        s.render(clear=False)
        out.append(s)
    compare_scenes(out[0], out[1], "uniform blocks reassigned")


@pytest.mark.parametrize("depth_test,clear_depth", [(A.DEPTH_TEST_LESS_THAN, 1.0), (A.DEPTH_TEST_LESS_EQUAL, 1.0),
                                                    (A.DEPTH_TEST_GREATER_THAN, 0.0), (A.DEPTH_TEST_GREATER_EQUAL, 0.0)])
@pytest.mark.parametrize("spread", [1e-4, 1e-6])
def test_depth_bound_on_slivers(ctxs, depth_test, clear_depth, spread):
    """The ordered raster skips scan-lines whose depth bound cannot pass;
    near-degenerate slivers with depths packed within `spread` put the
    rounding of the walk's barycentrics at the test's edge. Two frames, so
    the second starts from a depth buffer the first wrote."""
    g, o = ctxs
    for seed in (121, 122):
        sg, so = render_both(E.sliver_soup, g, o, frames=2, seed=seed, depth_test=depth_test, clear_depth=clear_depth,
                             z_spread=spread)
        compare_scenes(sg, so, f"slivers {depth_test} spread {spread} seed {seed}")
