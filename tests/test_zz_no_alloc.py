"""slg_draw_noalloc, the draw whose scratch is one fixed device array, against
slg_draw on the same scenes: two no-allocation calls in a row, then slg_draw,
then one more no-allocation call, each frame compared with slg_draw's.
Tolerance: depth bit-exact (NaN matches NaN), RGBA8 colour within 1 LSB,
float colour within 1e-5 relative -- the same bar as the oracle parity tests.
The file name sorts last so that it also runs after every other GPU test."""
import numpy as np
import pytest

from softlight_gb300 import api as A
from softlight_gb300 import scenes as S

import edge_scenes as E

pytestmark = pytest.mark.gpu

MAX_TRIS = 1024   # SLG_NOALLOC_MAX_TRIANGLES
MAX_TILES = 64    # SLG_NOALLOC_MAX_TILES


@pytest.fixture()
def ctx(gpu_lib):
    c = gpu_lib.Context()
    yield c
    c.close()


def frame(scene, noalloc, visibility=False):
    """One frame drawn call by call; returns every colour attachment, the
    depth and (when enabled) the visibility map."""
    c = scene.ctx
    for k in range(len(scene.attachments)):
        c.clear_color_buffer(scene.fbo, k, scene.clear_color)
    c.clear_depth_buffer(scene.fbo, scene.clear_depth)
    for (mesh, n, shader) in scene.draws:
        assert n == 1
        if noalloc:
            c.draw_noalloc(mesh, shader, scene.fbo)
        else:
            c.draw(mesh, shader, scene.fbo)
    c.finish()
    vis = c.fbo_read_visibility(scene.fbo, (scene.height, scene.width)) if visibility else None
    return scene.read_colors(), scene.read_depth(), vis


def assert_color(cg, cw, label):
    if cg.dtype == np.uint8:
        diff = np.abs(cg.astype(np.int16) - cw.astype(np.int16))
        assert diff.max(initial=0) <= 1, f"{label}: colour differs by {diff.max()} LSB"
    else:
        scale = np.maximum(np.abs(cw), 1e-30)
        ok = (np.abs(cg - cw) <= 1e-5 * scale) | (cg == cw) | (np.isnan(cg) & np.isnan(cw))
        assert ok.all(), f"{label}: float colour differs"


def assert_same(got, want, label):
    cg, dg, vg = got
    cw, dw, vw = want
    bad = (dg.view(np.uint32) != dw.view(np.uint32)) & ~(np.isnan(dg) & np.isnan(dw))
    assert not bad.any(), f"{label}: {int(bad.sum())} depth texels differ"
    assert len(cg) == len(cw)
    for k, (a, b) in enumerate(zip(cg, cw)):
        assert_color(a, b, f"{label} attachment {k}")
    if vw is not None:
        assert np.array_equal(vg, vw), f"{label}: visibility map differs at {int((vg != vw).sum())} pixels"


def check_scene(scene, label, visibility=False):
    first = frame(scene, noalloc=True, visibility=visibility)
    second = frame(scene, noalloc=True, visibility=visibility)
    want = frame(scene, noalloc=False, visibility=visibility)
    third = frame(scene, noalloc=True, visibility=visibility)   # now with the context's uploaded resource tables
    scene.ctx.clear_framebuffer(scene.fbo, 0, scene.clear_color, scene.clear_depth)
    scene.ctx.finish()
    blank = scene.read_color()
    touched = np.any(want[0][0] != blank, axis=-1) if want[0][0].ndim == 3 else (want[0][0] != blank)
    assert touched.sum() > 100, f"{label}: scene covers too little"
    assert_same(first, want, f"{label} call 1")
    assert_same(second, want, f"{label} call 2")
    assert_same(third, want, f"{label} call 3")


def test_opaque_soup_with_clipping(ctx):
    s = E.random_soup(ctx, num_tris=MAX_TRIS, width=256, height=256, seed=31)
    check_scene(s, "opaque soup")


def test_blended_soup_ordered_path(ctx):
    s = E.random_soup(ctx, num_tris=600, width=200, height=160, seed=32,
                      blend=A.BLEND_ALPHA, depth_mask=A.DEPTH_MASK_OFF)
    check_scene(s, "blended soup")


def test_float_target(ctx):
    s = E.random_soup(ctx, num_tris=400, width=128, height=96, seed=33,
                      color_type=A.COLOR_RGBA_FLOAT, program=A.PROGRAM_VCOLOR_TEXF)
    check_scene(s, "float target")


def test_largest_framebuffer_at_64px_tiles(ctx):
    ctx.set_tile_size(64, 64)
    s = E.random_soup(ctx, num_tris=800, width=512, height=512, seed=34)
    check_scene(s, "512x512 at 64x64 tiles")


def test_limits_rejected_before_any_work(ctx):
    s = E.random_soup(ctx, num_tris=MAX_TRIS + 1, width=64, height=64, seed=35)
    c = s.ctx
    c.clear_framebuffer(s.fbo, 0, s.clear_color, s.clear_depth)
    mesh, _, shader = s.draws[0]
    with pytest.raises(A.SLError, match=str(MAX_TRIS)):
        c.draw_noalloc(mesh, shader, s.fbo)
    c.finish()
    assert (s.read_depth() == s.clear_depth).all()

    big = E.random_soup(ctx, num_tris=100, width=257, height=256, seed=36)  # 9 x 8 tiles of 32 x 32
    big.ctx.clear_framebuffer(big.fbo, 0, big.clear_color, big.clear_depth)
    big.ctx.finish()
    before = big.read_depth()   # 257 x 256 % 3 == 2: the reference's clear leaves the last texel
    mesh, _, shader = big.draws[0]
    with pytest.raises(A.SLError, match=str(MAX_TILES)):
        big.ctx.draw_noalloc(mesh, shader, big.fbo)
    big.ctx.finish()
    assert np.array_equal(big.read_depth(), before)


def test_lines(ctx):
    s = E.random_lines(ctx, num_lines=600, width=128, height=96, seed=37, persp=True)
    check_scene(s, "lines")


def test_blended_lines(ctx):
    s = E.random_lines(ctx, num_lines=500, width=128, height=96, seed=38, blend=A.BLEND_ALPHA)
    check_scene(s, "blended lines")


def test_wireframe(ctx):
    s = E.random_soup(ctx, num_tris=500, width=160, height=120, seed=39, wire=True)
    check_scene(s, "wireframe")


def test_points(ctx):
    s = E.random_points(ctx, num_points=1000, width=128, height=96, seed=40)
    check_scene(s, "points")


def test_multiple_render_targets(ctx):
    s = E.mrt(ctx, num_tris=500, width=128, height=96, seed=41)
    check_scene(s, "four render targets")


def test_visibility_map(ctx):
    s = E.random_soup(ctx, num_tris=MAX_TRIS, width=200, height=150, seed=42)
    ctx.fbo_enable_visibility(s.fbo, True)
    check_scene(s, "visibility map", visibility=True)
    # the checks slg_draw makes for a framebuffer with a visibility map
    blended = s.add_shader(A.PROGRAM_VCOLOR_TEX_ALPHA, 2, S.vcolor_uniforms(np.eye(4), 0), cull=A.CULL_OFF,
                           blend=A.BLEND_ALPHA)
    mesh = s.draws[0][0]
    for draw in (ctx.draw, ctx.draw_noalloc):
        with pytest.raises(A.SLError, match="opaque draws only"):
            draw(mesh, blended, s.fbo)
    ctx.finish()


def test_device_status_reported_at_finish(ctx):
    """A blended wireframe triangle whose pixels are revisited after 600
    queued fragments is reported at slg_finish (SLG_ERR_OVERFLOW), through
    draw_noalloc as through draw."""
    # 1024 x 64 pixels: 32 x 2 tiles of 32 x 32, the most the static scratch takes
    s = S.Scene(ctx, "wire_queue_small", 1024, 64)
    pts = [(30.0, 1.0), (994.0, 1.0), (515.0, 63.0)]
    verts = np.zeros((3, 9), np.float32)
    for i, (x, y) in enumerate(pts):
        verts[i, :3] = (2.0 * x / 1024 - 1.0, 2.0 * y / 64 - 1.0, 0.5)
    mesh = s.add_mesh(verts, None, stride=36)
    mesh.mode = A.RENDER_MODE_TRI_WIRE
    sh = s.add_shader(A.PROGRAM_FLAT_COLOR, 0, S.flat_uniforms(np.eye(4), (0.3, 0.2, 0.1, 0.5)),
                      cull=A.CULL_OFF, blend=A.BLEND_ADDITIVE)
    for draw in (ctx.draw, ctx.draw_noalloc, ctx.draw_noalloc):
        ctx.clear_framebuffer(s.fbo, 0, s.clear_color, s.clear_depth)
        draw(mesh, sh, s.fbo)
        with pytest.raises(A.SLError, match="600 queued fragments"):
            ctx.finish()
        ctx.finish()   # the status was cleared when it was reported
