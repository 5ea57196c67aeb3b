"""The CUDA draw path, through the C ABI, against golden fixtures produced by
SoftLight's own draw-path sources (tests/golden). Depth bit-exact (NaN
payloads aside), colour within 1 LSB / 1e-5 relative; each scene runs with
both raster strategies and two tile sizes."""
import os

import numpy as np
import pytest

import golden_scenes as G
from parity import compare_colors

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", sorted(G.SCENES))
@pytest.mark.parametrize("mode,tile", [(0, (16, 16)), (1, (32, 32)), (3, (8, 8))])
def test_gpu_matches_reference_golden(gpu_lib, name, mode, tile):
    builder, kw = G.SCENES[name]
    ctx = gpu_lib.Context()
    ctx.set_raster_mode(mode)
    ctx.set_tile_size(*tile)
    scene = builder(ctx, **kw)
    if name in G.GPU_REPORTED:
        from softlight_gb300 import api as A
        with pytest.raises(A.SLError, match=G.GPU_REPORTED[name]):
            scene.render()
            ctx.finish()
        ctx.close()
        return
    scene.render()
    ctx.finish()
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    gd = d["depth"]
    dd = scene.read_depth()
    bits = {2: np.uint16, 4: np.uint32, 8: np.uint64}[dd.dtype.itemsize]
    bad = (dd.view(bits) != gd.view(bits)) & ~(np.isnan(dd) & np.isnan(gd))
    assert not bad.any(), f"{name}: {int(bad.sum())} depth texels differ from the reference"
    for k in range(len(scene.attachments)):
        compare_colors(scene.read_color(k), d["color" if k == 0 else f"color{k}"], f"{name} attachment {k}")
    ctx.close()


def test_gpu_blits_match_reference_golden(gpu_lib):
    """SL_Context::blit on the GPU: scaled reads in every format pair, a
    rectangle blit into a patterned texture and a whole-texture blit, bit for
    bit against the reference's outputs (tests/golden/blits.npz)."""
    want = np.load(os.path.join(GOLDEN, "blits.npz"))
    ctx = gpu_lib.Context()
    got = G.blit_cases(ctx)
    ctx.close()
    assert set(got) == set(want.files)
    for name in want.files:
        a, b = got[name], want[name]
        same = np.array_equal(a.view(np.uint8), b.view(np.uint8)) or (
            a.dtype == np.float32 and np.array_equal(np.isnan(a), np.isnan(b))
            and np.array_equal(np.nan_to_num(a), np.nan_to_num(b)))
        assert same, f"blit {name} differs from the reference"


@pytest.mark.parametrize("mode,tile", [(0, (16, 16)), (1, (32, 32)), (3, (8, 8))])
def test_gpu_scene_graph_matches_reference_golden(gpu_lib, mode, tile):
    """SL_SceneGraph::update and the mesh-node traversal on the GPU (update
    kernel, draw-list kernel, one batched launch per frame): model matrices,
    colour and depth bit for bit against the reference's three frames
    (tests/golden/scene_graph.npz), in three raster configurations."""
    want = np.load(os.path.join(GOLDEN, "scene_graph.npz"))

    def make_ctx():
        c = gpu_lib.Context()
        c.set_raster_mode(mode)
        c.set_tile_size(*tile)
        return c
    got = G.scene_graph_cases(make_ctx)
    assert set(got) == set(want.files)
    for name in want.files:
        a, b = got[name], want[name]
        assert a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8)), f"scene graph {name} differs from the reference"


def test_gpu_blit_rejects_out_of_bounds_rectangles(gpu_lib):
    from softlight_gb300 import api as A
    ctx = gpu_lib.Context()
    t = ctx.create_texture()
    ctx.texture_init(t, A.COLOR_RGBA_8U, 32, 32, 1)
    u = ctx.create_texture()
    ctx.texture_init(u, A.COLOR_RGBA_8U, 16, 16, 1)
    with pytest.raises(A.SLError, match="below the destination"):
        ctx.blit_rect(u, t, (0, 0, 32, 32), (0, 0, 16, 17))
    with pytest.raises(A.SLError, match="reads outside"):
        ctx.blit_rect(u, t, (0, 0, 32, 40), (0, 0, 16, 16))
    with pytest.raises(A.SLError, match="inverted"):
        ctx.blit_rect(u, t, (8, 0, 4, 32), (0, 0, 16, 16))
    with pytest.raises(A.SLError, match="same texture"):
        ctx.blit(t, t)
    ctx.close()
