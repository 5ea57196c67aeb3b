"""The CUDA draw path, through the C ABI, against golden fixtures produced by
SoftLight's own draw-path sources (tests/golden). Depth bit-exact (NaN
payloads aside), colour within 1 LSB / 1e-5 relative; each scene runs with
both raster strategies and two tile sizes."""
import os

import numpy as np
import pytest

import golden_scenes as G

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", sorted(G.SCENES))
@pytest.mark.parametrize("mode,tile", [(0, (16, 16)), (1, (32, 32)), (0, (8, 8))])
def test_gpu_matches_reference_golden(gpu_lib, name, mode, tile):
    builder, kw = G.SCENES[name]
    ctx = gpu_lib.Context()
    ctx.set_raster_mode(mode)
    ctx.set_tile_size(*tile)
    scene = builder(ctx, **kw)
    scene.render()
    ctx.finish()
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    gc, gd = d["color"], d["depth"]
    c, dd = scene.read_color(), scene.read_depth()
    bad = (dd.view(np.uint32) != gd.view(np.uint32)) & ~(np.isnan(dd) & np.isnan(gd))
    assert not bad.any(), f"{name}: {int(bad.sum())} depth texels differ from the reference"
    if c.dtype == np.uint8:
        diff = np.abs(c.astype(np.int16) - gc.astype(np.int16)).max(initial=0)
        assert diff <= 1, f"{name}: colour differs by {diff} LSB"
    else:
        ok = (np.abs(c - gc) <= 1e-5 * np.maximum(np.abs(gc), 1e-30)) | (c == gc) | (np.isnan(c) & np.isnan(gc))
        assert ok.all(), f"{name}: float colour differs"
    ctx.close()
