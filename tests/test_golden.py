"""The CPU oracle against golden fixtures produced by SoftLight's own draw-path
sources (tests/golden/make_golden.py), and - where the reference tree is
present - against the reference build directly. These pin the oracle: the
fixtures are the reference's outputs on the same seeded inputs."""
import json
import os

import numpy as np
import pytest

import golden_scenes as G
from golden.make_golden import digest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _reference_available():
    import importlib.util
    spec = importlib.util.spec_from_file_location("ref_build", os.path.join(os.path.dirname(HERE), "oracle", "ref_build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.available()


REFERENCE_PRESENT = _reference_available()


def load(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    return d["color"], d["depth"]


def same(a, b):
    if a.dtype.kind == "f":
        bits = {2: np.uint16, 4: np.uint32, 8: np.uint64}[a.dtype.itemsize]
        return a.dtype == b.dtype and (np.array_equal(a.view(bits), b.view(bits)) or
                                       (np.array_equal(np.isnan(a), np.isnan(b)) and
                                        np.array_equal(np.where(np.isnan(a), 0, a).view(bits), np.where(np.isnan(b), 0, b).view(bits))))
    return np.array_equal(a, b)


def test_index_matches_fixtures():
    with open(os.path.join(GOLDEN, "index.json")) as fh:
        index = json.load(fh)
    assert set(index) == set(G.SCENES)
    for name, meta in index.items():
        c, d = load(name)
        assert digest(c) == meta["color_sha256"], name
        assert digest(d) == meta["depth_sha256"], name


@pytest.mark.parametrize("name", sorted(G.SCENES))
def test_oracle_matches_reference_golden(oracle_mod, name):
    builder, kw = G.SCENES[name]
    ctx = oracle_mod.Context()
    scene = builder(ctx, **kw)
    scene.render()
    gc, gd = load(name)
    c, d = scene.read_color(), scene.read_depth()
    assert same(d, gd), f"{name}: depth differs from the reference in {int((d != gd).sum())} texels"
    assert same(c, gc), f"{name}: colour differs from the reference"
    fixture = np.load(os.path.join(GOLDEN, name + ".npz"))
    for k in range(1, len(scene.attachments)):
        assert same(scene.read_color(k), fixture[f"color{k}"]), f"{name}: colour attachment {k} differs from the reference"
    ctx.close()


def test_oracle_blits_match_reference_golden(oracle_mod):
    """SL_Context::blit: scaled reads in every format pair, a rectangle blit
    and a whole-texture blit, against the reference's outputs."""
    want = np.load(os.path.join(GOLDEN, "blits.npz"))
    ctx = oracle_mod.Context()
    got = G.blit_cases(ctx)
    ctx.close()
    assert set(got) == set(want.files)
    for name in want.files:
        assert same(got[name], want[name]), f"blit {name} differs from the reference"


def test_oracle_scene_graph_matches_reference_golden(oracle_mod):
    """SL_SceneGraph::update and the mesh-node traversal over three frames
    (dirty propagation including a child the reference's update leaves
    stale, an FPS-view transform, a lines-mode submesh skipped, frustum
    culling): model matrices, colour and depth bit for bit against the
    reference's (tests/golden/scene_graph.npz)."""
    want = np.load(os.path.join(GOLDEN, "scene_graph.npz"))
    got = G.scene_graph_cases(oracle_mod.Context)
    assert set(got) == set(want.files)
    for name in want.files:
        assert same(got[name], want[name]), f"scene graph {name} differs from the reference"


def test_oracle_scene_graph_rejections(oracle_mod):
    """Bad ids, a non-Lambert shader and paths deeper than 64 nodes fail."""
    from softlight_gb300 import api as A
    from softlight_gb300 import scenes as S
    ctx = oracle_mod.Context()
    s = S.build_scene_graph(ctx, groups=2, per_group=2)
    T = A.make_transform
    with pytest.raises(A.SLError, match="invalid parent"):
        ctx.scene_insert_node(s.scene, 10 ** 6, [], T())
    with pytest.raises(A.SLError, match="invalid submesh"):
        ctx.scene_insert_node(s.scene, A.SCENE_ROOT, [99], T())
    with pytest.raises(A.SLError, match="invalid scene"):
        ctx.scene_update(77)
    with pytest.raises(A.SLError, match="unknown transform type"):
        ctx.scene_insert_node(s.scene, A.SCENE_ROOT, [], T(type=9))
    parent = A.SCENE_ROOT
    for _ in range(64):
        parent = ctx.scene_insert_node(s.scene, parent, [], T())
    with pytest.raises(A.SLError, match="at most 64"):
        ctx.scene_insert_node(s.scene, parent, [], T())
    flat = s.add_shader(A.PROGRAM_FLAT_COLOR, 0, S.flat_uniforms(np.eye(4), (1, 1, 1, 1)))
    with pytest.raises(A.SLError, match="LAMBERT_TEX"):
        ctx.scene_draw(s.scene, s.fbo, flat, np.eye(4), np.eye(4))
    ctx.close()


@pytest.mark.skipif(not REFERENCE_PRESENT, reason="reference tree not present")
def test_reference_scene_graph_matches_oracle_live(oracle_mod):
    """The reference's SL_SceneGraph, SL_Transform and sl_is_visible, built
    from its sources, against the oracle on a larger graph over four frames."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import ref_build
    from softlight_gb300.api import SLContext, open_library
    from softlight_gb300 import scenes as S
    lib = open_library(ref_build.build_ref(), "slr_", gpu=False)
    r = SLContext(lib, "slr_", gpu=False)
    o = oracle_mod.Context()
    sr = S.build_scene_graph(r, groups=9, per_group=7, seed=33, cull_fov=30.0)
    so = S.build_scene_graph(o, groups=9, per_group=7, seed=33, cull_fov=30.0)
    for _ in range(4):
        sr.render()
        so.render()
        assert same(sr.read_models(), so.read_models())
        assert same(sr.read_depth(), so.read_depth())
        assert same(sr.read_color(), so.read_color())


@pytest.mark.parametrize("threads", [2, 5])
def test_oracle_threads_match_one_thread(oracle_mod, threads):
    """The oracle's multi-threaded mode (used for the CPU baseline timing)
    reproduces the one-thread result."""
    from softlight_gb300 import scenes as S
    ref = oracle_mod.Context(num_threads=1)
    par = oracle_mod.Context(num_threads=threads)
    a = S.build_c2(ref, num_instances=4, width=200, height=120, tex_size=64)
    b = S.build_c2(par, num_instances=4, width=200, height=120, tex_size=64)
    a.render()
    b.render()
    assert np.array_equal(a.read_color(), b.read_color())
    assert same(a.read_depth(), b.read_depth())


@pytest.mark.skipif(not REFERENCE_PRESENT, reason="reference tree not present")
@pytest.mark.parametrize("name", ["c1_sphere_160x120", "c3_soup_2000_160x96", "multi_draw", "soup_not_equal",
                                  "lines_persp_clip_cull", "line_alias"])
def test_reference_build_matches_oracle_live(oracle_mod, name):
    """Builds the reference sources (oracle/ref_build.py) and renders live."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import ref_build
    from softlight_gb300.api import SLContext, open_library
    lib = open_library(ref_build.build_ref(), "slr_", gpu=False)
    builder, kw = G.SCENES[name]
    r = SLContext(lib, "slr_", gpu=False)
    o = oracle_mod.Context()
    sr, so = builder(r, **kw), builder(o, **kw)
    sr.render()
    so.render()
    assert same(sr.read_depth(), so.read_depth())
    assert same(sr.read_color(), so.read_color())
