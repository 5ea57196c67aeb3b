"""Workloads with golden fixtures (tests/golden/*.npz): reduced-size versions
of the benchmark configurations plus the edge-case scenes, small enough that
the fixtures stay a few hundred KB and the CPU oracle renders each in well
under a second."""
import numpy as np

from softlight_gb300 import api as A
from softlight_gb300 import scenes as S

import edge_scenes as E

SCENES = {
    "c1_sphere_160x120": (S.build_c1, dict(width=160, height=120)),
    "c2_instanced_32_240x136": (S.build_c2, dict(num_instances=32, width=240, height=136, tex_size=128)),
    "c3_soup_2000_160x96": (S.build_c3, dict(num_tris=2000, width=160, height=96, tex_size=128)),
    "c4_batch_10_192x108": (S.build_c4, dict(num_draws=10, width=192, height=108, tex_size=32)),
    "soup_depth_off_mask_on": (E.random_soup, dict(depth_test=A.DEPTH_TEST_OFF, depth_mask=1, clear_depth=0.5, num_tris=500)),
    "soup_less_equal_mask_off": (E.random_soup, dict(depth_test=A.DEPTH_TEST_LESS_EQUAL, depth_mask=0, clear_depth=0.999)),
    "soup_greater_mask_on": (E.random_soup, dict(depth_test=A.DEPTH_TEST_GREATER_THAN, depth_mask=1, clear_depth=0.0)),
    "soup_not_equal": (E.random_soup, dict(depth_test=A.DEPTH_TEST_NOT_EQUAL, depth_mask=1, clear_depth=0.999)),
    "soup_blend_premultiplied": (E.random_soup, dict(blend=A.BLEND_PREMULTIPLED_ALPHA)),
    "soup_blend_additive_float": (E.random_soup, dict(blend=A.BLEND_ADDITIVE, color_type=A.COLOR_RGBA_FLOAT)),
    "soup_blend_screen": (E.random_soup, dict(blend=A.BLEND_SCREEN)),
    "soup_cull_front": (E.random_soup, dict(cull=A.CULL_FRONT_FACE)),
    "soup_cull_off_u16": (E.random_soup, dict(cull=A.CULL_OFF, indexed=np.uint16, num_tris=120)),
    "soup_texf": (E.random_soup, dict(program=A.PROGRAM_VCOLOR_TEXF, color_type=A.COLOR_RGBA_FLOAT)),
    "big_triangles": (E.big_triangles, dict()),
    "multi_draw": (E.multi_draw, dict()),
    "flat_triangle": (E.flat_triangle, dict(width=128, height=96)),
    "points_less": (E.random_points, dict()),
    "points_blend_alpha": (E.random_points, dict(blend=A.BLEND_ALPHA, depth_mask=A.DEPTH_MASK_OFF, seed=42)),
    "points_u16_depth_off": (E.random_points, dict(indexed=np.uint16, depth_test=A.DEPTH_TEST_OFF, seed=43)),
    "points_gequal_float": (E.random_points, dict(depth_test=A.DEPTH_TEST_GREATER_EQUAL, clear_depth=-1.0,
                                                  color_type=A.COLOR_RGBA_FLOAT, seed=44)),
    "points_not_equal": (E.random_points, dict(depth_test=A.DEPTH_TEST_NOT_EQUAL, clear_depth=0.5, seed=45)),
    "point_edges": (E.point_edges, dict()),
    "lines_less": (E.random_lines, dict()),
    "lines_persp_clip_cull": (E.random_lines, dict(persp=True, seed=62, num_lines=1500, width=120, height=80)),
    "lines_blend_alpha": (E.random_lines, dict(blend=A.BLEND_ALPHA, depth_mask=A.DEPTH_MASK_OFF, seed=63)),
    "lines_u16_gequal_float": (E.random_lines, dict(indexed=np.uint16, depth_test=A.DEPTH_TEST_GREATER_EQUAL,
                                                    clear_depth=-1.0, color_type=A.COLOR_RGBA_FLOAT, seed=64)),
    "lines_instanced_odd_end": (E.random_lines, dict(num_instances=3, seed=65, odd_end=True)),
    "lines_not_equal_700x40": (E.random_lines, dict(depth_test=A.DEPTH_TEST_NOT_EQUAL, clear_depth=0.5, seed=66,
                                                    num_lines=3000, width=700, height=40)),
    "line_edges": (E.line_edges, dict()),
    "line_alias": (E.line_alias, dict()),
    "line_alias_wide_occluded": (E.line_alias_wide, dict(occluded=True)),
    "line_alias_wide_open": (E.line_alias_wide, dict(occluded=False)),
    "line_alias_wide_occluded_blend": (E.line_alias_wide, dict(occluded=True, blend=A.BLEND_ALPHA)),
    "wire_soup_less": (E.random_soup, dict(wire=True)),
    "wire_soup_u16_cull_off": (E.random_soup, dict(wire=True, cull=A.CULL_OFF, indexed=np.uint16, num_tris=120, seed=12)),
    "wire_soup_blend_alpha": (E.random_soup, dict(wire=True, blend=A.BLEND_ALPHA, seed=13)),
    "wire_soup_not_equal": (E.random_soup, dict(wire=True, depth_test=A.DEPTH_TEST_NOT_EQUAL, clear_depth=0.5, seed=14)),
    "wire_soup_instanced_float": (E.random_soup, dict(wire=True, num_instances=2, color_type=A.COLOR_RGBA_FLOAT, seed=15)),
    "wire_big_triangles": (E.big_triangles, dict(wire=True)),
    "wire_big_blend_additive": (E.big_triangles, dict(wire=True, blend=A.BLEND_ADDITIVE)),
    "wire_queue_additive": (E.wire_queue, dict()),
    "mrt_4_mixed_formats": (E.mrt, dict()),
    "mrt_3_blend_alpha": (E.mrt, dict(types=(A.COLOR_RGBA_8U, A.COLOR_RGBA_8U, A.COLOR_RGBA_FLOAT), num_outputs=3,
                                      blend=A.BLEND_ALPHA, seed=102)),
    "mrt_2_of_3_then_single": (E.mrt, dict(types=(A.COLOR_RGBA_8U, A.COLOR_RGBA_FLOAT, A.COLOR_R_FLOAT), num_outputs=2,
                                           seed=103, single_after=True)),
    "mrt_wire_additive": (E.mrt, dict(prim="wire", blend=A.BLEND_ADDITIVE, seed=104)),
    "mrt_lines": (E.mrt, dict(prim="line", types=(A.COLOR_RGBA_8U, A.COLOR_RGBA_FLOAT), num_outputs=2, seed=105)),
    "mrt_points_premultiplied": (E.mrt, dict(prim="point", blend=A.BLEND_PREMULTIPLED_ALPHA, seed=106, num_tris=2000)),
    "soup_half_depth_less": (E.random_soup, dict(depth_type=A.COLOR_R_HALF)),
    "soup_half_depth_lequal": (E.random_soup, dict(depth_type=A.COLOR_R_HALF, depth_test=A.DEPTH_TEST_LESS_EQUAL, seed=21)),
    "soup_half_depth_not_equal_blend": (E.random_soup, dict(depth_type=A.COLOR_R_HALF, depth_test=A.DEPTH_TEST_NOT_EQUAL,
                                                            clear_depth=0.5, blend=A.BLEND_ALPHA, seed=22)),
    "soup_double_depth_greater": (E.random_soup, dict(depth_type=A.COLOR_R_DOUBLE, depth_test=A.DEPTH_TEST_GREATER_THAN,
                                                      clear_depth=0.1, seed=23)),
    "wire_double_depth": (E.random_soup, dict(depth_type=A.COLOR_R_DOUBLE, wire=True, seed=24)),
    "lines_half_depth": (E.random_lines, dict(depth_type=A.COLOR_R_HALF, seed=25)),
    # fragment programs that discard (SL_FragmentShader returning false: no
    # colour, depth still written) and that read / write SL_FragCoordXYZ
    "cutout_soup": (E.program_soup, dict(program=A.PROGRAM_VCOLOR_TEX_CUTOUT)),
    "cutout_soup_blend_alpha": (E.program_soup, dict(program=A.PROGRAM_VCOLOR_TEX_CUTOUT, blend=A.BLEND_ALPHA, seed=52)),
    "cutout_soup_depth_off": (E.program_soup, dict(program=A.PROGRAM_VCOLOR_TEX_CUTOUT, depth_test=A.DEPTH_TEST_OFF,
                                                   alpha_ref=0.2, seed=53)),
    "cutout_wire": (E.program_soup, dict(program=A.PROGRAM_VCOLOR_TEX_CUTOUT, prim="wire", seed=54)),
    "cutout_lines_instanced": (E.program_soup, dict(program=A.PROGRAM_VCOLOR_TEX_CUTOUT, prim="line", seed=55,
                                                    num_instances=2)),
    "cutout_points": (E.program_soup, dict(program=A.PROGRAM_VCOLOR_TEX_CUTOUT, prim="point", seed=56, num_tris=1000)),
    "fragcoord_soup_float": (E.program_soup, dict(program=A.PROGRAM_FRAG_COORD, color_type=A.COLOR_RGBA_FLOAT, seed=57)),
    "fragcoord_soup_greater_nodoor": (E.program_soup, dict(program=A.PROGRAM_FRAG_COORD, depth_test=A.DEPTH_TEST_GREATER_THAN,
                                                           clear_depth=-1.0, screen_door=0, depth_scale=-1.0,
                                                           depth_bias=0.0, seed=58)),
    "fragcoord_wire_half_depth": (E.program_soup, dict(program=A.PROGRAM_FRAG_COORD, prim="wire", depth_type=A.COLOR_R_HALF,
                                                       seed=59)),
    "fragcoord_lines_float": (E.program_soup, dict(program=A.PROGRAM_FRAG_COORD, prim="line", color_type=A.COLOR_RGBA_FLOAT,
                                                   seed=60)),
    "fragcoord_points_float": (E.program_soup, dict(program=A.PROGRAM_FRAG_COORD, prim="point", color_type=A.COLOR_RGBA_FLOAT,
                                                    seed=61, num_tris=1000)),
    # draw_multiple over meshes with overlapping primIndex ranges: blended,
    # the reference's 1024-bin flush groups are sorted by primIndex
    "multi_mesh_blend_alpha": (E.multi_mesh, dict()),
    "multi_mesh_blend_additive_le": (E.multi_mesh, dict(blend=A.BLEND_ADDITIVE, depth_test=A.DEPTH_TEST_LESS_EQUAL, seed=92,
                                                        num_meshes=4, num_tris=500)),
    "multi_mesh_wire_blend": (E.multi_mesh, dict(modes=(A.RENDER_MODE_TRI_WIRE, A.RENDER_MODE_TRI_WIRE, A.RENDER_MODE_TRI_WIRE),
                                                 seed=93)),
    "multi_mesh_mixed_modes_blend": (E.multi_mesh, dict(modes=(A.RENDER_MODE_TRIANGLES, A.RENDER_MODE_INDEXED_TRI_WIRE,
                                                               A.RENDER_MODE_INDEXED_TRIANGLES), seed=94)),
    "multi_mesh_opaque": (E.multi_mesh, dict(blend=A.BLEND_OFF, seed=95)),
}

# every colour format: four per scene through the G-buffer program, unblended
# and alpha-blended over a clear colour, and the out-of-range / NaN writes
for _g, _types in enumerate(E.FORMAT_GROUPS):
    for _blend, _bname in [(A.BLEND_OFF, "opaque"), (A.BLEND_ALPHA, "alpha")]:
        SCENES[f"formats_{_types[0]}_{_types[-1]}_{_bname}"] = (
            E.mrt, dict(types=_types, num_outputs=4, blend=_blend, seed=140 + _types[0], width=48, height=40,
                        num_tris=120, clear_color=(0.2, 0.4, 0.6, 0.8)))
for _t in range(33):
    SCENES[f"format_edges_{_t}"] = (E.format_edges, dict(color_type=_t))

# Scenes whose draws the GPU path reports as not reproduced (SLError at
# finish), with the reason: a blended wireframe triangle revisits a pixel
# after 600 queued fragments (the reference's queue flush points).
GPU_REPORTED = {
    "wire_queue_additive": "queue flush order",
}



# (name, source: "color" | "depth" | "colorf", destination type, width, height)
BLIT_READS = [
    ("rgba8_to_rgba8_80x50", "color", A.COLOR_RGBA_8U, 80, 50),
    ("rgba8_to_rgbaf_213x97", "color", A.COLOR_RGBA_FLOAT, 213, 97),
    ("rgba8_to_rf_100x75", "color", A.COLOR_R_FLOAT, 100, 75),
    ("rf_to_rgba8_160x120", "depth", A.COLOR_RGBA_8U, 160, 120),
    ("rf_to_rgbaf_57x33", "depth", A.COLOR_RGBA_FLOAT, 57, 33),
    ("rf_to_rf_320x240", "depth", A.COLOR_R_FLOAT, 320, 240),
    ("rgbaf_to_rgba8_120x90", "colorf", A.COLOR_RGBA_8U, 120, 90),
    ("rgbaf_to_rf_96x80", "colorf", A.COLOR_R_FLOAT, 96, 80),
    ("rgbaf_to_rgbaf_50x40", "colorf", A.COLOR_RGBA_FLOAT, 50, 40),
]


def blit_cases(ctx):
    """Blits (SL_Context::blit) of rendered attachments through ctx: scaled
    reads into host buffers of every supported format, a rectangle blit into
    a patterned texture and a whole-texture blit. Returns {name: array}."""
    out = {}
    s = S.build_c1(ctx, width=160, height=120)
    s.render()
    f = E.random_soup(ctx, program=A.PROGRAM_VCOLOR_TEXF, color_type=A.COLOR_RGBA_FLOAT)
    f.render()
    src = {"color": s.color_tex, "depth": s.depth_tex, "colorf": f.color_tex}
    for name, which, ctype, w, h in BLIT_READS:
        out[name] = ctx.blit_read(src[which], ctype, w, h)

    dst = ctx.create_texture()
    ctx.texture_init(dst, A.COLOR_RGBA_8U, 200, 150, 1)
    ctx.texture_set_texels(dst, (np.arange(200 * 150 * 4) % 251).astype(np.uint8).reshape(150, 200, 4))
    ctx.blit_rect(dst, s.color_tex, (10, 5, 150, 100), (20, 30, 180, 140))
    out["rect_rgba8_into_pattern"] = ctx.texture_read(dst, (150, 200, 4), np.uint8)

    dstf = ctx.create_texture()
    ctx.texture_init(dstf, A.COLOR_RGBA_FLOAT, 64, 48, 1)
    ctx.texture_set_texels(dstf, np.full((48, 64, 4), 0.25, np.float32))
    ctx.blit(dstf, s.depth_tex)
    out["whole_rf_to_rgbaf_64x48"] = ctx.texture_read(dstf, (48, 64, 4), np.float32)
    return out


# The scene graph (SL_SceneGraph): three frames of build_scene_graph, culled
# against a 40-degree frustum and unculled; per frame the model matrices,
# colour and depth.
SCENE_GRAPH_VARIANTS = {"cull40": 40.0, "nocull": None}
SCENE_GRAPH_FRAMES = 3


def scene_graph_cases(make_ctx):
    """{variant}_{models,color,depth}_f{k} arrays, one new context per variant."""
    from softlight_gb300 import scenes as S
    out = {}
    for variant, fov in SCENE_GRAPH_VARIANTS.items():
        ctx = make_ctx()
        scene = S.build_scene_graph(ctx, cull_fov=fov)
        for k in range(SCENE_GRAPH_FRAMES):
            scene.render()
            out[f"{variant}_models_f{k}"] = scene.read_models()
            out[f"{variant}_color_f{k}"] = scene.read_color()
            out[f"{variant}_depth_f{k}"] = scene.read_depth()
        ctx.close()
    return out
