"""Workloads with golden fixtures (tests/golden/*.npz): reduced-size versions
of the BASELINE configurations plus the edge-case scenes, small enough that
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
}
