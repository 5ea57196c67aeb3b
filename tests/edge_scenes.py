"""Small seeded workloads for edge cases of the draw path (test-only)."""
import math

import numpy as np

from softlight_gb300 import api as A
from softlight_gb300 import scenes as S


def random_soup(ctx, num_tris=300, width=96, height=80, seed=11, blend=A.BLEND_OFF,
                depth_test=A.DEPTH_TEST_LESS_THAN, depth_mask=A.DEPTH_MASK_ON, cull=A.CULL_BACK_FACE,
                color_type=A.COLOR_RGBA_8U, program=A.PROGRAM_VCOLOR_TEX_ALPHA, indexed=None, clear_depth=1.0,
                max_area=None, wire=False, num_instances=1, depth_type=A.COLOR_R_FLOAT):
    """Triangle soup like the c3 workload at a small size, with the pipeline
    state as parameters. indexed: None (non-indexed) or a numpy index dtype;
    wire: draw the triangles as wireframe (SL_RENDER_MODE_[INDEXED_]TRI_WIRE)."""
    s = S.Scene(ctx, f"soup_{seed}", width, height, color_type=color_type, depth_type=depth_type)
    verts, proj = S.soup_triangles(num_tris, width, height, seed=seed)
    if max_area is not None:
        pass
    if indexed is None:
        mesh = s.add_mesh(verts, None, stride=36)
    else:
        n = verts.shape[0]
        perm = np.random.default_rng(seed + 1).permutation(n)
        inv = np.empty_like(perm)
        inv[perm] = np.arange(n)
        shuffled = verts[perm]
        idx = inv.astype(indexed)
        if np.dtype(indexed).itemsize == 1:
            assert n <= 256
        mesh = s.add_mesh(shuffled, idx, stride=36)
    if program == A.PROGRAM_VCOLOR_TEXF:
        tex = s.add_texture_rgbaf(S.value_noise(64, 64, seed=seed, octaves=2).astype(np.float32))
    else:
        tex = s.add_texture_rgba8(S.to_rgba8(S.value_noise(64, 64, seed=seed, octaves=2, alpha=1.0)))
    if wire:
        mesh.mode = A.RENDER_MODE_TRI_WIRE if indexed is None else A.RENDER_MODE_INDEXED_TRI_WIRE
    ub = S.vcolor_uniforms(proj, tex)
    sh = s.add_shader(program, 2, ub, cull=cull, depth_test=depth_test, depth_mask=depth_mask, blend=blend)
    s.draws.append((mesh, num_instances, sh))
    s.num_triangles = num_tris
    s.clear_depth = clear_depth
    return s


def big_triangles(ctx, width=300, height=200, seed=5, wire=False, blend=A.BLEND_OFF):
    """A few triangles spanning many tiles (long catch-up chains), one of
    them screen-filling, plus equal-depth overlaps (order ties); optionally
    as wireframe."""
    s = S.Scene(ctx, "big", width, height)
    rng = np.random.default_rng(seed)
    tris = []
    for k in range(6):
        z = -5.0 if k < 3 else -5.0 - k
        p = rng.uniform(-6, 6, (3, 2))
        tris.append([(p[0, 0], p[0, 1], z), (p[1, 0], p[1, 1], z), (p[2, 0], p[2, 1], z)])
    tris.append([(-50, -50, -8.0), (50, -50, -8.0), (0, 60, -8.0)])
    verts = []
    for t in tris:
        c = rng.uniform(0.2, 1.0, 4)
        for v in t:
            verts.append([*v, *c, *rng.uniform(0, 1, 2)])
    verts = np.asarray(verts, dtype=np.float32)
    mesh = s.add_mesh(verts, None, stride=36)
    tex = s.add_texture_rgba8(S.checker(32, 32, 4))
    proj = S.perspective(60.0, width / height, 0.1, 100.0)
    if wire:
        mesh.mode = A.RENDER_MODE_TRI_WIRE
    sh = s.add_shader(A.PROGRAM_VCOLOR_TEX_ALPHA, 2, S.vcolor_uniforms(proj, tex), cull=A.CULL_OFF, blend=blend)
    s.draws.append((mesh, 1, sh))
    s.num_triangles = len(tris)
    return s


def multi_draw(ctx, width=128, height=96, batched=False, seed=21, lon=16, lat=8):
    """Several draws with different programs and depth states into one frame,
    issued one by one or as one batch (lon x lat sphere segments)."""
    s = S.Scene(ctx, "multi", width, height)
    verts, idx = S.uv_sphere(lon, lat)
    sphere = s.add_mesh(verts, idx)
    tex = s.add_texture_rgba8(S.checker(64, 64, 8))
    vp = S.perspective(60.0, width / height, 0.1, 100.0) @ S.look_at((0, 0, 6), (0, 0, 0), (0, 1, 0))
    light = np.asarray([0.2, 0.9, 0.4]) / np.linalg.norm([0.2, 0.9, 0.4])
    rng = np.random.default_rng(seed)
    for k in range(5):
        model = S.translate(rng.uniform(-2, 2, 3)) @ S.random_rotation(rng) @ S.scale(rng.uniform(0.5, 1.5))
        ub = S.lambert_uniforms(vp, model, [*light, 0.0], [0.1, 0.1, 0.1, 0.0], tex)
        sh = s.add_shader(A.PROGRAM_LAMBERT_TEX, 2, ub,
                          depth_test=(A.DEPTH_TEST_LESS_THAN, A.DEPTH_TEST_LESS_EQUAL)[k % 2])
        s.draws.append((sphere, 1, sh))
    soup, proj = S.soup_triangles(60, width, height, seed=seed)
    mesh = s.add_mesh(soup, None, stride=36)
    sh = s.add_shader(A.PROGRAM_VCOLOR_TEX_ALPHA, 2, S.vcolor_uniforms(proj, tex), blend=A.BLEND_ALPHA)
    s.draws.append((mesh, 1, sh))
    s.batched = batched
    return s


def flat_triangle(ctx, width=640, height=480):
    """The reference's headless draw test scene shape: one triangle, flat colour,
    depth test off (softlight/tests/sl_draw_test.cpp:108-194)."""
    s = S.Scene(ctx, "flat", width, height)
    verts = np.asarray([[-0.9, -0.9, 0.0, 0, 0, 0, 0, 0, 0],
                        [0.9, -0.9, 0.0, 0, 0, 0, 0, 0, 0],
                        [0.0, 0.9, 0.0, 0, 0, 0, 0, 0, 0]], dtype=np.float32)
    mesh = s.add_mesh(verts, None, stride=36)
    sh = s.add_shader(A.PROGRAM_FLAT_COLOR, 0, S.flat_uniforms(np.eye(4), (1.0, 0.5, 0.25, 1.0)),
                      cull=A.CULL_OFF, depth_test=A.DEPTH_TEST_OFF, depth_mask=A.DEPTH_MASK_OFF)
    s.draws.append((mesh, 1, sh))
    return s


def random_points(ctx, num_points=3000, width=64, height=48, seed=41, blend=A.BLEND_OFF,
                  depth_test=A.DEPTH_TEST_LESS_THAN, depth_mask=A.DEPTH_MASK_ON, indexed=None,
                  color_type=A.COLOR_RGBA_8U, clear_depth=1.0, num_instances=1):
    """Point draw (SL_RENDER_MODE_POINTS): seeded points in and around the
    view volume, dense enough that many share a pixel; vertex colour x RGBA8
    texture program with vertex alpha."""
    rng = np.random.default_rng(seed)
    s = S.Scene(ctx, f"points_{seed}", width, height, color_type=color_type)
    pos = np.stack([rng.uniform(-1.3, 1.3, num_points), rng.uniform(-1.3, 1.3, num_points),
                    rng.uniform(-1.2, 1.2, num_points)], 1)
    col = np.concatenate([rng.uniform(0.0, 1.0, (num_points, 3)), rng.uniform(0.2, 1.0, (num_points, 1))], 1)
    uv = rng.uniform(-0.5, 1.5, (num_points, 2))
    verts = np.concatenate([pos, col, uv], 1).astype(np.float32)
    tex = s.add_texture_rgba8(S.to_rgba8(S.value_noise(32, 32, seed=seed, octaves=2, alpha=1.0)))
    if indexed is None:
        mesh = s.add_mesh(verts, None, stride=36)
        mesh.mode = A.RENDER_MODE_POINTS
    else:
        order = rng.permutation(num_points)
        mesh = s.add_mesh(verts, order.astype(indexed), stride=36)
        mesh.mode = A.RENDER_MODE_INDEXED_POINTS
    sh = s.add_shader(A.PROGRAM_VCOLOR_TEX_ALPHA, 2, S.vcolor_uniforms(np.eye(4), tex), cull=A.CULL_OFF,
                      depth_test=depth_test, depth_mask=depth_mask, blend=blend)
    s.draws.append((mesh, num_instances, sh))
    s.num_triangles = num_points
    s.clear_depth = clear_depth
    return s


def random_lines(ctx, num_lines=400, width=64, height=48, seed=61, blend=A.BLEND_OFF,
                 depth_test=A.DEPTH_TEST_LESS_THAN, depth_mask=A.DEPTH_MASK_ON, indexed=None,
                 color_type=A.COLOR_RGBA_8U, clear_depth=1.0, num_instances=1, persp=False, odd_end=False,
                 depth_type=A.COLOR_R_FLOAT):
    """Line draw (SL_RENDER_MODE_LINES): seeded segments in and around the
    view volume, so that many are clipped to the viewport (and, with
    `persp`, some cross the camera plane and are culled); vertex colour x
    RGBA8 texture program with vertex alpha, the uv interpolated along the
    line. `odd_end` ends the element range on an odd count: the last line
    reads the vertex after elementEnd, as the reference's loop does."""
    rng = np.random.default_rng(seed)
    s = S.Scene(ctx, f"lines_{seed}", width, height, color_type=color_type, depth_type=depth_type)
    n = 2 * num_lines
    if persp:
        pos = np.stack([rng.uniform(-3.0, 3.0, n), rng.uniform(-2.0, 2.0, n), rng.uniform(-2.5, 3.5, n)], 1)
        mvp = S.perspective(60.0, width / height, 0.1, 10.0) @ S.translate((0.0, 0.0, -3.0))
    else:
        pos = np.stack([rng.uniform(-1.6, 1.6, n), rng.uniform(-1.6, 1.6, n), rng.uniform(-1.2, 1.2, n)], 1)
        mvp = np.eye(4)
    col = np.concatenate([rng.uniform(0.0, 1.0, (n, 3)), rng.uniform(0.2, 1.0, (n, 1))], 1)
    uv = rng.uniform(-0.5, 1.5, (n, 2))
    verts = np.concatenate([pos, col, uv], 1).astype(np.float32)
    tex = s.add_texture_rgba8(S.to_rgba8(S.value_noise(32, 32, seed=seed, octaves=2, alpha=1.0)))
    if indexed is None:
        mesh = s.add_mesh(verts, None, stride=36)
        mesh.mode = A.RENDER_MODE_LINES
    else:
        order = rng.permutation(n)
        mesh = s.add_mesh(verts, order.astype(indexed), stride=36)
        mesh.mode = A.RENDER_MODE_INDEXED_LINES
    if odd_end:
        mesh.elementEnd -= 1
    sh = s.add_shader(A.PROGRAM_VCOLOR_TEX_ALPHA, 2, S.vcolor_uniforms(mvp, tex), cull=A.CULL_OFF,
                      depth_test=depth_test, depth_mask=depth_mask, blend=blend)
    s.draws.append((mesh, num_instances, sh))
    s.num_triangles = num_lines
    s.clear_depth = clear_depth
    return s


def line_edges(ctx, width=40, height=30):
    """Lines at the edges of the reference's line path, identity transform,
    flat colour, depth LESS: a full-width line (its x = W end lands on the
    next row), a vertical line at x = W (every pixel lands one row down), the
    diagonal whose last pixel (W, H) falls past the buffer, lines clipped at
    one or both ends, lines wholly outside, zero-length lines inside and
    outside, a line whose z leaves the volume (clipped with nothing to cut),
    steep and shallow lines in all octants."""
    s = S.Scene(ctx, "line_edges", width, height)
    segs = [
        ((-1.0, -0.2, 0.1), (1.0, -0.2, 0.1)),
        ((1.0, -0.9, 0.2), (1.0, 0.9, 0.2)),
        ((-1.0, -1.0, 0.0), (1.0, 1.0, 0.3)),
        ((-2.0, 0.3, -0.5), (2.0, -0.4, 0.5)),
        ((0.2, -3.0, 0.0), (-0.1, 0.5, 0.4)),
        ((1.5, 1.5, 0.0), (2.0, 2.0, 0.0)),
        ((0.1, 0.1, 0.0), (0.1, 0.1, 0.0)),
        ((1.4, 0.1, 0.0), (1.4, 0.1, 0.0)),
        ((-0.5, 0.6, -2.0), (0.5, 0.7, 0.5)),
        ((-0.9, 0.9, -0.1), (-0.8, -0.95, 0.6)),
        ((0.95, 0.2, 0.0), (-0.95, 0.25, -0.2)),
        ((0.3, -0.8, 0.7), (0.35, 0.85, -0.7)),
        ((-0.7, 0.4, 0.9), (0.6, 0.45, 0.9)),
        ((0.0, 0.0, 0.5), (1.0, 0.0, -0.5)),
    ]
    verts = np.zeros((2 * len(segs), 9), np.float32)
    for i, (a, b) in enumerate(segs):
        verts[2 * i, :3] = a
        verts[2 * i + 1, :3] = b
    mesh = s.add_mesh(verts, None, stride=36)
    mesh.mode = A.RENDER_MODE_LINES
    sh = s.add_shader(A.PROGRAM_FLAT_COLOR, 0, S.flat_uniforms(np.eye(4), (0.25, 1.0, 0.5, 1.0)),
                      cull=A.CULL_OFF, depth_test=A.DEPTH_TEST_LESS_THAN, depth_mask=A.DEPTH_MASK_ON)
    s.draws.append((mesh, 1, sh))
    return s


def mixed_prims(ctx, width=160, height=120, batched=False, blend_lines=False, seed=81):
    """Triangles, lines and points into one frame, issued draw by draw or as
    one batch (one launch holding all three record kinds); opaque with one
    depth rule (order-free raster), or with blended lines (ordered raster)."""
    rng = np.random.default_rng(seed)
    s = S.Scene(ctx, "mixed", width, height)
    tex = s.add_texture_rgba8(S.to_rgba8(S.value_noise(32, 32, seed=seed, octaves=2, alpha=1.0)))
    soup, proj = S.soup_triangles(300, width, height, seed=seed)
    tris = s.add_mesh(soup, None, stride=36)
    s.draws.append((tris, 1, s.add_shader(A.PROGRAM_VCOLOR_TEX_ALPHA, 2, S.vcolor_uniforms(proj, tex), cull=A.CULL_OFF)))
    n = 1200
    pos = np.stack([rng.uniform(-1.4, 1.4, n), rng.uniform(-1.4, 1.4, n), rng.uniform(-1.0, 1.0, n)], 1)
    col = np.concatenate([rng.uniform(0.0, 1.0, (n, 3)), rng.uniform(0.2, 1.0, (n, 1))], 1)
    verts = np.concatenate([pos, col, rng.uniform(-0.5, 1.5, (n, 2))], 1).astype(np.float32)
    lines = s.add_mesh(verts, None, stride=36)
    lines.mode = A.RENDER_MODE_LINES
    blend = A.BLEND_ALPHA if blend_lines else A.BLEND_OFF
    s.draws.append((lines, 1, s.add_shader(A.PROGRAM_VCOLOR_TEX_ALPHA, 2, S.vcolor_uniforms(np.eye(4), tex),
                                           cull=A.CULL_OFF, blend=blend)))
    points = s.add_mesh(verts[::-1].copy(), None, stride=36)
    points.mode = A.RENDER_MODE_POINTS
    s.draws.append((points, 1, s.add_shader(A.PROGRAM_VCOLOR_TEX_ALPHA, 2, S.vcolor_uniforms(np.eye(4), tex),
                                            cull=A.CULL_OFF)))
    s.batched = batched
    return s


def wire_queue(ctx, blend=A.BLEND_ADDITIVE, width=700, height=80):
    """One blended wireframe triangle with a long top edge and a sharp bottom
    vertex: its scan-lines near the vertex are narrower than the edges' moves,
    so their pixels are visited twice, after more than 600 queued fragments,
    where SoftLight's queue may be flushed between the two visits."""
    s = S.Scene(ctx, "wire_queue", width, height)
    pts = [(20.0, 10.0), (680.0, 10.0), (350.0, 70.0)]
    verts = np.zeros((3, 9), np.float32)
    for i, (x, y) in enumerate(pts):
        verts[i, :3] = (2.0 * x / width - 1.0, 2.0 * y / height - 1.0, 0.5)
    mesh = s.add_mesh(verts, None, stride=36)
    mesh.mode = A.RENDER_MODE_TRI_WIRE
    sh = s.add_shader(A.PROGRAM_FLAT_COLOR, 0, S.flat_uniforms(np.eye(4), (0.3, 0.2, 0.1, 0.5)),
                      cull=A.CULL_OFF, depth_test=A.DEPTH_TEST_LESS_THAN, depth_mask=A.DEPTH_MASK_ON, blend=blend)
    s.draws.append((mesh, 1, sh))
    return s


MRT_FORMATS = (A.COLOR_RGBA_8U, A.COLOR_RGBA_FLOAT, A.COLOR_R_FLOAT, A.COLOR_RGBA_8U)


def mrt(ctx, types=MRT_FORMATS, num_outputs=4, prim="tri", blend=A.BLEND_OFF, depth_test=A.DEPTH_TEST_LESS_THAN,
        num_tris=300, width=96, height=80, seed=101, single_after=False, batched=False, clear_color=None):
    """Multiple render targets: the G-buffer program writes num_outputs
    outputs into colour attachments of the given formats (output k to
    attachment k), as filled triangles, wireframe, lines or points of a
    triangle soup. single_after adds a one-output draw into the same
    framebuffer (it writes attachment 0 only)."""
    s = S.Scene(ctx, f"mrt_{seed}", width, height)
    s.set_color_attachments(list(types))
    if clear_color is not None:
        s.clear_color = clear_color
    verts, proj = S.soup_triangles(num_tris, width, height, seed=seed)
    mesh = s.add_mesh(verts, None, stride=36)
    mesh.mode = {"tri": A.RENDER_MODE_TRIANGLES, "wire": A.RENDER_MODE_TRI_WIRE,
                 "line": A.RENDER_MODE_LINES, "point": A.RENDER_MODE_POINTS}[prim]
    tex = s.add_texture_rgba8(S.to_rgba8(S.value_noise(32, 32, seed=seed, octaves=2, alpha=1.0)))
    sh = s.add_shader(A.PROGRAM_GBUFFER, 2, S.vcolor_uniforms(proj, tex), cull=A.CULL_OFF, depth_test=depth_test,
                      blend=blend, num_outputs=num_outputs)
    s.draws.append((mesh, 1, sh))
    if single_after:
        soup, proj2 = S.soup_triangles(num_tris // 2, width, height, seed=seed + 1)
        mesh2 = s.add_mesh(soup, None, stride=36)
        sh2 = s.add_shader(A.PROGRAM_VCOLOR_TEX_ALPHA, 2, S.vcolor_uniforms(proj2, tex), cull=A.CULL_OFF,
                           depth_test=depth_test, blend=blend)
        s.draws.append((mesh2, 1, sh2))
    s.num_triangles = num_tris
    s.batched = batched
    return s


# the 28 component formats in groups of four, then the five packed ones
FORMAT_GROUPS = tuple(tuple(range(4 * g, 4 * g + 4)) for g in range(7)) + ((28, 29, 30, 31), (32, 28, 21, 5))


def format_edges(ctx, color_type, width=8, height=6):
    """One colour attachment of the given format: the left half gets an
    unblended flat colour outside [0, 1] (-0.25, 1.5, 3.0, 0.5), the right
    half an alpha-blended colour of alpha 0 over a cleared alpha 0 (0 / 0:
    NaN components), the conversions where formats differ most."""
    s = S.Scene(ctx, f"format_edges_{color_type}", width, height)
    s.set_color_attachments([color_type])
    s.clear_color = (0.1, 0.2, 0.3, 0.0)
    for x0, x1, col, blend in [(-1.0, 0.0, (-0.25, 1.5, 3.0, 0.5), A.BLEND_OFF), (0.0, 1.0, (0.3, 0.6, 0.9, 0.0), A.BLEND_ALPHA)]:
        verts = np.zeros((6, 9), np.float32)
        verts[:, :3] = [(x0, -1, 0), (x1, -1, 0), (x1, 1, 0), (x0, -1, 0), (x1, 1, 0), (x0, 1, 0)]
        mesh = s.add_mesh(verts, None, stride=36)
        sh = s.add_shader(A.PROGRAM_FLAT_COLOR, 0, S.flat_uniforms(np.eye(4), col), cull=A.CULL_OFF,
                          depth_test=A.DEPTH_TEST_OFF, depth_mask=A.DEPTH_MASK_OFF, blend=blend)
        s.draws.append((mesh, 1, sh))
    return s


LINE_ALIAS_PIXEL = (10, 0)   # (row, column) that both ends of line_alias's line address


def line_alias(ctx, width=40, height=30):
    """A full-width line whose last pixel (x = W, row 9) is stored at the
    address of its first pixel (x = 0, row 10). SoftLight tests both against
    the depth before the line (fewer than 600 fragments are queued before the
    last one, so the queue is written after both tests) and writes them in
    walk order: the later, farther fragment wins there. Depth LESS, z from
    0.2 to 0.5."""
    s = S.Scene(ctx, "line_alias", width, height)
    verts = np.zeros((2, 9), np.float32)
    verts[0, :3] = (-1.0, -0.32, 0.2)
    verts[1, :3] = (1.0, -0.38, 0.5)
    mesh = s.add_mesh(verts, None, stride=36)
    mesh.mode = A.RENDER_MODE_LINES
    sh = s.add_shader(A.PROGRAM_FLAT_COLOR, 0, S.flat_uniforms(np.eye(4), (1.0, 1.0, 1.0, 1.0)),
                      cull=A.CULL_OFF, depth_test=A.DEPTH_TEST_LESS_THAN, depth_mask=A.DEPTH_MASK_ON)
    s.draws.append((mesh, 1, sh))
    return s


def line_alias_wide(ctx, occluded=True, batched=False, blend=A.BLEND_OFF, width=700, height=20):
    """A 700-wide framebuffer and a line from (0, row 10) to (W, row 9), its
    last pixel stored at its first. With `occluded`, a nearer quad hides
    columns 50..690 of rows 7..12 first: fewer than 600 of the line's
    fragments are queued before its last step, so SoftLight tests that step
    against the depth before the line; unoccluded, the queue is flushed in
    between and the test follows the first step's write."""
    s = S.Scene(ctx, f"line_alias_wide_{int(occluded)}", width, height)
    if occluded:
        xa, xb = 50.0 / (width / 2) - 1.0, 690.0 / (width / 2) - 1.0
        quad = np.zeros((6, 9), np.float32)
        quad[:, :3] = [(xa, -0.3, 0.0), (xb, -0.3, 0.0), (xb, 0.3, 0.0), (xa, -0.3, 0.0), (xb, 0.3, 0.0), (xa, 0.3, 0.0)]
        mesh = s.add_mesh(quad, None, stride=36)
        sh = s.add_shader(A.PROGRAM_FLAT_COLOR, 0, S.flat_uniforms(np.eye(4), (0.2, 0.2, 0.9, 1.0)),
                          cull=A.CULL_OFF, depth_test=A.DEPTH_TEST_LESS_THAN, depth_mask=A.DEPTH_MASK_ON)
        s.draws.append((mesh, 1, sh))
    verts = np.zeros((2, 9), np.float32)
    verts[0, :3] = (-1.0, 0.05, 0.2)
    verts[1, :3] = (1.0, -0.05, 0.5)
    line = s.add_mesh(verts, None, stride=36)
    line.mode = A.RENDER_MODE_LINES
    sh = s.add_shader(A.PROGRAM_FLAT_COLOR, 0, S.flat_uniforms(np.eye(4), (1.0, 0.8, 0.1, 0.6)),
                      cull=A.CULL_OFF, depth_test=A.DEPTH_TEST_LESS_THAN, depth_mask=A.DEPTH_MASK_ON, blend=blend)
    s.draws.append((line, 1, sh))
    s.batched = batched
    return s


def point_edges(ctx, width=40, height=30):
    """Points placed at the edges of the reference's point addressing: x = W
    lands on the next row's first pixel (linear index x + W*y), x = W on the
    last row falls past the buffer and is dropped, w <= 0 and |x| > w are
    culled; identity transform, flat colour, depth off."""
    s = S.Scene(ctx, "point_edges", width, height)
    pts = [(1.0, 0.0, 0.0), (1.0, -1.0, 0.0), (1.0, 1.0, 0.0), (-1.0, -1.0, 0.0), (0.999, 0.999, 0.0),
           (1.0001, 0.0, 0.0), (0.0, 0.0, 1.0), (0.0, 0.0, -1.0), (0.5, -0.5, 0.5), (-1.0, 1.0, 0.0)]
    verts = np.zeros((len(pts), 9), np.float32)
    verts[:, :3] = pts
    mesh = s.add_mesh(verts, None, stride=36)
    mesh.mode = A.RENDER_MODE_POINTS
    sh = s.add_shader(A.PROGRAM_FLAT_COLOR, 0, S.flat_uniforms(np.eye(4), (1.0, 0.5, 0.25, 1.0)),
                      cull=A.CULL_OFF, depth_test=A.DEPTH_TEST_OFF, depth_mask=A.DEPTH_MASK_OFF)
    s.draws.append((mesh, 1, sh))
    return s


def program_soup(ctx, program, num_tris=300, width=96, height=80, seed=51, prim="tri", blend=A.BLEND_OFF,
                 depth_test=A.DEPTH_TEST_LESS_THAN, depth_mask=A.DEPTH_MASK_ON, color_type=A.COLOR_RGBA_8U,
                 depth_type=A.COLOR_R_FLOAT, alpha_ref=0.3, depth_scale=0.5, depth_bias=0.25, screen_door=3,
                 clear_depth=1.0, num_instances=1):
    """A triangle soup drawn as filled triangles, wireframe, lines or points
    with one of the programs that need the ordered raster: the alpha-cutout
    program (SLG_PROGRAM_VCOLOR_TEX_CUTOUT: discards where vertex alpha x
    texel alpha < alpha_ref, over a texture with varying alpha) or the
    fragment-coordinate program (SLG_PROGRAM_FRAG_COORD: colour from x, y and
    depth, screen-door discard, depth written as depth * scale + bias)."""
    s = S.Scene(ctx, f"prog_{program}_{seed}", width, height, color_type=color_type, depth_type=depth_type)
    verts, proj = S.soup_triangles(num_tris, width, height, seed=seed)
    mesh = s.add_mesh(verts, None, stride=36)
    mesh.mode = {"tri": A.RENDER_MODE_TRIANGLES, "wire": A.RENDER_MODE_TRI_WIRE,
                 "line": A.RENDER_MODE_LINES, "point": A.RENDER_MODE_POINTS}[prim]
    if program == A.PROGRAM_VCOLOR_TEX_CUTOUT:
        tex = s.add_texture_rgba8(S.to_rgba8(S.value_noise(32, 32, seed=seed, octaves=2)))
        ub = S.cutout_uniforms(proj, tex, alpha_ref)
    else:
        ub = S.fragcoord_uniforms(proj, 1.0 / width, 1.0 / height, depth_scale, depth_bias, screen_door)
    sh = s.add_shader(program, 2, ub, cull=A.CULL_OFF, depth_test=depth_test, depth_mask=depth_mask, blend=blend)
    s.draws.append((mesh, num_instances, sh))
    s.num_triangles = num_tris
    s.clear_depth = clear_depth
    return s


def multi_mesh(ctx, num_tris=700, num_meshes=3, width=128, height=96, seed=91, blend=A.BLEND_ALPHA,
               modes=None, depth_test=A.DEPTH_TEST_LESS_THAN):
    """One SL_Context::draw_multiple call over several triangle soups of the
    same size, so their primIndex ranges (element indices within each mesh)
    overlap: with blending, the reference's flush groups of 1024 bins are
    sorted by primIndex and interleave the meshes. `modes` gives each mesh's
    render mode (the first mesh's decides the processor and raster mode;
    indexed modes get an identity-permuted index buffer)."""
    s = S.Scene(ctx, f"multi_mesh_{seed}", width, height)
    tex = s.add_texture_rgba8(S.to_rgba8(S.value_noise(32, 32, seed=seed, octaves=2, alpha=1.0)))
    proj = None
    for k in range(num_meshes):
        verts, proj = S.soup_triangles(num_tris, width, height, seed=seed + k)
        mode = modes[k] if modes else A.RENDER_MODE_TRIANGLES
        indexed = mode in (A.RENDER_MODE_INDEXED_TRIANGLES, A.RENDER_MODE_INDEXED_TRI_WIRE)
        idx = np.random.default_rng(seed + 10 + k).permutation(verts.shape[0]).astype(np.uint32) if indexed else None
        if idx is not None:
            inv = np.empty_like(idx)
            inv[idx] = np.arange(idx.size, dtype=np.uint32)
            verts, idx = verts[idx], inv
        mesh = s.add_mesh(verts, idx, stride=36)
        mesh.mode = mode
        s.draws.append((mesh, 1, None))
    sh = s.add_shader(A.PROGRAM_VCOLOR_TEX_ALPHA, 2, S.vcolor_uniforms(proj, tex), cull=A.CULL_OFF, blend=blend,
                      depth_test=depth_test)
    s.draws = [(m, 1, sh) for (m, _, _) in s.draws]
    s.multiple = True
    s.num_triangles = num_tris * num_meshes
    return s


def sliver_soup(ctx, num_tris=1500, width=320, height=200, seed=121, depth_test=A.DEPTH_TEST_LESS_THAN,
                blend=A.BLEND_ALPHA, clear_depth=1.0, z_base=0.5, z_spread=1e-4):
    """Near-degenerate triangles for the ordered raster's depth bound: long
    slivers (up to the screen's width, 0.01..3 px thick) and small ones,
    placed directly in clip space (identity transform) with depths packed
    within z_spread of each other, so the rounding of the walk's
    barycentrics decides many depth tests."""
    rng = np.random.default_rng(seed)
    s = S.Scene(ctx, f"slivers_{seed}", width, height)
    verts = np.zeros((3 * num_tris, 9), np.float32)
    for t in range(num_tris):
        p0 = rng.uniform([-1.1, -1.1], [1.1, 1.1])
        ang = rng.uniform(0, 2 * math.pi)
        length = rng.choice([rng.uniform(0.01, 0.2), rng.uniform(0.5, 2.5)])
        d = length * np.array([math.cos(ang), math.sin(ang)])
        thick = rng.uniform(0.01, 3.0) * 2.0 / height
        n = np.array([-d[1], d[0]]) / max(np.linalg.norm(d), 1e-9)
        p1 = p0 + d
        p2 = p0 + d * rng.uniform(0.0, 1.0) + n * thick
        z = z_base + rng.uniform(-z_spread, z_spread, 3)
        for k, p in enumerate((p0, p1, p2)):
            verts[3 * t + k, :3] = (p[0], p[1], z[k])
            verts[3 * t + k, 3:7] = (*rng.uniform(0.0, 1.0, 3), rng.uniform(0.3, 1.0))
            verts[3 * t + k, 7:9] = rng.uniform(0.0, 1.0, 2)
    mesh = s.add_mesh(verts, None, stride=36)
    tex = s.add_texture_rgba8(S.to_rgba8(S.value_noise(32, 32, seed=seed, octaves=2, alpha=1.0)))
    sh = s.add_shader(A.PROGRAM_VCOLOR_TEX_ALPHA, 2, S.vcolor_uniforms(np.eye(4), tex), cull=A.CULL_OFF,
                      depth_test=depth_test, blend=blend)
    s.draws.append((mesh, 1, sh))
    s.clear_depth = clear_depth
    return s
