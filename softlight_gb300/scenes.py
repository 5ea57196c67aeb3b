"""Seeded procedural workloads for the draw path.

Each builder creates its resources through an SLContext (GPU or any other
implementation of include/slg.h) with identical calls and data, and returns
a Scene whose render() clears the framebuffer and issues the draws. All
inputs are synthetic: procedural meshes (UV spheres, tori, grids, triangle
soup), procedural textures (checker, value noise) and matrices computed in
float64 and stored as float32.

Configurations (the benchmark workloads C1-C5):
  c1  one 64x32 UV sphere (4096 tris), 256^2 RGBA8 checker, Lambert, 640x480
  c2  the sphere x1024 instances, 1024^2 noise texture, Blinn-Phong 4 lights, 1920x1080
  c3  2M-triangle soup, 30% back-facing, 10% crossing the near plane, alpha blend, 1920x1080
  c4  256 uneven meshes (12..65k tris) each with its own 512^2 texture, Lambert+ambient, 3840x2160
  c5  10k-triangle noise-displaced sphere, per-vertex colours x 256^2 float RGBA texture,
      512x512 float target with a visibility map (the differentiable render)
"""
import math
import struct

import numpy as np

from . import api as A

# ---------------------------------------------------------------------------
# matrices (column-major float32, as ls::math::mat4)
# ---------------------------------------------------------------------------


def perspective(fov_y_deg, aspect, near, far):
    f = 1.0 / math.tan(math.radians(fov_y_deg) / 2.0)
    m = np.zeros((4, 4), dtype=np.float64)  # row-major math matrix
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 2] = (far + near) / (near - far)
    m[2, 3] = 2.0 * far * near / (near - far)
    m[3, 2] = -1.0
    return m


def look_at(eye, target, up):
    eye, target, up = (np.asarray(v, dtype=np.float64) for v in (eye, target, up))
    f = target - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def translate(t):
    m = np.eye(4)
    m[:3, 3] = t
    return m


def scale(s):
    m = np.eye(4)
    m[0, 0] = m[1, 1] = m[2, 2] = s
    return m


def quat_to_mat(q):
    w, x, y, z = q
    m = np.eye(4)
    m[:3, :3] = [
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ]
    return m


def random_rotation(rng):
    """Uniform random rotation (Shoemake's subgroup algorithm)."""
    u1, u2, u3 = rng.random(3)
    a, b = math.sqrt(1 - u1), math.sqrt(u1)
    q = (b * math.cos(2 * math.pi * u3), a * math.sin(2 * math.pi * u2),
         a * math.cos(2 * math.pi * u2), b * math.sin(2 * math.pi * u3))
    return quat_to_mat(q)


def col_major(m):
    """float64 row-major 4x4 -> 16 float32 in column-major order."""
    return np.asarray(m, dtype=np.float64).T.astype(np.float32).reshape(16)


# ---------------------------------------------------------------------------
# geometry: interleaved float32 pos3 / uv2 / normal3 (32-byte vertices)
# ---------------------------------------------------------------------------


def _orient_outward(verts, idx, center=(0.0, 0.0, 0.0)):
    """Flip triangles so (v1-v0)x(v2-v0) points away from `center`
    (counter-clockwise seen from outside = front-facing)."""
    p = verts[:, :3].astype(np.float64)
    t = idx.reshape(-1, 3)
    n = np.cross(p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]])
    c = (p[t[:, 0]] + p[t[:, 1]] + p[t[:, 2]]) / 3.0 - np.asarray(center)
    flip = (n * c).sum(1) < 0
    t = t.copy()
    t[flip, 1], t[flip, 2] = t[flip, 2].copy(), t[flip, 1].copy()
    return t.reshape(-1)


def uv_sphere(lon=64, lat=32, radius=1.0):
    """(lon+1)*(lat+1) vertices and lon*lat*2 triangles (pole quads included)."""
    th = np.linspace(0.0, math.pi, lat + 1)
    ph = np.linspace(0.0, 2.0 * math.pi, lon + 1)
    T, P = np.meshgrid(th, ph, indexing="ij")
    n = np.stack([np.sin(T) * np.cos(P), np.cos(T), -np.sin(T) * np.sin(P)], -1)
    uv = np.stack([P / (2 * math.pi), T / math.pi], -1)
    verts = np.concatenate([n * radius, uv, n], -1).reshape(-1, 8)
    idx = []
    for i in range(lat):
        for j in range(lon):
            a = i * (lon + 1) + j
            b = a + lon + 1
            idx += [a, b, a + 1, a + 1, b, b + 1]
    idx = np.asarray(idx, dtype=np.uint32)
    return verts.astype(np.float32), _orient_outward(verts, idx).astype(np.uint32)


def torus(seg_major, seg_minor, R=1.0, r=0.35):
    u = np.linspace(0.0, 2 * math.pi, seg_major + 1)
    v = np.linspace(0.0, 2 * math.pi, seg_minor + 1)
    U, V = np.meshgrid(u, v, indexing="ij")
    cx, cz = np.cos(U), np.sin(U)
    pos = np.stack([(R + r * np.cos(V)) * cx, r * np.sin(V), (R + r * np.cos(V)) * cz], -1)
    nrm = np.stack([np.cos(V) * cx, np.sin(V), np.cos(V) * cz], -1)
    uv = np.stack([U / (2 * math.pi), V / (2 * math.pi)], -1)
    verts = np.concatenate([pos, uv, nrm], -1).reshape(-1, 8)
    idx = []
    for i in range(seg_major):
        for j in range(seg_minor):
            a = i * (seg_minor + 1) + j
            b = a + seg_minor + 1
            idx += [a, b, a + 1, a + 1, b, b + 1]
    idx = np.asarray(idx, dtype=np.uint32)
    # orient against the tube centre of each triangle
    p = verts[:, :3]
    t = idx.reshape(-1, 3)
    ctr = p[t].mean(1)
    ang = np.arctan2(ctr[:, 2], ctr[:, 0])
    tube = np.stack([R * np.cos(ang), np.zeros_like(ang), R * np.sin(ang)], -1)
    nrmt = np.cross(p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]])
    flip = (nrmt * (ctr - tube)).sum(1) < 0
    t = t.copy()
    t[flip, 1], t[flip, 2] = t[flip, 2].copy(), t[flip, 1].copy()
    return verts.astype(np.float32), t.reshape(-1).astype(np.uint32)


def grid(nx, ny, size=2.0):
    """A flat nx*ny-cell grid in the xy plane facing +z."""
    xs = np.linspace(-size / 2, size / 2, nx + 1)
    ys = np.linspace(-size / 2, size / 2, ny + 1)
    Y, X = np.meshgrid(ys, xs, indexing="ij")
    pos = np.stack([X, Y, np.zeros_like(X)], -1)
    uv = np.stack([(X + size / 2) / size, (Y + size / 2) / size], -1)
    nrm = np.zeros_like(pos)
    nrm[..., 2] = 1.0
    verts = np.concatenate([pos, uv, nrm], -1).reshape(-1, 8)
    idx = []
    for i in range(ny):
        for j in range(nx):
            a = i * (nx + 1) + j
            b = a + nx + 1
            idx += [a, a + 1, b, a + 1, b + 1, b]
    return verts.astype(np.float32), np.asarray(idx, dtype=np.uint32)


# ---------------------------------------------------------------------------
# textures
# ---------------------------------------------------------------------------


def checker(w, h, cells, c0=(230, 80, 40, 255), c1=(40, 90, 220, 255)):
    y, x = np.mgrid[0:h, 0:w]
    m = ((x // (w // cells)) + (y // (h // cells))) % 2
    out = np.where(m[..., None] == 0, np.asarray(c0, np.uint8), np.asarray(c1, np.uint8))
    return out.astype(np.uint8)


def value_noise(w, h, seed, octaves=4, base=8, channels=4, alpha=None):
    """Seeded value noise in [0,1): sum of bilinearly upsampled random lattices."""
    rng = np.random.default_rng(seed)
    acc = np.zeros((h, w, channels), dtype=np.float64)
    amp, tot = 1.0, 0.0
    for o in range(octaves):
        g = base << o
        lat = rng.random((g + 1, g + 1, channels))
        ys = np.linspace(0, g, h, endpoint=False)
        xs = np.linspace(0, g, w, endpoint=False)
        y0, x0 = ys.astype(int), xs.astype(int)
        fy, fx = (ys - y0)[:, None, None], (xs - x0)[None, :, None]
        v = (lat[y0][:, x0] * (1 - fy) * (1 - fx) + lat[y0 + 1][:, x0] * fy * (1 - fx)
             + lat[y0][:, x0 + 1] * (1 - fy) * fx + lat[y0 + 1][:, x0 + 1] * fy * fx)
        acc += amp * v
        tot += amp
        amp *= 0.5
    acc /= tot
    if alpha is not None and channels == 4:
        acc[..., 3] = alpha
    return acc


def to_rgba8(x):
    return np.clip(np.floor(x * 256.0), 0, 255).astype(np.uint8)


# ---------------------------------------------------------------------------
# uniform blocks (byte layouts of include/slg_programs.h)
# ---------------------------------------------------------------------------


def lambert_uniforms(vp, model, light_dir, ambient, tex_id):
    return (col_major(vp).tobytes() + col_major(model).tobytes()
            + np.asarray(light_dir, np.float32).tobytes() + np.asarray(ambient, np.float32).tobytes()
            + struct.pack("<4I", tex_id, 0, 0, 0))


def blinn_uniforms(vp, cam, light_pos, light_col, ambient, specularity, attenuation, tex_id, inst_buf):
    return (col_major(vp).tobytes() + np.asarray(cam, np.float32).tobytes()
            + np.asarray(light_pos, np.float32).reshape(16).tobytes()
            + np.asarray(light_col, np.float32).reshape(16).tobytes()
            + np.asarray(ambient, np.float32).tobytes()
            + struct.pack("<ffII", specularity, attenuation, tex_id, inst_buf))


def vcolor_uniforms(mvp, tex_id):
    return col_major(mvp).tobytes() + struct.pack("<4I", tex_id, 0, 0, 0)


def cutout_uniforms(mvp, tex_id, alpha_ref):
    """slg_cutout_uniforms: the vertex-colour block plus the alpha test's reference."""
    return col_major(mvp).tobytes() + struct.pack("<If2I", tex_id, alpha_ref, 0, 0)


def fragcoord_uniforms(mvp, inv_w, inv_h, depth_scale=1.0, depth_bias=0.0, screen_door=0):
    """slg_fragcoord_uniforms of SLG_PROGRAM_FRAG_COORD."""
    return col_major(mvp).tobytes() + struct.pack("<4fI3I", inv_w, inv_h, depth_scale, depth_bias, screen_door, 0, 0, 0)


def flat_uniforms(mvp, rgba):
    return col_major(mvp).tobytes() + np.asarray(rgba, np.float32).tobytes()


# ---------------------------------------------------------------------------
# scene
# ---------------------------------------------------------------------------


class Scene:
    """Resources of one workload in one context plus its frame sequence."""

    def __init__(self, ctx, name, width, height, color_type=A.COLOR_RGBA_8U, depth_type=A.COLOR_R_FLOAT):
        self.ctx, self.name, self.width, self.height = ctx, name, width, height
        self.color_type = color_type
        self.depth_type = depth_type
        self.color_tex = ctx.create_texture()
        ctx.texture_init(self.color_tex, color_type, width, height, 1)
        self.depth_tex = ctx.create_texture()
        ctx.texture_init(self.depth_tex, depth_type, width, height, 1)
        self.fbo = ctx.create_framebuffer()
        ctx.fbo_reserve_color_buffers(self.fbo, 1)
        ctx.fbo_attach_color_buffer(self.fbo, 0, self.color_tex)
        ctx.fbo_attach_depth_buffer(self.fbo, self.depth_tex)
        self.attachments = [(self.color_tex, color_type)]
        self.clear_color = (0.0, 0.0, 0.0, 1.0)
        self.clear_depth = 1.0
        self.draws = []          # list of (kind, args)
        self.num_triangles = 0   # submitted triangles per frame
        self.batched = False
        self.frame_ubos = []     # (ubo id, bytes) re-uploaded per frame in e2e timing
        self.texture_bytes = 0
        self.geometry_bytes = 0
        self.blending = False

    def set_color_attachments(self, types):
        """Colour attachments 0..len(types)-1 of the given formats (multiple
        render targets, SL_Framebuffer::reserve_color_buffers and
        attach_color_buffer); attachment 0 replaces the default one."""
        ctx = self.ctx
        ctx.fbo_reserve_color_buffers(self.fbo, len(types))
        self.attachments = []
        for k, t in enumerate(types):
            tex = ctx.create_texture()
            ctx.texture_init(tex, t, self.width, self.height, 1)
            ctx.fbo_attach_color_buffer(self.fbo, k, tex)
            self.attachments.append((tex, t))
        self.color_tex, self.color_type = self.attachments[0]

    def add_texture_rgba8(self, img):
        t = self.ctx.create_texture()
        h, w = img.shape[:2]
        self.ctx.texture_init(t, A.COLOR_RGBA_8U, w, h, 1)
        self.ctx.texture_set_texels(t, img)
        self.texture_bytes += img.nbytes
        return t

    def add_texture_rgbaf(self, img):
        t = self.ctx.create_texture()
        h, w = img.shape[:2]
        self.ctx.texture_init(t, A.COLOR_RGBA_FLOAT, w, h, 1)
        self.ctx.texture_set_texels(t, np.ascontiguousarray(img, dtype=np.float32))
        self.texture_bytes += img.nbytes
        return t

    def add_mesh(self, verts, indices=None, stride=32):
        ctx = self.ctx
        vbo = ctx.create_vbo()
        ctx.vbo_init(vbo, verts)
        vao = ctx.create_vao()
        ctx.vao_set_vertex_buffer(vao, vbo)
        ctx.vao_set_binding(vao, 0, 0, stride, 3, A.VERTEX_DATA_FLOAT)
        self.geometry_bytes += verts.nbytes
        if indices is not None:
            ibo = ctx.create_ibo()
            ctx.ibo_init(ibo, indices)
            ctx.vao_set_index_buffer(vao, ibo)
            self.geometry_bytes += indices.nbytes
            mesh = A.Mesh(vao, 0, indices.size, A.RENDER_MODE_INDEXED_TRIANGLES, 0)
        else:
            mesh = A.Mesh(vao, 0, verts.shape[0], A.RENDER_MODE_TRIANGLES, 0)
        return mesh

    def add_shader(self, program, num_varyings, ubo_bytes, cull=A.CULL_BACK_FACE, depth_test=A.DEPTH_TEST_LESS_THAN,
                   depth_mask=A.DEPTH_MASK_ON, blend=A.BLEND_OFF, num_outputs=1):
        ctx = self.ctx
        ubo = ctx.create_ubo()
        ctx.ubo_assign(ubo, ubo_bytes)
        self.frame_ubos.append((ubo, ubo_bytes))
        self.blending = self.blending or blend != A.BLEND_OFF
        vs = A.VertexShader(num_varyings, cull, program)
        fs = A.FragmentShader(num_varyings, num_outputs, blend, depth_test, depth_mask, program)
        return ctx.create_shader(vs, fs, ubo)

    def render(self, clear=True):
        ctx = self.ctx
        if clear:
            ctx.clear_framebuffer(self.fbo, 0, self.clear_color, self.clear_depth)
            for k in range(1, len(self.attachments)):
                ctx.clear_color_buffer(self.fbo, k, self.clear_color)
        if getattr(self, "multiple", False):
            # one SL_Context::draw_multiple call over every mesh, with the first draw's shader
            ctx.draw_multiple([m for (m, _, _) in self.draws], self.draws[0][2], self.fbo)
        elif self.batched:
            cmds = [A.DrawCmd(m, n, s) for (m, n, s) in self.draws]
            ctx.draw_batch(cmds, self.fbo)
        else:
            for (m, n, s) in self.draws:
                if n == 1:
                    ctx.draw(m, s, self.fbo)
                else:
                    ctx.draw_instanced(m, n, s, self.fbo)

    def read_color(self, k=0):
        tex, ctype = self.attachments[k]
        nc, dtype = A.color_layout(ctype)
        shape = (self.height, self.width) if nc == 1 else (self.height, self.width, nc)
        return self.ctx.texture_read(tex, shape, np.dtype(dtype))

    def read_colors(self):
        return [self.read_color(k) for k in range(len(self.attachments))]

    def read_depth(self):
        dtype = {A.COLOR_R_HALF: np.float16, A.COLOR_R_DOUBLE: np.float64}.get(self.depth_type, np.float32)
        return self.ctx.texture_read(self.depth_tex, (self.height, self.width), dtype)

    def framebuffer_bytes(self):
        return self.width * self.height * (A.BYTES_PER_COLOR[self.color_type] + 4)


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------


def build_c1(ctx, width=640, height=480):
    """Single UV sphere, 64 x 32 segments, Lambert, 256^2 checker, 640x480."""
    s = Scene(ctx, "c1_sphere_640x480", width, height)
    verts, idx = uv_sphere(64, 32)
    mesh = s.add_mesh(verts, idx)
    tex = s.add_texture_rgba8(checker(256, 256, 8))
    vp = perspective(60.0, width / height, 0.1, 100.0) @ look_at((0, 0, 3), (0, 0, 0), (0, 1, 0))
    light = np.asarray([1.0, 1.0, 1.0]) / math.sqrt(3.0)
    ub = lambert_uniforms(vp, np.eye(4), [*light, 0.0], [0.0, 0.0, 0.0, 0.0], tex)
    sh = s.add_shader(A.PROGRAM_LAMBERT_TEX, 2, ub)
    s.draws.append((mesh, 1, sh))
    s.num_triangles = idx.size // 3
    return s


def c2_instance_matrices(num_instances, seed=2):
    rng = np.random.default_rng(seed)
    mats = np.empty((num_instances, 16), dtype=np.float32)
    for i in range(num_instances):
        t = rng.uniform(-20.0, 20.0, 3)
        r = random_rotation(rng)
        sc = rng.uniform(0.2, 2.0)
        mats[i] = col_major(translate(t) @ r @ scale(sc))
    return mats


def build_c2(ctx, num_instances=1024, width=1920, height=1080, tex_size=1024):
    """The sphere instanced num_instances times, Blinn-Phong with 4 point lights, 1080p."""
    s = Scene(ctx, f"c2_instanced_{num_instances}_{width}x{height}", width, height)
    verts, idx = uv_sphere(64, 32)
    mesh = s.add_mesh(verts, idx)
    tex = s.add_texture_rgba8(to_rgba8(value_noise(tex_size, tex_size, seed=2, alpha=1.0)))
    mats = c2_instance_matrices(num_instances)
    inst_buf = ctx.create_vbo()
    ctx.vbo_init(inst_buf, mats)
    s.instance_matrices = (inst_buf, mats)
    eye = (0.0, 0.0, 45.0)
    vp = perspective(60.0, width / height, 0.1, 200.0) @ look_at(eye, (0, 0, 0), (0, 1, 0))
    lights = [(-15, 15, 25, 1), (15, 15, 25, 1), (0, -20, 20, 1), (0, 25, -10, 1)]
    colors = [(1.0, 0.9, 0.8, 1.0), (0.6, 0.7, 1.0, 1.0), (0.9, 0.5, 0.4, 1.0), (0.5, 1.0, 0.6, 1.0)]
    ub = blinn_uniforms(vp, (*eye, 1.0), lights, colors, (0.08, 0.08, 0.08, 1.0), 0.5, 0.0008, tex, inst_buf)
    sh = s.add_shader(A.PROGRAM_BLINN_PHONG_INST, 3, ub)
    s.draws.append((mesh, num_instances, sh))
    s.num_triangles = (idx.size // 3) * num_instances
    s.geometry_bytes += mats.nbytes
    return s


def soup_triangles(num_tris, width, height, seed=3, near=0.1, fov=60.0):
    """Triangle soup in view space: screen-uniform centroids, log-uniform screen
    area in [0.5, 20000] px, aspect <= 8, 30% reversed winding, 10% with one
    vertex behind the near plane. Returns float32 [3*num_tris, 9]
    (pos3, rgba4, uv2) vertices and the projection matrix."""
    rng = np.random.default_rng(seed)
    aspect = width / height
    proj = perspective(fov, aspect, near, 500.0)
    f = 1.0 / math.tan(math.radians(fov) / 2.0)
    n = num_tris
    cx = rng.uniform(0, width, n)
    cy = rng.uniform(0, height, n)
    area = np.exp(rng.uniform(math.log(0.5), math.log(20000.0), n))
    elong = np.exp(rng.uniform(0.0, math.log(8.0), n))
    ang = rng.uniform(0, 2 * math.pi, n)
    depth = rng.uniform(2.0, 400.0, n)
    # triangle (0,0),(a,0),(b,c) in a local frame, area = a*c/2
    base = np.sqrt(2.0 * area * elong)
    hgt = 2.0 * area / base
    off = rng.uniform(-0.5, 0.5, n) * base
    local = np.stack([np.stack([-base / 3, -hgt / 3], -1),
                      np.stack([2 * base / 3, -hgt / 3], -1),
                      np.stack([off, 2 * hgt / 3], -1)], 1)  # (n,3,2) CCW
    ca, sa = np.cos(ang)[:, None], np.sin(ang)[:, None]
    sx = cx[:, None] + local[..., 0] * ca - local[..., 1] * sa
    sy = cy[:, None] + local[..., 0] * sa + local[..., 1] * ca
    # screen -> NDC -> view space at depth d
    ndx = sx / width * 2.0 - 1.0
    ndy = sy / height * 2.0 - 1.0
    d = depth[:, None] * (1.0 + rng.uniform(-0.05, 0.05, (n, 3)))
    vx = ndx * d * aspect / f
    vy = ndy * d / f
    vz = -d
    back = rng.random(n) < 0.30
    vx[back, 1], vx[back, 2] = vx[back, 2].copy(), vx[back, 1].copy()
    vy[back, 1], vy[back, 2] = vy[back, 2].copy(), vy[back, 1].copy()
    vz[back, 1], vz[back, 2] = vz[back, 2].copy(), vz[back, 1].copy()
    cross = rng.random(n) < 0.10
    k = rng.integers(0, 3, n)
    ci = np.nonzero(cross)[0]
    vz[ci, k[ci]] = rng.uniform(0.05, 2.0, ci.size)  # behind the camera
    rgba = np.concatenate([rng.uniform(0.1, 1.0, (n, 3)), rng.uniform(0.2, 1.0, (n, 1))], 1)
    uv = rng.uniform(0.0, 4.0, (n, 3, 2))
    pos = np.stack([vx, vy, vz], -1)
    col = np.repeat(rgba[:, None, :], 3, 1)
    verts = np.concatenate([pos, col, uv], -1).reshape(-1, 9).astype(np.float32)
    return verts, proj


def build_c3(ctx, num_tris=2_000_000, width=1920, height=1080, tex_size=2048):
    """Alpha-blended triangle soup with clipping at 1080p."""
    s = Scene(ctx, f"c3_soup_{num_tris}_{width}x{height}", width, height)
    verts, proj = soup_triangles(num_tris, width, height)
    mesh = s.add_mesh(verts, None, stride=36)
    tex = s.add_texture_rgba8(to_rgba8(value_noise(tex_size, tex_size, seed=3, alpha=1.0)))
    ub = vcolor_uniforms(proj, tex)
    sh = s.add_shader(A.PROGRAM_VCOLOR_TEX_ALPHA, 2, ub, blend=A.BLEND_ALPHA)
    s.draws.append((mesh, 1, sh))
    s.num_triangles = num_tris
    return s


def c4_mesh_plan(num_draws, seed=4, lo=12, hi=65000):
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(math.log(lo), math.log(hi), num_draws))
    plan = []
    for i, c in enumerate(counts):
        kind = ("sphere", "torus", "grid")[i % 3]
        if kind == "sphere":
            lat = max(2, int(round(math.sqrt(c / 4.0))))
            plan.append((kind, 2 * lat, lat))
        elif kind == "torus":
            mi = max(3, int(round(math.sqrt(c / 6.0))))
            plan.append((kind, 3 * mi, mi))
        else:
            g = max(1, int(round(math.sqrt(c / 2.0))))
            plan.append((kind, g, g))
    return plan, rng


def build_c4(ctx, num_draws=256, width=3840, height=2160, tex_size=512, batched=True):
    """num_draws independent meshes with uneven triangle counts, one texture
    and model matrix each, Lambert + ambient, 2160p."""
    s = Scene(ctx, f"c4_batch_{num_draws}_{width}x{height}", width, height)
    plan, rng = c4_mesh_plan(num_draws)
    eye = (0.0, 0.0, 60.0)
    vp = perspective(60.0, width / height, 0.1, 300.0) @ look_at(eye, (0, 0, 0), (0, 1, 0))
    light = np.asarray([0.3, 0.8, 0.5])
    light = light / np.linalg.norm(light)
    tris = 0
    for i, (kind, a, b) in enumerate(plan):
        if kind == "sphere":
            verts, idx = uv_sphere(a, b)
        elif kind == "torus":
            verts, idx = torus(a, b)
        else:
            verts, idx = grid(a, b)
        mesh = s.add_mesh(verts, idx)
        tex = s.add_texture_rgba8(to_rgba8(value_noise(tex_size, tex_size, seed=1000 + i, octaves=3, alpha=1.0)))
        t = rng.uniform([-45, -25, -30], [45, 25, 10])
        model = translate(t) @ random_rotation(rng) @ scale(rng.uniform(1.0, 5.0))
        ub = lambert_uniforms(vp, model, [*light, 0.0], [0.1, 0.1, 0.1, 0.0], tex)
        sh = s.add_shader(A.PROGRAM_LAMBERT_TEX, 2, ub)
        s.draws.append((mesh, 1, sh))
        tris += idx.size // 3
    s.num_triangles = tris
    s.batched = batched
    return s


def quat_axis_angle(axis, angle):
    """Unit quaternion (x, y, z, w) of a rotation by angle about axis."""
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    h = math.sin(0.5 * angle)
    return (float(a[0] * h), float(a[1] * h), float(a[2] * h), float(math.cos(0.5 * angle)))


class GraphScene(Scene):
    """A scene graph (SL_SceneGraph) drawn through the library's scene entry
    points: per frame, clear, the frame's transform changes, update, then
    the mesh-node traversal as one draw list."""

    def __init__(self, ctx, name, width, height):
        super().__init__(ctx, name, width, height)
        self.scene = ctx.create_scene()
        self.num_nodes = 0
        self.shader = None
        self.projection = np.eye(4)
        self.view = np.eye(4)
        self.cull_projection = None   # frustum of the culling test (None: no culling)
        self.frame = 0
        self.animate = None      # callable(scene, frame) setting transforms

    def node(self, parent, sub_meshes, transform):
        n = self.ctx.scene_insert_node(self.scene, parent, list(sub_meshes), transform)
        self.num_nodes += 1
        return n

    def render(self, clear=True):
        ctx = self.ctx
        if clear:
            ctx.clear_framebuffer(self.fbo, 0, self.clear_color, self.clear_depth)
        if self.animate is not None:
            self.animate(self, self.frame)
        ctx.scene_update(self.scene)
        ctx.scene_draw(self.scene, self.fbo, self.shader, self.projection, self.view, self.cull_projection)
        self.frame += 1

    def read_models(self):
        return self.ctx.scene_read_models(self.scene, self.num_nodes)


def build_scene_graph(ctx, width=320, height=240, groups=6, per_group=5, seed=21, tex_size=64, lon=24, lat=12, cull_fov=40.0):
    """A scene graph of `groups` group nodes in a ring, each with `per_group`
    mesh-node children (some with two submeshes, one with a lines-mode
    submesh the traversal skips, one with a grandchild), an FPS-view
    transform on one child, a group far outside the frustum, and two
    children inserted after all groups (so their subtrees are not
    contiguous: the reference's update leaves the second one stale when its
    group changes). Frames 1, 2, ... rotate group 3, move one child and one
    grandchild. Lambert with one texture per mesh, cull on back faces; submeshes
    culled against a cull_fov-degree frustum (None: no culling), narrower than
    the drawn 55 degrees."""
    rng = np.random.default_rng(seed)
    s = GraphScene(ctx, f"scene_graph_{groups}x{per_group}", width, height)
    shapes = [uv_sphere(lon, lat), torus(lon, max(6, lat // 2)), grid(8, 8)]
    meshes = []
    tris = []
    for k, (verts, idx) in enumerate(shapes):
        mesh = s.add_mesh(verts, idx)
        tex = s.add_texture_rgba8(to_rgba8(value_noise(tex_size, tex_size, seed=seed + k, octaves=2, alpha=1.0)))
        mesh.materialId = ctx.scene_insert_material(s.scene, tex)
        meshes.append(ctx.scene_insert_mesh(s.scene, mesh, verts[:, :3].max(0), verts[:, :3].min(0)))
        tris.append(idx.size // 3)
    lines = A.Mesh(mesh.vaoId, 0, (shapes[2][1].size // 2) * 2, A.RENDER_MODE_INDEXED_LINES, mesh.materialId)
    lines_id = ctx.scene_insert_mesh(s.scene, lines, (1, 1, 1), (-1, -1, -1))
    light = np.asarray([0.4, 0.8, 0.45])
    light = light / np.linalg.norm(light)
    s.projection = perspective(55.0, width / height, 0.5, 60.0)
    s.view = look_at((0.0, 6.0, 17.0), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0))
    # a narrower culling frustum than the drawn one, so culling shows in the image
    s.cull_projection = perspective(cull_fov, width / height, 0.5, 60.0) if cull_fov else None
    s.shader = s.add_shader(A.PROGRAM_LAMBERT_TEX, 2, lambert_uniforms(np.eye(4), np.eye(4), [*light, 0.0],
                                                                       [0.12, 0.12, 0.12, 0.0], 0))
    T = A.make_transform
    group_ids, children = [], []
    num_tris = 0
    for g in range(groups):
        ang = 2.0 * math.pi * g / groups
        gpos = (9.0 * math.cos(ang), float(rng.uniform(-2.0, 2.0)), 9.0 * math.sin(ang) - 3.0)
        gn = s.node(A.SCENE_ROOT, [], T(gpos, (1.0, 1.0, 1.0), quat_axis_angle(rng.normal(size=3), rng.uniform(0, math.pi))))
        group_ids.append(gn)
        for c in range(per_group):
            subs = [meshes[(g + c) % 3]]
            if c % 3 == 0:
                subs.append(meshes[(g + c + 1) % 3])
            if c == 1:
                subs.append(lines_id)
            pos = rng.uniform(-3.0, 3.0, 3)
            sc = rng.uniform(0.4, 1.2, 3)
            cn = s.node(gn, subs, T(pos, sc, quat_axis_angle(rng.normal(size=3), rng.uniform(0, math.pi)),
                                    type=1 if (g == 2 and c == 0) else 0))
            num_tris += sum(tris[m] for m in subs if m < len(tris))
            children.append(cn)
            if c == 2:
                gc = s.node(cn, [meshes[0]], T((0.0, 1.6, 0.0), (0.5, 0.5, 0.5), (0.0, 0.0, 0.0, 1.0)))
                num_tris += tris[0]
                children.append(gc)
    far = s.node(A.SCENE_ROOT, [], T((0.0, 0.0, 200.0)))
    s.node(far, [meshes[1]], T())
    num_tris += tris[1]
    late0 = s.node(group_ids[0], [meshes[1]], T((0.0, -2.5, 0.0), (0.7, 0.7, 0.7)))
    late3 = s.node(group_ids[min(3, groups - 1)], [meshes[0]], T((0.0, 2.5, 0.0), (0.8, 0.8, 0.8)))
    num_tris += tris[1] + tris[0]
    s.num_triangles = num_tris
    s.late_children = (late0, late3)
    g3 = group_ids[min(3, groups - 1)]
    g3_pos = (9.0 * math.cos(2.0 * math.pi * min(3, groups - 1) / groups), 0.5, 9.0 * math.sin(2.0 * math.pi * min(3, groups - 1) / groups) - 3.0)
    mover = children[1]
    grand = children[3] if len(children) > 3 else children[-1]

    def animate(scene, frame):
        if frame == 0:
            return
        scene.ctx.scene_set_transform(scene.scene, g3, T(g3_pos, (1.0, 1.0, 1.0), quat_axis_angle((0.2, 1.0, 0.1), 0.4 * frame)))
        scene.ctx.scene_set_transform(scene.scene, mover, T((0.5 * frame - 1.0, 0.3, 0.2), (0.9, 0.9, 0.9),
                                                            quat_axis_angle((1.0, 0.0, 0.3), 0.3 * frame)))
        if frame % 2 == 0:
            scene.ctx.scene_set_transform(scene.scene, grand, T((0.0, 1.6 + 0.1 * frame, 0.0), (0.5, 0.6, 0.5)))

    s.animate = animate
    return s


def displaced_sphere(lon=100, lat=50, seed=5, amplitude=0.1, waves=6):
    """UV sphere (lon*lat*2 triangles) with radius 1 + amplitude * noise(n),
    noise a seeded sum of sinusoids of the direction: positions (V x 3),
    uvs (V x 2), triangle indices."""
    verts, idx = uv_sphere(lon, lat)
    n = verts[:, 5:8].astype(np.float64)
    rng = np.random.default_rng(seed)
    freq = rng.normal(size=(waves, 3)) * 2.5
    phase = rng.uniform(0.0, 2.0 * math.pi, waves)
    amp = rng.uniform(0.3, 1.0, waves)
    noise = (amp[None, :] * np.sin(n @ freq.T + phase[None, :])).sum(1) / amp.sum()
    pos = n * (1.0 + amplitude * noise)[:, None]
    return pos.astype(np.float32), verts[:, 3:5].copy(), idx


def c5_uv(uv):
    """The differentiable scene's texture coordinates: the sphere's (j/lon,
    i/lat) grid scaled and offset so that no mesh edge lies on a texel
    boundary (where the bilinear derivative jumps) and no triangle spans the
    repeat seam."""
    return (np.asarray(uv, np.float64) * [0.97, 0.93] + [0.0157, 0.0347]).astype(np.float32)


class DiffScene(Scene):
    """One opaque vertex-colour x float-texture draw whose per-vertex
    positions and colours and whose texels are parameters: the scene of the
    differentiable render."""

    def set_params(self, pos=None, col=None, tex=None):
        if pos is not None:
            self.pos = np.ascontiguousarray(pos, np.float32)
        if col is not None:
            self.col = np.ascontiguousarray(col, np.float32)
        if tex is not None:
            self.tex = np.ascontiguousarray(tex, np.float32)
            self.ctx.texture_set_texels(self.tex_id, self.tex)
        if pos is not None or col is not None:
            self.ctx.vbo_assign(self.vbo, self.vertex_array())

    def vertex_array(self):
        return np.concatenate([self.pos, self.col, self.uv], 1).astype(np.float32)


def build_c5(ctx, width=512, height=512, tex_size=256, lon=100, lat=50, seed=5, index_dtype=np.uint32):
    """Differentiable render: a 10k-triangle noise-displaced sphere with
    float32 per-vertex colours and a tex_size^2 float32 RGBA texture,
    vertex colour x texture, depth LESS, 512x512 RGBA float target.
    index_dtype None draws the triangles non-indexed (vertices expanded)."""
    s = DiffScene(ctx, f"c5_diff_{width}x{height}", width, height, color_type=A.COLOR_RGBA_FLOAT)
    s.clear_color = (0.0, 0.0, 0.0, 0.0)
    pos, uv, idx = displaced_sphere(lon, lat, seed)
    uv = c5_uv(uv)
    if index_dtype is None:
        pos, uv, idx = pos[idx], uv[idx], None
    rng = np.random.default_rng(seed + 1)
    col = np.concatenate([rng.uniform(0.3, 1.0, (pos.shape[0], 3)), np.ones((pos.shape[0], 1))], 1)
    ntri = pos.shape[0] // 3 if idx is None else idx.size // 3
    s.tri = np.arange(3 * ntri).reshape(-1, 3) if idx is None else idx.reshape(-1, 3).astype(np.int64)
    s.pos, s.uv = pos, uv.astype(np.float32)
    s.col = col.astype(np.float32)
    s.tex = value_noise(tex_size, tex_size, seed=seed + 2, octaves=3).astype(np.float32)
    s.vbo = ctx.create_vbo()
    ctx.vbo_init(s.vbo, s.vertex_array())
    vao = ctx.create_vao()
    ctx.vao_set_vertex_buffer(vao, s.vbo)
    ctx.vao_set_binding(vao, 0, 0, 36, 3, A.VERTEX_DATA_FLOAT)
    if idx is None:
        mesh = A.Mesh(vao, 0, 3 * ntri, A.RENDER_MODE_TRIANGLES, 0)
        s.geometry_bytes = s.vertex_array().nbytes
    else:
        ibo = ctx.create_ibo()
        ctx.ibo_init(ibo, idx.astype(index_dtype))
        ctx.vao_set_index_buffer(vao, ibo)
        mesh = A.Mesh(vao, 0, idx.size, A.RENDER_MODE_INDEXED_TRIANGLES, 0)
        s.geometry_bytes = s.vertex_array().nbytes + idx.astype(index_dtype).nbytes
    s.tex_id = s.add_texture_rgbaf(s.tex)
    s.mvp = perspective(60.0, width / height, 0.1, 100.0) @ look_at((0, 0, 2.5), (0, 0, 0), (0, 1, 0))
    sh = s.add_shader(A.PROGRAM_VCOLOR_TEXF, 2, vcolor_uniforms(s.mvp, s.tex_id))
    s.mesh, s.shader = mesh, sh
    s.draws.append((mesh, 1, sh))
    s.num_triangles = ntri
    if ctx.gpu:
        ctx.fbo_enable_visibility(s.fbo)   # the CPU restatement has no visibility map
    return s


def c5_perturbed(s, seed=6, col_sigma=0.05, tex_sigma=0.05, pos_sigma=0.05):
    """Seeded perturbation of a c5 scene's parameters (the target's)."""
    rng = np.random.default_rng(seed)
    pos = s.pos + rng.normal(0.0, pos_sigma, s.pos.shape).astype(np.float32)
    col = s.col + rng.normal(0.0, col_sigma, s.col.shape).astype(np.float32)
    tex = s.tex + rng.normal(0.0, tex_sigma, s.tex.shape).astype(np.float32)
    return pos, col, tex


BUILDERS = {"c1": build_c1, "c2": build_c2, "c3": build_c3, "c4": build_c4, "c5": build_c5}
