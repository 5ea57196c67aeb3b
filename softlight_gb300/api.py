"""ctypes binding of the draw-path C ABI (include/slg.h), shaped like SoftLight's
SL_Context (softlight/include/softlight/SL_Context.hpp:59-306).

`SLContext` wraps any library that exports the slg.h entry points under a
given symbol prefix. The product library is softlight_gb300/libslg.so
(prefix "slg_"); `Context()` opens it and raises if it is missing, so there is
no silent CPU fallback.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libslg.so")

INVALID_ID = (1 << 64) - 1

# enums (values of include/slg.h, which mirror the reference's)
VERTEX_DATA_BYTE, VERTEX_DATA_SHORT, VERTEX_DATA_INT, VERTEX_DATA_LONG, VERTEX_DATA_FLOAT = 0, 1, 2, 3, 4
RENDER_MODE_POINTS, RENDER_MODE_INDEXED_POINTS = 0x01, 0x03
RENDER_MODE_LINES, RENDER_MODE_INDEXED_LINES = 0x04, 0x0C
RENDER_MODE_TRI_WIRE, RENDER_MODE_INDEXED_TRI_WIRE = 0x50, 0x70
RENDER_MODE_TRIANGLES, RENDER_MODE_INDEXED_TRIANGLES = 0x10, 0x30
CULL_BACK_FACE, CULL_FRONT_FACE, CULL_OFF = 0, 1, 2
DEPTH_TEST_OFF, DEPTH_TEST_LESS_THAN, DEPTH_TEST_LESS_EQUAL, DEPTH_TEST_GREATER_THAN = 0, 1, 2, 3
DEPTH_TEST_GREATER_EQUAL, DEPTH_TEST_EQUAL, DEPTH_TEST_NOT_EQUAL = 4, 5, 6
DEPTH_MASK_OFF, DEPTH_MASK_ON = 0, 1
BLEND_OFF, BLEND_ALPHA, BLEND_PREMULTIPLED_ALPHA, BLEND_ADDITIVE, BLEND_SCREEN = 0, 1, 2, 3, 4
# SL_ColorDataType 0..27: (R, RG, RGB, RGBA) x (8U, 16U, 32U, 64U, HALF, FLOAT, DOUBLE)
COLOR_COMPONENT_DTYPES = ("uint8", "uint16", "uint32", "uint64", "float16", "float32", "float64")
for _n, _prefix in enumerate(("R", "RG", "RGB", "RGBA")):
    for _k, _suffix in enumerate(("8U", "16U", "32U", "64U", "HALF", "FLOAT", "DOUBLE")):
        globals()[f"COLOR_{_prefix}_{_suffix}"] = 7 * _n + _k
# packed formats (SL_ColorCompressed.hpp): one integer per texel
COLOR_RGB_332, COLOR_RGB_565, COLOR_RGBA_5551, COLOR_RGBA_4444, COLOR_RGBA_1010102 = 28, 29, 30, 31, 32
PACKED_FORMATS = {28: ("uint8", (3, 3, 2)), 29: ("uint16", (5, 6, 5)), 30: ("uint16", (5, 5, 5, 1)),
                  31: ("uint16", (4, 4, 4, 4)), 32: ("uint32", (10, 10, 10, 2))}
COLOR_TYPES = tuple(range(33))
PROGRAM_LAMBERT_TEX, PROGRAM_BLINN_PHONG_INST, PROGRAM_VCOLOR_TEX_ALPHA = 1, 2, 3
PROGRAM_VCOLOR_TEXF, PROGRAM_FLAT_COLOR, PROGRAM_GBUFFER = 4, 5, 6
PROGRAM_VCOLOR_TEX_CUTOUT, PROGRAM_FRAG_COORD = 7, 8
PROGRAM_USER_FIRST = 256
PROGRAM_DISCARDS, PROGRAM_WRITES_DEPTH = 1, 2

BYTES_PER_COLOR = {t: (t // 7 + 1) * (1, 2, 4, 8, 2, 4, 8)[t % 7] for t in range(28)}
BYTES_PER_COLOR.update({28: 1, 29: 2, 30: 2, 31: 2, 32: 4})


def color_layout(t):
    """(components, numpy dtype name) of a colour format; a packed format is
    one integer per texel."""
    if t in PACKED_FORMATS:
        return 1, PACKED_FORMATS[t][0]
    return t // 7 + 1, COLOR_COMPONENT_DTYPES[t % 7]


class Mesh(C.Structure):
    """SL_Mesh (softlight/include/softlight/SL_Mesh.hpp:30-39)."""
    _fields_ = [("vaoId", C.c_size_t), ("elementBegin", C.c_size_t), ("elementEnd", C.c_size_t),
                ("mode", C.c_uint32), ("materialId", C.c_uint32)]


class Transform(C.Structure):
    """SL_Transform's parameters (softlight/include/softlight/SL_Transform.hpp:60-75):
    orientation is a quaternion (x, y, z, w); type an SL_TransformType."""
    _fields_ = [("position", C.c_float * 3), ("scaling", C.c_float * 3), ("orientation", C.c_float * 4),
                ("type", C.c_uint32)]


SCENE_ROOT = 2 ** (8 * C.sizeof(C.c_size_t)) - 1   # SCENE_NODE_ROOT_ID


def make_transform(position=(0.0, 0.0, 0.0), scaling=(1.0, 1.0, 1.0), orientation=(0.0, 0.0, 0.0, 1.0), type=0):
    t = Transform()
    t.position[:] = [float(v) for v in position]
    t.scaling[:] = [float(v) for v in scaling]
    t.orientation[:] = [float(v) for v in orientation]
    t.type = type
    return t


class VertexShader(C.Structure):
    """SL_VertexShader (softlight/include/softlight/SL_Shader.hpp:58)."""
    _fields_ = [("numVaryings", C.c_uint8), ("cullMode", C.c_uint8), ("program", C.c_uint32)]


class FragmentShader(C.Structure):
    """SL_FragmentShader (softlight/include/softlight/SL_Shader.hpp:89)."""
    _fields_ = [("numVaryings", C.c_uint8), ("numOutputs", C.c_uint8), ("blend", C.c_uint8),
                ("depthTest", C.c_uint8), ("depthMask", C.c_uint8), ("program", C.c_uint32)]


class DrawCmd(C.Structure):
    _fields_ = [("mesh", Mesh), ("numInstances", C.c_size_t), ("shaderId", C.c_size_t)]


class SLError(RuntimeError):
    pass


class ProgramInfo(C.Structure):
    """slg_program_info (include/slg.h): one registered program."""
    _fields_ = [("id", C.c_uint32), ("vertexBytes", C.c_uint32), ("flags", C.c_uint32)]


# (name, restype, argtypes) for every entry point of include/slg.h
_SIGNATURES = [
    ("context_create", C.c_int, [C.POINTER(C.c_void_p)]),
    ("context_destroy", None, [C.c_void_p]),
    ("last_error", C.c_char_p, [C.c_void_p]),
    ("num_threads", C.c_uint, [C.c_void_p, C.c_uint]),
    ("create_vbo", C.c_size_t, [C.c_void_p]),
    ("vbo_init", C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p]),
    ("vbo_assign", C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.c_size_t]),
    ("create_ibo", C.c_size_t, [C.c_void_p]),
    ("ibo_init", C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t, C.c_int, C.c_void_p]),
    ("create_vao", C.c_size_t, [C.c_void_p]),
    ("vao_set_vertex_buffer", C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t]),
    ("vao_set_index_buffer", C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t]),
    ("vao_set_binding", C.c_int, [C.c_void_p, C.c_size_t, C.c_uint, C.c_ssize_t, C.c_ssize_t, C.c_uint, C.c_int]),
    ("create_texture", C.c_size_t, [C.c_void_p]),
    ("texture_init", C.c_int, [C.c_void_p, C.c_size_t, C.c_int, C.c_uint16, C.c_uint16, C.c_uint16]),
    ("texture_set_texels", C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]),
    ("texture_read", C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]),
    ("create_framebuffer", C.c_size_t, [C.c_void_p]),
    ("fbo_reserve_color_buffers", C.c_int, [C.c_void_p, C.c_size_t, C.c_uint]),
    ("fbo_attach_color_buffer", C.c_int, [C.c_void_p, C.c_size_t, C.c_uint, C.c_size_t]),
    ("fbo_attach_depth_buffer", C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t]),
    ("create_ubo", C.c_size_t, [C.c_void_p]),
    ("ubo_assign", C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]),
    ("create_shader", C.c_size_t, [C.c_void_p, C.POINTER(VertexShader), C.POINTER(FragmentShader), C.c_size_t]),
    ("clear_framebuffer", C.c_int, [C.c_void_p, C.c_size_t, C.c_uint, C.POINTER(C.c_double), C.c_double]),
    ("clear_color_buffer", C.c_int, [C.c_void_p, C.c_size_t, C.c_uint, C.POINTER(C.c_double)]),
    ("clear_depth_buffer", C.c_int, [C.c_void_p, C.c_size_t, C.c_double]),
    ("draw", C.c_int, [C.c_void_p, C.POINTER(Mesh), C.c_size_t, C.c_size_t]),
    ("draw_instanced", C.c_int, [C.c_void_p, C.POINTER(Mesh), C.c_size_t, C.c_size_t, C.c_size_t]),
    ("draw_multiple", C.c_int, [C.c_void_p, C.POINTER(Mesh), C.c_size_t, C.c_size_t, C.c_size_t]),
    ("draw_batch", C.c_int, [C.c_void_p, C.POINTER(DrawCmd), C.c_size_t, C.c_size_t]),
    ("blit", C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t]),
    ("blit_rect", C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t] + [C.c_uint16] * 8),
    ("blit_read", C.c_int, [C.c_void_p, C.c_size_t, C.c_int, C.c_uint16, C.c_uint16, C.c_void_p, C.c_size_t]),
    ("finish", C.c_int, [C.c_void_p]),
    ("create_scene", C.c_size_t, [C.c_void_p]),
    ("scene_insert_mesh", C.c_int, [C.c_void_p, C.c_size_t, C.POINTER(Mesh), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                    C.POINTER(C.c_size_t)]),
    ("scene_insert_material", C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t, C.POINTER(C.c_size_t)]),
    ("scene_insert_node", C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t, C.POINTER(C.c_size_t),
                                    C.POINTER(Transform), C.POINTER(C.c_size_t)]),
    ("scene_set_transform", C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t, C.POINTER(Transform)]),
    ("scene_update", C.c_int, [C.c_void_p, C.c_size_t]),
    ("scene_read_models", C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]),
    ("scene_draw", C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t, C.POINTER(C.c_float), C.POINTER(C.c_float),
                             C.POINTER(C.c_float)]),
]

# GPU-only entry points (include/slg.h, "GPU-only controls")
_GPU_SIGNATURES = [
    ("context_stream", C.c_void_p, [C.c_void_p]),
    ("set_tile_size", C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    ("profile_stages", C.c_int, [C.c_void_p, C.c_int]),
    ("stage_times", C.c_int, [C.c_void_p, C.POINTER(C.c_float)]),
    ("set_raster_mode", C.c_int, [C.c_void_p, C.c_int]),
    ("untiled_raster", C.c_int, [C.c_void_p]),
    ("set_vertex_block", C.c_int, [C.c_void_p, C.c_int]),
    ("set_batch_graphs", C.c_int, [C.c_void_p, C.c_int]),
    ("autotune", C.c_int, [C.c_void_p, C.POINTER(DrawCmd), C.c_size_t, C.c_size_t, C.POINTER(C.c_double),
                           C.c_double, C.POINTER(C.c_int)]),
    ("draw_noalloc", C.c_int, [C.c_void_p, C.POINTER(Mesh), C.c_size_t, C.c_size_t]),
    ("set_scratch_caps", C.c_int, [C.c_void_p, C.c_size_t, C.c_size_t, C.c_uint]),
    ("ubo_assign_many", C.c_int, [C.c_void_p, C.POINTER(C.c_size_t), C.c_size_t, C.c_void_p, C.c_size_t, C.c_size_t]),
    ("register_programs", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(ProgramInfo), C.c_size_t]),
    ("fbo_enable_visibility", C.c_int, [C.c_void_p, C.c_size_t, C.c_int]),
    ("fbo_read_visibility", C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]),
    ("diff_shade", C.c_int, [C.c_void_p, C.POINTER(Mesh), C.c_size_t, C.c_size_t, C.c_void_p, C.c_size_t]),
    ("draw_adjoint", C.c_int, [C.c_void_p, C.POINTER(Mesh), C.c_size_t, C.c_size_t, C.c_void_p, C.c_size_t,
                               C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t]),
]


def exported_symbols(prefix="slg_", gpu=True):
    """Names of the C ABI entry points a conforming library must export."""
    sigs = _SIGNATURES + (_GPU_SIGNATURES if gpu else [])
    return [prefix + n for n, _, _ in sigs]


_LIB_CACHE = {}


def open_library(path, prefix, gpu):
    """dlopen a library exporting the slg.h ABI under `prefix` and bind its
    signatures. Raises OSError if the file is missing."""
    key = (os.path.realpath(path), prefix)
    if key in _LIB_CACHE:
        return _LIB_CACHE[key]
    if not os.path.exists(path):
        raise OSError(f"draw-path library not found: {path} (run softlight_gb300.build.build())")
    lib = C.CDLL(path)
    for name, res, args in _SIGNATURES + (_GPU_SIGNATURES if gpu else []):
        fn = getattr(lib, prefix + name)
        fn.restype = res
        fn.argtypes = args
    _LIB_CACHE[key] = lib
    return lib


class SLContext:
    """SL_Context-shaped wrapper over one context of an slg.h library."""

    def __init__(self, lib, prefix="slg_", gpu=True):
        self._lib = lib
        self._p = prefix
        self.gpu = gpu
        h = C.c_void_p()
        rc = self._fn("context_create")(C.byref(h))
        if rc != 0:
            raise SLError(f"context_create failed ({rc})")
        self._h = h
        self._keep = []

    # -- plumbing -----------------------------------------------------------
    def _fn(self, name):
        return getattr(self._lib, self._p + name)

    def _call(self, name, *args):
        rc = self._fn(name)(self._h, *args)
        if rc != 0:
            raise SLError(f"{self._p}{name} failed ({rc}): {self.last_error()}")
        return rc

    def _id(self, name, *args):
        r = self._fn(name)(self._h, *args)
        if r == INVALID_ID:
            raise SLError(f"{self._p}{name} failed: {self.last_error()}")
        return r

    def last_error(self):
        s = self._fn("last_error")(self._h)
        return s.decode() if s else ""

    def close(self):
        if getattr(self, "_h", None):
            self._fn("context_destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- resources ----------------------------------------------------------
    def num_threads(self, n=0):
        return self._fn("num_threads")(self._h, n)

    def create_vbo(self):
        return self._id("create_vbo")

    def vbo_init(self, vbo, data):
        a = np.ascontiguousarray(data)
        self._call("vbo_init", vbo, a.nbytes, a.ctypes.data_as(C.c_void_p))

    def vbo_assign(self, vbo, data, offset=0):
        a = np.ascontiguousarray(data)
        self._call("vbo_assign", vbo, a.ctypes.data_as(C.c_void_p), offset, a.nbytes)

    def create_ibo(self):
        return self._id("create_ibo")

    def ibo_init(self, ibo, indices):
        a = np.ascontiguousarray(indices)
        t = {np.dtype(np.uint8): VERTEX_DATA_BYTE, np.dtype(np.uint16): VERTEX_DATA_SHORT,
             np.dtype(np.uint32): VERTEX_DATA_INT}[a.dtype]
        self._call("ibo_init", ibo, a.size, t, a.ctypes.data_as(C.c_void_p))

    def create_vao(self):
        return self._id("create_vao")

    def vao_set_vertex_buffer(self, vao, vbo):
        self._call("vao_set_vertex_buffer", vao, vbo)

    def vao_set_index_buffer(self, vao, ibo):
        self._call("vao_set_index_buffer", vao, ibo)

    def vao_set_binding(self, vao, bind_id, offset, stride, num_components=3, data_type=VERTEX_DATA_FLOAT):
        self._call("vao_set_binding", vao, bind_id, offset, stride, num_components, data_type)

    def create_texture(self):
        return self._id("create_texture")

    def texture_init(self, tex, color_type, w, h, d=1):
        self._call("texture_init", tex, color_type, w, h, d)

    def texture_set_texels(self, tex, data):
        a = np.ascontiguousarray(data)
        self._call("texture_set_texels", tex, a.ctypes.data_as(C.c_void_p), a.nbytes)

    def texture_read(self, tex, shape, dtype, out=None):
        """Copy a texture's texels into a numpy array of `shape`/`dtype`."""
        if out is None:
            out = np.empty(shape, dtype=dtype)
        self._call("texture_read", tex, out.ctypes.data_as(C.c_void_p), out.nbytes)
        return out

    def create_framebuffer(self):
        return self._id("create_framebuffer")

    def fbo_reserve_color_buffers(self, fbo, n):
        self._call("fbo_reserve_color_buffers", fbo, n)

    def fbo_attach_color_buffer(self, fbo, index, tex):
        self._call("fbo_attach_color_buffer", fbo, index, tex)

    def fbo_attach_depth_buffer(self, fbo, tex):
        self._call("fbo_attach_depth_buffer", fbo, tex)

    def create_ubo(self):
        return self._id("create_ubo")

    def ubo_assign(self, ubo, data):
        """data: bytes or a numpy array, passed to the C ABI without a copy."""
        if isinstance(data, np.ndarray):
            a = np.ascontiguousarray(data)
            self._call("ubo_assign", ubo, a.ctypes.data_as(C.c_void_p), a.nbytes)
        else:
            b = bytes(data)
            self._call("ubo_assign", ubo, C.cast(C.c_char_p(b), C.c_void_p), len(b))

    def create_shader(self, vs, fs, ubo=INVALID_ID):
        return self._id("create_shader", C.byref(vs), C.byref(fs), ubo)

    # -- frame --------------------------------------------------------------
    def clear_framebuffer(self, fbo, attachment, rgba, depth):
        c = (C.c_double * 4)(*rgba)
        self._call("clear_framebuffer", fbo, attachment, c, depth)

    def clear_color_buffer(self, fbo, attachment, rgba):
        c = (C.c_double * 4)(*rgba)
        self._call("clear_color_buffer", fbo, attachment, c)

    def clear_depth_buffer(self, fbo, depth):
        self._call("clear_depth_buffer", fbo, depth)

    def draw(self, mesh, shader, fbo):
        self._call("draw", C.byref(mesh), shader, fbo)

    def draw_instanced(self, mesh, num_instances, shader, fbo):
        self._call("draw_instanced", C.byref(mesh), num_instances, shader, fbo)

    def draw_multiple(self, meshes, shader, fbo):
        arr = (Mesh * len(meshes))(*meshes)
        self._call("draw_multiple", arr, len(meshes), shader, fbo)

    def draw_batch(self, cmds, fbo):
        arr = (DrawCmd * len(cmds))(*cmds)
        self._call("draw_batch", arr, len(cmds), fbo)

    # scene graph (SL_SceneGraph)
    def create_scene(self):
        return self._id("create_scene")

    def scene_insert_mesh(self, scene, mesh, max_point, min_point):
        out = C.c_size_t()
        hi = (C.c_float * 3)(*[float(v) for v in max_point])
        lo = (C.c_float * 3)(*[float(v) for v in min_point])
        self._call("scene_insert_mesh", scene, C.byref(mesh), hi, lo, C.byref(out))
        return out.value

    def scene_insert_material(self, scene, texture):
        out = C.c_size_t()
        self._call("scene_insert_material", scene, texture, C.byref(out))
        return out.value

    def scene_insert_node(self, scene, parent, sub_meshes, transform):
        out = C.c_size_t()
        ids = (C.c_size_t * max(1, len(sub_meshes)))(*sub_meshes)
        self._call("scene_insert_node", scene, parent, len(sub_meshes), ids, C.byref(transform), C.byref(out))
        return out.value

    def scene_set_transform(self, scene, node, transform):
        self._call("scene_set_transform", scene, node, C.byref(transform))

    def scene_update(self, scene):
        self._call("scene_update", scene)

    def scene_read_models(self, scene, num_nodes):
        out = np.zeros((num_nodes, 16), np.float32)
        self._call("scene_read_models", scene, out.ctypes.data_as(C.c_void_p), num_nodes)
        return out

    def scene_draw(self, scene, fbo, shader, projection, view, cull_projection=None):
        """projection, view, cull_projection: 4x4 row-major numpy matrices
        (passed column-major); no culling when cull_projection is None."""
        def cm(m):
            return np.ascontiguousarray(np.asarray(m, np.float32).T).ravel()
        p, v = cm(projection), cm(view)
        cp = cm(cull_projection) if cull_projection is not None else None
        self._call("scene_draw", scene, fbo, shader, p.ctypes.data_as(C.POINTER(C.c_float)),
                   v.ctypes.data_as(C.POINTER(C.c_float)),
                   cp.ctypes.data_as(C.POINTER(C.c_float)) if cp is not None else None)

    def set_scratch_caps(self, entries=0, clip_records=0, sort_keys=0):
        """slg_set_scratch_caps: start the scratch buffers small (overflow
        recovery tests)."""
        self._call("set_scratch_caps", entries, clip_records, sort_keys)

    def ubo_assign_many(self, ids, blocks):
        """slg_ubo_assign_many: blocks is a C-contiguous uint8 array of shape
        (len(ids), numBytes); row k goes to uniform block ids[k]."""
        arr = (C.c_size_t * len(ids))(*ids)
        self._call("ubo_assign_many", arr, len(ids), blocks.ctypes.data_as(C.c_void_p), blocks.strides[0], blocks.shape[1])

    def register_programs(self, ops_ptr, programs):
        """slg_register_programs: ops_ptr is the address of an
        slg_pipeline_ops table (a caller's compiled program set); programs
        is a list of (id, vertex bytes, flags)."""
        arr = (ProgramInfo * len(programs))(*[ProgramInfo(*p) for p in programs])
        self._call("register_programs", C.c_void_p(ops_ptr), arr, len(programs))

    def draw_noalloc(self, mesh, shader, fbo):
        """slg_draw with its scratch in a fixed device array (no allocation)."""
        self._call("draw_noalloc", C.byref(mesh), shader, fbo)

    # -- differentiable rendering (device pointers as integers) -------------
    def fbo_enable_visibility(self, fbo, enable=True):
        self._call("fbo_enable_visibility", fbo, 1 if enable else 0)

    def fbo_read_visibility(self, fbo, shape):
        out = np.empty(shape, np.uint32)
        self._call("fbo_read_visibility", fbo, out.ctypes.data_as(C.c_void_p), out.size)
        return out

    def diff_shade(self, mesh, shader, fbo, image_ptr, count):
        self._call("diff_shade", C.byref(mesh), shader, fbo, C.c_void_p(image_ptr), count)

    def draw_adjoint(self, mesh, shader, fbo, d_image_ptr, d_image_count, d_vertices_ptr, d_vertex_count,
                     d_texels_ptr, d_texel_count):
        self._call("draw_adjoint", C.byref(mesh), shader, fbo, C.c_void_p(d_image_ptr), d_image_count,
                   C.c_void_p(d_vertices_ptr), d_vertex_count, C.c_void_p(d_texels_ptr), d_texel_count)

    def blit(self, out_tex, in_tex):
        self._call("blit", out_tex, in_tex)

    def blit_rect(self, out_tex, in_tex, src, dst):
        """src = (x0, y0, x1, y1) in the input texture, dst likewise in the output."""
        self._call("blit_rect", out_tex, in_tex, *src, *dst)

    def blit_read(self, in_tex, color_type, width, height):
        """The texture scaled into a width x height host image of color_type."""
        shape = (height, width) if color_type == COLOR_R_FLOAT else (height, width, 4)
        dtype = np.uint8 if color_type == COLOR_RGBA_8U else np.float32
        out = np.empty(shape, dtype)
        self._call("blit_read", in_tex, color_type, width, height, out.ctypes.data_as(C.c_void_p), out.nbytes)
        return out

    def finish(self):
        self._call("finish")

    # -- GPU-only -----------------------------------------------------------
    def stream_handle(self):
        return self._fn("context_stream")(self._h)

    def set_tile_size(self, w, h):
        self._call("set_tile_size", w, h)

    def profile_stages(self, enable=True):
        self._call("profile_stages", 1 if enable else 0)

    def set_raster_mode(self, mode):
        self._call("set_raster_mode", mode)

    def untiled_raster(self):
        """Whether order-free triangle / point launches run untiled."""
        return bool(self._fn("untiled_raster")(self._h))

    def set_vertex_block(self, threads):
        self._call("set_vertex_block", threads)

    def set_batch_graphs(self, enable=True):
        self._call("set_batch_graphs", 1 if enable else 0)

    def autotune(self, cmds, fbo, rgba=(0.0, 0.0, 0.0, 1.0), depth=1.0):
        """Picks the fastest tile size and vertex block for clear + draw_batch;
        returns (tileW, tileH, vertex block)."""
        arr = (DrawCmd * len(cmds))(*cmds)
        c = (C.c_double * 4)(*rgba)
        out = (C.c_int * 3)()
        self._call("autotune", arr, len(cmds), fbo, c, depth, out)
        return tuple(out)

    def stage_times(self):
        ms = (C.c_float * 4)()
        self._call("stage_times", ms)
        return list(ms)


def Context():
    """A context of the GPU library; raises OSError when libslg.so is absent."""
    lib = open_library(LIB_PATH, "slg_", gpu=True)
    return SLContext(lib, "slg_", gpu=True)
