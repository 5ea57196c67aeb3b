/*
 * slg.h - C ABI of the GB300 draw path (SoftLight-compatible).
 *
 * Every entry point mirrors a member of SoftLight's SL_Context or of one of
 * the resource objects it owns; the reference interface each one replaces is
 * cited beside it (paths relative to the SoftLight source tree). Resource ids
 * are size_t handles exactly as in SL_Context; set-up calls return
 * SLG_INVALID_ID or a negative status on error, draws return a status where
 * SL_Context::draw returns void (the facade in slg_context.hpp keeps the
 * void signature). The text of the last error is available through
 * slg_last_error().
 *
 * Only plain C types cross this boundary: no CUDA, torch or C++ types.
 */
#ifndef SLG_H
#define SLG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SLG_INVALID_ID ((size_t)-1)

/* status codes */
enum slg_status
{
    SLG_OK              = 0,
    SLG_ERR_INVALID_ID  = -1, /* unknown resource id */
    SLG_ERR_INVALID_ARG = -2, /* bad size, type or state */
    SLG_ERR_CUDA        = -3, /* a CUDA runtime call failed */
    SLG_ERR_OVERFLOW    = -4, /* an internal buffer was too small (retried internally) */
    SLG_ERR_TIMEOUT     = -5, /* a bounded device-side wait ran out */
    SLG_ERR_NO_MEMORY   = -6
};

/* SL_DataType (softlight/include/softlight/SL_Geometry.hpp:30) */
enum slg_data_type
{
    SLG_VERTEX_DATA_BYTE = 0,
    SLG_VERTEX_DATA_SHORT,
    SLG_VERTEX_DATA_INT,
    SLG_VERTEX_DATA_LONG,
    SLG_VERTEX_DATA_FLOAT,
    SLG_VERTEX_DATA_DOUBLE,
    SLG_VERTEX_DATA_INVALID
};

/* SL_RenderMode (softlight/include/softlight/SL_Mesh.hpp:16) */
enum slg_render_mode
{
    SLG_RENDER_MODE_POINTS            = 0x01,
    SLG_RENDER_MODE_INDEXED_POINTS    = 0x03,
    SLG_RENDER_MODE_LINES             = 0x04,
    SLG_RENDER_MODE_INDEXED_LINES     = 0x0C,
    SLG_RENDER_MODE_TRIANGLES         = 0x10,
    SLG_RENDER_MODE_INDEXED_TRIANGLES = 0x30,
    SLG_RENDER_MODE_TRI_WIRE          = 0x50,
    SLG_RENDER_MODE_INDEXED_TRI_WIRE  = 0x70
};

/* SL_CullMode, SL_DepthTest, SL_DepthMask, SL_BlendMode
 * (softlight/include/softlight/SL_PipelineState.hpp:15-66) */
enum slg_cull_mode  { SLG_CULL_BACK_FACE = 0, SLG_CULL_FRONT_FACE, SLG_CULL_OFF };
enum slg_depth_test
{
    SLG_DEPTH_TEST_OFF = 0,
    SLG_DEPTH_TEST_LESS_THAN,
    SLG_DEPTH_TEST_LESS_EQUAL,
    SLG_DEPTH_TEST_GREATER_THAN,
    SLG_DEPTH_TEST_GREATER_EQUAL,
    SLG_DEPTH_TEST_EQUAL,
    SLG_DEPTH_TEST_NOT_EQUAL
};
enum slg_depth_mask { SLG_DEPTH_MASK_OFF = 0, SLG_DEPTH_MASK_ON };
enum slg_blend_mode
{
    SLG_BLEND_OFF = 0,
    SLG_BLEND_ALPHA,
    SLG_BLEND_PREMULTIPLED_ALPHA,
    SLG_BLEND_ADDITIVE,
    SLG_BLEND_SCREEN
};

/* SL_ColorDataType (softlight/include/softlight/SL_Color.hpp:31), values the
 * reference's: R / RG / RGB / RGBA (type / 7 + 1 components) of u8, u16,
 * u32, u64, half, float, double (type % 7), densely packed, then five
 * packed formats. Colour attachments and clears accept all 33; depth attachments R_HALF, R_FLOAT,
 * R_DOUBLE; sampled textures RGBA_8U or RGBA_FLOAT; blits R_FLOAT, RGBA_8U,
 * RGBA_FLOAT. */
enum slg_color_type
{
    SLG_COLOR_R_8U        = 0,
    SLG_COLOR_R_16U       = 1,
    SLG_COLOR_R_32U       = 2,
    SLG_COLOR_R_64U       = 3,
    SLG_COLOR_R_HALF      = 4,
    SLG_COLOR_R_FLOAT     = 5,
    SLG_COLOR_R_DOUBLE    = 6,
    SLG_COLOR_RG_8U       = 7,
    SLG_COLOR_RG_16U      = 8,
    SLG_COLOR_RG_32U      = 9,
    SLG_COLOR_RG_64U      = 10,
    SLG_COLOR_RG_HALF     = 11,
    SLG_COLOR_RG_FLOAT    = 12,
    SLG_COLOR_RG_DOUBLE   = 13,
    SLG_COLOR_RGB_8U      = 14,
    SLG_COLOR_RGB_16U     = 15,
    SLG_COLOR_RGB_32U     = 16,
    SLG_COLOR_RGB_64U     = 17,
    SLG_COLOR_RGB_HALF    = 18,
    SLG_COLOR_RGB_FLOAT   = 19,
    SLG_COLOR_RGB_DOUBLE  = 20,
    SLG_COLOR_RGBA_8U     = 21,
    SLG_COLOR_RGBA_16U    = 22,
    SLG_COLOR_RGBA_32U    = 23,
    SLG_COLOR_RGBA_64U    = 24,
    SLG_COLOR_RGBA_HALF   = 25,
    SLG_COLOR_RGBA_FLOAT  = 26,
    SLG_COLOR_RGBA_DOUBLE = 27,
    /* packed, one integer per texel, fields from bit 0 up
     * (softlight/include/softlight/SL_ColorCompressed.hpp) */
    SLG_COLOR_RGB_332      = 28,   /* u8:  r 3, g 3, b 2 */
    SLG_COLOR_RGB_565      = 29,   /* u16: r 5, g 6, b 5 */
    SLG_COLOR_RGBA_5551    = 30,   /* u16: r 5, g 5, b 5, a 1 */
    SLG_COLOR_RGBA_4444    = 31,   /* u16: r 4, g 4, b 4, a 4 */
    SLG_COLOR_RGBA_1010102 = 32    /* u32: r 10, g 10, b 10, a 2 */
};

/* Built-in device shader programs. In SoftLight a shader is a host function
 * pointer (SL_VertexShader::shader, SL_FragmentShader::shader,
 * softlight/include/softlight/SL_Shader.hpp:58-92); on the GPU it is a
 * __device__ function compiled into a pipeline instance, named by this id. */
enum slg_shader_program
{
    SLG_PROGRAM_LAMBERT_TEX        = 1, /* textured Lambert + ambient, per-draw model matrix */
    SLG_PROGRAM_BLINN_PHONG_INST   = 2, /* textured Blinn-Phong, 4 point lights, per-instance matrices */
    SLG_PROGRAM_VCOLOR_TEX_ALPHA   = 3, /* vertex colour x RGBA8 texture, vertex alpha */
    SLG_PROGRAM_VCOLOR_TEXF        = 4, /* vertex colour x RGBA float texture */
    SLG_PROGRAM_FLAT_COLOR         = 5, /* uniform colour, no varyings */
    SLG_PROGRAM_GBUFFER            = 6, /* up to four outputs for multiple render targets (vertex-colour layout) */
    SLG_PROGRAM_VCOLOR_TEX_CUTOUT  = 7, /* vertex colour x RGBA8 texture with an alpha test: discards below alphaRef */
    SLG_PROGRAM_FRAG_COORD         = 8, /* fragment position and depth as colour; screen-door discard; writes depth */
    SLG_PROGRAM_USER_FIRST         = 256 /* ids from here on name programs registered with slg_register_programs */
};

/* SL_Mesh (softlight/include/softlight/SL_Mesh.hpp:30-39), same layout */
typedef struct slg_mesh
{
    size_t   vaoId;
    size_t   elementBegin;
    size_t   elementEnd;
    uint32_t mode;
    uint32_t materialId;
} slg_mesh;

/* SL_VertexShader (softlight/include/softlight/SL_Shader.hpp:58) */
typedef struct slg_vertex_shader
{
    uint8_t  numVaryings;
    uint8_t  cullMode;
    uint32_t program;     /* slg_shader_program */
} slg_vertex_shader;

/* SL_FragmentShader (softlight/include/softlight/SL_Shader.hpp:89) */
typedef struct slg_fragment_shader
{
    uint8_t  numVaryings;
    uint8_t  numOutputs;
    uint8_t  blend;
    uint8_t  depthTest;
    uint8_t  depthMask;
    uint32_t program;     /* slg_shader_program */
} slg_fragment_shader;

/* One draw of a batch: the arguments of one SL_Context::draw or
 * draw_instanced call (softlight/src/SL_Context.cpp:714-740). */
typedef struct slg_draw_cmd
{
    slg_mesh mesh;
    size_t   numInstances;
    size_t   shaderId;
} slg_draw_cmd;

typedef struct slg_context slg_context;

/* SL_Context::SL_Context / ~SL_Context (softlight/src/SL_Context.cpp:21-50) */
int         slg_context_create(slg_context** outCtx);
void        slg_context_destroy(slg_context* ctx);
const char* slg_last_error(const slg_context* ctx);

/* SL_Context::num_threads (softlight/src/SL_Context.cpp:1135,1145): accepted,
 * returns the value stored; the GPU path does not use host threads. */
unsigned slg_num_threads(slg_context* ctx, unsigned n);

/* SL_Context::create_vbo + SL_VertexBuffer::init/assign
 * (softlight/src/SL_Context.cpp:335; softlight/src/SL_VertexBuffer.cpp:96) */
size_t slg_create_vbo(slg_context* ctx);
int    slg_vbo_init(slg_context* ctx, size_t vboId, size_t numBytes, const void* data);
int    slg_vbo_assign(slg_context* ctx, size_t vboId, const void* data, size_t offset, size_t numBytes);

/* SL_Context::create_ibo + SL_IndexBuffer::init
 * (softlight/src/SL_Context.cpp:386; softlight/src/SL_IndexBuffer.cpp:138) */
size_t slg_create_ibo(slg_context* ctx);
int    slg_ibo_init(slg_context* ctx, size_t iboId, size_t numElements, int indexType, const void* data);

/* SL_Context::create_vao + SL_VertexArray::set_vertex_buffer / set_index_buffer /
 * set_binding (softlight/src/SL_Context.cpp:181;
 * softlight/include/softlight/SL_VertexArray.hpp:56-85,176,216) */
size_t slg_create_vao(slg_context* ctx);
int    slg_vao_set_vertex_buffer(slg_context* ctx, size_t vaoId, size_t vboId);
int    slg_vao_set_index_buffer(slg_context* ctx, size_t vaoId, size_t iboId);
int    slg_vao_set_binding(slg_context* ctx, size_t vaoId, unsigned bindId, ptrdiff_t offset,
                           ptrdiff_t stride, unsigned numComponents, int dataType);

/* SL_Context::create_texture + SL_Texture::init / set_texels / data
 * (softlight/src/SL_Context.cpp:232; softlight/src/SL_Texture.cpp:276;
 * softlight/include/softlight/SL_Texture.hpp:77-181) */
size_t slg_create_texture(slg_context* ctx);
int    slg_texture_init(slg_context* ctx, size_t texId, int colorType, uint16_t w, uint16_t h, uint16_t d);
int    slg_texture_set_texels(slg_context* ctx, size_t texId, const void* data, size_t numBytes);
/* Device-to-host read of a texture (replaces SL_Context::blit to a swapchain,
 * softlight/src/SL_Context.cpp:747-880): copies w*h*d texels. */
int    slg_texture_read(slg_context* ctx, size_t texId, void* dst, size_t numBytes);

/* SL_Context::blit(outTextureId, inTextureId) and its rectangle form
 * (softlight/src/SL_Context.cpp:747-812; SL_BlitProcessor::blit_nearest,
 * softlight/src/SL_BlitProcessor.cpp:621-660): nearest-neighbour scaled copy
 * with a vertical flip and the reference's colour-format conversions between
 * any two of the supported texture types. Rectangles whose reads would fall
 * outside the source texture, or writes outside the destination, are
 * rejected (the reference does not check them). */
int slg_blit(slg_context* ctx, size_t outTextureId, size_t inTextureId);
int slg_blit_rect(slg_context* ctx, size_t outTextureId, size_t inTextureId, uint16_t srcX0, uint16_t srcY0,
                  uint16_t srcX1, uint16_t srcY1, uint16_t dstX0, uint16_t dstY0, uint16_t dstX1, uint16_t dstY1);
/* SL_Context::blit(SL_TextureView& buffer, textureId) (softlight/src/SL_Context.cpp:816-880)
 * into host memory: the whole texture scaled into a dstW x dstH buffer of
 * dstColorType texels (a window's back buffer in the reference), read back
 * at once. */
int slg_blit_read(slg_context* ctx, size_t inTextureId, int dstColorType, uint16_t dstW, uint16_t dstH, void* dst,
                  size_t numBytes);

/* SL_Context::create_framebuffer + SL_Framebuffer::reserve_color_buffers /
 * attach_color_buffer / attach_depth_buffer (softlight/src/SL_Context.cpp:284;
 * softlight/src/SL_Framebuffer.cpp:823,855,908) */
size_t slg_create_framebuffer(slg_context* ctx);
int    slg_fbo_reserve_color_buffers(slg_context* ctx, size_t fboId, unsigned numColorBuffers);
int    slg_fbo_attach_color_buffer(slg_context* ctx, size_t fboId, unsigned index, size_t texId);
int    slg_fbo_attach_depth_buffer(slg_context* ctx, size_t fboId, size_t texId);

/* SL_Context::create_ubo (softlight/src/SL_Context.cpp:437) + SL_UniformBuffer (1024 bytes,
 * softlight/include/softlight/SL_UniformBuffer.hpp:12-20). Texture and buffer
 * references inside a uniform block are ids, not host pointers. */
size_t slg_create_ubo(slg_context* ctx);
int    slg_ubo_assign(slg_context* ctx, size_t uboId, const void* data, size_t numBytes);

/* slg_ubo_assign for many blocks in one call: block k (numBytes bytes at
 * blocks + k * blockStride) into uboIds[k]. No single reference
 * counterpart: it replaces a caller loop of SL_UniformBuffer writes (one
 * per draw of a frame, softlight/tests/sl_large_scene_test.cpp:690-720).
 * All ids are checked before any block is written. */
int    slg_ubo_assign_many(slg_context* ctx, const size_t* uboIds, size_t count, const void* blocks, size_t blockStride,
                           size_t numBytes);

/* SL_Context::create_shader (softlight/src/SL_Context.cpp:488-606): same
 * validation, SLG_INVALID_ID where the reference returns (size_t)-1. */
size_t slg_create_shader(slg_context* ctx, const slg_vertex_shader* vs,
                         const slg_fragment_shader* fs, size_t uboId);

/*-----------------------------------------------------------------------------
 * Caller-defined shader programs. SoftLight takes shaders as host function
 * pointers over SL_VertexParam / SL_FragmentParam
 * (softlight/include/softlight/SL_Shader.hpp:41-119) handed to
 * SL_Context::create_shader (softlight/src/SL_Context.cpp:488-606). Here a
 * caller writes its programs as __device__ functions over parameter structs
 * of the same shape (slg::VertexParam / slg::FragmentParam in
 * include/slg_shader.cuh), compiles the draw-path kernels for them in its
 * own CUDA translation unit (SLG_DEFINE_PROGRAMS) and registers the result
 * here; slg_create_shader then takes their ids like the built-in ones. The
 * vertex and fragment program of one shader come from the same set.
-----------------------------------------------------------------------------*/
#define SLG_PIPELINE_ABI_VERSION 1u

/* The kernels of one program set, behind plain function pointers (the frame
 * and stream are the library's launch description and cudaStream_t). */
typedef struct slg_pipeline_ops
{
    uint32_t abiVersion;   /* SLG_PIPELINE_ABI_VERSION the set was compiled against */
    uint32_t frameBytes;   /* size of the launch description it was compiled against */
    int (*set_attributes)(void);
    int (*launch_vertex)(const void* frame, void* stream);
    int (*launch_raster)(const void* frame, void* stream);
} slg_pipeline_ops;

/* What the host needs to know about a program to launch it correctly. */
#define SLG_PROGRAM_DISCARDS     1u  /* the fragment program may return false (SL_FragmentShader semantics) */
#define SLG_PROGRAM_WRITES_DEPTH 2u  /* the fragment program may change coord.depth */

typedef struct slg_program_info
{
    uint32_t id;           /* >= SLG_PROGRAM_USER_FIRST, not yet registered in the context */
    uint32_t vertexBytes;  /* bytes the vertex program reads per vertex at binding 0's offset (checked against the buffer) */
    uint32_t flags;        /* SLG_PROGRAM_DISCARDS | SLG_PROGRAM_WRITES_DEPTH */
} slg_program_info;

/* Registers the programs of one compiled set. Launches whose fragment
 * programs discard or write depth take the ordered raster; a program that
 * returns false without SLG_PROGRAM_DISCARDS is reported at slg_finish
 * (SLG_ERR_INVALID_ARG). Vertex programs must be pure functions of the
 * vertex, the instance and the resources they read: the vertex stage may
 * run them once per vertex instead of once per triangle corner. */
int slg_register_programs(slg_context* ctx, const slg_pipeline_ops* ops, const slg_program_info* programs, size_t numPrograms);

/* SL_Context::clear_framebuffer / clear_color_buffer / clear_depth_buffer
 * (softlight/src/SL_Context.cpp:881-969). As in SL_ClearProcessor
 * (softlight/src/SL_ClearProcessor.cpp:22-33) the clear reaches the texels
 * its thread partition covers for the slg_num_threads count: with one thread
 * and width * height % 3 == 2 the last texel keeps its value. */
int slg_clear_framebuffer(slg_context* ctx, size_t fboId, unsigned attachment, const double rgba[4], double depth);
int slg_clear_color_buffer(slg_context* ctx, size_t fboId, unsigned attachment, const double rgba[4]);
int slg_clear_depth_buffer(slg_context* ctx, size_t fboId, double depth);

/* SL_Context::draw / draw_instanced / draw_multiple
 * (softlight/include/softlight/SL_Context.hpp:215-225; softlight/src/SL_Context.cpp:714-740).
 * Render modes: [INDEXED_]TRIANGLES, [INDEXED_]TRI_WIRE, [INDEXED_]LINES and
 * [INDEXED_]POINTS. A blended wireframe triangle that revisits a pixel after
 * 600 queued fragments is reported at finish (SLG_ERR_OVERFLOW: the
 * reference's queue flush order is not reproduced). A partial last primitive reads
 * the elements after elementEnd as the reference does, and those reads are
 * validated. Line draws need a framebuffer of at most 10922 x 10922 (the
 * reference's int16 Bresenham error term) and no visibility map. */
int slg_draw(slg_context* ctx, const slg_mesh* m, size_t shaderId, size_t fboId);
int slg_draw_instanced(slg_context* ctx, const slg_mesh* m, size_t numInstances, size_t shaderId, size_t fboId);
int slg_draw_multiple(slg_context* ctx, const slg_mesh* meshes, size_t numMeshes, size_t shaderId, size_t fboId);

/* slg_draw that allocates nothing. No counterpart in the reference: SoftLight
 * draws on the host and has no device scratch to allocate.
 *
 * slg_draw grows its scratch buffers with cudaMalloc when a draw needs more;
 * callers that must not allocate mid-frame (a fixed device-memory budget, a
 * thread that must not meet cudaMalloc's implicit device synchronisation, an
 * allocator hook that forbids new allocations) use this variant, whose
 * scratch is one file-scope device array of about 4.8 MiB sized for the
 * worst case of the limits below. Same arguments, results and errors as
 * slg_draw (device-side conditions such as a blended wireframe revisit after
 * 600 queued fragments are reported at slg_finish through the context's own
 * status words; a framebuffer with a visibility map gets the same checks and
 * the map is written), plus:
 *  - limits: at most SLG_NOALLOC_MAX_TRIANGLES triangles per call and a
 *    framebuffer of at most SLG_NOALLOC_MAX_TILES tiles of the context's tile
 *    size (256x256 pixels at the default 32x32); larger draws are rejected
 *    with SLG_ERR_INVALID_ARG and a message naming the limit, before any work
 *    is queued;
 *  - the first call on a device looks up the array's device address
 *    (cudaGetSymbolAddress, with that device current) and caches it; make
 *    that first call before any stream capture;
 *  - the pipeline's counters (overflow and clip counts, status words, per-tile
 *    triangle counts) must start at zero; each call clears them itself with
 *    one cudaMemsetAsync on the context's stream before its kernels;
 *  - all contexts on a device share the one array: calls whose work overlaps
 *    on the device (two contexts, or two host threads) race on it and must be
 *    serialised by the caller. */
#define SLG_NOALLOC_MAX_TRIANGLES 1024
#define SLG_NOALLOC_MAX_TILES 64
int slg_draw_noalloc(slg_context* ctx, const slg_mesh* m, size_t shaderId, size_t fboId);

/* Many draws (each possibly instanced, each with its own shader/uniforms) in
 * one launch sequence with the same result as issuing them one by one with
 * slg_draw / slg_draw_instanced. No single reference counterpart: it replaces
 * a caller loop over SL_Context::draw (softlight/tests/sl_instancing_test.cpp:236-279). */
int slg_draw_batch(slg_context* ctx, const slg_draw_cmd* cmds, size_t numCmds, size_t fboId);

/*-----------------------------------------------------------------------------
 * Scene graph (SL_SceneGraph, softlight/include/softlight/SL_SceneGraph.hpp:215)
 * and the draw list of its mesh nodes. Nodes keep their insertion order
 * (a parent precedes its children); update follows SL_SceneGraph::update
 * (softlight/src/SL_SceneGraph.cpp:259-299) on the device; draw traverses
 * the mesh nodes as SoftLight's scene demos do
 * (softlight/tests/sl_large_scene_test.cpp:678-740) and draws the result as
 * one batched launch whose uniform blocks and culling are written on the
 * device.
-----------------------------------------------------------------------------*/
/* SL_Transform's parameters (softlight/include/softlight/SL_Transform.hpp:60-75) */
typedef struct slg_transform
{
    float    position[3];
    float    scaling[3];
    float    orientation[4];  /* quaternion x, y, z, w */
    uint32_t type;            /* SL_TransformType: 0 model, 1 view FPS, 2 view arc,
                                 3 view FPS locked y, 4 view arc locked y */
} slg_transform;

#define SLG_SCENE_ROOT ((size_t)-1)   /* SCENE_NODE_ROOT_ID */

size_t slg_create_scene(slg_context* ctx);

/* SL_SceneGraph::insert_mesh (SL_SceneGraph.cpp:1212-1223): a mesh and its
 * bounding box (points with w = 1). Mesh nodes also append a default box
 * (max 1, min -1) to the same list, as the reference does, and culling reads
 * the box at the submesh's mesh index. */
int slg_scene_insert_mesh(slg_context* ctx, size_t sceneId, const slg_mesh* mesh, const float maxPoint[3],
                          const float minPoint[3], size_t* outMeshId);

/* A material (SL_Material) reduced to its ambient texture, the one the
 * demos' traversal binds; slg_mesh.materialId indexes these. */
int slg_scene_insert_material(slg_context* ctx, size_t sceneId, size_t ambientTextureId, size_t* outMaterialId);

/* SL_SceneGraph::insert_empty_node (numSubMeshes == 0) or insert_mesh_node
 * (SL_SceneGraph.cpp:1180-1258): the node is appended (the reference's
 * reparent call leaves it in place) with a dirty transform and an identity
 * model matrix until the next update. Paths from a root hold at most 64
 * nodes. */
int slg_scene_insert_node(slg_context* ctx, size_t sceneId, size_t parentId, size_t numSubMeshes, const size_t* subMeshIds,
                          const slg_transform* transform, size_t* outNodeId);

/* SL_Transform::position / scaling / orientation / type of a node's
 * current transform: marks it dirty. */
int slg_scene_set_transform(slg_context* ctx, size_t sceneId, size_t nodeId, const slg_transform* transform);

/* SL_SceneGraph::update: recomputes the model matrices of the nodes the
 * reference's loop recomputes (each dirty node and the nodes after it up to
 * the first whose parent precedes it). */
int slg_scene_update(slg_context* ctx, size_t sceneId);

/* The model matrices (mModelMatrices, 16 floats per node, column-major). */
int slg_scene_read_models(slg_context* ctx, size_t sceneId, float* out, size_t numNodes);

/* Draws every triangle-mode submesh of every mesh node in node order with
 * shaderId's state and a copy of its uniform block: program
 * SLG_PROGRAM_LAMBERT_TEX, vpMatrix = projection * view, modelMatrix = the
 * node's model matrix, textureId = the material's ambient texture. With a
 * cullProjection (the demos pass a fixed perspective), a submesh whose
 * bounding box fails sl_is_visible(box, view * model, frustum planes of
 * cullProjection) (softlight/src/SL_Camera.cpp:25-85) is skipped; NULL
 * draws them all. Shader and uniform-block ids for the draws are created on
 * first use and kept by the scene. */
int slg_scene_draw(slg_context* ctx, size_t sceneId, size_t fboId, size_t shaderId, const float projection[16],
                   const float view[16], const float cullProjection[16]);

/* Wait for all queued work (SL_Context::draw is synchronous in the reference;
 * here results are synchronous at slg_finish / slg_texture_read). */
int slg_finish(slg_context* ctx);

/*-----------------------------------------------------------------------------
 * GPU-only controls (no reference counterpart: SoftLight's only runtime knob
 * is num_threads).
-----------------------------------------------------------------------------*/
/* The cudaStream_t the context enqueues its work on, as an opaque pointer. */
void* slg_context_stream(slg_context* ctx);

/* Screen-tile size of the binning and raster stages. Supported sizes:
 * 8x8, 16x16, 32x16, 32x32 (default), 64x32, 64x64. */
int slg_set_tile_size(slg_context* ctx, int tileW, int tileH);

/* When enabled, every draw records CUDA events around its four stages;
 * slg_stage_times returns the last draw's stage durations in milliseconds:
 * [0] vertex/set-up, [1] tile scan, [2] bin fill, [3] raster+shade. */
int slg_profile_stages(slg_context* ctx, int enable);
int slg_stage_times(slg_context* ctx, float ms[4]);

/* Capacities of the scratch buffers for the next launches: tile-list
 * entries, clipped-triangle records and keys of the shared-memory tile sort
 * (0 keeps a value). A launch that needs more sets a capacity bit, writes
 * nothing, and the work queued after it is skipped; at the next
 * synchronisation point (slg_finish, slg_texture_read, ...) the buffer is
 * grown and the recorded operations are replayed from that launch, so the
 * frame comes out complete. Normal use never needs this call: buffers start
 * large and grow on their own. It starts a context small so that the
 * recovery path can be exercised; a launch with more triangle slots than
 * any before resets the sizes. A sort-key cap also makes blended launches
 * fill their tile lists by atomics and sort them per tile (otherwise they
 * are filled in key order and need no sort). */
int slg_set_scratch_caps(slg_context* ctx, size_t maxEntries, size_t maxClipRecords, unsigned maxSortKeys);

/* Raster strategy: 0 (default) picks the order-free resolve for launches
 * without blending and with one order-independent depth rule, else the
 * ordered per-pixel replay; the order-free resolve of triangle and point
 * launches with one colour target runs untiled (every record walked once
 * into per-pixel best words) when slg_autotune found that faster, on screen
 * tiles otherwise. 1 forces the ordered replay, 2 keeps order-free launches
 * on tiles, 3 runs them untiled where they qualify. All give the same
 * image. */
int slg_set_raster_mode(slg_context* ctx, int mode);

/* Whether order-free triangle and point launches run untiled (1) or on
 * screen tiles (0) under the current raster mode and autotuner pick. */
int slg_untiled_raster(const slg_context* ctx);

/* Threads per block of the vertex/set-up stage, i.e. triangles per CTA: 64,
 * 128 (default) or 256. */
int slg_set_vertex_block(slg_context* ctx, int threads);

/* When enabled, slg_draw_batch captures its launch sequence into a CUDA
 * graph and replays it on later calls with the same draws and launch
 * parameters (uniform-block contents may change between replays). */
int slg_set_batch_graphs(slg_context* ctx, int enable);

/* Autotuner: renders clear(rgba, depth) + slg_draw_batch(cmds) with every
 * supported tile size and vertex block size, then untiled (order-free
 * launches of triangles and points) with every vertex block size, keeps the
 * fastest for the context and returns it in out = {tileW, tileH, vertex
 * block}; slg_untiled_raster tells whether the untiled raster won. The
 * framebuffer holds the last trial's frame afterwards. */
int slg_autotune(slg_context* ctx, const slg_draw_cmd* cmds, size_t numCmds, size_t fboId,
                 const double rgba[4], double depth, int out[3]);

/*-----------------------------------------------------------------------------
 * Differentiable rendering (no reference counterpart: SoftLight has no
 * adjoint). Covers one opaque SLG_PROGRAM_VCOLOR_TEXF draw per framebuffer
 * frame. The model: the draw's exact coverage is frozen as a visibility map;
 * at each covered pixel (x, y) the perspective-correct barycentrics of the
 * visible triangle's unsnapped clip-space vertices at the pixel's NDC point
 * interpolate vertex colour and uv, the float texture is sampled bilinearly
 * (REPEAT, the draw path's texel addressing), and out = colour * texel.
 * Device buffers below are plain device (or managed, or pinned host)
 * pointers; work is queued on the context's stream (slg_context_stream).
-----------------------------------------------------------------------------*/
/* Attach (enable != 0) or drop a visibility map: one uint32 per pixel of the
 * depth attachment, cleared to 0 with the depth buffer; every opaque draw
 * into the framebuffer then writes, where its fragment wins the depth test,
 * 1 + the index of the winning triangle within the draw. Draws that blend or
 * mix depth rules are rejected while it is attached. */
int slg_fbo_enable_visibility(slg_context* ctx, size_t fboId, int enable);
int slg_fbo_read_visibility(slg_context* ctx, size_t fboId, uint32_t* dst, size_t count);

/* The model's image for the draw (mesh, shader) over the framebuffer's
 * visibility map: width*height RGBA floats into `image` (device, 16-byte
 * aligned). The model covers a pixel when its visible triangle's
 * barycentrics there are all >= -1 (within one triangle height of the
 * unsnapped triangle; snapping lets slivers cover pixels far outside it)
 * and the triangle is not a sliver (twice its area in clip-space xy/w at
 * the pixel >= 0.02 x the sum of its squared edge lengths there); every
 * other pixel takes the framebuffer's colour when colour attachment 0 is
 * RGBA float, else 0, and carries no gradient. */
int slg_diff_shade(slg_context* ctx, const slg_mesh* mesh, size_t shaderId, size_t fboId, float* image, size_t count);

/* Adjoint of slg_diff_shade: for dL/d image (width*height RGBA floats),
 * ADDS dL/d vertex position, colour and uv into dVertices -- floats laid
 * out like the draw's vertex buffer (pos[3], rgba[4], uv[2] at binding 0's
 * offset and stride) -- and dL/d texel into dTexels (texW*texH RGBA floats).
 * Recomputes every pixel's barycentrics, varyings and texture footprint
 * from the buffers; stores nothing from the forward but the visibility map.
 * Accumulates with FP32 atomics staged per 32x8 pixel tile in shared
 * memory, so the summation order (and the last bits) vary between runs. */
int slg_draw_adjoint(slg_context* ctx, const slg_mesh* mesh, size_t shaderId, size_t fboId, const float* dImage,
                     size_t dImageCount, float* dVertices, size_t dVertexCount, float* dTexels, size_t dTexelCount);

#ifdef __cplusplus
}
#endif

#endif /* SLG_H */
