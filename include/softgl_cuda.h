/*
 * softgl_cuda.h — C ABI of the GB300 (sm_103a) renderer back-end.
 *
 * Every entry point mirrors one method of SoftGLRender's back-end abstraction so that a C++
 * `RendererCUDA : public SoftGL::Renderer` (or any FFI caller) can forward to it one-to-one:
 *
 *   SoftGL::Renderer            src/Render/Renderer.h:24-59
 *   SoftGL::FrameBuffer         src/Render/Framebuffer.h:20-91
 *   SoftGL::Texture/TextureDesc src/Render/Texture.h:17-105
 *   SoftGL::VertexArray(Object) src/Render/Vertex.h:15-37
 *   SoftGL::ShaderProgram       src/Render/ShaderProgram.h:15-58
 *   SoftGL::UniformBlock/Sampler/ShaderResources  src/Render/Uniform.h:20-64
 *   SoftGL::RenderStates/ClearStates              src/Render/RenderStates.h:13-99
 *
 * ABI rules: plain C types only; resources are opaque non-zero 32-bit handles owned by a context;
 * every call returns an sglc_status (0 = SGLC_OK) and never aborts the process; the text of the
 * last failure of a context is available from sglc_last_error(). All enum values are the
 * reference's own enum values (same order), so a binding passes them through unchanged.
 *
 * Execution model: one context = one CUDA device + one CUDA stream. Draws are enqueued
 * asynchronously; sglc_wait_idle() synchronises (RendererSoft::waitIdle is a no-op because its
 * draw() is synchronous, RendererSoft.cpp:136-168). Reads of attachments synchronise implicitly.
 */
#ifndef SOFTGL_CUDA_H_
#define SOFTGL_CUDA_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define SGLC_API __attribute__((visibility("default")))
#else
#define SGLC_API
#endif

typedef int32_t sglc_status;
typedef int32_t sglc_handle; /* 0 is the null handle */
typedef struct sglc_context sglc_context;

enum {
  SGLC_OK = 0,
  SGLC_ERR_INVALID_HANDLE = 1,
  SGLC_ERR_INVALID_VALUE = 2,
  SGLC_ERR_OUT_OF_MEMORY = 3,
  SGLC_ERR_DEVICE = 4,       /* a CUDA runtime call failed */
  SGLC_ERR_UNSUPPORTED = 5,  /* valid in the reference API, not implemented by this back-end */
  SGLC_ERR_OVERFLOW = 6,     /* a device-side capacity (clip vertices, tile lists) was exceeded */
  SGLC_ERR_NO_DEVICE = 7,
};

/* ---- enums: values equal to the reference's enums ---------------------------------------- */
/* TextureType (Texture.h:58-61) */
enum { SGLC_TEXTURE_2D = 0, SGLC_TEXTURE_CUBE = 1 };
/* TextureFormat (Texture.h:63-66) */
enum { SGLC_FORMAT_RGBA8 = 0, SGLC_FORMAT_FLOAT32 = 1 };
/* FilterMode (Texture.h:24-31) */
enum {
  SGLC_FILTER_NEAREST = 0, SGLC_FILTER_LINEAR, SGLC_FILTER_NEAREST_MIPMAP_NEAREST,
  SGLC_FILTER_LINEAR_MIPMAP_NEAREST, SGLC_FILTER_NEAREST_MIPMAP_LINEAR, SGLC_FILTER_LINEAR_MIPMAP_LINEAR
};
/* WrapMode (Texture.h:17-22) */
enum { SGLC_WRAP_REPEAT = 0, SGLC_WRAP_MIRRORED_REPEAT, SGLC_WRAP_CLAMP_TO_EDGE, SGLC_WRAP_CLAMP_TO_BORDER };
/* BorderColor (Texture.h:42-45) */
enum { SGLC_BORDER_BLACK = 0, SGLC_BORDER_WHITE = 1 };
/* BufferLayout (Base/Buffer.h:14-18): compile-time in the reference, per texture here */
enum { SGLC_LAYOUT_LINEAR = 0, SGLC_LAYOUT_TILED = 1, SGLC_LAYOUT_MORTON = 2 };
/* DepthFunction / BlendFactor / BlendFunction / PolygonMode / PrimitiveType (RenderStates.h:13-77) */
enum {
  SGLC_DEPTH_NEVER = 0, SGLC_DEPTH_LESS, SGLC_DEPTH_EQUAL, SGLC_DEPTH_LEQUAL,
  SGLC_DEPTH_GREATER, SGLC_DEPTH_NOTEQUAL, SGLC_DEPTH_GEQUAL, SGLC_DEPTH_ALWAYS
};
enum {
  SGLC_BLEND_ZERO = 0, SGLC_BLEND_ONE, SGLC_BLEND_SRC_COLOR, SGLC_BLEND_SRC_ALPHA, SGLC_BLEND_DST_COLOR,
  SGLC_BLEND_DST_ALPHA, SGLC_BLEND_ONE_MINUS_SRC_COLOR, SGLC_BLEND_ONE_MINUS_SRC_ALPHA,
  SGLC_BLEND_ONE_MINUS_DST_COLOR, SGLC_BLEND_ONE_MINUS_DST_ALPHA
};
enum { SGLC_FUNC_ADD = 0, SGLC_FUNC_SUBTRACT, SGLC_FUNC_REVERSE_SUBTRACT, SGLC_FUNC_MIN, SGLC_FUNC_MAX };
enum { SGLC_POLYGON_POINT = 0, SGLC_POLYGON_LINE, SGLC_POLYGON_FILL };
enum { SGLC_PRIMITIVE_POINT = 0, SGLC_PRIMITIVE_LINE, SGLC_PRIMITIVE_TRIANGLE };

/* Shading models. 1..3 are ShadingModel (Viewer/Material.h:24-33) loaded by
 * ViewerSoftware::loadShaders (ViewerSoftware.h:54-69); 100+ are device shaders with no
 * reference counterpart, used by the synthetic benchmark scenes. */
enum {
  SGLC_SHADING_BASE_COLOR = 1,          /* Shader/Software/BasicSoft.h:62-79 */
  SGLC_SHADING_BLINN_PHONG = 2,         /* Shader/Software/BlinnPhongSoft.h:181-325 (point light) */
  SGLC_SHADING_PBR = 3,                 /* Shader/Software/PbrSoft.h:106-323 */
  SGLC_SHADING_SKYBOX = 4,              /* Shader/Software/SkyboxSoft.h:42-107 (equirectangular or cube) */
  SGLC_SHADING_IBL_IRRADIANCE = 5,      /* Shader/Software/IBLIrradianceSoft.h:40-105 */
  SGLC_SHADING_IBL_PREFILTER = 6,       /* Shader/Software/IBLPrefilterSoft.h:44-172 */
  SGLC_SHADING_FXAA = 7,                /* Shader/Software/FxaaSoft.h:37-267 (QuadFilter screen pass) */
  SGLC_SHADING_BLINN_PHONG_DIR = 100,   /* Blinn-Phong, directional light, shininess 32 */
  SGLC_SHADING_VERTEX_COLOR = 101,      /* per-vertex RGBA colour */
};

/* TextureDesc (Texture.h:76-85) plus the storage layout (reference: compile-time macro). */
typedef struct sglc_texture_desc {
  int32_t width;
  int32_t height;
  int32_t type;        /* SGLC_TEXTURE_* */
  int32_t format;      /* SGLC_FORMAT_* */
  uint32_t usage;      /* TextureUsage bits (Texture.h:68-74) */
  int32_t use_mipmaps;
  int32_t multi_sample;
  int32_t layout;      /* SGLC_LAYOUT_* (sampled textures; attachments are stored linearly) */
} sglc_texture_desc;

/* SamplerDesc (Texture.h:47-56) */
typedef struct sglc_sampler_desc {
  int32_t filter_min;
  int32_t filter_mag;
  int32_t wrap_s;
  int32_t wrap_t;
  int32_t wrap_r;
  int32_t border_color;
} sglc_sampler_desc;

/* RenderStates (RenderStates.h:79-92) with BlendParameters (:53-73) flattened. */
typedef struct sglc_render_states {
  int32_t blend;
  int32_t blend_func_rgb;
  int32_t blend_src_rgb;
  int32_t blend_dst_rgb;
  int32_t blend_func_alpha;
  int32_t blend_src_alpha;
  int32_t blend_dst_alpha;
  int32_t depth_test;
  int32_t depth_mask;
  int32_t depth_func;
  int32_t cull_face;
  int32_t primitive_type;
  int32_t polygon_mode;
  float line_width;
} sglc_render_states;

/* ClearStates (RenderStates.h:94-99) */
typedef struct sglc_clear_states {
  int32_t depth_flag;
  int32_t color_flag;
  float clear_color[4];
  float clear_depth;
} sglc_clear_states;

/* Per-draw counters (no reference counterpart; the viewer shows only a triangle count). */
typedef struct sglc_draw_stats {
  int64_t vertices_in;
  int64_t triangles_in;
  int64_t clip_vertices;      /* vertices created by frustum clipping */
  int64_t primitives;         /* after clipping (originals + appended fan triangles) */
  int64_t bin_entries;        /* (tile, triangle) pairs */
  int64_t fragments_shaded;   /* fragment-shader invocations (stats level 2) */
  float geometry_ms;          /* device time of vertex + clip + setup (stats level >= 1) */
  float binning_ms;           /* pair emission + sort + tile ranges, including the count read-back */
  float raster_ms;            /* tile raster + shading + ROP + resolve */
  int32_t kernel_launches;    /* kernels this back-end launched for the draw */
  float coverage_ms;          /* deferred shading: coverage + depth kernel (stats level >= 1; else 0) */
  float shading_ms;           /* deferred shading: fragment-shader kernel */
  float rop_ms;               /* deferred shading: colour operations + resolve kernel */
} sglc_draw_stats;

/* ---- context (Renderer::create / destroy, Renderer.h:27-28) ---------------------------------- */
SGLC_API sglc_status sglc_create(sglc_context **out, int32_t device);
SGLC_API sglc_status sglc_destroy(sglc_context *ctx);
SGLC_API const char *sglc_last_error(sglc_context *ctx);
/* Release one resource handle (the shared_ptr reset of the reference). */
SGLC_API sglc_status sglc_release(sglc_context *ctx, sglc_handle h);

/* ---- framebuffer (Renderer::createFrameBuffer, Renderer.h:31; FrameBuffer, Framebuffer.h:20-91) */
SGLC_API sglc_status sglc_create_framebuffer(sglc_context *ctx, int32_t offscreen, sglc_handle *out);
SGLC_API sglc_status sglc_framebuffer_set_color_attachment(sglc_context *ctx, sglc_handle fb, sglc_handle tex,
                                                           int32_t layer, int32_t level);
SGLC_API sglc_status sglc_framebuffer_set_depth_attachment(sglc_context *ctx, sglc_handle fb, sglc_handle tex);
SGLC_API sglc_status sglc_framebuffer_is_valid(sglc_context *ctx, sglc_handle fb, int32_t *valid);

/* ---- texture (Renderer::createTexture, Renderer.h:34; Texture, Texture.h:87-105) ------------- */
SGLC_API sglc_status sglc_create_texture(sglc_context *ctx, const sglc_texture_desc *desc, sglc_handle *out);
SGLC_API sglc_status sglc_texture_set_sampler_desc(sglc_context *ctx, sglc_handle tex,
                                                   const sglc_sampler_desc *sampler);
SGLC_API sglc_status sglc_texture_init_image_data(sglc_context *ctx, sglc_handle tex);
/* Texture::setImageData: one linear width*height image per layer (1 for 2D, 6 for cube faces in
 * CubeMapFace order); the mip chain is generated on the device when use_mipmaps is set. */
SGLC_API sglc_status sglc_texture_set_image_data(sglc_context *ctx, sglc_handle tex, int32_t layer_count,
                                                 const void *const *layers, size_t bytes_per_layer);
/* Upload one mip level of one layer (the reference fills levels by rendering into a level
 * attachment, Environment.cpp:152-195; this uploads the same bytes directly). */
SGLC_API sglc_status sglc_texture_set_level_data(sglc_context *ctx, sglc_handle tex, int32_t layer, int32_t level,
                                                 const void *data, size_t bytes);
/* Texture::dumpImage analogue: copy one level of one layer to host memory in linear order.
 * For multi-sample textures `resolved` = 0 returns the 4 interleaved samples per pixel
 * (RGBA8: 16 B/pixel; FLOAT32: 16 B/pixel) and 1 returns the resolved RGBA8 image. */
SGLC_API sglc_status sglc_texture_read_image(sglc_context *ctx, sglc_handle tex, int32_t layer, int32_t level,
                                             int32_t resolved, void *out, size_t bytes);
/* TextureSoft::storeToFile / TextureSoft::loadFromFile (TextureSoft.h:166-215), the format of the
 * viewer's IBL texture cache (IBLGenerator::storeToCache / loadFromCache, Environment.cpp:205-239):
 * for every layer, for every mip level, the level's raw texels in the storage order of its buffer
 * layout (Buffer::convertIndex, Buffer.h:31-33, 151-157, 193-202), padding texels of the Tiled 4x4 /
 * Morton 32x32 layouts included; 4 B per texel (RGBA8 or FLOAT32), 4 samples per texel for a
 * multi-sample texture. Attachments and multi-sample textures are stored Linear. A texture with no
 * image data writes and reads nothing. Load reads exactly the bytes it needs (a longer file is
 * accepted, a shorter one fails with SGLC_ERR_INVALID_VALUE and leaves the texture unchanged);
 * an unopenable path fails with SGLC_ERR_INVALID_VALUE. */
SGLC_API sglc_status sglc_texture_store_to_file(sglc_context *ctx, sglc_handle tex, const char *path);
SGLC_API sglc_status sglc_texture_load_from_file(sglc_context *ctx, sglc_handle tex, const char *path);

/* ---- vertex array (Renderer::createVertexArrayObject, Renderer.h:37; VertexSoft.h:16-31) ----
 * Lengths are in bytes, as VertexArray::vertexesBufferLength / indexBufferLength (Vertex.h:33-36). */
SGLC_API sglc_status sglc_create_vertex_array(sglc_context *ctx, const void *vertexes, size_t vertexes_len,
                                              size_t stride, const int32_t *indices, size_t indices_len,
                                              sglc_handle *out);
SGLC_API sglc_status sglc_vertex_array_update(sglc_context *ctx, sglc_handle vao, const void *data, size_t len);

/* ---- shader program (Renderer::createShaderProgram, Renderer.h:40; ShaderProgramSoft.h:26-70) */
SGLC_API sglc_status sglc_create_shader_program(sglc_context *ctx, sglc_handle *out);
SGLC_API sglc_status sglc_program_add_define(sglc_context *ctx, sglc_handle prog, const char *name);
/* ShaderProgramSoft::SetShaders(VS, FS): selects the device vertex/fragment shader pair. */
SGLC_API sglc_status sglc_program_set_shaders(sglc_context *ctx, sglc_handle prog, int32_t shading_model);

/* ---- pipeline states (Renderer::createPipelineStates, Renderer.h:43) ------------------------- */
SGLC_API sglc_status sglc_create_pipeline_states(sglc_context *ctx, const sglc_render_states *states,
                                                 sglc_handle *out);

/* ---- uniforms (Renderer::createUniformBlock/Sampler, Renderer.h:46-47; UniformSoft.h:15-90) -- */
SGLC_API sglc_status sglc_create_uniform_block(sglc_context *ctx, const char *name, int32_t size, sglc_handle *out);
SGLC_API sglc_status sglc_uniform_block_set_sub_data(sglc_context *ctx, sglc_handle ub, const void *data,
                                                     int32_t len, int32_t offset);
SGLC_API sglc_status sglc_uniform_block_set_data(sglc_context *ctx, sglc_handle ub, const void *data, int32_t len);
SGLC_API sglc_status sglc_create_uniform_sampler(sglc_context *ctx, const char *name, int32_t type, int32_t format,
                                                 sglc_handle *out);
SGLC_API sglc_status sglc_uniform_sampler_set_texture(sglc_context *ctx, sglc_handle us, sglc_handle tex);
/* ShaderResources (Uniform.h:60-64): two maps keyed by the caller's integer key. */
SGLC_API sglc_status sglc_create_shader_resources(sglc_context *ctx, sglc_handle *out);
SGLC_API sglc_status sglc_shader_resources_set_block(sglc_context *ctx, sglc_handle res, int32_t key, sglc_handle ub);
SGLC_API sglc_status sglc_shader_resources_set_sampler(sglc_context *ctx, sglc_handle res, int32_t key,
                                                       sglc_handle us);

/* ---- pipeline (Renderer.h:50-58; RendererSoft.cpp:61-168) ------------------------------------ */
SGLC_API sglc_status sglc_begin_render_pass(sglc_context *ctx, sglc_handle fb, const sglc_clear_states *states);
SGLC_API sglc_status sglc_set_viewport(sglc_context *ctx, int32_t x, int32_t y, int32_t width, int32_t height);
SGLC_API sglc_status sglc_set_vertex_array(sglc_context *ctx, sglc_handle vao);
SGLC_API sglc_status sglc_set_shader_program(sglc_context *ctx, sglc_handle prog);
SGLC_API sglc_status sglc_set_shader_resources(sglc_context *ctx, sglc_handle res);
SGLC_API sglc_status sglc_set_pipeline_states(sglc_context *ctx, sglc_handle states);
SGLC_API sglc_status sglc_draw(sglc_context *ctx);
SGLC_API sglc_status sglc_end_render_pass(sglc_context *ctx);
SGLC_API sglc_status sglc_wait_idle(sglc_context *ctx);
/* RendererSoft::setEnableEarlyZ (RendererSoft.h:53). */
SGLC_API sglc_status sglc_set_enable_early_z(sglc_context *ctx, int32_t enable);

/* ---- extensions (no reference counterpart) --------------------------------------------------- */
/* Batched views: the bound vertex array, program and pipeline states drawn once per view, view v
 * into framebuffers[v] with the uniform blocks of resources[v] (samplers are taken from
 * resources[0] and shared). The result is identical to, for each view in order:
 * beginRenderPass(framebuffers[v], clear) (no clear when `clear` is null); setShaderResources(
 * resources[v]); draw(); endRenderPass(). All views' attachments must have view 0's sizes, formats
 * and sample count. The GPU runs every view in one pipeline pass (one launch per stage over all
 * (view, triangle) and (view, tile) work items). At most 2^20 views per call. */
SGLC_API sglc_status sglc_draw_views(sglc_context *ctx, const sglc_handle *framebuffers, const sglc_handle *resources,
                                     int32_t count, const sglc_clear_states *clear);
/* Multi-scene draw: independent scenes that share the bound program, pipeline states and samplers
 * but not geometry or frame size, scene s drawn from vertex_arrays[s] into framebuffers[s] with
 * the uniform blocks of resources[s]. The result is identical to, for each scene in order:
 * beginRenderPass(framebuffers[s], clear); setViewPort(0, 0, W, H) with the scene's attachment size;
 * setVertexArrayObject(vertex_arrays[s]); setShaderResources(resources[s]); draw(); endRenderPass().
 * Attachments may differ in size between scenes, not in presence or sample count; vertex arrays
 * must share their stride; every scene's resources must bind the textures and sampler states that
 * resources[0] binds (SGLC_ERR_INVALID_VALUE otherwise). The GPU runs all scenes in one pipeline
 * pass: one launch per stage over every (scene, vertex), (scene, triangle) and (scene, tile) work
 * item, the raster stage taking tiles from one heaviest-first queue across the scenes. It replaces
 * the per-scene loop over Renderer calls that RendererSoft runs one block task queue for at a time
 * (RendererSoft.cpp:731-737 feeding ThreadPool.h:100-110). At most 2^20 scenes per call. */
SGLC_API sglc_status sglc_draw_scenes(sglc_context *ctx, const sglc_handle *vertex_arrays,
                                      const sglc_handle *framebuffers, const sglc_handle *resources, int32_t count,
                                      const sglc_clear_states *clear);
/* Counters of the last draw (synchronises). */
SGLC_API sglc_status sglc_get_draw_stats(sglc_context *ctx, sglc_draw_stats *out);
/* 0: no instrumentation; 1: per-stage device timings of each draw; 2: also count fragments. */
SGLC_API sglc_status sglc_set_stats_level(sglc_context *ctx, int32_t level);
/* The CUDA stream the context enqueues on (as an opaque pointer, cudaStream_t). */
SGLC_API sglc_status sglc_get_stream(sglc_context *ctx, void **stream);
/* Height of the raster tiles that heavy shading models' deferred kernels work on: 16 (16x16
 * pixels, 256 threads per tile, the default) or 8 (16x8 pixels, 128 threads); other draws use
 * 16x16. Picked by the autotuner (softglrender_gb300/autotune.py). */
SGLC_API sglc_status sglc_set_tile_size(sglc_context *ctx, int32_t tile);
/* 1 (default): shading models with a heavy fragment shader (Blinn-Phong, PBR, skybox / IBL, FXAA)
 * rasterise in three kernels: coverage and depth, then the fragment shader over every fragment, then
 * the colour operations in each pixel's order. 0: one fused raster kernel. Same images either way. */
SGLC_API sglc_status sglc_set_deferred_shading(sglc_context *ctx, int32_t enable);
/* 1 (default): the deferred raster kernels write each whole 16x16 tile's colour, resolved colour
 * and depth back from shared memory with TMA bulk tensor stores (single-view draws on attachments
 * whose rows are a multiple of 16 bytes); 0: every thread stores its own pixel. Same images. */
SGLC_API sglc_status sglc_set_tma_store(sglc_context *ctx, int32_t enable);

/* ---- synchronisation-free draws and CUDA graphs (no reference counterpart) ------------------- */
/* Working-array capacities of a draw (a batched draw counts all its views together). */
typedef struct sglc_capacity {
  int64_t clip_vertices;         /* vertices created by frustum clipping */
  int64_t clip_polygons;         /* triangles clipped into polygons of more than 3 vertices */
  int64_t appended_primitives;   /* fan triangles appended after clipping */
  int64_t bin_entries;           /* (tile, triangle) pairs */
  int32_t heavy_first;           /* 1: raster the longest tile lists first; 0: tiles in index order */
  int64_t fragments;             /* fragment records of deferred shading (0: those draws use the
                                    single raster kernel) */
} sglc_capacity;
/* With capacities set, draws size their working arrays from them instead of reading counts back
 * from the device after the setup stage: a draw then never waits for the GPU, and draws can be
 * captured in a CUDA graph. Work beyond a capacity is dropped and recorded in sticky overflow flags
 * (sglc_get_overflow); the images of such a draw are then unspecified. Null restores the default
 * (exact sizing with one count read-back per draw). */
SGLC_API sglc_status sglc_set_capacity(sglc_context *ctx, const sglc_capacity *cap);
/* The largest counts the draws since the last call needed (draws with exact sizing only; fragments:
 * the records deferred-shading draws used, in whole chunks of 32), as capacities (heavy_first = 1);
 * resets them. Used to calibrate sglc_set_capacity. */
SGLC_API sglc_status sglc_get_peak_counts(sglc_context *ctx, sglc_capacity *out);
/* Synchronises, returns and clears the overflow flags of the draws since the last call: bit 0 clip
 * vertices, 1 clip polygons, 2 appended primitives, 3 bin entries, 4 an index outside the vertex
 * array, 5 fragment records, 6 a tensor-core wait of the neural shader timed out (that draw's
 * colours are unspecified). */
SGLC_API sglc_status sglc_get_overflow(sglc_context *ctx, int32_t *flags);
typedef struct sglc_graph sglc_graph;
/* Capture everything enqueued on the context between begin and end into a CUDA graph. Draws in the
 * capture must run with capacities set, and the same sequence must have run once uncaptured so
 * that every working array is already sized (a capture that would need to grow one fails). Reads
 * of attachments and other synchronising calls are not allowed inside a capture. */
SGLC_API sglc_status sglc_graph_begin(sglc_context *ctx);
SGLC_API sglc_status sglc_graph_end(sglc_context *ctx, sglc_graph **out);
/* Enqueue one replay of the graph on its context's stream. Refused (SGLC_ERR_INVALID_VALUE) once the
 * context has freed or grown any buffer or resource since the capture; other contexts' frees do
 * not affect it, so graphs of several contexts can be captured and replayed concurrently. */
SGLC_API sglc_status sglc_graph_launch(sglc_graph *graph);
SGLC_API sglc_status sglc_graph_destroy(sglc_graph *graph);

/* ---- neural IBL shader (no reference counterpart) ------------------------------------------- */
/* A small MLP (12 inputs, 6-frequency encoding, 2 x 64 ReLU, 3 outputs; BF16 weights, FP32
 * accumulation on the tensor cores) that stands in for the image-based-lighting term of the PBR
 * shader (PbrSoft.h:296-309). It is trained on records that the plain PBR shader captures while it
 * renders, by tensor-core forward / backward / Adam kernels, and bound to a PBR program to replace
 * the irradiance and prefiltered-cube evaluation inside the fragment stage. Records are 16 floats:
 * N.xyz, V.xyz, roughness, metallic, albedo texel rgb, max(dot(N, V), 0), sqrt of the IBL term
 * rgb (before ambient occlusion), 0. Parameters are FP32 in the order W1[64][156], b1[64],
 * W2[64][64], b2[64], W3[3][64], b3[3] (sglc_neural_param_count() floats). All calls run on the
 * owning context's stream and synchronise before returning, except sglc_neural_capture. */
typedef struct sglc_neural sglc_neural;
typedef struct sglc_neural_train_params {
  int32_t steps;          /* Adam steps to run */
  int32_t batch;          /* records per step, drawn uniformly with replacement */
  float lr, beta1, beta2, eps;
  uint64_t seed;          /* record sampling: index = mix64(seed ^ step << 32 ^ row) % records */
} sglc_neural_train_params;

SGLC_API sglc_status sglc_neural_create(sglc_context *ctx, uint64_t seed, sglc_neural **out);
SGLC_API sglc_status sglc_neural_destroy(sglc_neural *net);
SGLC_API int64_t sglc_neural_param_count(void);
SGLC_API sglc_status sglc_neural_set_params(sglc_neural *net, const float *params, int64_t count);
SGLC_API sglc_status sglc_neural_get_params(sglc_neural *net, float *params, int64_t count);
/* Replace the record set with `count` host records. */
SGLC_API sglc_status sglc_neural_set_records(sglc_neural *net, const float *records, int64_t count);
SGLC_API sglc_status sglc_neural_get_records(sglc_neural *net, float *records, int64_t first, int64_t count);
/* Start capturing: every `stride`-th fragment the plain PBR shader shades on `ctx` (in the order
 * the shading threads reach the capture counter) appends a record, up to `capacity` records (the
 * rest are dropped); capacity 0 stops. */
SGLC_API sglc_status sglc_neural_capture(sglc_context *ctx, sglc_neural *net, int64_t capacity, int32_t stride);
SGLC_API sglc_status sglc_neural_record_count(sglc_neural *net, int64_t *count);
/* Adam on mean squared error; `loss` receives the last step's batch loss. */
SGLC_API sglc_status sglc_neural_train(sglc_neural *net, const sglc_neural_train_params *params, float *loss);
/* Gradient of the mean squared error over records [first, first + count) (no update). */
SGLC_API sglc_status sglc_neural_gradients(sglc_neural *net, int64_t first, int64_t count, float *grads,
                                           float *loss);
/* Network outputs (3 floats per record) for records [first, first + count). */
SGLC_API sglc_status sglc_neural_infer(sglc_neural *net, int64_t first, int64_t count, float *out);
/* Bind a network to a PBR program: its IBL term comes from the network (null unbinds, restoring
 * the plain shader). The network must outlive its use by draws. */
SGLC_API sglc_status sglc_program_set_neural_shader(sglc_context *ctx, sglc_handle prog, sglc_neural *net);
/* Test hook of the neural shading kernels (no counterpart in the reference): flag 1 makes every
 * completed tensor-core wait report a timeout, so a test can check that timeouts reach the host
 * (sglc_get_overflow bit 6) without a real one. 0 restores normal operation. */
SGLC_API sglc_status sglc_neural_set_test_flags(sglc_context *ctx, int32_t flags);

/* ---- allocation-free draw ----------------------------------------------------------------- */
/* One vertex-colour draw (position vec3 padded to 16 B + RGBA float colour, 32-B stride; the
 * vertex-colour shading model above) into caller-owned device buffers, for callers that cannot
 * call cudaMalloc: code whose device memory is owned by a host framework's pool, real-time
 * render threads that must not enter the CUDA allocator, library code that must not grow the
 * process's footprint. No counterpart in the reference. It allocates nothing: its working memory
 * is one fixed device array of at most 24 MiB inside the library, held by every GPU that loads
 * the library until the process exits, so there is no context to create. Limits: 65,536 vertices,
 * 32,768 triangles, width and height <= 1024, 262,144 (tile, triangle) bin entries; larger inputs
 * are rejected with SGLC_ERR_INVALID_VALUE and a message in `error`.
 * The attachments are read and written in place (no clear; viewport = the whole attachment),
 * linear, 4 interleaved samples per pixel when samples = 4. Everything is enqueued on `stream`
 * (a cudaStream_t, 0 = default stream), which is synchronised once at the end to read the
 * capacity flags (SGLC_ERR_OVERFLOW: the attachments' contents are then unspecified).
 * The first call on a device (per CUDA context current on it) looks up the array's device
 * address; make it before any stream capture. The array exists once per context that loads the
 * library, and a device reset gives a new context whose address is looked up again. All calls in
 * one context share the array: calls that overlap on the GPU (different streams or threads) race
 * and must be serialised by the caller. */
typedef struct sglc_noalloc_draw {
  const void *vertexes;           /* device, vertex_count * stride bytes */
  int32_t vertex_count;
  int32_t stride;                 /* bytes; must be 32 */
  const int32_t *indices;         /* device, 3 * triangle_count */
  int32_t triangle_count;
  const void *uniforms_model;     /* host, 256-B UniformsModel (Material.h:70-76) */
  const void *uniforms_material;  /* host, 48-B UniformsMaterial (Material.h:78-85) */
  int32_t width;
  int32_t height;
  int32_t samples;                /* 1 or 4 */
  uint32_t *color;                /* device RGBA8, width * height * samples */
  uint32_t *resolved;             /* device RGBA8, width * height (samples = 4 only) */
  float *depth;                   /* device, width * height * samples */
  sglc_render_states states;
  int32_t early_z;
  char *error;                    /* optional: receives a message when the call fails */
  size_t error_len;
} sglc_noalloc_draw;

SGLC_API sglc_status sglc_draw_vertex_color_noalloc(const sglc_noalloc_draw *draw, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SOFTGL_CUDA_H_ */
