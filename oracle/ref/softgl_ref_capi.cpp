/*
 * Test infrastructure (checker only; never linked into the product).
 *
 * The C ABI of include/softgl_cuda.h, implemented with prefix `sglr_` over the UNMODIFIED
 * reference SoftGL::RendererSoft compiled from the reference sources by oracle/ref/Makefile.
 * Python tests drive this library, the CPU restatement (oracle/softgl_oracle.cpp, prefix
 * `sglo_`) and the CUDA product (prefix `sglc_`) with the same call sequence, which is the
 * sequence Viewer::pipelineDraw issues (src/Viewer/Viewer.cpp:388-396).
 *
 * Everything here forwards to the reference objects; the only additions are handle tables, the
 * shader-pair loading that ViewerSoftware::loadShaders does (src/Viewer/ViewerSoftware.h:54-69),
 * and read-back of attachments in linear order (Buffer::get, src/Base/Buffer.h:86-99).
 */
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "Render/Software/RendererSoft.h"
#include "Render/Software/TextureSoft.h"
#include "Render/Software/FramebufferSoft.h"
#include "Render/Software/UniformSoft.h"
#include "Viewer/Shader/Software/BasicSoft.h"
#include "Viewer/Shader/Software/BlinnPhongSoft.h"
#include "Viewer/Shader/Software/PbrSoft.h"
#include "Viewer/Shader/Software/SkyboxSoft.h"
#include "Viewer/Shader/Software/IBLIrradianceSoft.h"
#include "Viewer/Shader/Software/IBLPrefilterSoft.h"
#include "Viewer/Shader/Software/FxaaSoft.h"
#include "extra_shaders_soft.h"
#include "softgl_cuda.h"

using namespace SoftGL;

namespace {

struct Object {
  std::shared_ptr<FrameBuffer> fb;
  std::shared_ptr<Texture> tex;
  std::shared_ptr<VertexArrayObject> vao;
  std::shared_ptr<ShaderProgram> prog;
  std::shared_ptr<PipelineStates> states;
  std::shared_ptr<UniformBlock> ub;
  std::shared_ptr<UniformSampler> us;
  std::shared_ptr<ShaderResources> res;
};

struct Ctx {
  RendererSoft renderer;
  std::map<int, Object> objects;
  int next = 1;
  std::string err;
  // the reference keeps raw pointers to bound objects; hold them alive like the Viewer does
  std::shared_ptr<FrameBuffer> boundFb;
  std::shared_ptr<VertexArrayObject> boundVao;
  std::shared_ptr<ShaderProgram> boundProg;
  std::shared_ptr<ShaderResources> boundRes;
  std::shared_ptr<PipelineStates> boundStates;

  int add(const Object &o) {
    int h = next++;
    objects[h] = o;
    return h;
  }
  Object *get(int h) {
    auto it = objects.find(h);
    return it == objects.end() ? nullptr : &it->second;
  }
  sglc_status fail(sglc_status s, const std::string &msg) {
    err = msg;
    return s;
  }
};

#define CTX_CHECK(c) \
  if (!(c)) return SGLC_ERR_INVALID_HANDLE;

template<typename T>
bool readTexture(TextureSoft<T> *tex, int layer, int level, int resolved, uint8_t *out, size_t bytes) {
  auto &img = tex->getImage(layer);
  if (level < 0 || level >= (int) img.levels.size()) return false;
  auto &buf = img.getBuffer(level);
  int w = buf->width, h = buf->height;
  if (buf->multiSample && !resolved) {
    if (bytes < (size_t) w * h * sizeof(glm::tvec4<T>) || !buf->bufferMs4x) return false;
    auto *dst = reinterpret_cast<glm::tvec4<T> *>(out);
    for (int y = 0; y < h; y++)
      for (int x = 0; x < w; x++) dst[y * w + x] = *buf->bufferMs4x->get(x, y);
    return true;
  }
  if (bytes < (size_t) w * h * sizeof(T)) return false;
  if (!buf->buffer) {
    memset(out, 0, (size_t) w * h * sizeof(T));
    return true;
  }
  auto *dst = reinterpret_cast<T *>(out);
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) dst[y * w + x] = *buf->buffer->get(x, y);
  return true;
}

template<typename T>
bool writeLevel(TextureSoft<T> *tex, int layer, int level, const uint8_t *data, size_t bytes) {
  auto &img = tex->getImage(layer);
  if (level < 0 || level >= (int) img.levels.size()) return false;
  auto &buf = img.getBuffer(level);
  if (!buf->buffer || bytes < (size_t) buf->width * buf->height * sizeof(T)) return false;
  auto *src = reinterpret_cast<const T *>(data);
  for (int y = 0; y < buf->height; y++)
    for (int x = 0; x < buf->width; x++) buf->buffer->set(x, y, src[y * buf->width + x]);
  return true;
}

}  // namespace

#define SOFT_SHADERS(ns) \
  ps->SetShaders(std::make_shared<ns::VS>(), std::make_shared<ns::FS>())

extern "C" {

sglc_status sglr_create(sglc_context **out, int32_t device) {
  (void) device;
  auto *c = new Ctx();
  c->renderer.create();
  *out = reinterpret_cast<sglc_context *>(c);
  return SGLC_OK;
}

sglc_status sglr_destroy(sglc_context *ctx) {
  delete reinterpret_cast<Ctx *>(ctx);
  return SGLC_OK;
}

const char *sglr_last_error(sglc_context *ctx) {
  return reinterpret_cast<Ctx *>(ctx)->err.c_str();
}

sglc_status sglr_release(sglc_context *ctx, sglc_handle h) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  if (!c->objects.erase(h)) return c->fail(SGLC_ERR_INVALID_HANDLE, "release: unknown handle");
  return SGLC_OK;
}

sglc_status sglr_create_framebuffer(sglc_context *ctx, int32_t offscreen, sglc_handle *out) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object o;
  o.fb = c->renderer.createFrameBuffer(offscreen != 0);
  *out = c->add(o);
  return SGLC_OK;
}

sglc_status sglr_framebuffer_set_color_attachment(sglc_context *ctx, sglc_handle fb, sglc_handle tex,
                                                  int32_t layer, int32_t level) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *f = c->get(fb), *t = c->get(tex);
  CTX_CHECK(f && f->fb && t && t->tex);
  if (t->tex->type == TextureType_CUBE) {
    f->fb->setColorAttachment(t->tex, (CubeMapFace) layer, level);
  } else {
    f->fb->setColorAttachment(t->tex, level);
  }
  return SGLC_OK;
}

sglc_status sglr_framebuffer_set_depth_attachment(sglc_context *ctx, sglc_handle fb, sglc_handle tex) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *f = c->get(fb), *t = c->get(tex);
  CTX_CHECK(f && f->fb && t && t->tex);
  f->fb->setDepthAttachment(t->tex);
  return SGLC_OK;
}

sglc_status sglr_framebuffer_is_valid(sglc_context *ctx, sglc_handle fb, int32_t *valid) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *f = c->get(fb);
  CTX_CHECK(f && f->fb);
  *valid = f->fb->isValid() ? 1 : 0;
  return SGLC_OK;
}

sglc_status sglr_create_texture(sglc_context *ctx, const sglc_texture_desc *d, sglc_handle *out) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  TextureDesc desc;
  desc.width = d->width;
  desc.height = d->height;
  desc.type = (TextureType) d->type;
  desc.format = (TextureFormat) d->format;
  desc.usage = d->usage;
  desc.useMipmaps = d->use_mipmaps != 0;
  desc.multiSample = d->multi_sample != 0;
  Object o;
  o.tex = c->renderer.createTexture(desc);
  if (!o.tex) return c->fail(SGLC_ERR_INVALID_VALUE, "createTexture returned null");
  *out = c->add(o);
  return SGLC_OK;
}

sglc_status sglr_texture_set_sampler_desc(sglc_context *ctx, sglc_handle tex, const sglc_sampler_desc *s) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *t = c->get(tex);
  CTX_CHECK(t && t->tex);
  SamplerDesc sd;
  sd.filterMin = (FilterMode) s->filter_min;
  sd.filterMag = (FilterMode) s->filter_mag;
  sd.wrapS = (WrapMode) s->wrap_s;
  sd.wrapT = (WrapMode) s->wrap_t;
  sd.wrapR = (WrapMode) s->wrap_r;
  sd.borderColor = (BorderColor) s->border_color;
  t->tex->setSamplerDesc(sd);
  return SGLC_OK;
}

sglc_status sglr_texture_init_image_data(sglc_context *ctx, sglc_handle tex) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *t = c->get(tex);
  CTX_CHECK(t && t->tex);
  t->tex->initImageData();
  return SGLC_OK;
}

sglc_status sglr_texture_set_image_data(sglc_context *ctx, sglc_handle tex, int32_t layer_count,
                                        const void *const *layers, size_t bytes_per_layer) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *t = c->get(tex);
  CTX_CHECK(t && t->tex);
  auto &tx = *t->tex;
  size_t need = (size_t) tx.width * tx.height * 4;
  if (bytes_per_layer < need) return c->fail(SGLC_ERR_INVALID_VALUE, "setImageData: short buffer");
  if (tx.format == TextureFormat_RGBA8) {
    std::vector<std::shared_ptr<Buffer<RGBA>>> bufs;
    for (int i = 0; i < layer_count; i++) {
      auto b = Buffer<RGBA>::makeDefault(tx.width, tx.height);
      auto *src = reinterpret_cast<const RGBA *>(layers[i]);
      for (int y = 0; y < tx.height; y++)
        for (int x = 0; x < tx.width; x++) b->set(x, y, src[y * tx.width + x]);
      bufs.push_back(b);
    }
    tx.setImageData(bufs);
  } else {
    std::vector<std::shared_ptr<Buffer<float>>> bufs;
    for (int i = 0; i < layer_count; i++) {
      auto b = Buffer<float>::makeDefault(tx.width, tx.height);
      auto *src = reinterpret_cast<const float *>(layers[i]);
      for (int y = 0; y < tx.height; y++)
        for (int x = 0; x < tx.width; x++) b->set(x, y, src[y * tx.width + x]);
      bufs.push_back(b);
    }
    tx.setImageData(bufs);
  }
  return SGLC_OK;
}

sglc_status sglr_texture_set_level_data(sglc_context *ctx, sglc_handle tex, int32_t layer, int32_t level,
                                        const void *data, size_t bytes) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *t = c->get(tex);
  CTX_CHECK(t && t->tex);
  bool ok;
  if (t->tex->format == TextureFormat_RGBA8) {
    ok = writeLevel(dynamic_cast<TextureSoft<RGBA> *>(t->tex.get()), layer, level, (const uint8_t *) data, bytes);
  } else {
    ok = writeLevel(dynamic_cast<TextureSoft<float> *>(t->tex.get()), layer, level, (const uint8_t *) data, bytes);
  }
  return ok ? SGLC_OK : c->fail(SGLC_ERR_INVALID_VALUE, "set_level_data: bad level or size");
}

sglc_status sglr_texture_read_image(sglc_context *ctx, sglc_handle tex, int32_t layer, int32_t level,
                                    int32_t resolved, void *out, size_t bytes) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *t = c->get(tex);
  CTX_CHECK(t && t->tex);
  bool ok;
  if (t->tex->format == TextureFormat_RGBA8) {
    ok = readTexture(dynamic_cast<TextureSoft<RGBA> *>(t->tex.get()), layer, level, resolved, (uint8_t *) out, bytes);
  } else {
    ok = readTexture(dynamic_cast<TextureSoft<float> *>(t->tex.get()), layer, level, resolved, (uint8_t *) out, bytes);
  }
  return ok ? SGLC_OK : c->fail(SGLC_ERR_INVALID_VALUE, "read_image: bad level or size");
}

sglc_status sglr_texture_store_to_file(sglc_context *ctx, sglc_handle tex, const char *path) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *t = c->get(tex);
  CTX_CHECK(t && t->tex && path);
  FILE *probe = fopen(path, "ab");   // storeToFile only logs a failed open
  if (!probe) return c->fail(SGLC_ERR_INVALID_VALUE, "store_to_file: failed to open file");
  fclose(probe);
  if (t->tex->format == TextureFormat_RGBA8) dynamic_cast<TextureSoft<RGBA> *>(t->tex.get())->storeToFile(path);
  else dynamic_cast<TextureSoft<float> *>(t->tex.get())->storeToFile(path);
  return SGLC_OK;
}

sglc_status sglr_texture_load_from_file(sglc_context *ctx, sglc_handle tex, const char *path) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *t = c->get(tex);
  CTX_CHECK(t && t->tex && path);
  bool ok;
  if (t->tex->format == TextureFormat_RGBA8) ok = dynamic_cast<TextureSoft<RGBA> *>(t->tex.get())->loadFromFile(path);
  else ok = dynamic_cast<TextureSoft<float> *>(t->tex.get())->loadFromFile(path);
  return ok ? SGLC_OK : c->fail(SGLC_ERR_INVALID_VALUE, "load_from_file: failed");
}

sglc_status sglr_create_vertex_array(sglc_context *ctx, const void *vertexes, size_t vertexes_len, size_t stride,
                                     const int32_t *indices, size_t indices_len, sglc_handle *out) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  VertexArray va;
  va.vertexSize = stride;
  va.vertexesDesc.push_back({stride / 4, stride, 0});
  va.vertexesBuffer = (uint8_t *) vertexes;
  va.vertexesBufferLength = vertexes_len;
  va.indexBuffer = (int32_t *) indices;
  va.indexBufferLength = indices_len;
  Object o;
  o.vao = c->renderer.createVertexArrayObject(va);
  *out = c->add(o);
  return SGLC_OK;
}

sglc_status sglr_vertex_array_update(sglc_context *ctx, sglc_handle vao, const void *data, size_t len) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *v = c->get(vao);
  CTX_CHECK(v && v->vao);
  v->vao->updateVertexData((void *) data, len);
  return SGLC_OK;
}

sglc_status sglr_create_shader_program(sglc_context *ctx, sglc_handle *out) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object o;
  o.prog = c->renderer.createShaderProgram();
  *out = c->add(o);
  return SGLC_OK;
}

sglc_status sglr_program_add_define(sglc_context *ctx, sglc_handle prog, const char *name) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *p = c->get(prog);
  CTX_CHECK(p && p->prog);
  p->prog->addDefine(name);
  return SGLC_OK;
}

sglc_status sglr_program_set_shaders(sglc_context *ctx, sglc_handle prog, int32_t shading) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *p = c->get(prog);
  CTX_CHECK(p && p->prog);
  auto *ps = dynamic_cast<ShaderProgramSoft *>(p->prog.get());
  switch (shading) {
    case SGLC_SHADING_BASE_COLOR: SOFT_SHADERS(ShaderBasic); break;
    case SGLC_SHADING_BLINN_PHONG: SOFT_SHADERS(ShaderBlinnPhong); break;
    case SGLC_SHADING_PBR: SOFT_SHADERS(ShaderPbrIBL); break;
    case SGLC_SHADING_SKYBOX: SOFT_SHADERS(ShaderSkybox); break;
    case SGLC_SHADING_IBL_IRRADIANCE: SOFT_SHADERS(ShaderIBLIrradiance); break;
    case SGLC_SHADING_IBL_PREFILTER: SOFT_SHADERS(ShaderIBLPrefilter); break;
    case SGLC_SHADING_FXAA: SOFT_SHADERS(ShaderFXAA); break;
    case SGLC_SHADING_BLINN_PHONG_DIR: SOFT_SHADERS(ShaderBlinnPhongDir); break;
    case SGLC_SHADING_VERTEX_COLOR: SOFT_SHADERS(ShaderVertexColor); break;
    default: return c->fail(SGLC_ERR_UNSUPPORTED, "unknown shading model");
  }
  return SGLC_OK;
}

sglc_status sglr_create_pipeline_states(sglc_context *ctx, const sglc_render_states *s, sglc_handle *out) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  RenderStates rs;
  rs.blend = s->blend != 0;
  rs.blendParams.blendFuncRgb = (BlendFunction) s->blend_func_rgb;
  rs.blendParams.blendSrcRgb = (BlendFactor) s->blend_src_rgb;
  rs.blendParams.blendDstRgb = (BlendFactor) s->blend_dst_rgb;
  rs.blendParams.blendFuncAlpha = (BlendFunction) s->blend_func_alpha;
  rs.blendParams.blendSrcAlpha = (BlendFactor) s->blend_src_alpha;
  rs.blendParams.blendDstAlpha = (BlendFactor) s->blend_dst_alpha;
  rs.depthTest = s->depth_test != 0;
  rs.depthMask = s->depth_mask != 0;
  rs.depthFunc = (DepthFunction) s->depth_func;
  rs.cullFace = s->cull_face != 0;
  rs.primitiveType = (PrimitiveType) s->primitive_type;
  rs.polygonMode = (PolygonMode) s->polygon_mode;
  rs.lineWidth = s->line_width;
  Object o;
  o.states = c->renderer.createPipelineStates(rs);
  *out = c->add(o);
  return SGLC_OK;
}

sglc_status sglr_create_uniform_block(sglc_context *ctx, const char *name, int32_t size, sglc_handle *out) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object o;
  o.ub = c->renderer.createUniformBlock(name, size);
  *out = c->add(o);
  return SGLC_OK;
}

sglc_status sglr_uniform_block_set_sub_data(sglc_context *ctx, sglc_handle ub, const void *data, int32_t len,
                                            int32_t offset) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *u = c->get(ub);
  CTX_CHECK(u && u->ub);
  u->ub->setSubData((void *) data, len, offset);
  return SGLC_OK;
}

sglc_status sglr_uniform_block_set_data(sglc_context *ctx, sglc_handle ub, const void *data, int32_t len) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *u = c->get(ub);
  CTX_CHECK(u && u->ub);
  u->ub->setData((void *) data, len);
  return SGLC_OK;
}

sglc_status sglr_create_uniform_sampler(sglc_context *ctx, const char *name, int32_t type, int32_t format,
                                        sglc_handle *out) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  TextureDesc desc;
  desc.type = (TextureType) type;
  desc.format = (TextureFormat) format;
  Object o;
  o.us = c->renderer.createUniformSampler(name, desc);
  *out = c->add(o);
  return SGLC_OK;
}

sglc_status sglr_uniform_sampler_set_texture(sglc_context *ctx, sglc_handle us, sglc_handle tex) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *u = c->get(us), *t = c->get(tex);
  CTX_CHECK(u && u->us && t && t->tex);
  u->us->setTexture(t->tex);
  return SGLC_OK;
}

sglc_status sglr_create_shader_resources(sglc_context *ctx, sglc_handle *out) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object o;
  o.res = std::make_shared<ShaderResources>();
  *out = c->add(o);
  return SGLC_OK;
}

sglc_status sglr_shader_resources_set_block(sglc_context *ctx, sglc_handle res, int32_t key, sglc_handle ub) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *r = c->get(res), *u = c->get(ub);
  CTX_CHECK(r && r->res && u && u->ub);
  r->res->blocks[key] = u->ub;
  return SGLC_OK;
}

sglc_status sglr_shader_resources_set_sampler(sglc_context *ctx, sglc_handle res, int32_t key, sglc_handle us) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *r = c->get(res), *u = c->get(us);
  CTX_CHECK(r && r->res && u && u->us);
  r->res->samplers[key] = u->us;
  return SGLC_OK;
}

sglc_status sglr_begin_render_pass(sglc_context *ctx, sglc_handle fb, const sglc_clear_states *s) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *f = c->get(fb);
  CTX_CHECK(f && f->fb);
  ClearStates cs;
  cs.depthFlag = s->depth_flag != 0;
  cs.colorFlag = s->color_flag != 0;
  cs.clearColor = glm::vec4(s->clear_color[0], s->clear_color[1], s->clear_color[2], s->clear_color[3]);
  cs.clearDepth = s->clear_depth;
  c->boundFb = f->fb;
  c->renderer.beginRenderPass(c->boundFb, cs);
  return SGLC_OK;
}

sglc_status sglr_set_viewport(sglc_context *ctx, int32_t x, int32_t y, int32_t w, int32_t h) {
  reinterpret_cast<Ctx *>(ctx)->renderer.setViewPort(x, y, w, h);
  return SGLC_OK;
}

sglc_status sglr_set_vertex_array(sglc_context *ctx, sglc_handle vao) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *v = c->get(vao);
  CTX_CHECK(v && v->vao);
  c->boundVao = v->vao;
  c->renderer.setVertexArrayObject(c->boundVao);
  return SGLC_OK;
}

sglc_status sglr_set_shader_program(sglc_context *ctx, sglc_handle prog) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *p = c->get(prog);
  CTX_CHECK(p && p->prog);
  c->boundProg = p->prog;
  c->renderer.setShaderProgram(c->boundProg);
  return SGLC_OK;
}

sglc_status sglr_set_shader_resources(sglc_context *ctx, sglc_handle res) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *r = c->get(res);
  CTX_CHECK(r && r->res);
  c->boundRes = r->res;
  c->renderer.setShaderResources(c->boundRes);
  return SGLC_OK;
}

sglc_status sglr_set_pipeline_states(sglc_context *ctx, sglc_handle st) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  Object *s = c->get(st);
  CTX_CHECK(s && s->states);
  c->boundStates = s->states;
  c->renderer.setPipelineStates(c->boundStates);
  return SGLC_OK;
}

sglc_status sglr_draw(sglc_context *ctx) {
  reinterpret_cast<Ctx *>(ctx)->renderer.draw();
  return SGLC_OK;
}

sglc_status sglr_end_render_pass(sglc_context *ctx) {
  reinterpret_cast<Ctx *>(ctx)->renderer.endRenderPass();
  return SGLC_OK;
}

// The batched draw on the reference: the views drawn one after another in their own render passes
// (RendererSoft has no batching).
sglc_status sglr_draw_views(sglc_context *ctx, const sglc_handle *fbs, const sglc_handle *res, int32_t count,
                            const sglc_clear_states *clear) {
  sglc_clear_states none{0, 0, {0.f, 0.f, 0.f, 0.f}, 1.f};
  for (int v = 0; v < count; v++) {
    sglc_status s = sglr_begin_render_pass(ctx, fbs[v], clear ? clear : &none);
    if (!s) s = sglr_set_shader_resources(ctx, res[v]);
    if (!s) s = sglr_draw(ctx);
    if (!s) s = sglr_end_render_pass(ctx);
    if (s) return s;
  }
  return SGLC_OK;
}

// The multi-scene draw on the reference: each scene in its own render pass, viewport over its whole
// frame (the larger of its attachments), its own vertex array.
sglc_status sglr_draw_scenes(sglc_context *ctx, const sglc_handle *vaos, const sglc_handle *fbs, const sglc_handle *res,
                             int32_t count, const sglc_clear_states *clear) {
  auto *c = reinterpret_cast<Ctx *>(ctx);
  sglc_clear_states none{0, 0, {0.f, 0.f, 0.f, 0.f}, 1.f};
  for (int v = 0; v < count; v++) {
    Object *f = c->get(fbs[v]);
    CTX_CHECK(f && f->fb);
    int w = 0, h = 0;
    for (const FrameBufferAttachment *a : {&f->fb->getColorAttachment(), &f->fb->getDepthAttachment()})
      if (a->tex) {
        w = std::max(w, (int) a->tex->getLevelWidth(a->level));
        h = std::max(h, (int) a->tex->getLevelHeight(a->level));
      }
    sglc_status s = sglr_begin_render_pass(ctx, fbs[v], clear ? clear : &none);
    if (!s) s = sglr_set_viewport(ctx, 0, 0, w, h);
    if (!s) s = sglr_set_vertex_array(ctx, vaos[v]);
    if (!s) s = sglr_set_shader_resources(ctx, res[v]);
    if (!s) s = sglr_draw(ctx);
    if (!s) s = sglr_end_render_pass(ctx);
    if (s) return s;
  }
  return SGLC_OK;
}

// Capacities only change how the GPU back-end sizes its working arrays; RendererSoft has none.
sglc_status sglr_set_capacity(sglc_context *, const sglc_capacity *) { return SGLC_OK; }
sglc_status sglr_get_peak_counts(sglc_context *, sglc_capacity *out) {
  if (out) *out = sglc_capacity{0, 0, 0, 0, 1};
  return SGLC_OK;
}
sglc_status sglr_get_overflow(sglc_context *, int32_t *flags) {
  if (flags) *flags = 0;
  return SGLC_OK;
}

sglc_status sglr_wait_idle(sglc_context *ctx) {
  reinterpret_cast<Ctx *>(ctx)->renderer.waitIdle();
  return SGLC_OK;
}

sglc_status sglr_set_enable_early_z(sglc_context *ctx, int32_t enable) {
  reinterpret_cast<Ctx *>(ctx)->renderer.setEnableEarlyZ(enable != 0);
  return SGLC_OK;
}

sglc_status sglr_get_draw_stats(sglc_context *ctx, sglc_draw_stats *out) {
  memset(out, 0, sizeof(*out));
  return SGLC_OK;
}

sglc_status sglr_get_stream(sglc_context *ctx, void **stream) {
  *stream = nullptr;
  return SGLC_OK;
}

sglc_status sglr_set_stats_level(sglc_context *ctx, int32_t level) {
  (void) ctx;
  (void) level;
  return SGLC_OK;
}

sglc_status sglr_set_deferred_shading(sglc_context *ctx, int32_t enable) {
  (void) ctx;
  (void) enable;
  return SGLC_OK;
}

sglc_status sglr_set_tma_store(sglc_context *ctx, int32_t enable) {
  (void) ctx;
  (void) enable;
  return SGLC_OK;
}

sglc_status sglr_set_tile_size(sglc_context *ctx, int32_t tile) {
  (void) ctx;
  (void) tile;
  return SGLC_OK;
}

}  // extern "C"
