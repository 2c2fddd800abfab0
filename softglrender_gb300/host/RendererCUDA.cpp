/*
 * RendererCUDA: forwarding of SoftGL::Renderer to the C ABI (see RendererCUDA.h).
 */
#include "RendererCUDA.h"

#include <vector>

#include "Base/ImageUtils.h"
#include "Base/Logger.h"

namespace SoftGL {

static sglc_texture_desc toDesc(const TextureDesc &d) {
  sglc_texture_desc t{};
  t.width = d.width;
  t.height = d.height;
  t.type = (int32_t) d.type;
  t.format = (int32_t) d.format;
  t.usage = d.usage;
  t.use_mipmaps = d.useMipmaps;
  t.multi_sample = d.multiSample;
  t.layout = SGLC_LAYOUT_LINEAR;
  return t;
}

bool RendererCUDA::check(sglc_status s, const char *what) {
  if (s != SGLC_OK) {
    LOGE("%s failed (%d): %s", what, s, ctx_ ? sglc_last_error(ctx_) : "no context");
    return false;
  }
  return true;
}

bool RendererCUDA::create() {
  if (ctx_) return true;
  return check(sglc_create(&ctx_, device_), "sglc_create");
}

void RendererCUDA::destroy() {
  if (ctx_) sglc_destroy(ctx_);
  ctx_ = nullptr;
}

// ---- resources ------------------------------------------------------------------------------
TextureCUDA::TextureCUDA(RendererCUDA *r, const TextureDesc &desc, sglc_handle h) : renderer(r), handle(h) {
  width = desc.width;
  height = desc.height;
  type = desc.type;
  format = desc.format;
  usage = desc.usage;
  useMipmaps = desc.useMipmaps;
  multiSample = desc.multiSample;
  tag = desc.tag;
}

void TextureCUDA::setSamplerDesc(SamplerDesc &s) {
  sglc_sampler_desc d{(int32_t) s.filterMin, (int32_t) s.filterMag, (int32_t) s.wrapS, (int32_t) s.wrapT,
                      (int32_t) s.wrapR, (int32_t) s.borderColor};
  renderer->check(sglc_texture_set_sampler_desc(renderer->ctx(), handle, &d), "setSamplerDesc");
}

void TextureCUDA::initImageData() {
  renderer->check(sglc_texture_init_image_data(renderer->ctx(), handle), "initImageData");
}

template<typename T>
static void uploadLayers(TextureCUDA *t, const std::vector<std::shared_ptr<Buffer<T>>> &buffers) {
  // Buffer<T> may use a tiled / Morton layout: linearise through get(x, y) (Buffer.h:86-92)
  std::vector<std::vector<T>> lin(buffers.size());
  std::vector<const void *> ptrs;
  for (size_t i = 0; i < buffers.size(); i++) {
    auto &b = buffers[i];
    lin[i].resize((size_t) t->width * t->height);
    for (int y = 0; y < t->height; y++)
      for (int x = 0; x < t->width; x++) lin[i][(size_t) y * t->width + x] = *b->get(x, y);
    ptrs.push_back(lin[i].data());
  }
  t->renderer->check(sglc_texture_set_image_data(t->renderer->ctx(), t->handle, (int32_t) ptrs.size(), ptrs.data(),
                                                 (size_t) t->width * t->height * sizeof(T)),
                     "setImageData");
}

void TextureCUDA::setImageData(const std::vector<std::shared_ptr<Buffer<RGBA>>> &buffers) { uploadLayers(this, buffers); }
void TextureCUDA::setImageData(const std::vector<std::shared_ptr<Buffer<float>>> &buffers) { uploadLayers(this, buffers); }

void TextureCUDA::dumpImage(const char *path, uint32_t layer, uint32_t level) {
  if (multiSample) return;   // as TextureSoft::dumpImageSoft
  int w = getLevelWidth(level), h = getLevelHeight(level);
  std::vector<uint32_t> px((size_t) w * h);
  if (!renderer->check(sglc_texture_read_image(renderer->ctx(), handle, layer, level, 0, px.data(), px.size() * 4),
                       "dumpImage"))
    return;
  if (format == TextureFormat_FLOAT32) {
    std::vector<RGBA> rgba((size_t) w * h);
    ImageUtils::convertFloatImage(rgba.data(), reinterpret_cast<float *>(px.data()), w, h);
    ImageUtils::writeImage(path, w, h, 4, rgba.data(), w * 4, true);
  } else {
    ImageUtils::writeImage(path, w, h, 4, px.data(), w * 4, true);
  }
}

bool TextureCUDA::loadFromFile(const char *path) {
  return renderer->check(sglc_texture_load_from_file(renderer->ctx(), handle, path), "loadFromFile");
}

void TextureCUDA::storeToFile(const char *path) {
  renderer->check(sglc_texture_store_to_file(renderer->ctx(), handle, path), "storeToFile");
}

bool TextureCUDA::setLevelData(uint32_t layer, uint32_t level, const void *data, size_t bytes) {
  return renderer->check(sglc_texture_set_level_data(renderer->ctx(), handle, (int32_t) layer, (int32_t) level, data,
                                                     bytes),
                         "setLevelData");
}

bool TextureCUDA::readImage(void *out, size_t bytes, uint32_t layer, uint32_t level, bool resolved) {
  return renderer->check(sglc_texture_read_image(renderer->ctx(), handle, (int32_t) layer, (int32_t) level,
                                                 resolved ? 1 : 0, out, bytes),
                         "readImage");
}

bool FrameBufferCUDA::isValid() {
  int32_t v = 0;
  renderer->check(sglc_framebuffer_is_valid(renderer->ctx(), handle, &v), "isValid");
  return v != 0;
}

void FrameBufferCUDA::setColorAttachment(std::shared_ptr<Texture> &color, int level) {
  FrameBuffer::setColorAttachment(color, level);
  auto *t = dynamic_cast<TextureCUDA *>(color.get());
  renderer->check(sglc_framebuffer_set_color_attachment(renderer->ctx(), handle, t->handle, 0, level),
                  "setColorAttachment");
}

void FrameBufferCUDA::setColorAttachment(std::shared_ptr<Texture> &color, CubeMapFace face, int level) {
  FrameBuffer::setColorAttachment(color, face, level);
  auto *t = dynamic_cast<TextureCUDA *>(color.get());
  renderer->check(sglc_framebuffer_set_color_attachment(renderer->ctx(), handle, t->handle, (int32_t) face, level),
                  "setColorAttachment");
}

void FrameBufferCUDA::setDepthAttachment(std::shared_ptr<Texture> &depth) {
  FrameBuffer::setDepthAttachment(depth);
  auto *t = dynamic_cast<TextureCUDA *>(depth.get());
  renderer->check(sglc_framebuffer_set_depth_attachment(renderer->ctx(), handle, t->handle), "setDepthAttachment");
}

void VertexArrayObjectCUDA::updateVertexData(void *data, size_t length) {
  renderer->check(sglc_vertex_array_update(renderer->ctx(), handle, data, length), "updateVertexData");
}

void ShaderProgramCUDA::addDefine(const std::string &def) {
  renderer->check(sglc_program_add_define(renderer->ctx(), handle, def.c_str()), "addDefine");
}

bool ShaderProgramCUDA::setShadingModel(int shadingModel) {
  return renderer->check(sglc_program_set_shaders(renderer->ctx(), handle, shadingModel), "setShaders");
}

void UniformBlockCUDA::setSubData(void *data, int len, int offset) {
  renderer->check(sglc_uniform_block_set_sub_data(renderer->ctx(), handle, data, len, offset), "setSubData");
}

void UniformBlockCUDA::setData(void *data, int len) {
  renderer->check(sglc_uniform_block_set_data(renderer->ctx(), handle, data, len), "setData");
}

void UniformSamplerCUDA::setTexture(const std::shared_ptr<Texture> &tex) {
  auto *t = dynamic_cast<TextureCUDA *>(tex.get());
  renderer->check(sglc_uniform_sampler_set_texture(renderer->ctx(), handle, t->handle), "setTexture");
}

// ---- factories ------------------------------------------------------------------------------
std::shared_ptr<FrameBuffer> RendererCUDA::createFrameBuffer(bool offscreen) {
  sglc_handle h = 0;
  if (!check(sglc_create_framebuffer(ctx_, offscreen, &h), "createFrameBuffer")) return nullptr;
  return std::make_shared<FrameBufferCUDA>(this, offscreen, h);
}

std::shared_ptr<Texture> RendererCUDA::createTexture(const TextureDesc &desc) {
  sglc_texture_desc d = toDesc(desc);
  sglc_handle h = 0;
  if (!check(sglc_create_texture(ctx_, &d, &h), "createTexture")) return nullptr;
  return std::make_shared<TextureCUDA>(this, desc, h);
}

std::shared_ptr<VertexArrayObject> RendererCUDA::createVertexArrayObject(const VertexArray &va) {
  sglc_handle h = 0;
  size_t stride = va.vertexesDesc.empty() ? 0 : va.vertexesDesc[0].stride;   // VertexSoft.h:18
  if (!check(sglc_create_vertex_array(ctx_, va.vertexesBuffer, va.vertexesBufferLength, stride, va.indexBuffer,
                                      va.indexBufferLength, &h),
             "createVertexArrayObject"))
    return nullptr;
  return std::make_shared<VertexArrayObjectCUDA>(this, h);
}

std::shared_ptr<ShaderProgram> RendererCUDA::createShaderProgram() {
  sglc_handle h = 0;
  if (!check(sglc_create_shader_program(ctx_, &h), "createShaderProgram")) return nullptr;
  return std::make_shared<ShaderProgramCUDA>(this, h);
}

std::shared_ptr<PipelineStates> RendererCUDA::createPipelineStates(const RenderStates &rs) {
  const BlendParameters &b = rs.blendParams;
  sglc_render_states s{rs.blend, b.blendFuncRgb, b.blendSrcRgb, b.blendDstRgb, b.blendFuncAlpha, b.blendSrcAlpha,
                       b.blendDstAlpha, rs.depthTest, rs.depthMask, rs.depthFunc, rs.cullFace, rs.primitiveType,
                       rs.polygonMode, rs.lineWidth};
  sglc_handle h = 0;
  if (!check(sglc_create_pipeline_states(ctx_, &s, &h), "createPipelineStates")) return nullptr;
  return std::make_shared<PipelineStatesCUDA>(rs, h);
}

std::shared_ptr<UniformBlock> RendererCUDA::createUniformBlock(const std::string &name, int size) {
  sglc_handle h = 0;
  if (!check(sglc_create_uniform_block(ctx_, name.c_str(), size, &h), "createUniformBlock")) return nullptr;
  return std::make_shared<UniformBlockCUDA>(this, name, size, h);
}

std::shared_ptr<UniformSampler> RendererCUDA::createUniformSampler(const std::string &name, const TextureDesc &desc) {
  sglc_handle h = 0;
  if (!check(sglc_create_uniform_sampler(ctx_, name.c_str(), desc.type, desc.format, &h), "createUniformSampler"))
    return nullptr;
  return std::make_shared<UniformSamplerCUDA>(this, name, desc.type, desc.format, h);
}

// ---- pipeline ---------------------------------------------------------------------------------
void RendererCUDA::beginRenderPass(std::shared_ptr<FrameBuffer> &frameBuffer, const ClearStates &states) {
  auto *fb = dynamic_cast<FrameBufferCUDA *>(frameBuffer.get());
  if (!fb) return;   // RendererSoft::beginRenderPass returns on a foreign FBO (RendererSoft.cpp:62-66)
  sglc_clear_states c{states.depthFlag, states.colorFlag,
                      {states.clearColor.r, states.clearColor.g, states.clearColor.b, states.clearColor.a},
                      states.clearDepth};
  check(sglc_begin_render_pass(ctx_, fb->handle, &c), "beginRenderPass");
}

void RendererCUDA::setViewPort(int x, int y, int width, int height) {
  check(sglc_set_viewport(ctx_, x, y, width, height), "setViewPort");
}

void RendererCUDA::setVertexArrayObject(std::shared_ptr<VertexArrayObject> &vao) {
  auto *v = dynamic_cast<VertexArrayObjectCUDA *>(vao.get());
  if (v) check(sglc_set_vertex_array(ctx_, v->handle), "setVertexArrayObject");
}

void RendererCUDA::setShaderProgram(std::shared_ptr<ShaderProgram> &program) {
  auto *p = dynamic_cast<ShaderProgramCUDA *>(program.get());
  if (p) check(sglc_set_shader_program(ctx_, p->handle), "setShaderProgram");
}

// ShaderProgram::bindResources (ShaderProgram.h:27-54): the C ABI copies the blocks into the bound
// program now and binds the samplers by reference, as UniformSoft does
void RendererCUDA::setShaderResources(std::shared_ptr<ShaderResources> &resources) {
  if (!resources) return;
  const sglc_handle h = resourcesHandle(resources);
  if (h) check(sglc_set_shader_resources(ctx_, h), "setShaderResources");
}

sglc_handle RendererCUDA::resourcesHandle(const std::shared_ptr<ShaderResources> &resources) {
  if (!resources) return 0;
  sglc_handle &h = resources_[resources.get()];
  if (!h && !check(sglc_create_shader_resources(ctx_, &h), "createShaderResources")) return 0;
  for (auto &kv : resources->blocks) {
    auto *b = dynamic_cast<UniformBlockCUDA *>(kv.second.get());
    if (b) check(sglc_shader_resources_set_block(ctx_, h, kv.first, b->handle), "setShaderResources");
  }
  for (auto &kv : resources->samplers) {
    auto *s = dynamic_cast<UniformSamplerCUDA *>(kv.second.get());
    if (s) check(sglc_shader_resources_set_sampler(ctx_, h, kv.first, s->handle), "setShaderResources");
  }
  return h;
}

void RendererCUDA::setPipelineStates(std::shared_ptr<PipelineStates> &states) {
  auto *s = dynamic_cast<PipelineStatesCUDA *>(states.get());
  if (s) check(sglc_set_pipeline_states(ctx_, s->handle), "setPipelineStates");
}

void RendererCUDA::draw() { check(sglc_draw(ctx_), "draw"); }

void RendererCUDA::endRenderPass() { check(sglc_end_render_pass(ctx_), "endRenderPass"); }

void RendererCUDA::waitIdle() { check(sglc_wait_idle(ctx_), "waitIdle"); }

void RendererCUDA::setEnableEarlyZ(bool enable) { check(sglc_set_enable_early_z(ctx_, enable), "setEnableEarlyZ"); }

}  // namespace SoftGL
