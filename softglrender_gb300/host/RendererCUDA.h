/*
 * RendererCUDA: SoftGL::Renderer (src/Render/Renderer.h:24-59) backed by the sm_103a library through
 * the C ABI of include/softgl_cuda.h. This header is the reference-side binding: it compiles inside the
 * reference tree (it includes the reference's Render/*.h), next to RendererSoft, and links against
 * libsoftgl_cuda.so. Every virtual forwards to one sglc_* call; resource objects keep their sglc handle.
 */
#pragma once

#include <memory>
#include <string>
#include <unordered_map>

#include "Render/Renderer.h"
#include "Render/Uniform.h"
#include "softgl_cuda.h"

namespace SoftGL {

class RendererCUDA;

class TextureCUDA : public Texture {
 public:
  TextureCUDA(RendererCUDA *r, const TextureDesc &desc, sglc_handle h);
  int getId() const override { return handle; }
  void setSamplerDesc(SamplerDesc &sampler) override;
  void initImageData() override;
  void setImageData(const std::vector<std::shared_ptr<Buffer<RGBA>>> &buffers) override;
  void setImageData(const std::vector<std::shared_ptr<Buffer<float>>> &buffers) override;
  void dumpImage(const char *path, uint32_t layer, uint32_t level) override;
  // TextureSoft::loadFromFile / storeToFile (TextureSoft.h:166-215): the IBL cache format
  bool loadFromFile(const char *path);
  void storeToFile(const char *path);
  // One level of one layer from host memory (the reference fills prefiltered IBL levels by
  // rendering into a level attachment, Environment.cpp:152-195; a cached chain uploads directly)
  bool setLevelData(uint32_t layer, uint32_t level, const void *data, size_t bytes);
  // The pixels dumpImage writes, copied to host memory in linear row order (the software back-end's
  // callers read TextureSoft's buffers directly): RGBA8 4 B, FLOAT32 4 B per sample; a multi-sample
  // texture gives its 4 interleaved samples per pixel, or with `resolved` its resolved RGBA8 image
  bool readImage(void *out, size_t bytes, uint32_t layer, uint32_t level, bool resolved);

  RendererCUDA *renderer;
  sglc_handle handle;
};

class FrameBufferCUDA : public FrameBuffer {
 public:
  FrameBufferCUDA(RendererCUDA *r, bool offscreen, sglc_handle h) : FrameBuffer(offscreen), renderer(r), handle(h) {}
  int getId() const override { return handle; }
  bool isValid() override;
  void setColorAttachment(std::shared_ptr<Texture> &color, int level) override;
  void setColorAttachment(std::shared_ptr<Texture> &color, CubeMapFace face, int level) override;
  void setDepthAttachment(std::shared_ptr<Texture> &depth) override;

  RendererCUDA *renderer;
  sglc_handle handle;
};

class VertexArrayObjectCUDA : public VertexArrayObject {
 public:
  VertexArrayObjectCUDA(RendererCUDA *r, sglc_handle h) : renderer(r), handle(h) {}
  int getId() const override { return handle; }
  void updateVertexData(void *data, size_t length) override;

  RendererCUDA *renderer;
  sglc_handle handle;
};

class ShaderProgramCUDA : public ShaderProgram {
 public:
  ShaderProgramCUDA(RendererCUDA *r, sglc_handle h) : renderer(r), handle(h) {}
  int getId() const override { return handle; }
  void addDefine(const std::string &def) override;
  // ShaderProgramSoft::SetShaders(VS, FS) analogue: selects the device shader pair (SGLC_SHADING_*)
  bool setShadingModel(int shadingModel);

  RendererCUDA *renderer;
  sglc_handle handle;
};

class PipelineStatesCUDA : public PipelineStates {
 public:
  PipelineStatesCUDA(const RenderStates &states, sglc_handle h) : PipelineStates(states), handle(h) {}
  sglc_handle handle;
};

class UniformBlockCUDA : public UniformBlock {
 public:
  UniformBlockCUDA(RendererCUDA *r, const std::string &name, int size, sglc_handle h)
      : UniformBlock(name, size), renderer(r), handle(h) {}
  int getLocation(ShaderProgram &program) override { return 0; }
  void bindProgram(ShaderProgram &program, int location) override {}
  void setSubData(void *data, int len, int offset) override;
  void setData(void *data, int len) override;

  RendererCUDA *renderer;
  sglc_handle handle;
};

class UniformSamplerCUDA : public UniformSampler {
 public:
  UniformSamplerCUDA(RendererCUDA *r, const std::string &name, TextureType type, TextureFormat format, sglc_handle h)
      : UniformSampler(name, type, format), renderer(r), handle(h) {}
  int getLocation(ShaderProgram &program) override { return 0; }
  void bindProgram(ShaderProgram &program, int location) override {}
  void setTexture(const std::shared_ptr<Texture> &tex) override;

  RendererCUDA *renderer;
  sglc_handle handle;
};

class RendererCUDA : public Renderer {
 public:
  explicit RendererCUDA(int device = 0) : device_(device) {}
  ~RendererCUDA() { destroy(); }

  RendererType type() override { return Renderer_SOFT; }   // the reference enum has no CUDA entry
  bool create() override;
  void destroy() override;

  std::shared_ptr<FrameBuffer> createFrameBuffer(bool offscreen) override;
  std::shared_ptr<Texture> createTexture(const TextureDesc &desc) override;
  std::shared_ptr<VertexArrayObject> createVertexArrayObject(const VertexArray &vertexArray) override;
  std::shared_ptr<ShaderProgram> createShaderProgram() override;
  std::shared_ptr<PipelineStates> createPipelineStates(const RenderStates &renderStates) override;
  std::shared_ptr<UniformBlock> createUniformBlock(const std::string &name, int size) override;
  std::shared_ptr<UniformSampler> createUniformSampler(const std::string &name, const TextureDesc &desc) override;

  void beginRenderPass(std::shared_ptr<FrameBuffer> &frameBuffer, const ClearStates &states) override;
  void setViewPort(int x, int y, int width, int height) override;
  void setVertexArrayObject(std::shared_ptr<VertexArrayObject> &vao) override;
  void setShaderProgram(std::shared_ptr<ShaderProgram> &program) override;
  void setShaderResources(std::shared_ptr<ShaderResources> &resources) override;
  void setPipelineStates(std::shared_ptr<PipelineStates> &states) override;
  void draw() override;
  void endRenderPass() override;
  void waitIdle() override;

  // RendererSoft::setEnableEarlyZ (RendererSoft.h:53)
  void setEnableEarlyZ(bool enable);

  // logs a failed call the way the reference reports errors (LOGE + continue)
  bool check(sglc_status s, const char *what);
  sglc_context *ctx() const { return ctx_; }
  // the C-ABI handle of a ShaderResources with its current blocks and samplers (0 on failure), for
  // the batched extensions (sglc_draw_views, sglc_draw_scenes) called with the context above
  sglc_handle resourcesHandle(const std::shared_ptr<ShaderResources> &resources);

 private:
  int device_;
  sglc_context *ctx_ = nullptr;
  std::unordered_map<const ShaderResources *, sglc_handle> resources_;
};

}  // namespace SoftGL
