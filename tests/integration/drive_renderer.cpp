// Drives RendererCUDA through the reference's SoftGL::Renderer interface only (the calls
// Viewer::pipelineDraw makes, src/Viewer/Viewer.cpp:388-396). Exit code 0 when the sequence runs;
// on a host without a GPU, create() must fail cleanly and the program reports it (exit code 3).
#include <cstdio>
#include <memory>

#include "RendererCUDA.h"

using namespace SoftGL;

int main() {
  std::shared_ptr<Renderer> renderer = std::make_shared<RendererCUDA>(0);
  if (!renderer->create()) {
    printf("no device\n");
    return 3;
  }
  TextureDesc cd;
  cd.width = 64;
  cd.height = 48;
  cd.format = TextureFormat_RGBA8;
  cd.usage = TextureUsage_AttachmentColor;
  auto color = renderer->createTexture(cd);
  color->initImageData();
  TextureDesc dd = cd;
  dd.format = TextureFormat_FLOAT32;
  dd.usage = TextureUsage_AttachmentDepth;
  auto depth = renderer->createTexture(dd);
  depth->initImageData();
  auto fbo = renderer->createFrameBuffer(true);
  fbo->setColorAttachment(color, 0);
  fbo->setDepthAttachment(depth);
  float verts[3][8] = {{-0.5f, -0.5f, 0.f, 0.f, 1.f, 0.f, 0.f, 1.f},
                       {0.5f, -0.5f, 0.f, 0.f, 0.f, 1.f, 0.f, 1.f},
                       {0.f, 0.5f, 0.f, 0.f, 0.f, 0.f, 1.f, 1.f}};
  int32_t idx[3] = {0, 1, 2};
  VertexArray va;
  va.vertexSize = 32;
  va.vertexesDesc.push_back({8, 32, 0});
  va.vertexesBuffer = reinterpret_cast<uint8_t *>(verts);
  va.vertexesBufferLength = sizeof(verts);
  va.indexBuffer = idx;
  va.indexBufferLength = sizeof(idx);
  auto vao = renderer->createVertexArrayObject(va);
  auto program = renderer->createShaderProgram();
  std::dynamic_pointer_cast<ShaderProgramCUDA>(program)->setShadingModel(SGLC_SHADING_VERTEX_COLOR);
  float model[64] = {0};
  for (int i = 0; i < 4; i++) model[4 + i * 4 + i] = model[20 + i * 4 + i] = 1.f;   // identity model and MVP
  auto ubModel = renderer->createUniformBlock("UniformsModel", 256);
  ubModel->setData(model, 256);
  auto resources = std::make_shared<ShaderResources>();
  resources->blocks[1] = ubModel;
  RenderStates rs;
  rs.depthTest = true;
  auto states = renderer->createPipelineStates(rs);
  ClearStates cs;
  cs.colorFlag = cs.depthFlag = true;
  renderer->beginRenderPass(fbo, cs);
  renderer->setViewPort(0, 0, 64, 48);
  renderer->setVertexArrayObject(vao);
  renderer->setShaderProgram(program);
  renderer->setShaderResources(resources);
  renderer->setPipelineStates(states);
  renderer->draw();
  renderer->endRenderPass();
  renderer->waitIdle();
  printf("drawn\n");
  return 0;
}
