// Test infrastructure: drives RendererCUDA through the reference's SoftGL::Renderer interface only,
// with the calls Viewer::pipelineDraw makes (src/Viewer/Viewer.cpp:388-396) around the resource set-up
// the viewer does (textures through Buffer<RGBA> / Buffer<float>, uniform blocks, samplers, pipeline
// states; Viewer.cpp:600-690).
//
//   drive_renderer                 one vertex-colour triangle (exit code 0 once drawn)
//   drive_renderer SCENE OUTPUT    the scene file written by tests/integration/scene_file.py; after
//                                  the last pass the attachments of every pass (colour, resolved
//                                  colour where multi-sampled, depth) are read back into OUTPUT
//   drive_renderer SCENE OUTPUT multi
//                                  the same resources, every pass's first draw then drawn by one
//                                  multi-scene call (sglc_draw_scenes with the binding's handles,
//                                  pass 0's program, states and clear), as a C++ caller batches
//                                  independent scenes
//
// On a host without a GPU, create() must fail cleanly and the program reports it (exit code 3).
// Level-0 images are handed over in tiled and Morton Buffer<T> layouts, so the binding's
// linearisation (Buffer::get) is exercised as well.
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "RendererCUDA.h"

using namespace SoftGL;

namespace {

struct Reader {
  std::vector<uint8_t> b;
  size_t p = 0;
  bool ok = true;
  void get(void *out, size_t n) {
    if (p + n > b.size()) {
      ok = false;
      memset(out, 0, n);
      return;
    }
    memcpy(out, b.data() + p, n);
    p += n;
  }
  int32_t i() {
    int32_t v;
    get(&v, 4);
    return v;
  }
  int64_t q() {
    int64_t v;
    get(&v, 8);
    return v;
  }
  float f() {
    float v;
    get(&v, 4);
    return v;
  }
  std::string s() {
    int32_t n = i();
    std::string r(n > 0 ? (size_t) n : 0, '\0');
    if (n > 0) get(&r[0], (size_t) n);
    return r;
  }
  std::vector<uint8_t> blob() {
    int64_t n = q();
    std::vector<uint8_t> r(n > 0 && ok ? (size_t) n : 0);
    if (!r.empty()) get(r.data(), r.size());
    return r;
  }
};

template<typename T>
std::shared_ptr<Buffer<T>> makeBuffer(int w, int h, const std::vector<uint8_t> &img, int flavour) {
  std::shared_ptr<Buffer<T>> b;
  if (flavour == 1) b = std::make_shared<TiledBuffer<T>>();
  else if (flavour == 2) b = std::make_shared<MortonBuffer<T>>();
  else b = std::make_shared<Buffer<T>>();
  b->create(w, h);
  const T *src = reinterpret_cast<const T *>(img.data());
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) b->set(x, y, src[(size_t) y * w + x]);
  return b;
}

struct Draw {
  std::shared_ptr<VertexArrayObject> vao;
  std::shared_ptr<ShaderProgram> program;
  std::shared_ptr<ShaderResources> resources;
  std::shared_ptr<PipelineStates> states;
};

struct Pass {
  int width = 0, height = 0, samples = 1;
  ClearStates clear;
  std::shared_ptr<FrameBuffer> fbo;
  std::shared_ptr<Texture> color, depth;
  std::vector<Draw> draws;
};

int triangle(std::shared_ptr<Renderer> &renderer) {
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

int scene(std::shared_ptr<Renderer> &renderer, const char *scenePath, const char *outPath, bool multi) {
  Reader in;
  FILE *f = fopen(scenePath, "rb");
  if (!f) {
    printf("cannot open %s\n", scenePath);
    return 2;
  }
  for (int c; (c = fgetc(f)) != EOF;) in.b.push_back((uint8_t) c);
  fclose(f);
  char magic[8];
  in.get(magic, 8);
  if (memcmp(magic, "SGLSCN01", 8) != 0) {
    printf("not a scene file\n");
    return 2;
  }
  std::vector<Pass> passes(in.i());
  std::map<int, std::shared_ptr<Texture>> textures;   // shared between draws by id
  for (auto &p : passes) {
    p.width = in.i();
    p.height = in.i();
    p.samples = in.i();
    bool hasColor = in.i() != 0, hasDepth = in.i() != 0;
    p.clear.depthFlag = in.i() != 0;
    p.clear.colorFlag = in.i() != 0;
    for (int k = 0; k < 4; k++) p.clear.clearColor[k] = in.f();
    p.clear.clearDepth = in.f();
    // attachments as the viewer creates them (Viewer.cpp:56-98)
    p.fbo = renderer->createFrameBuffer(true);
    TextureDesc ad;
    ad.width = p.width;
    ad.height = p.height;
    ad.multiSample = p.samples > 1;
    if (hasColor) {
      ad.format = TextureFormat_RGBA8;
      ad.usage = TextureUsage_AttachmentColor | TextureUsage_RendererOutput;
      p.color = renderer->createTexture(ad);
      p.color->initImageData();
      p.fbo->setColorAttachment(p.color, 0);
    }
    if (hasDepth) {
      ad.format = TextureFormat_FLOAT32;
      ad.usage = TextureUsage_AttachmentDepth;
      p.depth = renderer->createTexture(ad);
      p.depth->initImageData();
      p.fbo->setDepthAttachment(p.depth);
    }
    p.draws.resize(in.i());
    for (auto &d : p.draws) {
      int32_t stride = in.i();
      std::vector<uint8_t> vertexes = in.blob();
      int64_t nIdx = in.q();
      std::vector<int32_t> indices(nIdx > 0 && in.ok ? (size_t) nIdx : 0);
      if (!indices.empty()) in.get(indices.data(), indices.size() * 4);
      VertexArray va;
      va.vertexSize = stride;
      va.vertexesDesc.push_back({(size_t) stride / 4, (size_t) stride, 0});
      va.vertexesBuffer = vertexes.data();
      va.vertexesBufferLength = vertexes.size();
      va.indexBuffer = indices.data();
      va.indexBufferLength = indices.size() * sizeof(int32_t);
      d.vao = renderer->createVertexArrayObject(va);

      int32_t shading = in.i();
      d.program = renderer->createShaderProgram();
      for (int n = in.i(); n > 0; n--) d.program->addDefine(in.s());
      std::dynamic_pointer_cast<ShaderProgramCUDA>(d.program)->setShadingModel(shading);

      RenderStates rs;
      rs.blend = in.i() != 0;
      rs.blendParams.blendFuncRgb = (BlendFunction) in.i();
      rs.blendParams.blendSrcRgb = (BlendFactor) in.i();
      rs.blendParams.blendDstRgb = (BlendFactor) in.i();
      rs.blendParams.blendFuncAlpha = (BlendFunction) in.i();
      rs.blendParams.blendSrcAlpha = (BlendFactor) in.i();
      rs.blendParams.blendDstAlpha = (BlendFactor) in.i();
      rs.depthTest = in.i() != 0;
      rs.depthMask = in.i() != 0;
      rs.depthFunc = (DepthFunction) in.i();
      rs.cullFace = in.i() != 0;
      rs.primitiveType = (PrimitiveType) in.i();
      rs.polygonMode = (PolygonMode) in.i();
      rs.lineWidth = in.f();
      d.states = renderer->createPipelineStates(rs);

      d.resources = std::make_shared<ShaderResources>();
      for (int n = in.i(); n > 0; n--) {
        std::string name = in.s();
        int32_t key = in.i();
        std::vector<uint8_t> data = in.blob();
        auto ub = renderer->createUniformBlock(name, (int) data.size());
        ub->setData(data.data(), (int) data.size());
        d.resources->blocks[key] = ub;
      }
      int nTex = in.i();
      for (int k = 0; k < nTex && in.ok; k++) {
        int32_t id = in.i();
        std::string name = in.s();
        TextureDesc td;
        td.width = in.i();
        td.height = in.i();
        td.type = (TextureType) in.i();
        td.format = (TextureFormat) in.i();
        td.usage = (uint32_t) in.i();
        td.useMipmaps = in.i() != 0;
        td.multiSample = in.i() != 0;
        SamplerDesc sd;
        sd.filterMin = (FilterMode) in.i();
        sd.filterMag = (FilterMode) in.i();
        sd.wrapS = (WrapMode) in.i();
        sd.wrapT = (WrapMode) in.i();
        sd.wrapR = (WrapMode) in.i();
        sd.borderColor = (BorderColor) in.i();
        int32_t source = in.i();
        std::shared_ptr<Texture> &tex = textures[id];
        bool fresh = !tex;
        if (fresh) {
          tex = renderer->createTexture(td);
          tex->setSamplerDesc(sd);
        }
        if (source == 1) {   // explicit [level][layer] images
          int32_t levels = in.i(), layers = in.i();
          if (fresh) tex->initImageData();
          for (int lev = 0; lev < levels; lev++)
            for (int layer = 0; layer < layers; layer++) {
              std::vector<uint8_t> img = in.blob();
              if (fresh)
                std::dynamic_pointer_cast<TextureCUDA>(tex)->setLevelData(layer, lev, img.data(), img.size());
            }
        } else {             // level-0 image per layer; mip levels generated
          int32_t layers = in.i();
          std::vector<std::shared_ptr<Buffer<RGBA>>> rgba;
          std::vector<std::shared_ptr<Buffer<float>>> fl;
          for (int layer = 0; layer < layers; layer++) {
            std::vector<uint8_t> img = in.blob();
            int flavour = (id + layer) % 3;   // linear, tiled 4x4, Morton 32x32
            if (td.format == TextureFormat_RGBA8) rgba.push_back(makeBuffer<RGBA>(td.width, td.height, img, flavour));
            else fl.push_back(makeBuffer<float>(td.width, td.height, img, flavour));
          }
          if (fresh) {
            if (td.format == TextureFormat_RGBA8) tex->setImageData(rgba);
            else tex->setImageData(fl);
          }
        }
        auto us = renderer->createUniformSampler(name, td);
        us->setTexture(tex);
        d.resources->samplers[k] = us;
      }
    }
  }
  if (!in.ok) {
    printf("truncated scene file\n");
    return 2;
  }

  if (multi) {
    // one multi-scene draw over every pass's first draw (the passes share a shading model)
    auto cuda = std::dynamic_pointer_cast<RendererCUDA>(renderer);
    for (auto &p : passes)
      if (p.draws.empty()) {
        printf("multi: a pass without draws\n");
        return 2;
      }
    if (!cuda || passes.empty()) {
      printf("multi: needs a RendererCUDA and at least one pass\n");
      return 2;
    }
    std::vector<sglc_handle> vaos, fbos, res;
    for (auto &p : passes) {
      vaos.push_back(p.draws[0].vao->getId());
      fbos.push_back(p.fbo->getId());
      res.push_back(cuda->resourcesHandle(p.draws[0].resources));
    }
    renderer->setShaderProgram(passes[0].draws[0].program);
    renderer->setPipelineStates(passes[0].draws[0].states);
    const ClearStates &c = passes[0].clear;
    sglc_clear_states cs{c.depthFlag, c.colorFlag, {c.clearColor.r, c.clearColor.g, c.clearColor.b, c.clearColor.a},
                         c.clearDepth};
    if (!cuda->check(sglc_draw_scenes(cuda->ctx(), vaos.data(), fbos.data(), res.data(), (int32_t) passes.size(), &cs),
                     "drawScenes"))
      return 1;
  } else {
    // the frame: Viewer::drawFrame / pipelineDraw call order
    for (auto &p : passes) {
      renderer->beginRenderPass(p.fbo, p.clear);
      renderer->setViewPort(0, 0, p.width, p.height);
      for (auto &d : p.draws) {
        renderer->setVertexArrayObject(d.vao);
        renderer->setShaderProgram(d.program);
        renderer->setShaderResources(d.resources);
        renderer->setPipelineStates(d.states);
        renderer->draw();
      }
      renderer->endRenderPass();
    }
  }
  renderer->waitIdle();

  FILE *o = fopen(outPath, "wb");
  if (!o) return 2;
  bool ok = true;
  auto dump = [&](std::shared_ptr<Texture> &t, size_t bytes, bool resolved) {
    std::vector<uint8_t> px(bytes);
    ok = std::dynamic_pointer_cast<TextureCUDA>(t)->readImage(px.data(), bytes, 0, 0, resolved) && ok;
    fwrite(px.data(), 1, bytes, o);
  };
  for (auto &p : passes) {
    size_t pixels = (size_t) p.width * p.height;
    if (p.color) {
      dump(p.color, pixels * 4 * p.samples, false);
      if (p.samples > 1) dump(p.color, pixels * 4, true);
    }
    if (p.depth) dump(p.depth, pixels * 4 * p.samples, false);
  }
  fclose(o);
  printf(ok ? "rendered\n" : "read-back failed\n");
  return ok ? 0 : 1;
}

}  // namespace

int main(int argc, char **argv) {
  std::shared_ptr<Renderer> renderer = std::make_shared<RendererCUDA>(0);
  if (!renderer->create()) {
    printf("no device\n");
    return 3;
  }
  if (argc >= 3) return scene(renderer, argv[1], argv[2], argc >= 4 && strcmp(argv[3], "multi") == 0);
  return triangle(renderer);
}
