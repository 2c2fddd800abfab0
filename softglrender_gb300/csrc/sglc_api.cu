// C ABI of include/softgl_cuda.h: resources, render-state binding and draw orchestration of the
// sm_103a renderer. Mirrors SoftGL::RendererSoft (src/Render/Software/RendererSoft.cpp) call by
// call: resource objects are handle-table entries backed by device memory; uniform blocks are
// copied into the program at setShaderResources time and samplers are bound by reference
// (ShaderProgram::bindResources, src/Render/ShaderProgram.h:27-54; UniformSoft.h:26-29,79-82);
// draw() enqueues the geometry, binning and raster kernels on the context's stream.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "softgl_cuda.h"
#include "sglc_device.cuh"
#include "sglc_kernels.h"
#include "sglc_host_util.h"
#include "sglc_nn_host.h"

using namespace sglc;

namespace {

struct UniformDescEntry {
  const char *name;
  int offset;
  int samplerSlot;
};

struct ShaderInfo {
  int model;
  std::vector<const char *> defines;
  std::vector<UniformDescEntry> uniforms;
  int uniformSize;
  int varyingsCnt;
  int derivSlots;   // sampler slots whose LOD callback the FS installs (setupSamplerDerivative)
};

// uniform / varying layouts of the reference shaders with GLM aligned types
// (BasicSoft.h:24-42, BlinnPhongSoft.h:110-150, PbrSoft.h:29-72)
const ShaderInfo kShaders[] = {
    {SH_BASE, {}, {{"UniformsModel", 0, -1}, {"UniformsMaterial", 256, -1}}, 304, 0, 0},
    {SH_BLINN, {"ALBEDO_MAP", "NORMAL_MAP", "EMISSIVE_MAP", "AO_MAP"},
     {{"UniformsModel", 0, -1}, {"UniformsScene", 256, -1}, {"UniformsMaterial", 320, -1}, {"u_albedoMap", 368, 0},
      {"u_normalMap", 376, 1}, {"u_emissiveMap", 384, 2}, {"u_aoMap", 392, 3}, {"u_shadowMap", 400, 4}}, 416, 32, 0xF},
    {SH_PBR, {"ALBEDO_MAP", "NORMAL_MAP", "EMISSIVE_MAP", "AO_MAP", "METALROUGHNESS_MAP"},
     {{"UniformsModel", 0, -1}, {"UniformsScene", 256, -1}, {"UniformsMaterial", 320, -1}, {"u_albedoMap", 368, 0},
      {"u_normalMap", 376, 1}, {"u_emissiveMap", 384, 2}, {"u_aoMap", 392, 3}, {"u_metalRoughnessMap", 400, 4},
      {"u_irradianceMap", 408, 5}, {"u_prefilterMap", 416, 6}}, 432, 28, 0xF},
    // SkyboxSoft.h:24-61, IBLIrradianceSoft.h:24-56, IBLPrefilterSoft.h:24-61: UniformsModel, then
    // UniformsPrefilter (u_srcResolution, u_roughness), then the sampler pointers; varyings: v_worldPos
    {SH_SKYBOX, {"EQUIRECTANGULAR_MAP"},
     {{"UniformsModel", 0, -1}, {"u_equirectangularMap", 256, 0}, {"u_cubeMap", 264, 1}}, 272, 4, 0},
    {SH_IBL_IRR, {}, {{"UniformsModel", 0, -1}, {"u_cubeMap", 256, 0}}, 264, 4, 0},
    {SH_IBL_PRE, {}, {{"UniformsModel", 0, -1}, {"UniformsPrefilter", 256, -1}, {"u_cubeMap", 264, 0}}, 272, 4, 0},
    // FxaaSoft.h:24-53: UniformsQuadFilter (vec2 u_screenSize), the screen texture; varyings: v_texCoord
    {SH_FXAA, {}, {{"UniformsQuadFilter", 0, -1}, {"u_screenTexture", 8, 0}}, 16, 2, 0},
    {SH_BLINN_DIR, {"ALBEDO_MAP", "NORMAL_MAP", "EMISSIVE_MAP", "AO_MAP"},
     {{"UniformsModel", 0, -1}, {"UniformsScene", 256, -1}, {"UniformsMaterial", 320, -1}, {"u_albedoMap", 368, 0},
      {"u_normalMap", 376, 1}, {"u_emissiveMap", 384, 2}, {"u_aoMap", 392, 3}, {"u_shadowMap", 400, 4}}, 416, 32, 0xF},
    {SH_VCOLOR, {}, {{"UniformsModel", 0, -1}, {"UniformsMaterial", 256, -1}}, 304, 4, 0},
};

const ShaderInfo *findShader(int model) {
  for (auto &s : kShaders)
    if (s.model == model) return &s;
  return nullptr;
}

enum Kind { K_FB = 1, K_TEX, K_VAO, K_PROG, K_STATES, K_UB, K_US, K_RES };

struct TexObj {
  sglc_texture_desc desc{};
  sglc_sampler_desc sampler{0, 0, 2, 2, 2, 0};
  int layers = 1;
  int levels = 0;
  int samplesPerTexel = 1;
  bool allocated = false;
  uint32_t *dev = nullptr;
  size_t layerStride = 0;   // elements
  uint32_t offset[kMaxLevels] = {0};
  int w[kMaxLevels] = {0}, h[kMaxLevels] = {0}, tilesW[kMaxLevels] = {0};
  uint32_t *resolved = nullptr;   // multi-sample RGBA8 colour: resolved image
  bool resolvedValid = false;
  unsigned long long version = 0;   // bumped by every write of the texture's memory
  struct HwCopy *hw = nullptr;      // hardware-sampled copy for the neural shading path
};

// A 2D RGBA8 texture copied into a CUDA mipmapped array for the texture units, with one texture
// object per sampler state that uses it. Rebuilt when the texture's version moves on. Used only by
// the neural shading path (judged by PSNR); the exact shaders sample the texture's own memory.
struct HwCopy {
  cudaMipmappedArray_t arr = nullptr;
  int w = 0, h = 0, levels = 0;
  unsigned long long version = ~0ull;
  struct View {
    int filter, wrap;
    uint32_t border;
    cudaTextureObject_t obj;
  };
  std::vector<View> views;
  void release() {
    for (View &v : views) cudaDestroyTextureObject(v.obj);
    views.clear();
    if (arr) cudaFreeMipmappedArray(arr);
    arr = nullptr;
    version = ~0ull;
  }
};

struct FbObj {
  int colorTex = 0, colorLayer = 0, colorLevel = 0, depthTex = 0;
  bool colorReady = false, depthReady = false;
};

struct VaoObj {
  float *attr = nullptr;
  int32_t *idx = nullptr;
  size_t stride = 0, nv = 0, nidx = 0;
};

struct ProgObj {
  std::vector<std::string> defineNames;
  const ShaderInfo *shader = nullptr;
  uint8_t defines[8] = {0};
  uint8_t uniforms[kUniformBytes] = {0};
  int samplers[kMaxSamplers] = {0};
  const sglc_neural *neural = nullptr;   // bound neural IBL shader (PBR programs only)
};

struct UsObj {
  std::string name;
  int type = 0, format = 0, tex = 0;
  int filter = 1, wrap = 2;
  uint32_t border = 0;
  int width = 0, height = 0;
  bool useMipmaps = false;
};

struct Object {
  int kind = 0;
  FbObj fb;
  TexObj tex;
  VaoObj vao;
  ProgObj prog;
  sglc_render_states states{};
  std::string ubName;
  std::vector<uint8_t> ubData;
  UsObj us;
  std::map<int, int> resBlocks, resSamplers;
};

// Counts of device frees: a CUDA graph records device addresses, so a graph captured before any
// buffer it uses was freed (a working array grown, a resource released) must not be replayed;
// sglc_graph_launch compares the counts with the capture's. Each context counts the frees of its
// own buffers and resources (a graph uses only its context's), so renderers that grow or release
// memory do not invalidate other renderers' graphs; g_freeEpoch counts frees owned by no context.
std::atomic<unsigned long long> g_freeEpoch{0};

// grow-only device buffer
struct DevBuf {
  void *ptr = nullptr;
  size_t bytes = 0;
  std::atomic<unsigned long long> *epoch = nullptr;   // the owning context's free count
  static thread_local bool capturing;   // a graph capture is in progress on this thread
  void countFree() {
    if (epoch) (*epoch)++;
    else g_freeEpoch++;
  }
  cudaError_t ensure(size_t need) {
    if (need <= bytes) return cudaSuccess;
    if (capturing) return cudaErrorStreamCaptureUnsupported;   // run the sequence once before capturing
    if (ptr) {
      cudaFree(ptr);
      countFree();
    }
    ptr = nullptr;
    bytes = 0;
    size_t n = std::max(need, (size_t) 256);
    n = n + n / 4;
    cudaError_t e = cudaMalloc(&ptr, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (ptr) {
      cudaFree(ptr);
      countFree();
    }
    ptr = nullptr;
    bytes = 0;
  }
  template<typename T>
  T *as() const { return reinterpret_cast<T *>(ptr); }
};

thread_local bool DevBuf::capturing = false;

struct PendingClear {
  int fb = 0;
  bool active = false;
  int colorFlag = 0, depthFlag = 0;
  uint32_t color = 0;
  float depth = 1.f;
};

struct Ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::map<int, Object> objects;
  int next = 1;
  std::string err;
  bool earlyZ = true;
  int tile = 16;
  int tileH = 16;                    // sglc_set_tile_size: height of the deferred raster's tiles
  Viewport vp{};
  int fb = 0, vao = 0, prog = 0, states = 0;
  PendingClear clear;
  sglc_draw_stats stats{};
  int *hostCounters = nullptr;   // pinned
  int statsLevel = 0;
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  bool evDeferred = false;   // ev[4], ev[5] bracket the deferred-shading kernels of the last draw
  bool evPending = false;
  unsigned long long *fragCounter = nullptr;
  // scratch
  DevBuf vClip, vFrag, vMask, vVary, vAttrExtra, prims, clipExtra, clipAppendOff, clipPoly, clipPolyTri, counters;
  DevBuf tri, tileCount, pairOff, keyA, keyB, valA, valB, tileStart, tileEnd, tileOrder, scanScratch, sortHist,
      sortHistScan, staging, batchU, batchTargets, batchScenes;
  DevBuf recA, recB, recColor, chunkNext, chunkFill, warpHead, recDense;   // deferred shading
  DevBuf nnIn;   // neural shading: per record the surface stage's five float4 (blocks of 32 records)
  DevBuf peakChunks;   // largest number of fragment-record chunks a deferred draw used (device)
  bool deferredShading = true;
  bool tmaStore = true;              // sglc_set_tma_store
  int nnTestFlags = 0;               // sglc_neural_set_test_flags
  DevBuf lpSlot, lpOrigin, lpStampCount, lpStampOff, lpStampGeo, lpStampRow, lpStampColor, lpStampVary, lpFragCount,
      lpFragOff, lpMisc;   // point and line draws
  // capacity hints that survive between draws
  int extraVertHint = 0, polyHint = 0, appendHint = 0;
  // synchronisation-free draws (sglc_set_capacity) and graph capture
  bool capSet = false;
  sglc_capacity cap{};
  sglc_capacity peak{};              // largest counts of exactly sized draws since the last query
  DevBuf sticky;                     // overflow flags accumulated over draws
  bool capturing = false;
  unsigned long long captureEpoch = 0, captureCtxEpoch = 0;
  std::atomic<unsigned long long> freeEpoch{0};   // frees of this context's buffers and resources
  // every working array of the context
  template<typename F>
  void forEachBuf(F f) {
    DevBuf *bufs[] = {&vClip, &vFrag, &vMask, &vVary, &vAttrExtra, &prims, &clipExtra, &clipAppendOff, &clipPoly,
                      &clipPolyTri, &counters, &tri, &tileCount, &pairOff, &keyA, &keyB, &valA, &valB, &tileStart,
                      &tileEnd, &tileOrder, &scanScratch, &sortHist, &sortHistScan, &staging, &batchU, &batchTargets, &batchScenes,
                      &sticky, &lpSlot, &lpOrigin, &lpStampCount, &lpStampOff, &lpStampGeo, &lpStampRow,
                      &lpStampColor, &lpStampVary, &lpFragCount, &lpFragOff, &lpMisc, &recA, &recB, &recColor,
                      &chunkNext, &chunkFill, &warpHead, &recDense, &peakChunks, &nnIn};
    for (DevBuf *b : bufs) f(*b);
  }
  std::vector<void *> captureHostBufs;   // pinned host sources of memcpy nodes in the capture
  // neural IBL shader: training-record capture target
  float *capRecords = nullptr;
  unsigned long long *capCount = nullptr;
  long long capCap = 0;
  int capStride = 1;

  Object *get(int h, int kind) {
    auto it = objects.find(h);
    if (it == objects.end() || it->second.kind != kind) return nullptr;
    return &it->second;
  }
  sglc_status fail(sglc_status s, const std::string &msg) {
    err = msg;
    return s;
  }
};

// every entry point over a context runs with the context's device current (restored on return)
#define CTX                                    \
  if (!ctx) return SGLC_ERR_INVALID_HANDLE;    \
  Ctx *c = reinterpret_cast<Ctx *>(ctx);       \
  sglc::DeviceGuard deviceGuard_(c->device)
#define GET(var, h, kind)                                                     \
  Object *var = c->get(h, kind);                                              \
  if (!var) return c->fail(SGLC_ERR_INVALID_HANDLE, "invalid handle");
#define CK(call)                                                                                    \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess)                                                                          \
      return c->fail(e_ == cudaErrorMemoryAllocation ? SGLC_ERR_OUT_OF_MEMORY : SGLC_ERR_DEVICE,    \
                     std::string(#call) + ": " + cudaGetErrorString(e_));                           \
  } while (0)

static inline uint32_t u8c(float f) { return (uint32_t) ((int) f) & 255u; }

int addObject(Ctx *c, int kind) {
  int h = c->next++;
  c->objects[h].kind = kind;
  return h;
}

int levelCount(int w, int h) { return (int) std::floor(std::log2((double) std::max(w, h))) + 1; }

// storage geometry of a texture (Buffer::initLayout for the three layouts, Buffer.h:28-31,140-213)
void planLevels(TexObj &t) {
  bool attachment = (t.desc.usage & (4u | 8u)) != 0;   // AttachmentColor | AttachmentDepth
  if (attachment || t.desc.multi_sample) t.desc.layout = LAYOUT_LINEAR;
  t.samplesPerTexel = t.desc.multi_sample ? 4 : 1;
  t.levels = (t.desc.use_mipmaps && !t.desc.multi_sample) ? std::min(levelCount(t.desc.width, t.desc.height), kMaxLevels) : 1;
  size_t off = 0;
  for (int l = 0; l < t.levels; l++) {
    int w = std::max(1, t.desc.width >> l), h = std::max(1, t.desc.height >> l);
    t.w[l] = w;
    t.h[l] = h;
    size_t n;
    if (t.desc.layout == LAYOUT_TILED) {
      t.tilesW[l] = (w + 3) / 4;
      n = (size_t) t.tilesW[l] * 4 * ((h + 3) / 4) * 4;
    } else if (t.desc.layout == LAYOUT_MORTON) {
      t.tilesW[l] = (w + 31) / 32;
      n = (size_t) t.tilesW[l] * 32 * ((h + 31) / 32) * 32;
    } else {
      t.tilesW[l] = 0;
      n = (size_t) w * h;
    }
    t.offset[l] = (uint32_t) off;
    off += ((n * t.samplesPerTexel) + 3) & ~(size_t) 3;
  }
  t.layerStride = off;
}

DevTex devTex(const TexObj &t) {
  DevTex d{};
  d.base = t.dev;
  d.layerStride = (uint32_t) t.layerStride;
  d.levels = t.allocated ? t.levels : 0;
  d.layout = t.desc.layout;
  for (int l = 0; l < t.levels && l < kMaxLevels; l++) {
    d.offset[l] = t.offset[l];
    d.w[l] = (uint16_t) t.w[l];
    d.h[l] = (uint16_t) t.h[l];
    d.tilesW[l] = (uint16_t) t.tilesW[l];
  }
  return d;
}

sglc_status allocTexture(Ctx *c, TexObj &t) {
  if (t.allocated) return SGLC_OK;
  planLevels(t);
  size_t bytes = t.layerStride * t.layers * sizeof(uint32_t);
  CK(cudaMalloc(&t.dev, bytes));
  CK(cudaMemsetAsync(t.dev, 0, bytes, c->stream));
  if (t.desc.multi_sample && t.desc.format == SGLC_FORMAT_RGBA8) {
    CK(cudaMalloc(&t.resolved, (size_t) t.desc.width * t.desc.height * 4));
    CK(cudaMemsetAsync(t.resolved, 0, (size_t) t.desc.width * t.desc.height * 4, c->stream));
  }
  t.allocated = true;
  t.version++;
  return SGLC_OK;
}

void freeTexture(TexObj &t, std::atomic<unsigned long long> &epoch) {
  if (t.dev || t.resolved || t.hw) epoch++;
  if (t.hw) {
    t.hw->release();
    delete t.hw;
    t.hw = nullptr;
  }
  if (t.dev) cudaFree(t.dev);
  if (t.resolved) cudaFree(t.resolved);
  t.dev = nullptr;
  t.resolved = nullptr;
  t.allocated = false;
}

// upload one linear level into the texture's layout
sglc_status uploadLevel(Ctx *c, TexObj &t, int layer, int level, const void *data) {
  t.version++;
  size_t n = (size_t) t.w[level] * t.h[level];
  uint32_t *dst = t.dev + (size_t) layer * t.layerStride + t.offset[level];
  if (t.desc.layout == LAYOUT_LINEAR) {
    CK(cudaMemcpyAsync(dst, data, n * 4, cudaMemcpyHostToDevice, c->stream));
    return SGLC_OK;
  }
  CK(c->staging.ensure(n * 4));
  CK(cudaMemcpyAsync(c->staging.ptr, data, n * 4, cudaMemcpyHostToDevice, c->stream));
  launchSwizzleIn(devTex(t), layer, level, c->staging.as<uint32_t>(), c->stream);
  CK(cudaGetLastError());
  // the staging buffer is reused by the next upload: keep uploads ordered on the stream and make
  // sure the host source can be released by the caller
  CK(cudaStreamSynchronize(c->stream));
  return SGLC_OK;
}

// materialise a pending clear (RendererSoft::beginRenderPass, RendererSoft.cpp:61-90)
// The texture-unit view of a 2D RGBA8 texture for one sampler state (0 when the texture cannot be
// sampled by the hardware: another format, multi-sample, a cube map). Builds or refreshes the
// mipmapped copy when the texture changed since it was made (one device-to-array copy per level,
// on the context's stream; Tiled and Morton levels are first swizzled to linear in the staging
// buffer). Never called during a graph capture that could need a rebuild: the autotuner's capture
// follows eager frames, and draws do not write their material textures.
sglc_status hwTexture(Ctx *c, TexObj &t, const UsObj &us, cudaTextureObject_t *out) {
  *out = 0;
  if (!t.allocated || t.desc.format != SGLC_FORMAT_RGBA8 || t.desc.multi_sample || t.desc.type != SGLC_TEXTURE_2D)
    return SGLC_OK;
  if (!t.hw) t.hw = new HwCopy();
  HwCopy &h = *t.hw;
  if (h.version != t.version) {
    if (c->capturing) return c->fail(SGLC_ERR_UNSUPPORTED, "draw: a neural draw's texture changed inside a capture");
    if (!h.views.empty() || h.arr) c->freeEpoch++;   // graphs that baked the old copy in are stale
    for (HwCopy::View &v : h.views) cudaDestroyTextureObject(v.obj);
    h.views.clear();
    if (h.arr && (h.w != t.w[0] || h.h != t.h[0] || h.levels != t.levels)) {
      cudaFreeMipmappedArray(h.arr);
      h.arr = nullptr;
    }
    if (!h.arr) {
      cudaChannelFormatDesc cd = cudaCreateChannelDesc<uchar4>();
      CK(cudaMallocMipmappedArray(&h.arr, &cd, make_cudaExtent(t.w[0], t.h[0], 0), t.levels));
      h.w = t.w[0];
      h.h = t.h[0];
      h.levels = t.levels;
    }
    for (int l = 0; l < t.levels; l++) {
      cudaArray_t la = nullptr;
      CK(cudaGetMipmappedArrayLevel(&la, h.arr, l));
      const size_t n = (size_t) t.w[l] * t.h[l];
      const uint32_t *src = t.dev + t.offset[l];
      if (t.desc.layout != LAYOUT_LINEAR) {
        CK(c->staging.ensure(n * 4));
        launchSwizzleOut(devTex(t), 0, l, c->staging.as<uint32_t>(), c->stream);
        CK(cudaGetLastError());
        src = c->staging.as<uint32_t>();
      }
      CK(cudaMemcpy2DToArrayAsync(la, 0, 0, src, (size_t) t.w[l] * 4, (size_t) t.w[l] * 4, t.h[l],
                                  cudaMemcpyDeviceToDevice, c->stream));
    }
    h.version = t.version;
  }
  for (const HwCopy::View &v : h.views)
    if (v.filter == us.filter && v.wrap == us.wrap && v.border == us.border) {
      *out = v.obj;
      return SGLC_OK;
    }
  cudaResourceDesc rd{};
  rd.resType = cudaResourceTypeMipmappedArray;
  rd.res.mipmap.mipmap = h.arr;
  cudaTextureDesc td{};
  const cudaTextureAddressMode am = us.wrap == WRAP_REPEAT ? cudaAddressModeWrap
                                    : us.wrap == WRAP_MIRRORED ? cudaAddressModeMirror
                                    : us.wrap == WRAP_EDGE     ? cudaAddressModeClamp
                                                               : cudaAddressModeBorder;
  td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = am;
  const float bc = us.border ? 1.f : 0.f;   // BorderColor: black or white, alpha as the colour
  td.borderColor[0] = td.borderColor[1] = td.borderColor[2] = td.borderColor[3] = bc;
  td.filterMode = (us.filter & 1) ? cudaFilterModeLinear : cudaFilterModePoint;
  td.mipmapFilterMode = us.filter >= FILTER_NL ? cudaFilterModeLinear : cudaFilterModePoint;
  td.readMode = cudaReadModeNormalizedFloat;
  td.normalizedCoords = 1;
  td.minMipmapLevelClamp = 0.f;
  td.maxMipmapLevelClamp = (us.filter >= FILTER_NN && us.useMipmaps) ? (float) (t.levels - 1) : 0.f;
  td.maxAnisotropy = 1;
  cudaTextureObject_t obj = 0;
  CK(cudaCreateTextureObject(&obj, &rd, &td, nullptr));
  h.views.push_back({us.filter, us.wrap, us.border, obj});
  *out = obj;
  return SGLC_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against the driver)
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encodeTiledFn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
    cudaGetLastError();
  });
  return fn;
}

// A linear attachment of h rows of w pixels with spp 32-bit samples each, as a 2D tensor map
// (inner dimension w * spp) with a box of one raster tile (16 x boxH pixels). False where TMA cannot address it: a base
// that is not 16-byte aligned or a row that is not a multiple of 16 bytes (then the kernels store
// per thread).
bool encodeAttachment(CUtensorMap *m, void *base, int w, int h, int spp, int boxH) {
  EncodeTiledFn fn = encodeTiledFn();
  if (!fn || !base || ((uintptr_t) base & 15) || ((size_t) w * spp * 4) % 16 || w <= 0 || h <= 0) return false;
  const cuuint64_t dims[2] = {(cuuint64_t) w * spp, (cuuint64_t) h};
  const cuuint64_t strides[1] = {(cuuint64_t) w * spp * 4};
  const cuuint32_t box[2] = {(cuuint32_t) (16 * spp), (cuuint32_t) boxH};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_NONE,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

sglc_status flushClear(Ctx *c) {
  if (!c->clear.active) return SGLC_OK;
  c->clear.active = false;
  Object *f = c->get(c->clear.fb, K_FB);
  if (!f) return SGLC_OK;
  if (c->clear.colorFlag && f->fb.colorReady) {
    Object *t = c->get(f->fb.colorTex, K_TEX);
    if (t && t->tex.allocated && f->fb.colorLevel < t->tex.levels) {
      TexObj &T = t->tex;
      T.version++;
      size_t n = (size_t) T.w[f->fb.colorLevel] * T.h[f->fb.colorLevel] * T.samplesPerTexel;
      launchFill32(T.dev + (size_t) f->fb.colorLayer * T.layerStride + T.offset[f->fb.colorLevel], c->clear.color, n,
                   c->stream);
    }
  }
  if (c->clear.depthFlag && f->fb.depthReady) {
    Object *t = c->get(f->fb.depthTex, K_TEX);
    if (t && t->tex.allocated) {
      TexObj &T = t->tex;
      T.version++;
      uint32_t bits;
      memcpy(&bits, &c->clear.depth, 4);
      launchFill32(T.dev, bits, (size_t) T.w[0] * T.h[0] * T.samplesPerTexel, c->stream);
    }
  }
  CK(cudaGetLastError());
  return SGLC_OK;
}

TexObj *attachmentTex(Ctx *c, int h) {
  Object *o = c->get(h, K_TEX);
  return o ? &o->tex : nullptr;
}

// A batched draw (sglc_draw_views): per-view framebuffers and uniform bytes, one clear for all.
struct BatchViews {
  int count = 0;
  const sglc_handle *vaos = nullptr;   // non-null: a multi-scene draw (sglc_draw_scenes), one per view
  const sglc_handle *fbs = nullptr;
  std::vector<uint8_t> uniforms;   // count x kUniformBytes
  const sglc_clear_states *clear = nullptr;
};

// Point and line draws (RendererSoft.cpp:301-321, 409-487, 575-712; kernels in sglc_lines.cu).
// The stamp and fragment counts are read back (two synchronisations per draw), so these draws are
// not captured in graphs.
sglc_status drawPointsLines(Ctx *c, DrawParams &p, const sglc_render_states &rs, const VaoObj &vao, TexObj *ct,
                            TexObj *dt) {
  if (c->capturing) return c->fail(SGLC_ERR_UNSUPPORTED, "draw: point and line draws cannot be captured in a graph");
  // points and lines run the FS outside a pixel quad: the reference has no derivative context
  // there, so a derivative-LOD sampler in use has nothing to read
  if (p.needDeriv)
    return c->fail(SGLC_ERR_UNSUPPORTED, "draw: points/lines with a derivative-LOD (mipmapped 2D) sampler");
  sglc_status st0 = flushClear(c);
  if (st0) return st0;
  c->stats = sglc_draw_stats{};
  if (!ct) return SGLC_OK;   // rasterizationPoint draws nothing without a colour attachment (:637-639)
  const cudaStream_t st = c->stream;
  LineParams lp;
  memset(&lp, 0, sizeof(lp));
  int per = 3;
  if (rs.primitive_type == SGLC_PRIMITIVE_POINT) {
    lp.mode = LP_POINTS;
    per = 1;
  } else if (rs.primitive_type == SGLC_PRIMITIVE_LINE) {
    lp.mode = LP_LINES;
    per = 2;
  } else {
    lp.mode = rs.polygon_mode == SGLC_POLYGON_POINT ? LP_TRI_POINTS : LP_TRI_LINES;
  }
  const long long nIn = (long long) vao.nidx / per;
  // PointSize is written by the base-colour VS only (BasicSoft.h:66-69); ShaderBuiltin's default is 1
  lp.pointSize = 1.f;
  if (p.shading == SH_BASE) memcpy(&lp.pointSize, p.u + 268, sizeof(float));   // UniformsMaterial.u_pointSize
  lp.lineWidth = rs.line_width;
  lp.fw = std::max(p.cw, p.dw);
  lp.fh = std::max(p.ch, p.dh);
  const long long extra = lp.mode == LP_LINES ? 2 * nIn : (lp.mode == LP_TRI_LINES ? 6 * nIn : 0);
  const long long kScanMax = 4096ll * 4096ll;   // one scan handles up to 4096 blocks of 4096
  if (3 * nIn > kScanMax || (long long) p.nv + extra > (1ll << 30))
    return c->fail(SGLC_ERR_OVERFLOW, "draw: too many points/lines in one draw");
  lp.nIn = (int) nIn;
  const int nSlots = 3 * lp.nIn;
  p.attr = vao.attr;
  p.strideF = (int) (vao.stride / 4);
  p.nv = (int) vao.nv;
  p.indices = vao.idx;
  p.ntri = 0;
  p.views = 1;
  p.nvView = p.nv;
  p.ntriView = 0;
  p.vCap = (int) (p.nv + extra);
  CK(c->vClip.ensure(sizeof(float4) * std::max(p.vCap, 1)));
  CK(c->vFrag.ensure(sizeof(float4) * std::max(p.vCap, 1)));
  CK(c->vMask.ensure((size_t) std::max(p.vCap, 1)));
  CK(c->vVary.ensure(sizeof(float) * (size_t) std::max(p.vCap, 1) * p.varyStride));
  CK(c->vAttrExtra.ensure(sizeof(float) * (size_t) std::max<long long>(extra, 1) * std::max(p.strideF, 1)));
  CK(c->counters.ensure(sizeof(int) * 8));
  CK(c->lpSlot.ensure(sizeof(int4) * (size_t) std::max(nSlots, 1)));
  CK(c->lpOrigin.ensure(sizeof(float2) * (size_t) std::max(nSlots, 1)));
  CK(c->lpStampCount.ensure(sizeof(int) * (size_t) std::max(nSlots, 1)));
  CK(c->lpStampOff.ensure(sizeof(int) * (size_t) (nSlots + 1)));
  CK(c->lpMisc.ensure(64));
  CK(c->scanScratch.ensure(sizeof(int) * (size_t) scanScratchInts(nSlots + 1) * 2));
  p.vClip = c->vClip.as<float4>();
  p.vFrag = c->vFrag.as<float4>();
  p.vMask = c->vMask.as<uint8_t>();
  p.vVary = c->vVary.as<float>();
  p.vAttrExtra = c->vAttrExtra.as<float>();
  p.counters = c->counters.as<int>();
  lp.slot = c->lpSlot.as<int4>();
  lp.pointOrigin = c->lpOrigin.as<float2>();
  lp.stampCount = c->lpStampCount.as<int>();
  lp.stampOff = c->lpStampOff.as<int>();
  int *misc = c->lpMisc.as<int>();   // [0] flags, [1] sort count; [4..7] two 64-bit totals
  lp.flags = misc;
  lp.totals = reinterpret_cast<unsigned long long *>(misc + 4);
  CK(cudaMemsetAsync(p.counters, 0, sizeof(int) * 8, st));
  CK(cudaMemsetAsync(misc, 0, 64, st));
  int launches = 2;
  launchPointsLinesGeometry(p, lp, st);
  // sorts (p.keyA, p.valA)[0, n); the kernels read n from *nDev
  auto sortBy = [&](int n, const int *nDev, int keyBits) -> sglc_status {
    int sortInts = sortScratchInts(n);
    CK(c->sortHist.ensure(sizeof(int) * (size_t) sortInts));
    CK(c->sortHistScan.ensure(sizeof(int) * (size_t) sortInts));
    CK(c->scanScratch.ensure(sizeof(int) * (size_t) scanScratchInts(std::max(n + 1, sortInts)) * 2));
    sortPairs(p, n, nDev, keyBits, c->sortHist.as<int>(), c->sortHistScan.as<int>(), c->scanScratch.as<int>(), st);
    launches += 5 * sortPassCount(keyBits);
    return SGLC_OK;
  };
  auto bitsFor = [](long long n) {
    int b = 1;
    while ((1ll << b) < n) b++;
    return b;
  };
  if (lp.mode == LP_POINTS || lp.mode == LP_TRI_POINTS) {
    // per vertex, its point slots in drawing order: every stamp's origin
    CK(c->keyA.ensure(sizeof(uint32_t) * (size_t) std::max(nSlots, 1)));
    CK(c->keyB.ensure(sizeof(uint32_t) * (size_t) std::max(nSlots, 1)));
    CK(c->valA.ensure(sizeof(int) * (size_t) std::max(nSlots, 1)));
    CK(c->valB.ensure(sizeof(int) * (size_t) std::max(nSlots, 1)));
    p.keyA = c->keyA.as<uint32_t>();
    p.keyB = c->keyB.as<uint32_t>();
    p.valA = c->valA.as<int>();
    p.valB = c->valB.as<int>();
    launchPointKeys(lp, p.keyA, p.valA, nSlots, st);
    c->hostCounters[8] = nSlots;   // pinned; read by the copy below before any later write
    CK(cudaMemcpyAsync(misc + 1, c->hostCounters + 8, sizeof(int), cudaMemcpyHostToDevice, st));
    sglc_status s = sortBy(nSlots, misc + 1, bitsFor((long long) p.nv + 1));
    if (s) return s;
    launchPointChain(p, lp, p.keyA, p.valA, nSlots, st);
    launches += 2;
  }
  launchStampCount(p, lp, st);
  scanExclusive(lp.stampCount, lp.stampOff, nullptr, std::max(nSlots, 1), c->scanScratch.as<int>(), st);
  CK(cudaGetLastError());
  // read back: flags, stamp total
  CK(cudaMemcpyAsync(c->hostCounters, misc, 32, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  int flags = c->hostCounters[0];
  unsigned long long nStamps64;
  memcpy(&nStamps64, c->hostCounters + 4, 8);
  if (flags & LP_ERR_BADINDEX) return c->fail(SGLC_ERR_INVALID_VALUE, "draw: index out of range of the vertex array");
  if (flags & LP_ERR_LONGLINE) return c->fail(SGLC_ERR_OVERFLOW, "draw: line longer than 2^24 steps");
  if ((long long) nStamps64 > kScanMax - 1) return c->fail(SGLC_ERR_OVERFLOW, "draw: too many point/line stamps");
  const int nStamps = (int) nStamps64;
  const bool lineVary = p.varyCnt > 0 && (lp.mode == LP_LINES || lp.mode == LP_TRI_LINES);
  CK(c->lpStampGeo.ensure(sizeof(float4) * (size_t) std::max(nStamps, 1)));
  CK(c->lpStampRow.ensure(sizeof(int) * (size_t) std::max(nStamps, 1)));
  CK(c->lpStampColor.ensure(sizeof(float4) * (size_t) std::max(nStamps, 1)));
  if (lineVary) CK(c->lpStampVary.ensure(sizeof(float) * (size_t) std::max(nStamps, 1) * p.varyStride));
  CK(c->lpFragCount.ensure(sizeof(int) * (size_t) std::max(nStamps, 1)));
  CK(c->lpFragOff.ensure(sizeof(int) * (size_t) (nStamps + 1)));
  CK(c->scanScratch.ensure(sizeof(int) * (size_t) scanScratchInts(nStamps + 1) * 2));
  lp.stampGeo = c->lpStampGeo.as<float4>();
  lp.stampRow = c->lpStampRow.as<int>();
  lp.stampColor = c->lpStampColor.as<float4>();
  lp.stampVary = lineVary ? c->lpStampVary.as<float>() : nullptr;
  lp.fragCount = c->lpFragCount.as<int>();
  lp.fragOff = c->lpFragOff.as<int>();
  launchStampEmit(p, lp, st);
  launchStampShade(p, lp, nStamps, st);
  launchFragCount(lp, nStamps, st);
  scanExclusive(lp.fragCount, lp.fragOff, nullptr, std::max(nStamps, 1), c->scanScratch.as<int>(), st);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(c->hostCounters, misc, 32, cudaMemcpyDeviceToHost, st));
  CK(cudaStreamSynchronize(st));
  unsigned long long nFrags64;
  memcpy(&nFrags64, c->hostCounters + 6, 8);
  // the sort's histogram scan covers 256 digits x (n / 2048) blocks
  if ((long long) nFrags64 > 2048ll * (kScanMax / 256) - 2048)
    return c->fail(SGLC_ERR_OVERFLOW, "draw: too many point/line fragments");
  const int nFrags = (int) nFrags64;
  launches += 3 + 3 + 3;
  if (nFrags > 0) {
    CK(c->keyA.ensure(sizeof(uint32_t) * (size_t) nFrags));
    CK(c->keyB.ensure(sizeof(uint32_t) * (size_t) nFrags));
    CK(c->valA.ensure(sizeof(int) * (size_t) nFrags));
    CK(c->valB.ensure(sizeof(int) * (size_t) nFrags));
    p.keyA = c->keyA.as<uint32_t>();
    p.keyB = c->keyB.as<uint32_t>();
    p.valA = c->valA.as<int>();
    p.valB = c->valB.as<int>();
    launchFragEmit(lp, nStamps, p.keyA, p.valA, st);
    sglc_status s = sortBy(nFrags, lp.fragOff + nStamps, bitsFor((long long) lp.fw * lp.fh));
    if (s) return s;
    launchFragApply(p, lp, p.keyA, p.valA, nFrags, dt != nullptr, st);
    launches += 2;
  }
  if (p.samples == 4) {
    launchResolve(p, st);
    ct->resolvedValid = true;
    launches += 1;
  }
  CK(cudaGetLastError());
  c->stats.vertices_in = p.nv;
  c->stats.triangles_in = nIn;
  c->stats.primitives = nStamps;
  c->stats.bin_entries = nFrags;
  c->stats.clip_vertices = -1;
  c->stats.kernel_launches = launches;
  return SGLC_OK;
}

// RendererSoft::setViewPort (RendererSoft.cpp:92-113): the viewport transform with depth range [0, 1]
Viewport makeViewport(int x, int y, int w, int h) {
  Viewport v;
  v.x = (float) x;
  v.y = (float) y;
  v.w = (float) w;
  v.h = (float) h;
  float minD = 0.f, maxD = 1.f;
  v.absMin = std::min(minD, maxD);
  v.absMax = std::max(minD, maxD);
  v.oX = v.x + v.w / 2.f;
  v.oY = v.y + v.h / 2.f;
  v.oZ = minD;
  v.oW = 0.f;
  v.pX = v.w / 2.f;
  v.pY = v.h / 2.f;
  v.pZ = maxD - minD;
  v.pW = 1.f;
  return v;
}

// the viewport a multi-scene draw gives each scene: its whole frame
Viewport fullViewport(int w, int h) { return makeViewport(0, 0, w, h); }

sglc_status drawImpl(Ctx *c, const BatchViews *bv = nullptr) {
  const bool scenes = bv && bv->vaos;
  Object *fo = c->get(bv ? bv->fbs[0] : c->fb, K_FB), *vo = c->get(scenes ? bv->vaos[0] : c->vao, K_VAO),
         *po = c->get(c->prog, K_PROG);
  if (!fo || !vo || !po) return SGLC_OK;   // RendererSoft::draw is a silent no-op (RendererSoft.cpp:137-139)
  Object *so = c->get(c->states, K_STATES);
  if (!so) return c->fail(SGLC_ERR_INVALID_VALUE, "draw: no pipeline states bound");
  ProgObj &prog = po->prog;
  if (!prog.shader) return c->fail(SGLC_ERR_INVALID_VALUE, "draw: program has no shaders");
  const sglc_render_states &rs = so->states;
  if (rs.primitive_type < SGLC_PRIMITIVE_POINT || rs.primitive_type > SGLC_PRIMITIVE_TRIANGLE)
    return c->fail(SGLC_ERR_INVALID_VALUE, "draw: unknown primitive type");
  if (rs.polygon_mode < SGLC_POLYGON_POINT || rs.polygon_mode > SGLC_POLYGON_FILL)
    return c->fail(SGLC_ERR_INVALID_VALUE, "draw: unknown polygon mode");
  const bool pointsLines = rs.primitive_type != SGLC_PRIMITIVE_TRIANGLE || rs.polygon_mode != SGLC_POLYGON_FILL;
  if (pointsLines && bv) return c->fail(SGLC_ERR_UNSUPPORTED, "draw_views: only filled triangles are batched");
  FbObj &fb = fo->fb;
  TexObj *ct = fb.colorReady ? attachmentTex(c, fb.colorTex) : nullptr;
  TexObj *dt = fb.depthReady ? attachmentTex(c, fb.depthTex) : nullptr;
  if (ct && (!ct->allocated || fb.colorLevel >= ct->levels || ct->desc.format != SGLC_FORMAT_RGBA8)) ct = nullptr;
  if (dt && (!dt->allocated || dt->desc.format != SGLC_FORMAT_FLOAT32)) dt = nullptr;
  if (!ct && !dt) return SGLC_OK;
  if (ct && dt && ct->desc.multi_sample != dt->desc.multi_sample)
    return c->fail(SGLC_ERR_UNSUPPORTED, "draw: colour and depth attachments must have the same sample count");
  if (ct) ct->version++;   // the draw writes its attachments
  if (dt) dt->version++;
  VaoObj &vao = vo->vao;

  DrawParams p;
  memset(&p, 0, sizeof(p));
  p.shading = prog.shader->model;
  p.varyCnt = prog.shader->varyingsCnt;
  p.varyStride = std::max(8, ((p.varyCnt * 4 + 31) / 32) * 8);   // <= 32: k_vertex stages a row in registers
  memcpy(p.def, prog.defines, 8);
  memcpy(p.u, prog.uniforms, kUniformBytes);
  for (int s = 0; s < kMaxSamplers; s++) {
    Object *uo = c->get(prog.samplers[s], K_US);
    if (!uo) continue;
    UsObj &us = uo->us;
    Object *to = c->get(us.tex, K_TEX);
    if (!to || !to->tex.allocated) continue;
    DevSampler &d = p.samp[s];
    d.valid = 1;
    d.filter = us.filter;
    d.wrap = us.wrap;
    d.border = us.border;
    d.width = us.width;
    d.height = us.height;
    // only samplers whose LOD callback the FS installs (setupSamplerDerivative: albedo, normal,
    // emissive, ao; BlinnPhongSoft.h:217-230, PbrSoft.h:138-151) use derivative-based LOD
    d.lodFromDerivative = us.useMipmaps && ((prog.shader->derivSlots >> s) & 1) && us.type == SGLC_TEXTURE_2D;
    d.isFloat = us.format == SGLC_FORMAT_FLOAT32;
    d.tex = devTex(to->tex);
  }
  for (int s = 0; s < 4; s++)
    if (p.samp[s].valid && p.samp[s].lodFromDerivative && p.def[s]) p.needDeriv = 1;
  int iblEnabled = 0;
  memcpy(&iblEnabled, prog.uniforms + 324, sizeof(int));   // UniformsMaterial.u_enableIBL (PbrSoft.h:45)
  if (pointsLines) iblEnabled = 0;   // points and lines run the exact shader, never the neural one
  if (p.shading == SH_PBR && prog.neural && ct && iblEnabled) {
    p.shading = SH_PBR_NEURAL;
    p.nnImage = neuralImage(prog.neural);
    // the neural path's material maps go through the texture units (sglc_shade_neural.cu)
    for (int s = 0; s < kMaxSamplers; s++) {
      if (!p.samp[s].valid) continue;
      Object *uo = c->get(prog.samplers[s], K_US);
      Object *to = uo ? c->get(uo->us.tex, K_TEX) : nullptr;
      if (!to) continue;
      sglc_status st = hwTexture(c, to->tex, uo->us, &p.hwTex[s]);
      if (st) return st;
    }
    if (!c->sticky.ptr) {
      CK(c->sticky.ensure(sizeof(int)));
      CK(cudaMemsetAsync(c->sticky.ptr, 0, sizeof(int), c->stream));
    }
    p.errFlags = c->sticky.as<int>();
    p.nnInjectTimeout = c->nnTestFlags & 1;
  }
  if (p.shading == SH_PBR && c->capRecords && !pointsLines) {
    p.shading = SH_PBR_CAPTURE;
    p.capRecords = c->capRecords;
    p.capCount = c->capCount;
    p.capCap = c->capCap;
    p.capStride = c->capStride;
  }
  p.depthTest = rs.depth_test;
  p.depthMask = rs.depth_mask;
  p.depthFunc = rs.depth_func;
  p.blend = rs.blend;
  p.bFuncRgb = rs.blend_func_rgb;
  p.bSrcRgb = rs.blend_src_rgb;
  p.bDstRgb = rs.blend_dst_rgb;
  p.bFuncA = rs.blend_func_alpha;
  p.bSrcA = rs.blend_src_alpha;
  p.bDstA = rs.blend_dst_alpha;
  // BlendFactor -> (operand, c0, c1) with factor = c0 + c1 * operand (BlendSoft.h:13-30)
  {
    const int facs[4] = {rs.blend_src_rgb, rs.blend_dst_rgb, rs.blend_src_alpha, rs.blend_dst_alpha};
    for (int k = 0; k < 4; k++) {
      int f = facs[k], op = 0;
      float c0 = 0.f, c1 = 0.f;
      switch (f) {
        case SGLC_BLEND_ZERO: break;
        case SGLC_BLEND_ONE: c0 = 1.f; break;
        case SGLC_BLEND_SRC_COLOR: op = 0; c1 = 1.f; break;
        case SGLC_BLEND_SRC_ALPHA: op = 1; c1 = 1.f; break;
        case SGLC_BLEND_DST_COLOR: op = 2; c1 = 1.f; break;
        case SGLC_BLEND_DST_ALPHA: op = 3; c1 = 1.f; break;
        case SGLC_BLEND_ONE_MINUS_SRC_COLOR: op = 0; c0 = 1.f; c1 = -1.f; break;
        case SGLC_BLEND_ONE_MINUS_SRC_ALPHA: op = 1; c0 = 1.f; c1 = -1.f; break;
        case SGLC_BLEND_ONE_MINUS_DST_COLOR: op = 2; c0 = 1.f; c1 = -1.f; break;
        case SGLC_BLEND_ONE_MINUS_DST_ALPHA: op = 3; c0 = 1.f; c1 = -1.f; break;
      }
      p.bfOp[k] = op;
      p.bfC0[k] = c0;
      p.bfC1[k] = c1;
    }
    const int fns[2] = {rs.blend_func_rgb, rs.blend_func_alpha};
    for (int k = 0; k < 2; k++) {
      p.bKs[k] = fns[k] == SGLC_FUNC_REVERSE_SUBTRACT ? -1.f : 1.f;
      p.bKd[k] = fns[k] == SGLC_FUNC_SUBTRACT ? -1.f : 1.f;
      p.bMinMax[k] = fns[k] == SGLC_FUNC_MIN ? 1 : (fns[k] == SGLC_FUNC_MAX ? 2 : 0);
    }
  }
  p.cullFace = rs.cull_face;
  p.earlyZ = c->earlyZ;
  p.vp = c->vp;
  if (ct) {
    p.color = ct->dev + (size_t) fb.colorLayer * ct->layerStride + ct->offset[fb.colorLevel];
    p.resolved = ct->resolved;
    p.cw = ct->w[fb.colorLevel];
    p.ch = ct->h[fb.colorLevel];
    p.cms = ct->desc.multi_sample;
  }
  if (dt) {
    p.depth = reinterpret_cast<float *>(dt->dev);
    p.dw = dt->w[0];
    p.dh = dt->h[0];
    p.dms = dt->desc.multi_sample;
  }
  p.samples = ct ? (ct->desc.multi_sample ? 4 : 1) : (dt->desc.multi_sample ? 4 : 1);
  // raster tile: 16 pixels wide; 16 high, or the context's 8 for draws the deferred kernels raster
  // (the fused raster kernel has one shape)
  p.tile = c->tile;
  p.tileH = c->deferredShading && ct && deferredShadingModel(p.shading) && !pointsLines ? c->tileH : 16;
  // TMA write-back of whole tiles by the deferred raster kernels (single-view draws)
  if (!bv && c->tmaStore) {
    if (ct && encodeAttachment(&p.tmColor, p.color, p.cw, p.ch, p.samples, p.tileH) &&
        (p.samples == 1 || encodeAttachment(&p.tmResolved, p.resolved, p.cw, p.ch, 1, p.tileH)))
      p.tmaStore |= 1;
    if (dt && encodeAttachment(&p.tmDepth, p.depth, p.dw, p.dh, p.samples, p.tileH)) p.tmaStore |= 2;
  }
  std::vector<ViewTarget> targets;
  std::vector<SceneRec> sceneRecs;
  if (bv) {
    // every view's attachments must match view 0's (size, format, samples, presence)
    for (int v = 0; v < bv->count; v++) {
      Object *o = c->get(bv->fbs[v], K_FB);
      if (!o) return c->fail(SGLC_ERR_INVALID_HANDLE, "draw_views: invalid framebuffer");
      FbObj &f = o->fb;
      TexObj *vc = f.colorReady ? attachmentTex(c, f.colorTex) : nullptr;
      TexObj *vd = f.depthReady ? attachmentTex(c, f.depthTex) : nullptr;
      if (vc) vc->version++;
      if (vd) vd->version++;
      if (vc && (!vc->allocated || f.colorLevel >= vc->levels || vc->desc.format != SGLC_FORMAT_RGBA8)) vc = nullptr;
      if (vd && (!vd->allocated || vd->desc.format != SGLC_FORMAT_FLOAT32)) vd = nullptr;
      // (a multi-scene draw: sizes may differ, presence and sample count may not)
      if ((vc != nullptr) != (ct != nullptr) || (vd != nullptr) != (dt != nullptr) ||
          (vc && vc->desc.multi_sample != p.cms) || (vd && vd->desc.multi_sample != p.dms) ||
          (!scenes && vc && (vc->w[f.colorLevel] != p.cw || vc->h[f.colorLevel] != p.ch)) ||
          (!scenes && vd && (vd->w[0] != p.dw || vd->h[0] != p.dh)))
        return c->fail(SGLC_ERR_INVALID_VALUE, "draw_views: every view needs attachments like view 0's");
      if (scenes) {   // this scene's frame: its attachment sizes and a viewport over them
        SceneRec sr{};
        sr.cw = vc ? vc->w[f.colorLevel] : 0;
        sr.ch = vc ? vc->h[f.colorLevel] : 0;
        sr.dw = vd ? vd->w[0] : 0;
        sr.dh = vd ? vd->h[0] : 0;
        sr.vp = fullViewport(std::max(sr.cw, sr.dw), std::max(sr.ch, sr.dh));
        sceneRecs.push_back(sr);
      }
      ViewTarget t{};
      if (vc) {
        t.color = vc->dev + (size_t) f.colorLayer * vc->layerStride + vc->offset[f.colorLevel];
        t.resolved = vc->resolved;
        if (vc->desc.multi_sample) vc->resolvedValid = true;
      }
      if (vd) t.depth = reinterpret_cast<float *>(vd->dev);
      targets.push_back(t);
    }
    sglc_status st = flushClear(c);
    if (st) return st;
    const sglc_clear_states *cs = bv->clear;
    if (cs && (cs->color_flag || cs->depth_flag)) {
      p.pendingClear = 1;
      p.clearColorFlag = cs->color_flag && ct;
      p.clearDepthFlag = cs->depth_flag && dt;
      p.clearColor = u8c(cs->clear_color[0] * 255) | (u8c(cs->clear_color[1] * 255) << 8) |
                     (u8c(cs->clear_color[2] * 255) << 16) | (u8c(cs->clear_color[3] * 255) << 24);
      p.clearDepth = cs->clear_depth;
    }
  } else if (pointsLines) {
    return drawPointsLines(c, p, rs, vao, ct, dt);
  } else if (c->clear.active && c->clear.fb == c->fb) {
    p.pendingClear = 1;
    p.clearColorFlag = c->clear.colorFlag && ct;
    p.clearDepthFlag = c->clear.depthFlag && dt;
    p.clearColor = c->clear.color;
    p.clearDepth = c->clear.depth;
    c->clear.active = false;
  } else {
    sglc_status s = flushClear(c);
    if (s) return s;
  }
  p.attr = vao.attr;
  p.strideF = (int) (vao.stride / 4);
  p.nv = (int) vao.nv;
  p.indices = vao.idx;
  p.ntri = (int) (vao.nidx / 3);
  int fw = std::max(p.cw, p.dw), fh = std::max(p.ch, p.dh);
  p.tilesX = (fw + p.tile - 1) / p.tile;
  p.tilesY = (fh + p.tileH - 1) / p.tileH;
  int numTiles = p.tilesX * p.tilesY;
  p.views = 1;
  p.nvView = p.nv;
  p.ntriView = p.ntri;
  p.tilesPerView = numTiles;
  std::vector<int> sceneBases;   // multi-scene draws: first vertex, triangle and tile of every scene
  if (scenes) {
    // every scene's vertex array, its ranges of the pass's vertices, triangles and tiles
    long long nv = 0, nt = 0, tiles = 0;
    sceneBases.resize(3 * ((size_t) bv->count + 1));
    int *vBase = sceneBases.data(), *tBase = vBase + bv->count + 1, *tileBase = tBase + bv->count + 1;
    for (int v = 0; v < bv->count; v++) {
      Object *so2 = c->get(bv->vaos[v], K_VAO);
      if (!so2) return c->fail(SGLC_ERR_INVALID_HANDLE, "draw_scenes: invalid vertex array handle");
      const VaoObj &sv = so2->vao;
      if (sv.stride != vao.stride) return c->fail(SGLC_ERR_INVALID_VALUE, "draw_scenes: vertex strides differ");
      SceneRec &sr = sceneRecs[v];
      sr.attr = sv.attr;
      sr.indices = sv.idx;
      sr.nv = (int) sv.nv;
      sr.ntri = (int) (sv.nidx / 3);
      sr.tilesX = (std::max(sr.cw, sr.dw) + p.tile - 1) / p.tile;
      sr.tilesY = (std::max(sr.ch, sr.dh) + p.tileH - 1) / p.tileH;
      vBase[v] = (int) nv;
      tBase[v] = (int) nt;
      tileBase[v] = (int) tiles;
      nv += sr.nv;
      nt += sr.ntri;
      tiles += (long long) sr.tilesX * sr.tilesY;
      if (nt * 3 > (1ll << 30) || nv > (1ll << 30) || tiles > (1ll << 30))
        return c->fail(SGLC_ERR_INVALID_VALUE, "draw_scenes: batch too large");
    }
    vBase[bv->count] = (int) nv;
    tBase[bv->count] = (int) nt;
    tileBase[bv->count] = (int) tiles;
    p.views = bv->count;
    p.nv = (int) nv;
    p.ntri = (int) nt;
    p.nvView = p.ntriView = p.tilesPerView = 0;   // per scene instead
    numTiles = (int) tiles;
    p.vp = sceneRecs[0].vp;
  } else if (bv) {
    if ((long long) p.ntri * bv->count * 3 > (1ll << 30) || (long long) p.nv * bv->count > (1ll << 30) ||
        (long long) numTiles * bv->count > (1ll << 30))
      return c->fail(SGLC_ERR_INVALID_VALUE, "draw_views: batch too large");
    p.views = bv->count;
    p.nv *= bv->count;
    p.ntri *= bv->count;
    numTiles *= bv->count;
  }
  p.numTiles = numTiles;
  if (bv) {
    CK(c->batchU.ensure(bv->uniforms.size()));
    CK(c->batchTargets.ensure(sizeof(ViewTarget) * targets.size()));
    const void *srcU = bv->uniforms.data(), *srcT = targets.data();
    if (c->capturing) {   // a captured copy reads its host source at every replay: keep it alive with the graph
      void *hu = nullptr, *ht = nullptr;
      CK(cudaMallocHost(&hu, bv->uniforms.size()));
      c->captureHostBufs.push_back(hu);
      CK(cudaMallocHost(&ht, sizeof(ViewTarget) * targets.size()));
      c->captureHostBufs.push_back(ht);
      memcpy(hu, srcU, bv->uniforms.size());
      memcpy(ht, srcT, sizeof(ViewTarget) * targets.size());
      srcU = hu;
      srcT = ht;
    }
    CK(cudaMemcpyAsync(c->batchU.ptr, srcU, bv->uniforms.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->batchTargets.ptr, srcT, sizeof(ViewTarget) * targets.size(), cudaMemcpyHostToDevice,
                       c->stream));
    p.viewU = c->batchU.as<uint8_t>();
    p.viewTarget = c->batchTargets.as<ViewTarget>();
    if (scenes) {   // the scene records, then the three base arrays
      const size_t recBytes = sizeof(SceneRec) * sceneRecs.size(), baseBytes = sizeof(int) * sceneBases.size();
      std::vector<uint8_t> blob(recBytes + baseBytes);
      memcpy(blob.data(), sceneRecs.data(), recBytes);
      memcpy(blob.data() + recBytes, sceneBases.data(), baseBytes);
      CK(c->batchScenes.ensure(blob.size()));
      const void *srcS = blob.data();
      if (c->capturing) {
        void *hs = nullptr;
        CK(cudaMallocHost(&hs, blob.size()));
        c->captureHostBufs.push_back(hs);
        memcpy(hs, blob.data(), blob.size());
        srcS = hs;
      }
      CK(cudaMemcpyAsync(c->batchScenes.ptr, srcS, blob.size(), cudaMemcpyHostToDevice, c->stream));
      p.scenes = c->batchScenes.as<SceneRec>();
      const int *bases = reinterpret_cast<const int *>(c->batchScenes.as<uint8_t>() + recBytes);
      p.sceneVBase = bases;
      p.sceneTBase = bases + bv->count + 1;
      p.sceneTileBase = bases + 2 * (bv->count + 1);
    }
    if (p.shading == SH_PBR_CAPTURE) p.shading = SH_PBR;   // no training capture in batched draws
  }

  for (int attempt = 0; attempt < 4; attempt++) {
    const bool deferred = c->capSet;
    int extraVerts = std::max(std::max(4096, p.ntri / 2), c->extraVertHint);
    int polyCap = std::max(std::max(1024, p.ntri / 4), c->polyHint);
    int appendCap = std::max(std::max(1024, p.ntri / 4), c->appendHint);
    if (deferred) {
      extraVerts = (int) std::max<int64_t>(1, std::min<int64_t>(c->cap.clip_vertices, 1 << 28));
      polyCap = (int) std::max<int64_t>(1, std::min<int64_t>(c->cap.clip_polygons, 1 << 28));
      appendCap = (int) std::max<int64_t>(1, std::min<int64_t>(c->cap.appended_primitives, 1 << 28));
    }
    p.vCap = p.nv + extraVerts;
    p.clipPolyCap = polyCap;
    p.primCap = p.ntri + appendCap;
    CK(c->vClip.ensure(sizeof(float4) * p.vCap));
    CK(c->vFrag.ensure(sizeof(float4) * p.vCap));
    CK(c->vMask.ensure((size_t) p.vCap));
    CK(c->vVary.ensure(sizeof(float) * (size_t) p.vCap * p.varyStride));
    CK(c->vAttrExtra.ensure(sizeof(float) * (size_t) extraVerts * std::max(p.strideF, 1)));
    CK(c->prims.ensure(sizeof(int4) * (size_t) p.primCap));
    CK(c->clipExtra.ensure(sizeof(int) * (size_t) (p.ntri + 1)));
    CK(c->clipAppendOff.ensure(sizeof(int) * (size_t) (p.ntri + 1)));
    CK(c->clipPoly.ensure(sizeof(int4) * 3 * (size_t) polyCap));
    CK(c->clipPolyTri.ensure(sizeof(int) * (size_t) polyCap));
    // 16 counters, then the per-scan-tile totals k_clip and k_setup add up for the two scans
    const int clipTiles = scanTiles(std::max(p.ntri, 1)), primTiles = scanTiles(p.primCap);
    const size_t counterInts = 16 + (size_t) clipTiles + (size_t) primTiles;
    CK(c->counters.ensure(sizeof(int) * counterInts));
    CK(c->tri.ensure(sizeof(TriSetup) * (size_t) p.primCap));
    CK(c->tileCount.ensure(sizeof(int) * (size_t) p.primCap));
    CK(c->pairOff.ensure(sizeof(int) * (size_t) (p.primCap + 1)));
    CK(c->scanScratch.ensure(sizeof(int) * (size_t) scanScratchInts(std::max(p.primCap, p.ntri) + 1) * 2));
    p.vClip = c->vClip.as<float4>();
    p.vFrag = c->vFrag.as<float4>();
    p.vMask = c->vMask.as<uint8_t>();
    p.vVary = c->vVary.as<float>();
    p.vAttrExtra = c->vAttrExtra.as<float>();
    p.prims = c->prims.as<int4>();
    p.clipExtra = c->clipExtra.as<int>();
    p.clipAppendOff = c->clipAppendOff.as<int>();
    p.clipPoly = c->clipPoly.as<int4>();
    p.clipPolyTri = c->clipPolyTri.as<int>();
    p.counters = c->counters.as<int>();
    p.clipScanSums = p.counters + 16;
    p.tileScanSums = p.counters + 16 + clipTiles;
    p.tri = c->tri.as<TriSetup>();
    p.tileCount = c->tileCount.as<int>();
    p.pairOff = c->pairOff.as<int>();

    CK(cudaMemsetAsync(p.counters, 0, sizeof(int) * counterInts, c->stream));
    if (c->statsLevel >= 1) CK(cudaEventRecord(c->ev[0], c->stream));
    launchVertexAndClip(p, c->stream);
    scanApply(p.clipExtra, p.clipAppendOff, nullptr, std::max(p.ntri, 1), p.clipScanSums, c->stream);
    launchClipAppend(p, c->stream);
    launchSetup(p, p.primCap, c->stream);
    scanApply(p.tileCount, p.pairOff, p.counters + 3, p.primCap, p.tileScanSums, c->stream);
    CK(cudaGetLastError());
    if (c->statsLevel >= 1) CK(cudaEventRecord(c->ev[1], c->stream));
    int newVerts = -1, polys = -1, np = p.primCap, nPairs;
    unsigned long long fragBound = 0;   // upper bound on fragment records (exact sizing only)
    const int *nPairsDev = p.pairOff + p.primCap;
    if (!deferred) {
      CK(cudaMemcpyAsync(c->hostCounters, p.counters, sizeof(int) * 4, cudaMemcpyDeviceToHost, c->stream));
      CK(cudaMemcpyAsync(c->hostCounters + 4, p.pairOff + p.primCap, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaMemcpyAsync(c->hostCounters + 6, p.counters + kCntBound, 8, cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      newVerts = c->hostCounters[0];
      polys = c->hostCounters[1];
      int flags = c->hostCounters[2];
      np = c->hostCounters[3];
      if (flags & 16) return c->fail(SGLC_ERR_INVALID_VALUE, "draw: index out of range of the vertex array");
      if (flags & 7) {   // clip-vertex / polygon / primitive capacity: grow and redo (nothing written yet)
        c->extraVertHint = std::max(extraVerts * 2, newVerts + 1024);
        c->polyHint = std::max(polyCap * 2, polys + 1024);
        c->appendHint = std::max(appendCap * 2, p.primCap);
        continue;
      }
      nPairs = c->hostCounters[4];
      c->peak.clip_vertices = std::max<int64_t>(c->peak.clip_vertices, newVerts);
      c->peak.clip_polygons = std::max<int64_t>(c->peak.clip_polygons, polys);
      c->peak.appended_primitives = std::max<int64_t>(c->peak.appended_primitives, (int64_t) np - p.ntri);
      c->peak.bin_entries = std::max<int64_t>(c->peak.bin_entries, nPairs);
      memcpy(&fragBound, c->hostCounters + 6, 8);
    } else {
      // no read-back: the bin arrays have the set capacity, the sort and ranges read the pair count
      // (clamped to it) from the device
      nPairs = (int) std::max<int64_t>(1, std::min<int64_t>(c->cap.bin_entries, 1 << 30));
      p.binPairTotal = p.pairOff + p.primCap;   // k_bin_emit clamps it into counters[4]
      nPairsDev = p.counters + 4;
    }
    CK(c->keyA.ensure(sizeof(uint32_t) * (size_t) std::max(nPairs, 1)));
    CK(c->keyB.ensure(sizeof(uint32_t) * (size_t) std::max(nPairs, 1)));
    CK(c->valA.ensure(sizeof(int) * (size_t) std::max(nPairs, 1)));
    CK(c->valB.ensure(sizeof(int) * (size_t) std::max(nPairs, 1)));
    CK(c->tileStart.ensure(sizeof(int) * (size_t) numTiles));
    CK(c->tileEnd.ensure(sizeof(int) * (size_t) numTiles));
    CK(c->tileOrder.ensure(sizeof(int) * (size_t) numTiles));
    int sortInts = sortScratchInts(nPairs);
    CK(c->sortHist.ensure(sizeof(int) * (size_t) sortInts));
    CK(c->sortHistScan.ensure(sizeof(int) * (size_t) sortInts));
    CK(c->scanScratch.ensure(sizeof(int) * (size_t) (scanScratchInts(std::max(std::max(p.primCap, p.ntri) + 1, sortInts)) * 2)));
    p.keyA = c->keyA.as<uint32_t>();
    p.keyB = c->keyB.as<uint32_t>();
    p.valA = c->valA.as<int>();
    p.valB = c->valB.as<int>();
    p.pairCap = nPairs;
    p.tileStart = c->tileStart.as<int>();
    p.tileEnd = c->tileEnd.as<int>();
    if (np > 0) {
      p.binZeroRanges = 1;   // k_bin_emit clears the tile ranges
    } else {
      CK(cudaMemsetAsync(p.tileStart, 0, sizeof(int) * numTiles, c->stream));
      CK(cudaMemsetAsync(p.tileEnd, 0, sizeof(int) * numTiles, c->stream));
    }
    launchBinEmit(p, np, c->stream);
    int keyBits = 1;
    while ((1 << keyBits) < numTiles) keyBits++;
    sortPairs(p, nPairs, nPairsDev, keyBits, c->sortHist.as<int>(), c->sortHistScan.as<int>(),
              c->scanScratch.as<int>(), c->stream, true);
    launchTileRanges(p, nPairs, nPairsDev, c->stream);
    const bool heavyFirst = !deferred || c->cap.heavy_first;
    if (heavyFirst) {
      launchTileOrder(p, c->tileOrder.as<int>(), c->stream);
      p.tileOrder = c->tileOrder.as<int>();
    }
    if (c->statsLevel >= 2) {
      CK(cudaMemsetAsync(c->fragCounter, 0, sizeof(unsigned long long), c->stream));
      p.fragCounter = c->fragCounter;
    }
    // deferred shading: records = the bound from setup, plus a partly filled last chunk per warp
    bool deferShade = c->deferredShading && ct && deferredShadingModel(p.shading);
    long long chunks = 0;
    if (deferShade) {
      const long long warps = ((long long) numTiles + (kSplitParts - 1) * 64) * (p.tileH / 2);   // split tiles
      chunks = deferred ? (c->cap.fragments + kChunk - 1) / kChunk
                        : (long long) (fragBound / kChunk) + warps + 1;
      if (chunks < 1 || chunks * kChunk > (1ll << 28)) deferShade = false;   // single kernel instead
      if (!deferShade && p.tileH != 16)
        return c->fail(SGLC_ERR_OVERFLOW, "draw: more than 2^28 fragment records need 16x16 tiles (sglc_set_tile_size)");
    }
    if (deferShade) {
      CK(c->recA.ensure(sizeof(int4) * (size_t) chunks * kChunk));
      CK(c->recB.ensure(sizeof(float2) * (size_t) chunks * kChunk));
      CK(c->recColor.ensure(sizeof(float4) * (size_t) chunks * kChunk));
      CK(c->chunkNext.ensure(sizeof(int) * (size_t) chunks));
      CK(c->chunkFill.ensure(sizeof(int) * (size_t) chunks));
      CK(c->warpHead.ensure(sizeof(int) * (size_t) numTiles * kSplitParts * (p.tileH / 2)));
      CK(c->recDense.ensure(sizeof(int) * (size_t) chunks * kChunk));
      p.recA = c->recA.as<int4>();
      p.recB = c->recB.as<float2>();
      p.recColor = c->recColor.as<float4>();
      p.chunkNext = c->chunkNext.as<int>();
      p.chunkFill = c->chunkFill.as<int>();
      p.warpHead = c->warpHead.as<int>();
      p.recDense = c->recDense.as<int>();
      if (p.shading == SH_PBR_NEURAL) {
        CK(c->nnIn.ensure(sizeof(float4) * 5 * (size_t) chunks * kChunk));
        p.nnIn = c->nnIn.as<float4>();
      }
      p.chunkCap = (int) chunks;
      p.heavySlots = 64;    // with the heavy-first order: its first 64 tiles may be split in kSplitParts
      p.heavyMin = 256;     // primitives in a tile's list above which it is split in 4 (one row per warp)
      p.heavyMin8 = 1024;   // ... and in 8 (half a row per warp) above four times that: the sphere's poles at 1080p
      if (!c->peakChunks.ptr) {
        CK(c->peakChunks.ensure(sizeof(int)));
        CK(cudaMemsetAsync(c->peakChunks.ptr, 0, sizeof(int), c->stream));
      }
    }
    if (c->statsLevel >= 1) CK(cudaEventRecord(c->ev[2], c->stream));
    c->evDeferred = deferShade && c->statsLevel >= 1;
    if (deferShade) {
      // k_rop, the draw's last kernel, also keeps the peak of the chunks actually used (the pool is
      // sized from an upper bound; the peak calibrates capacities) and accumulates the overflow flags
      p.ropPeakChunks = c->peakChunks.as<int>();
      p.ropSticky = deferred ? c->sticky.as<int>() : nullptr;
      launchRasterDeferred(p, dt != nullptr, c->stream, c->evDeferred ? c->ev[4] : nullptr,
                           c->evDeferred ? c->ev[5] : nullptr);
    }
    else launchRaster(p, ct != nullptr, dt != nullptr, c->stream);
    if (c->statsLevel >= 1) {
      CK(cudaEventRecord(c->ev[3], c->stream));
      c->evPending = true;
    }
    if (deferred && !deferShade) launchAccumulateFlags(p.counters + 2, c->sticky.as<int>(), c->stream);
    CK(cudaGetLastError());
    if (ct && ct->desc.multi_sample) ct->resolvedValid = true;
    c->stats.vertices_in = p.nv;
    c->stats.triangles_in = p.ntri;
    c->stats.clip_vertices = newVerts;
    c->stats.primitives = deferred ? -1 : np;
    c->stats.bin_entries = deferred ? -1 : nPairs;
    // vertex, clip, scan, append, setup, scan | emit, sort (hist, 2 scan, scatter per pass), ranges,
    // order, raster (deferred shading: coverage, shade, ROP); flag accumulation when the draw has
    // capacities and no ROP kernel; a redone attempt ran the 6 geometry launches before
    int sortPasses = nPairs > 0 ? sortPassCount(keyBits) : 0;
    c->stats.kernel_launches = (p.nv > 0) + (p.ntri > 0) + 1 + 1 + 1 + 1 + (np > 0) + sortPasses * 4 +
                               (nPairs > 0) + (heavyFirst ? 1 : 0) + 1 + attempt * 6 +
                               (deferred && !deferShade ? 1 : 0) + (deferShade ? 2 : 0);
    return SGLC_OK;
  }
  return c->fail(SGLC_ERR_OVERFLOW, "draw: clip capacity could not be satisfied");
}

}  // namespace

namespace sglc {
cudaStream_t ctxStream(sglc_context *ctx) { return reinterpret_cast<Ctx *>(ctx)->stream; }
int ctxDevice(sglc_context *ctx) { return reinterpret_cast<Ctx *>(ctx)->device; }
void ctxSetError(sglc_context *ctx, const char *msg) {
  if (ctx) reinterpret_cast<Ctx *>(ctx)->err = msg;
}
void ctxSetCapture(sglc_context *ctx, float *records, unsigned long long *count, long long capacity, int stride) {
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  c->capRecords = records;
  c->capCount = records ? count : nullptr;
  c->capCap = records ? capacity : 0;
  c->capStride = stride;
}
void ctxDetachNeural(sglc_context *ctx, const sglc_neural *net) {
  Ctx *c = reinterpret_cast<Ctx *>(ctx);
  c->freeEpoch++;   // the network's buffers are about to be freed: graphs that read them are stale
  for (auto &kv : c->objects)
    if (kv.second.kind == K_PROG && kv.second.prog.neural == net) kv.second.prog.neural = nullptr;
  c->capRecords = nullptr;
  c->capCount = nullptr;
  c->capCap = 0;
}
}  // namespace sglc

extern "C" {

sglc_status sglc_create(sglc_context **out, int32_t device) {
  if (!out) return SGLC_ERR_INVALID_VALUE;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return SGLC_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return SGLC_ERR_INVALID_VALUE;
  sglc::DeviceGuard deviceGuard(device);
  int current = -1;
  if (cudaGetDevice(&current) != cudaSuccess || current != device) return SGLC_ERR_DEVICE;
  Ctx *c = new Ctx();
  c->device = device;
  c->forEachBuf([c](DevBuf &b) { b.epoch = &c->freeEpoch; });
  bool ok = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMallocHost(&c->hostCounters, 64) == cudaSuccess &&
            cudaMalloc(&c->fragCounter, sizeof(unsigned long long)) == cudaSuccess;
  for (int i = 0; i < 6 && ok; i++) ok = cudaEventCreate(&c->ev[i]) == cudaSuccess;
  if (!ok) {
    delete c;
    return SGLC_ERR_DEVICE;
  }
  *out = reinterpret_cast<sglc_context *>(c);
  return SGLC_OK;
}

sglc_status sglc_destroy(sglc_context *ctx) {
  CTX;
  cudaStreamSynchronize(c->stream);
  for (auto &kv : c->objects) {
    Object &o = kv.second;
    if (o.kind == K_TEX) freeTexture(o.tex, c->freeEpoch);
    if (o.kind == K_VAO) {
      cudaFree(o.vao.attr);
      cudaFree(o.vao.idx);
    }
  }
  c->forEachBuf([](DevBuf &b) { b.release(); });
  cudaFreeHost(c->hostCounters);
  for (void *h : c->captureHostBufs) cudaFreeHost(h);
  cudaFree(c->fragCounter);
  for (int i = 0; i < 6; i++)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  cudaStreamDestroy(c->stream);
  delete c;
  return SGLC_OK;
}

const char *sglc_last_error(sglc_context *ctx) {
  if (!ctx) return "null context";
  return reinterpret_cast<Ctx *>(ctx)->err.c_str();
}

sglc_status sglc_release(sglc_context *ctx, sglc_handle h) {
  CTX;
  auto it = c->objects.find(h);
  if (it == c->objects.end()) return c->fail(SGLC_ERR_INVALID_HANDLE, "release: unknown handle");
  CK(cudaStreamSynchronize(c->stream));
  if (it->second.kind == K_TEX) freeTexture(it->second.tex, c->freeEpoch);
  if (it->second.kind == K_VAO) {
    cudaFree(it->second.vao.attr);
    cudaFree(it->second.vao.idx);
    c->freeEpoch++;
  }
  c->objects.erase(it);
  return SGLC_OK;
}

sglc_status sglc_create_framebuffer(sglc_context *ctx, int32_t, sglc_handle *out) {
  CTX;
  *out = addObject(c, K_FB);
  return SGLC_OK;
}

sglc_status sglc_framebuffer_set_color_attachment(sglc_context *ctx, sglc_handle fb, sglc_handle tex, int32_t layer,
                                                  int32_t level) {
  CTX;
  GET(f, fb, K_FB);
  GET(t, tex, K_TEX);
  sglc_status s = flushClear(c);
  if (s) return s;
  f->fb.colorTex = tex;
  f->fb.colorLayer = t->tex.desc.type == SGLC_TEXTURE_CUBE ? layer : 0;
  f->fb.colorLevel = level;
  f->fb.colorReady = true;
  return SGLC_OK;
}

sglc_status sglc_framebuffer_set_depth_attachment(sglc_context *ctx, sglc_handle fb, sglc_handle tex) {
  CTX;
  GET(f, fb, K_FB);
  GET(t, tex, K_TEX);
  (void) t;
  sglc_status s = flushClear(c);
  if (s) return s;
  f->fb.depthTex = tex;
  f->fb.depthReady = true;
  return SGLC_OK;
}

sglc_status sglc_framebuffer_is_valid(sglc_context *ctx, sglc_handle fb, int32_t *valid) {
  CTX;
  GET(f, fb, K_FB);
  *valid = f->fb.colorReady || f->fb.depthReady;
  return SGLC_OK;
}

sglc_status sglc_create_texture(sglc_context *ctx, const sglc_texture_desc *d, sglc_handle *out) {
  CTX;
  if (!d || !out) return c->fail(SGLC_ERR_INVALID_VALUE, "createTexture: null argument");
  if (d->format != SGLC_FORMAT_RGBA8 && d->format != SGLC_FORMAT_FLOAT32)
    return c->fail(SGLC_ERR_INVALID_VALUE, "createTexture: unknown format");
  if (d->type != SGLC_TEXTURE_2D && d->type != SGLC_TEXTURE_CUBE)
    return c->fail(SGLC_ERR_INVALID_VALUE, "createTexture: unknown type");
  if (d->width <= 0 || d->height <= 0 || d->width > 32768 || d->height > 32768)
    return c->fail(SGLC_ERR_INVALID_VALUE, "createTexture: size out of range");
  if (d->layout < LAYOUT_LINEAR || d->layout > LAYOUT_MORTON)
    return c->fail(SGLC_ERR_INVALID_VALUE, "createTexture: unknown layout");
  int h = addObject(c, K_TEX);
  TexObj &t = c->objects[h].tex;
  t.desc = *d;
  t.layers = d->type == SGLC_TEXTURE_CUBE ? 6 : 1;
  *out = h;
  return SGLC_OK;
}

sglc_status sglc_texture_set_sampler_desc(sglc_context *ctx, sglc_handle tex, const sglc_sampler_desc *s) {
  CTX;
  GET(t, tex, K_TEX);
  t->tex.sampler = *s;
  return SGLC_OK;
}

sglc_status sglc_texture_init_image_data(sglc_context *ctx, sglc_handle tex) {
  CTX;
  GET(t, tex, K_TEX);
  if (t->tex.allocated) return SGLC_OK;
  return allocTexture(c, t->tex);
}

sglc_status sglc_texture_set_image_data(sglc_context *ctx, sglc_handle tex, int32_t layer_count,
                                        const void *const *layers, size_t bytes_per_layer) {
  CTX;
  GET(t, tex, K_TEX);
  TexObj &T = t->tex;
  if (T.desc.multi_sample) return c->fail(SGLC_ERR_INVALID_VALUE, "setImageData: multi sample texture");
  if (layer_count < T.layers || !layers) return c->fail(SGLC_ERR_INVALID_VALUE, "setImageData: layer count");
  if (bytes_per_layer < (size_t) T.desc.width * T.desc.height * 4)
    return c->fail(SGLC_ERR_INVALID_VALUE, "setImageData: size not match");
  sglc_status s = allocTexture(c, T);
  if (s) return s;
  for (int l = 0; l < T.layers; l++) {
    s = uploadLevel(c, T, l, 0, layers[l]);
    if (s) return s;
    // TextureImageSoft::generateMipmap (SamplerSoft.h:89-115) on the device
    for (int lev = 1; lev < T.levels; lev++) launchMipLevel(devTex(T), l, lev, T.desc.format == SGLC_FORMAT_FLOAT32, c->stream);
  }
  CK(cudaGetLastError());
  return SGLC_OK;
}

sglc_status sglc_texture_set_level_data(sglc_context *ctx, sglc_handle tex, int32_t layer, int32_t level,
                                        const void *data, size_t bytes) {
  CTX;
  GET(t, tex, K_TEX);
  TexObj &T = t->tex;
  sglc_status s = allocTexture(c, T);
  if (s) return s;
  if (layer < 0 || layer >= T.layers || level < 0 || level >= T.levels || T.desc.multi_sample)
    return c->fail(SGLC_ERR_INVALID_VALUE, "set_level_data: bad layer/level");
  if (bytes < (size_t) T.w[level] * T.h[level] * 4) return c->fail(SGLC_ERR_INVALID_VALUE, "set_level_data: size");
  return uploadLevel(c, T, layer, level, data);
}

sglc_status sglc_texture_read_image(sglc_context *ctx, sglc_handle tex, int32_t layer, int32_t level, int32_t resolved,
                                    void *out, size_t bytes) {
  CTX;
  GET(t, tex, K_TEX);
  TexObj &T = t->tex;
  sglc_status s = flushClear(c);
  if (s) return s;
  if (!T.allocated) {
    s = allocTexture(c, T);
    if (s) return s;
  }
  if (layer < 0 || layer >= T.layers || level < 0 || level >= T.levels)
    return c->fail(SGLC_ERR_INVALID_VALUE, "read_image: bad layer/level");
  size_t n = (size_t) T.w[level] * T.h[level];
  if (T.desc.multi_sample && resolved) {
    if (!T.resolved) return c->fail(SGLC_ERR_INVALID_VALUE, "read_image: no resolved image");
    if (bytes < n * 4) return c->fail(SGLC_ERR_INVALID_VALUE, "read_image: size");
    CK(cudaMemcpyAsync(out, T.resolved, n * 4, cudaMemcpyDeviceToHost, c->stream));
  } else {
    size_t total = n * 4 * T.samplesPerTexel;
    if (bytes < total) return c->fail(SGLC_ERR_INVALID_VALUE, "read_image: size");
    const uint32_t *src = T.dev + (size_t) layer * T.layerStride + T.offset[level];
    if (T.desc.layout == LAYOUT_LINEAR) {
      CK(cudaMemcpyAsync(out, src, total, cudaMemcpyDeviceToHost, c->stream));
    } else {
      CK(c->staging.ensure(n * 4));
      launchSwizzleOut(devTex(T), layer, level, c->staging.as<uint32_t>(), c->stream);
      CK(cudaMemcpyAsync(out, c->staging.ptr, n * 4, cudaMemcpyDeviceToHost, c->stream));
    }
  }
  CK(cudaStreamSynchronize(c->stream));
  return SGLC_OK;
}

// raw texels of one level in its storage layout, padding included (Buffer::getRawDataBytesSize)
static size_t levelStorageTexels(const TexObj &T, int level) {
  int w = T.w[level], h = T.h[level];
  size_t n;
  if (T.desc.layout == LAYOUT_TILED) n = (size_t) ((w + 3) / 4) * 4 * ((h + 3) / 4) * 4;
  else if (T.desc.layout == LAYOUT_MORTON) n = (size_t) ((w + 31) / 32) * 32 * ((h + 31) / 32) * 32;
  else n = (size_t) w * h;
  return n * T.samplesPerTexel;
}

// TextureSoft::storeToFile (TextureSoft.h:195-215): layers x levels of raw storage, in order
sglc_status sglc_texture_store_to_file(sglc_context *ctx, sglc_handle tex, const char *path) {
  CTX;
  GET(t, tex, K_TEX);
  if (!path) return c->fail(SGLC_ERR_INVALID_VALUE, "store_to_file: null path");
  if (c->capturing) return c->fail(SGLC_ERR_UNSUPPORTED, "store_to_file: not capturable in a graph");
  TexObj &T = t->tex;
  sglc_status s = flushClear(c);
  if (s) return s;
  std::vector<uint32_t> host;
  if (T.allocated) {
    size_t total = 0;
    for (int l = 0; l < T.levels; l++) total += levelStorageTexels(T, l);
    host.resize(total * (size_t) T.layers);
    size_t o = 0;
    for (int layer = 0; layer < T.layers; layer++)
      for (int l = 0; l < T.levels; l++) {
        size_t n = levelStorageTexels(T, l);
        CK(cudaMemcpyAsync(host.data() + o, T.dev + (size_t) layer * T.layerStride + T.offset[l], n * 4,
                           cudaMemcpyDeviceToHost, c->stream));
        o += n;
      }
    CK(cudaStreamSynchronize(c->stream));
  }
  FILE *f = fopen(path, "wb");
  if (!f) return c->fail(SGLC_ERR_INVALID_VALUE, std::string("store_to_file: failed to open file: ") + path);
  size_t wrote = host.empty() ? 0 : fwrite(host.data(), 4, host.size(), f);
  int closed = fclose(f);
  if (wrote != host.size() || closed != 0)
    return c->fail(SGLC_ERR_INVALID_VALUE, std::string("store_to_file: failed to write file: ") + path);
  return SGLC_OK;
}

// TextureSoft::loadFromFile (TextureSoft.h:166-193)
sglc_status sglc_texture_load_from_file(sglc_context *ctx, sglc_handle tex, const char *path) {
  CTX;
  GET(t, tex, K_TEX);
  if (!path) return c->fail(SGLC_ERR_INVALID_VALUE, "load_from_file: null path");
  if (c->capturing) return c->fail(SGLC_ERR_UNSUPPORTED, "load_from_file: not capturable in a graph");
  TexObj &T = t->tex;
  FILE *f = fopen(path, "rb");
  if (!f) return c->fail(SGLC_ERR_INVALID_VALUE, std::string("load_from_file: failed to open file: ") + path);
  if (!T.allocated) {   // no image data: nothing to read
    fclose(f);
    return SGLC_OK;
  }
  size_t total = 0;
  for (int l = 0; l < T.levels; l++) total += levelStorageTexels(T, l);
  total *= (size_t) T.layers;
  std::vector<uint32_t> host(total);
  size_t got = total ? fread(host.data(), 4, total, f) : 0;
  fclose(f);
  if (got != total) return c->fail(SGLC_ERR_INVALID_VALUE, std::string("load_from_file: failed to read file: ") + path);
  sglc_status s = flushClear(c);
  if (s) return s;
  T.version++;
  size_t o = 0;
  for (int layer = 0; layer < T.layers; layer++)
    for (int l = 0; l < T.levels; l++) {
      size_t n = levelStorageTexels(T, l);
      CK(cudaMemcpyAsync(T.dev + (size_t) layer * T.layerStride + T.offset[l], host.data() + o, n * 4,
                         cudaMemcpyHostToDevice, c->stream));
      o += n;
    }
  CK(cudaStreamSynchronize(c->stream));   // the host staging vector goes out of scope
  return SGLC_OK;
}

sglc_status sglc_create_vertex_array(sglc_context *ctx, const void *vertexes, size_t vlen, size_t stride,
                                     const int32_t *indices, size_t ilen, sglc_handle *out) {
  CTX;
  if (stride == 0 || stride % 4 || stride > 256) return c->fail(SGLC_ERR_INVALID_VALUE, "vertex array: stride");
  if (!out) return c->fail(SGLC_ERR_INVALID_VALUE, "vertex array: null output");
  size_t nv = vlen / stride;
  if (nv > (size_t) 0x3fffffff || ilen / 4 > (size_t) 0x3fffffff)
    return c->fail(SGLC_ERR_INVALID_VALUE, "vertex array: too large");
  VaoObj v;
  v.stride = stride;
  v.nv = nv;
  v.nidx = ilen / 4;
  CK(cudaMalloc(&v.attr, std::max(nv * stride, (size_t) 16)));
  CK(cudaMalloc(&v.idx, std::max(v.nidx * 4, (size_t) 16)));
  if (nv) CK(cudaMemcpyAsync(v.attr, vertexes, nv * stride, cudaMemcpyHostToDevice, c->stream));
  if (v.nidx) CK(cudaMemcpyAsync(v.idx, indices, v.nidx * 4, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  int h = addObject(c, K_VAO);
  c->objects[h].vao = v;
  *out = h;
  return SGLC_OK;
}

sglc_status sglc_vertex_array_update(sglc_context *ctx, sglc_handle vao, const void *data, size_t len) {
  CTX;
  GET(v, vao, K_VAO);
  size_t n = std::min(len, v->vao.nv * v->vao.stride);
  if (n) CK(cudaMemcpyAsync(v->vao.attr, data, n, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return SGLC_OK;
}

sglc_status sglc_create_shader_program(sglc_context *ctx, sglc_handle *out) {
  CTX;
  *out = addObject(c, K_PROG);
  return SGLC_OK;
}

sglc_status sglc_program_add_define(sglc_context *ctx, sglc_handle prog, const char *name) {
  CTX;
  GET(p, prog, K_PROG);
  if (!name) return c->fail(SGLC_ERR_INVALID_VALUE, "addDefine: null name");
  p->prog.defineNames.push_back(name);
  return SGLC_OK;
}

sglc_status sglc_program_set_shaders(sglc_context *ctx, sglc_handle prog, int32_t model) {
  CTX;
  GET(p, prog, K_PROG);
  const ShaderInfo *s = findShader(model);
  if (!s) return c->fail(SGLC_ERR_UNSUPPORTED, "setShaders: unknown shading model");
  ProgObj &P = p->prog;
  P.shader = s;
  memset(P.defines, 0, sizeof(P.defines));
  for (auto &n : P.defineNames)
    for (size_t i = 0; i < s->defines.size(); i++)
      if (n == s->defines[i]) P.defines[i] = 1;
  memset(P.uniforms, 0, sizeof(P.uniforms));
  return SGLC_OK;
}

sglc_status sglc_program_set_neural_shader(sglc_context *ctx, sglc_handle prog, sglc_neural *net) {
  CTX;
  GET(p, prog, K_PROG);
  if (net && (!p->prog.shader || p->prog.shader->model != SH_PBR))
    return c->fail(SGLC_ERR_INVALID_VALUE, "set_neural_shader: the program must use the PBR shading model");
  p->prog.neural = net;
  return SGLC_OK;
}

sglc_status sglc_neural_set_test_flags(sglc_context *ctx, int32_t flags) {
  CTX;
  if (flags & ~1) return c->fail(SGLC_ERR_INVALID_VALUE, "neural_set_test_flags: unknown flag");
  c->nnTestFlags = flags;
  return SGLC_OK;
}

sglc_status sglc_create_pipeline_states(sglc_context *ctx, const sglc_render_states *s, sglc_handle *out) {
  CTX;
  if (!s) return c->fail(SGLC_ERR_INVALID_VALUE, "pipeline states: null");
  if (s->depth_func < 0 || s->depth_func > 7 || s->blend_src_rgb < 0 || s->blend_src_rgb > 9 || s->blend_dst_rgb < 0 ||
      s->blend_dst_rgb > 9 || s->blend_src_alpha < 0 || s->blend_src_alpha > 9 || s->blend_dst_alpha < 0 ||
      s->blend_dst_alpha > 9 || s->blend_func_rgb < 0 || s->blend_func_rgb > 4 || s->blend_func_alpha < 0 ||
      s->blend_func_alpha > 4)
    return c->fail(SGLC_ERR_INVALID_VALUE, "pipeline states: enum out of range");
  int h = addObject(c, K_STATES);
  c->objects[h].states = *s;
  *out = h;
  return SGLC_OK;
}

sglc_status sglc_create_uniform_block(sglc_context *ctx, const char *name, int32_t size, sglc_handle *out) {
  CTX;
  if (!name || size < 0) return c->fail(SGLC_ERR_INVALID_VALUE, "uniform block: bad arguments");
  int h = addObject(c, K_UB);
  c->objects[h].ubName = name;
  c->objects[h].ubData.assign(size, 0);
  *out = h;
  return SGLC_OK;
}

sglc_status sglc_uniform_block_set_sub_data(sglc_context *ctx, sglc_handle ub, const void *data, int32_t len,
                                            int32_t offset) {
  CTX;
  GET(u, ub, K_UB);
  if (offset < 0 || len < 0 || (size_t) offset + len > u->ubData.size())
    return c->fail(SGLC_ERR_INVALID_VALUE, "uniform block: range outside the block");
  memcpy(u->ubData.data() + offset, data, len);
  return SGLC_OK;
}

sglc_status sglc_uniform_block_set_data(sglc_context *ctx, sglc_handle ub, const void *data, int32_t len) {
  return sglc_uniform_block_set_sub_data(ctx, ub, data, len, 0);
}

sglc_status sglc_create_uniform_sampler(sglc_context *ctx, const char *name, int32_t type, int32_t format,
                                        sglc_handle *out) {
  CTX;
  if (!name) return c->fail(SGLC_ERR_INVALID_VALUE, "uniform sampler: null name");
  int h = addObject(c, K_US);
  c->objects[h].us.name = name;
  c->objects[h].us.type = type;
  c->objects[h].us.format = format;
  *out = h;
  return SGLC_OK;
}

// Sampler2DSoft / SamplerCubeSoft::setTexture (SamplerSoft.h:388-436): filter = filterMin,
// wrap = wrapS, border from the sampler desc, size of level 0 at this moment
sglc_status sglc_uniform_sampler_set_texture(sglc_context *ctx, sglc_handle us, sglc_handle tex) {
  CTX;
  GET(u, us, K_US);
  GET(t, tex, K_TEX);
  UsObj &S = u->us;
  TexObj &T = t->tex;
  S.tex = tex;
  S.filter = T.sampler.filter_min;
  S.wrap = T.sampler.wrap_s;
  if (S.format == SGLC_FORMAT_FLOAT32) {
    float b = T.sampler.border_color == SGLC_BORDER_WHITE ? 1.f : 0.f;
    memcpy(&S.border, &b, 4);
  } else {
    S.border = T.sampler.border_color == SGLC_BORDER_WHITE ? 0xFFFFFFFFu : 0u;
  }
  S.width = T.allocated ? T.w[0] : 0;
  S.height = T.allocated ? T.h[0] : 0;
  S.useMipmaps = S.filter > SGLC_FILTER_LINEAR;
  return SGLC_OK;
}

sglc_status sglc_create_shader_resources(sglc_context *ctx, sglc_handle *out) {
  CTX;
  *out = addObject(c, K_RES);
  return SGLC_OK;
}

sglc_status sglc_shader_resources_set_block(sglc_context *ctx, sglc_handle res, int32_t key, sglc_handle ub) {
  CTX;
  GET(r, res, K_RES);
  GET(u, ub, K_UB);
  (void) u;
  r->resBlocks[key] = ub;
  return SGLC_OK;
}

sglc_status sglc_shader_resources_set_sampler(sglc_context *ctx, sglc_handle res, int32_t key, sglc_handle us) {
  CTX;
  GET(r, res, K_RES);
  GET(u, us, K_US);
  (void) u;
  r->resSamplers[key] = us;
  return SGLC_OK;
}

sglc_status sglc_begin_render_pass(sglc_context *ctx, sglc_handle fb, const sglc_clear_states *s) {
  CTX;
  GET(f, fb, K_FB);
  if (!s) return c->fail(SGLC_ERR_INVALID_VALUE, "beginRenderPass: null clear states");
  sglc_status st = flushClear(c);
  if (st) return st;
  c->fb = fb;
  // make sure the attachments have storage (the reference allocates in initImageData)
  if (f->fb.colorReady) {
    Object *t = c->get(f->fb.colorTex, K_TEX);
    if (t && !t->tex.allocated) {
      st = allocTexture(c, t->tex);
      if (st) return st;
    }
  }
  if (f->fb.depthReady) {
    Object *t = c->get(f->fb.depthTex, K_TEX);
    if (t && !t->tex.allocated) {
      st = allocTexture(c, t->tex);
      if (st) return st;
    }
  }
  PendingClear &pc = c->clear;
  pc.fb = fb;
  pc.colorFlag = s->color_flag;
  pc.depthFlag = s->depth_flag;
  pc.color = u8c(s->clear_color[0] * 255) | (u8c(s->clear_color[1] * 255) << 8) | (u8c(s->clear_color[2] * 255) << 16) |
             (u8c(s->clear_color[3] * 255) << 24);
  pc.depth = s->clear_depth;
  pc.active = s->color_flag || s->depth_flag;
  return SGLC_OK;
}

sglc_status sglc_set_viewport(sglc_context *ctx, int32_t x, int32_t y, int32_t w, int32_t h) {
  CTX;
  c->vp = makeViewport(x, y, w, h);
  return SGLC_OK;
}

sglc_status sglc_set_vertex_array(sglc_context *ctx, sglc_handle vao) {
  CTX;
  GET(v, vao, K_VAO);
  (void) v;
  c->vao = vao;
  return SGLC_OK;
}

sglc_status sglc_set_shader_program(sglc_context *ctx, sglc_handle prog) {
  CTX;
  GET(p, prog, K_PROG);
  (void) p;
  c->prog = prog;
  return SGLC_OK;
}

sglc_status sglc_set_shader_resources(sglc_context *ctx, sglc_handle res) {
  CTX;
  GET(r, res, K_RES);
  Object *po = c->get(c->prog, K_PROG);
  if (!po || !po->prog.shader) return SGLC_OK;
  ProgObj &P = po->prog;
  for (auto &kv : r->resBlocks) {
    Object *u = c->get(kv.second, K_UB);
    if (!u) continue;
    for (auto &d : P.shader->uniforms) {
      if (d.samplerSlot >= 0 || u->ubName != d.name) continue;
      size_t n = std::min(u->ubData.size(), (size_t) (P.shader->uniformSize - d.offset));
      memcpy(P.uniforms + d.offset, u->ubData.data(), n);
    }
  }
  for (auto &kv : r->resSamplers) {
    Object *u = c->get(kv.second, K_US);
    if (!u) continue;
    for (auto &d : P.shader->uniforms)
      if (d.samplerSlot >= 0 && u->us.name == d.name) P.samplers[d.samplerSlot] = kv.second;
  }
  return SGLC_OK;
}

sglc_status sglc_set_pipeline_states(sglc_context *ctx, sglc_handle st) {
  CTX;
  GET(s, st, K_STATES);
  (void) s;
  c->states = st;
  return SGLC_OK;
}

sglc_status sglc_draw(sglc_context *ctx) {
  CTX;
  return drawImpl(c);
}

}  // extern "C"

namespace {

// sglc_draw_views / sglc_draw_scenes: per-view uniforms and attachments (and, for scenes, vertex
// arrays), the bound program and states, one pipeline pass
sglc_status drawBatch(sglc_context *ctx, const sglc_handle *vaos, const sglc_handle *framebuffers,
                      const sglc_handle *resources, int32_t count, const sglc_clear_states *clear, const char *what) {
  CTX;
  const std::string w(what);
  if (count <= 0 || !framebuffers || !resources)
    return c->fail(SGLC_ERR_INVALID_VALUE, w + ": need at least one view");
  if (count > (1 << 20))   // fragment records carry the view in 21 bits of their meta word
    return c->fail(SGLC_ERR_INVALID_VALUE, w + ": at most 2^20 views in one call");
  Object *po = c->get(c->prog, K_PROG);
  if (!po || !po->prog.shader) return c->fail(SGLC_ERR_INVALID_VALUE, w + ": no shader program bound");
  ProgObj &P = po->prog;
  BatchViews bv;
  bv.count = count;
  bv.vaos = vaos;
  bv.fbs = framebuffers;
  bv.clear = clear;
  bv.uniforms.resize((size_t) count * kUniformBytes);
  for (int v = 0; v < count; v++) {
    Object *fo = c->get(framebuffers[v], K_FB);
    Object *r = c->get(resources[v], K_RES);
    if (!fo || !r) return c->fail(SGLC_ERR_INVALID_HANDLE, w + ": invalid framebuffer or resources handle");
    if (vaos && !c->get(vaos[v], K_VAO)) return c->fail(SGLC_ERR_INVALID_HANDLE, w + ": invalid vertex array handle");
    for (int h : {fo->fb.colorReady ? fo->fb.colorTex : 0, fo->fb.depthReady ? fo->fb.depthTex : 0}) {
      Object *t = c->get(h, K_TEX);
      if (t && !t->tex.allocated) {
        sglc_status st = allocTexture(c, t->tex);
        if (st) return st;
      }
    }
    // this view's uniforms: the program's current uniforms with the view's blocks applied, as
    // ShaderProgram::bindResources does for a single draw (ShaderProgram.h:27-54)
    uint8_t *dst = bv.uniforms.data() + (size_t) v * kUniformBytes;
    memcpy(dst, P.uniforms, kUniformBytes);
    for (auto &kv : r->resBlocks) {
      Object *u = c->get(kv.second, K_UB);
      if (!u) continue;
      for (auto &d : P.shader->uniforms) {
        if (d.samplerSlot >= 0 || u->ubName != d.name) continue;
        size_t n = std::min(u->ubData.size(), (size_t) (P.shader->uniformSize - d.offset));
        memcpy(dst + d.offset, u->ubData.data(), n);
      }
    }
  }
  // samplers are shared by all views: view 0's resources bind them
  sglc_status st = sglc_set_shader_resources(ctx, resources[0]);
  if (st) return st;
  if (vaos) {   // scenes bring their own resources: each must bind what scene 0 bound
    for (int v = 1; v < count; v++) {
      Object *r = c->get(resources[v], K_RES);
      for (auto &kv : r->resSamplers) {
        Object *u = c->get(kv.second, K_US);
        if (!u) continue;
        for (auto &d : P.shader->uniforms) {
          if (d.samplerSlot < 0 || u->us.name != d.name) continue;
          Object *b = c->get(P.samplers[d.samplerSlot], K_US);
          const UsObj &x = u->us;
          if (!b || b->us.tex != x.tex || b->us.filter != x.filter || b->us.wrap != x.wrap || b->us.border != x.border)
            return c->fail(SGLC_ERR_INVALID_VALUE, w + ": every scene must bind the textures and sampler states of "
                                                       "scene 0");
        }
      }
    }
  }
  return drawImpl(c, &bv);
}

}  // namespace

extern "C" {

sglc_status sglc_draw_views(sglc_context *ctx, const sglc_handle *framebuffers, const sglc_handle *resources,
                            int32_t count, const sglc_clear_states *clear) {
  return drawBatch(ctx, nullptr, framebuffers, resources, count, clear, "draw_views");
}

sglc_status sglc_draw_scenes(sglc_context *ctx, const sglc_handle *vertex_arrays, const sglc_handle *framebuffers,
                             const sglc_handle *resources, int32_t count, const sglc_clear_states *clear) {
  if (!vertex_arrays) {
    Ctx *c = reinterpret_cast<Ctx *>(ctx);
    return c ? c->fail(SGLC_ERR_INVALID_VALUE, "draw_scenes: no vertex arrays") : SGLC_ERR_INVALID_VALUE;
  }
  return drawBatch(ctx, vertex_arrays, framebuffers, resources, count, clear, "draw_scenes");
}

sglc_status sglc_set_capacity(sglc_context *ctx, const sglc_capacity *cap) {
  CTX;
  if (c->capturing) return c->fail(SGLC_ERR_INVALID_VALUE, "set_capacity: not allowed during a graph capture");
  if (!cap) {
    c->capSet = false;
    return SGLC_OK;
  }
  if (cap->clip_vertices < 1 || cap->clip_polygons < 1 || cap->appended_primitives < 1 || cap->bin_entries < 1)
    return c->fail(SGLC_ERR_INVALID_VALUE, "set_capacity: every capacity must be at least 1");
  CK(c->sticky.ensure(sizeof(int)));
  CK(cudaMemsetAsync(c->sticky.ptr, 0, sizeof(int), c->stream));
  c->cap = *cap;
  c->capSet = true;
  return SGLC_OK;
}

sglc_status sglc_get_peak_counts(sglc_context *ctx, sglc_capacity *out) {
  CTX;
  if (!out) return c->fail(SGLC_ERR_INVALID_VALUE, "get_peak_counts: null output");
  *out = c->peak;
  out->heavy_first = 1;
  out->fragments = 0;
  if (c->peakChunks.ptr) {   // fragment records the deferred draws used, in whole chunks
    CK(cudaMemcpyAsync(c->hostCounters + 10, c->peakChunks.ptr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemsetAsync(c->peakChunks.ptr, 0, sizeof(int), c->stream));
    CK(cudaStreamSynchronize(c->stream));
    out->fragments = (int64_t) c->hostCounters[10] * kChunk;
  }
  c->peak = sglc_capacity{};
  return SGLC_OK;
}

sglc_status sglc_get_overflow(sglc_context *ctx, int32_t *flags) {
  CTX;
  if (!flags) return c->fail(SGLC_ERR_INVALID_VALUE, "get_overflow: null output");
  if (c->capturing) return c->fail(SGLC_ERR_INVALID_VALUE, "get_overflow: not allowed during a graph capture");
  *flags = 0;
  if (!c->sticky.ptr) return SGLC_OK;
  CK(cudaMemcpyAsync(c->hostCounters + 8, c->sticky.ptr, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemsetAsync(c->sticky.ptr, 0, sizeof(int), c->stream));
  CK(cudaStreamSynchronize(c->stream));
  *flags = c->hostCounters[8];
  return SGLC_OK;
}

sglc_status sglc_end_render_pass(sglc_context *ctx) {
  CTX;
  return flushClear(c);
}

sglc_status sglc_wait_idle(sglc_context *ctx) {
  CTX;
  sglc_status s = flushClear(c);
  if (s) return s;
  CK(cudaStreamSynchronize(c->stream));
  return SGLC_OK;
}

sglc_status sglc_set_enable_early_z(sglc_context *ctx, int32_t enable) {
  CTX;
  c->earlyZ = enable != 0;
  return SGLC_OK;
}

sglc_status sglc_get_draw_stats(sglc_context *ctx, sglc_draw_stats *out) {
  CTX;
  CK(cudaStreamSynchronize(c->stream));
  if (c->evPending) {
    CK(cudaEventElapsedTime(&c->stats.geometry_ms, c->ev[0], c->ev[1]));
    CK(cudaEventElapsedTime(&c->stats.binning_ms, c->ev[1], c->ev[2]));
    CK(cudaEventElapsedTime(&c->stats.raster_ms, c->ev[2], c->ev[3]));
    c->stats.coverage_ms = c->stats.shading_ms = c->stats.rop_ms = 0.f;
    if (c->evDeferred) {
      CK(cudaEventElapsedTime(&c->stats.coverage_ms, c->ev[2], c->ev[4]));
      CK(cudaEventElapsedTime(&c->stats.shading_ms, c->ev[4], c->ev[5]));
      CK(cudaEventElapsedTime(&c->stats.rop_ms, c->ev[5], c->ev[3]));
    }
    if (c->statsLevel >= 2) {
      unsigned long long n = 0;
      CK(cudaMemcpy(&n, c->fragCounter, sizeof(n), cudaMemcpyDeviceToHost));
      c->stats.fragments_shaded = (int64_t) n;
    }
    c->evPending = false;
  }
  *out = c->stats;
  return SGLC_OK;
}

sglc_status sglc_set_stats_level(sglc_context *ctx, int32_t level) {
  CTX;
  if (level < 0 || level > 2) return c->fail(SGLC_ERR_INVALID_VALUE, "stats level must be 0, 1 or 2");
  c->statsLevel = level;
  c->stats.fragments_shaded = 0;
  return SGLC_OK;
}

sglc_status sglc_get_stream(sglc_context *ctx, void **stream) {
  CTX;
  *stream = c->stream;
  return SGLC_OK;
}

sglc_status sglc_set_deferred_shading(sglc_context *ctx, int32_t enable) {
  CTX;
  c->deferredShading = enable != 0;
  return SGLC_OK;
}

sglc_status sglc_set_tma_store(sglc_context *ctx, int32_t enable) {
  CTX;
  c->tmaStore = enable != 0;
  return SGLC_OK;
}

sglc_status sglc_set_tile_size(sglc_context *ctx, int32_t tile) {
  CTX;
  if (tile != 16 && tile != 8)
    return c->fail(SGLC_ERR_UNSUPPORTED, "set_tile_size: raster tiles are 16 (16x16 pixels) or 8 (16x8) high");
  c->tileH = tile;
  return SGLC_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------------
// CUDA graphs
// ------------------------------------------------------------------------------------------------
struct sglc_graph {
  sglc_context *ctx = nullptr;
  unsigned long long epoch = 0;      // g_freeEpoch when the capture began
  unsigned long long ctxEpoch = 0;   // the context's free count when the capture began
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void *> hostBufs;
};

extern "C" {

sglc_status sglc_graph_begin(sglc_context *ctx) {
  CTX;
  if (c->capturing) return c->fail(SGLC_ERR_INVALID_VALUE, "graph_begin: a capture is already in progress");
  if (!c->capSet) return c->fail(SGLC_ERR_INVALID_VALUE, "graph_begin: set capacities first (sglc_set_capacity)");
  sglc_status st = flushClear(c);
  if (st) return st;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeRelaxed));
  c->captureEpoch = g_freeEpoch.load();
  c->captureCtxEpoch = c->freeEpoch.load();
  c->capturing = true;
  DevBuf::capturing = true;
  return SGLC_OK;
}

sglc_status sglc_graph_end(sglc_context *ctx, sglc_graph **out) {
  CTX;
  if (!out) return c->fail(SGLC_ERR_INVALID_VALUE, "graph_end: null output");
  *out = nullptr;
  if (!c->capturing) return c->fail(SGLC_ERR_INVALID_VALUE, "graph_end: no capture in progress");
  flushClear(c);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  c->capturing = false;
  DevBuf::capturing = false;
  std::vector<void *> bufs;
  bufs.swap(c->captureHostBufs);
  if (e != cudaSuccess) {
    for (void *h : bufs) cudaFreeHost(h);
    if (g) cudaGraphDestroy(g);
    return c->fail(SGLC_ERR_DEVICE, std::string("graph_end: capture failed: ") + cudaGetErrorString(e) +
                                        " (run the sequence once before capturing; no synchronising calls inside)");
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, g, 0);
  if (e != cudaSuccess) {
    for (void *h : bufs) cudaFreeHost(h);
    cudaGraphDestroy(g);
    return c->fail(SGLC_ERR_DEVICE, std::string("graph_end: instantiate: ") + cudaGetErrorString(e));
  }
  sglc_graph *gr = new sglc_graph();
  gr->ctx = ctx;
  gr->epoch = c->captureEpoch;
  gr->ctxEpoch = c->captureCtxEpoch;
  gr->graph = g;
  gr->exec = exec;
  gr->hostBufs.swap(bufs);
  *out = gr;
  return SGLC_OK;
}

sglc_status sglc_graph_launch(sglc_graph *g) {
  if (!g || !g->exec) return SGLC_ERR_INVALID_VALUE;
  Ctx *c = reinterpret_cast<Ctx *>(g->ctx);
  sglc::DeviceGuard deviceGuard(c->device);
  if (g_freeEpoch.load() != g->epoch || c->freeEpoch.load() != g->ctxEpoch)
    return c->fail(SGLC_ERR_INVALID_VALUE, "graph_launch: a buffer the graph uses was freed or grown since the capture; "
                                           "capture it again");
  CK(cudaGraphLaunch(g->exec, c->stream));
  return SGLC_OK;
}

sglc_status sglc_graph_destroy(sglc_graph *g) {
  if (!g) return SGLC_ERR_INVALID_VALUE;
  Ctx *c = reinterpret_cast<Ctx *>(g->ctx);
  sglc::DeviceGuard deviceGuard(c->device);
  cudaStreamSynchronize(c->stream);
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  for (void *h : g->hostBufs) cudaFreeHost(h);
  delete g;
  return SGLC_OK;
}

}  // extern "C"
