/*
 * TEST INFRASTRUCTURE — the CPU oracle. Not part of the product: only tests/, the smoke check and
 * bench.py's CPU-baseline arm load it (through oracle/__init__.py), and only as the checker.
 *
 * A portable C++ restatement of SoftGLRender's software pipeline, RendererSoft
 * (src/Render/Software/RendererSoft.cpp), exporting the C ABI of include/softgl_cuda.h with the
 * symbol prefix `sglo_`. It follows the reference's algorithm step for step, including its
 * floating-point evaluation order, so that on identical inputs it reproduces the reference's
 * output; it is pinned against the reference itself (oracle/_ref, built from the reference
 * sources) by tests/test_oracle_vs_reference.py and against committed golden digests made by
 * tests/golden/make_golden.py. Unlike the reference it has no x86 intrinsics, so it also builds
 * on the Arm GPU host, where it checks the CUDA path and serves as the timed CPU baseline.
 *
 * Evaluation-order facts that matter (all single precision, no contraction, -ffp-contract=off):
 *  - glm mat4*vec4 = (m0*v0 + m1*v1) + (m2*v2 + m3*v3) per component (glm type_mat4x4.inl:540-572);
 *  - glm dot(vec4) on the SIMD path is DPPS: (p0+p1)+(p2+p3) (glm simd/geometric.h:46-49);
 *    dot(vec3) = (p0+p1)+p2, dot(vec2) = p0+p1 (glm func_geometric.inl:28-60);
 *  - normalize(vec3) = v * (1/sqrt(dot(v,v))) (glm func_geometric.inl:80-88, func_exponential.inl:134-139);
 *  - barycentric: cross of the SSE lanes then one division (RendererSoft.cpp:1021-1056);
 *  - varyings: out = fma(v2,b2, fma(v1,b1, v0*b0)) (AVX2/FMA path, RendererSoft.cpp:1116-1163);
 *  - RGBA8 mix/blend/store truncate to u8 (glm func_common.inl:104-132; RendererSoft.cpp:374).
 *
 * Parallel mode (sglo_set_threads > 1, used only for the CPU baseline): each thread owns a band of
 * rows and runs every primitive in order, writing only its own rows. Every pixel therefore sees the
 * same sequence of operations as in the single-threaded reference; the result is identical.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <vector>

#include "softgl_cuda.h"

namespace {

// ------------------------------------------------------------------------------------------------
// small vector math with the reference's evaluation order
// ------------------------------------------------------------------------------------------------
struct V2 { float x, y; };
struct V3 { float x, y, z; };
struct V4 { float x, y, z, w; };

static inline V3 v3(const V4 &a) { return {a.x, a.y, a.z}; }
static inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
static inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
static inline V3 operator-(float s, V3 a) { return {s - a.x, s - a.y, s - a.z}; }
static inline V3 operator+(V3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
static inline V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
static inline float dot3(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline float dot4(V4 a, V4 b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + a.w * b.w); }
static inline float gmax(float x, float y) { return (x < y) ? y : x; }
static inline float gmin(float x, float y) { return (y < x) ? y : x; }
static inline float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
static inline V3 normalize3(V3 v) {
  float inv = 1.0f / std::sqrt(dot3(v, v));
  return v * inv;
}
static inline V3 cross3(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline V3 pow3(V3 a, V3 b) { return {std::pow(a.x, b.x), std::pow(a.y, b.y), std::pow(a.z, b.z)}; }
static inline V3 max3(V3 a, V3 b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
static inline V3 min3(V3 a, V3 b) { return {gmin(a.x, b.x), gmin(a.y, b.y), gmin(a.z, b.z)}; }

// column-major matrices as stored in the uniform blocks
static inline V4 mul44(const float *m, V4 v) {
  V4 r;
  float *o = &r.x;
  for (int i = 0; i < 4; i++) {
    float a0 = m[0 + i] * v.x, a1 = m[4 + i] * v.y, a2 = m[8 + i] * v.z, a3 = m[12 + i] * v.w;
    o[i] = (a0 + a1) + (a2 + a3);
  }
  return r;
}
// glm::mat3(mat4) * vec3 : columns 0..2, rows 0..2 (type_mat3x3.inl:468-474)
static inline V3 mul33_of44(const float *m, V3 v) {
  return {m[0] * v.x + m[4] * v.y + m[8] * v.z, m[1] * v.x + m[5] * v.y + m[9] * v.z,
          m[2] * v.x + m[6] * v.y + m[10] * v.z};
}
// mat3 stored as 3 columns of vec3 padded to 16 B
static inline V3 mul33p(const float *m, V3 v) {
  return {m[0] * v.x + m[4] * v.y + m[8] * v.z, m[1] * v.x + m[5] * v.y + m[9] * v.z,
          m[2] * v.x + m[6] * v.y + m[10] * v.z};
}
static inline V3 load3(const float *p) { return {p[0], p[1], p[2]}; }
static inline uint8_t to_u8(float f) { return (uint8_t) (int) f; }

// ------------------------------------------------------------------------------------------------
// resources
// ------------------------------------------------------------------------------------------------
struct Level {
  int w = 0, h = 0;
  int samples = 1;
  std::vector<uint32_t> data;       // w*h*samples 32-bit texels (RGBA8 packed or float bits)
  std::vector<uint32_t> resolved;   // RGBA8 multi-sample colour: the resolved image
  bool hasResolved = false;
};

struct TextureObj {
  sglc_texture_desc desc{};
  sglc_sampler_desc sampler{0, 0, SGLC_WRAP_CLAMP_TO_EDGE, SGLC_WRAP_CLAMP_TO_EDGE, SGLC_WRAP_CLAMP_TO_EDGE, 0};
  int layers = 1;
  std::vector<std::vector<Level>> img;   // [layer][level]
};

struct FramebufferObj {
  int colorTex = 0, colorLayer = 0, colorLevel = 0;
  int depthTex = 0;
  bool colorReady = false, depthReady = false;
};

struct VaoObj {
  size_t stride = 0, vertexCnt = 0;
  std::vector<uint8_t> vertexes;
  std::vector<int32_t> indices;
};

struct UniformDesc {
  const char *name;
  int offset;
  int samplerSlot;   // -1 for a block
};

struct ShaderInfo {
  int model;
  std::vector<const char *> defines;
  std::vector<UniformDesc> uniforms;
  int uniformSize;
  int varyingsCnt;   // floats actually interpolated (sizeof(ShaderVaryings)/4)
  int derivSlots;    // sampler slots whose LOD callback the FS installs (setupSamplerDerivative)
};

// Uniform / varying layouts of the reference shaders with GLM aligned types (probe-checked):
// BlinnPhongSoft.h:110-150, PbrSoft.h:29-72, BasicSoft.h:24-42.
static const ShaderInfo kShaders[] = {
    {SGLC_SHADING_BASE_COLOR, {}, {{"UniformsModel", 0, -1}, {"UniformsMaterial", 256, -1}}, 304, 0, 0},
    {SGLC_SHADING_BLINN_PHONG, {"ALBEDO_MAP", "NORMAL_MAP", "EMISSIVE_MAP", "AO_MAP"},
     {{"UniformsModel", 0, -1}, {"UniformsScene", 256, -1}, {"UniformsMaterial", 320, -1},
      {"u_albedoMap", 368, 0}, {"u_normalMap", 376, 1}, {"u_emissiveMap", 384, 2}, {"u_aoMap", 392, 3},
      {"u_shadowMap", 400, 4}}, 416, 32, 0xF},
    {SGLC_SHADING_PBR, {"ALBEDO_MAP", "NORMAL_MAP", "EMISSIVE_MAP", "AO_MAP", "METALROUGHNESS_MAP"},
     {{"UniformsModel", 0, -1}, {"UniformsScene", 256, -1}, {"UniformsMaterial", 320, -1},
      {"u_albedoMap", 368, 0}, {"u_normalMap", 376, 1}, {"u_emissiveMap", 384, 2}, {"u_aoMap", 392, 3},
      {"u_metalRoughnessMap", 400, 4}, {"u_irradianceMap", 408, 5}, {"u_prefilterMap", 416, 6}}, 432, 28, 0xF},
    // SkyboxSoft.h:24-61, IBLIrradianceSoft.h:24-56, IBLPrefilterSoft.h:24-61
    {SGLC_SHADING_SKYBOX, {"EQUIRECTANGULAR_MAP"},
     {{"UniformsModel", 0, -1}, {"u_equirectangularMap", 256, 0}, {"u_cubeMap", 264, 1}}, 272, 4, 0},
    {SGLC_SHADING_IBL_IRRADIANCE, {}, {{"UniformsModel", 0, -1}, {"u_cubeMap", 256, 0}}, 264, 4, 0},
    {SGLC_SHADING_IBL_PREFILTER, {},
     {{"UniformsModel", 0, -1}, {"UniformsPrefilter", 256, -1}, {"u_cubeMap", 264, 0}}, 272, 4, 0},
    // FxaaSoft.h:24-53
    {SGLC_SHADING_FXAA, {}, {{"UniformsQuadFilter", 0, -1}, {"u_screenTexture", 8, 0}}, 16, 2, 0},
    {SGLC_SHADING_BLINN_PHONG_DIR, {"ALBEDO_MAP", "NORMAL_MAP", "EMISSIVE_MAP", "AO_MAP"},
     {{"UniformsModel", 0, -1}, {"UniformsScene", 256, -1}, {"UniformsMaterial", 320, -1},
      {"u_albedoMap", 368, 0}, {"u_normalMap", 376, 1}, {"u_emissiveMap", 384, 2}, {"u_aoMap", 392, 3},
      {"u_shadowMap", 400, 4}}, 416, 32, 0xF},
    {SGLC_SHADING_VERTEX_COLOR, {}, {{"UniformsModel", 0, -1}, {"UniformsMaterial", 256, -1}}, 304, 4, 0},
};

static const ShaderInfo *findShader(int model) {
  for (auto &s : kShaders)
    if (s.model == model) return &s;
  return nullptr;
}

enum { MAX_SAMPLERS = 8 };

struct ProgramObj {
  std::vector<std::string> defineNames;
  const ShaderInfo *shader = nullptr;
  uint8_t defines[8] = {0};
  std::vector<uint8_t> uniforms;
  int samplers[MAX_SAMPLERS] = {0};   // uniform sampler handles bound by location
};

struct UniformBlockObj {
  std::string name;
  std::vector<uint8_t> data;
};

// Sampler state captured by Sampler2DSoft/SamplerCubeSoft::setTexture (SamplerSoft.h:388-436).
struct UniformSamplerObj {
  std::string name;
  int type = 0, format = 0;
  int tex = 0;
  int filter = SGLC_FILTER_LINEAR;
  int wrap = SGLC_WRAP_CLAMP_TO_EDGE;
  uint32_t border = 0;
  int width = 0, height = 0;
  bool useMipmaps = false;
};

struct ResourcesObj {
  std::map<int, int> blocks, samplers;
};

struct Object {
  int kind = 0;   // 1 fb 2 tex 3 vao 4 prog 5 states 6 ub 7 us 8 res
  FramebufferObj fb;
  TextureObj tex;
  VaoObj vao;
  ProgramObj prog;
  sglc_render_states states{};
  UniformBlockObj ub;
  UniformSamplerObj us;
  ResourcesObj res;
};

// ------------------------------------------------------------------------------------------------
// texture sampling (SamplerSoft.h:117-266, 311-373)
// ------------------------------------------------------------------------------------------------
struct RGBAf { float r, g, b, a; };

static inline RGBAf unpack(uint32_t c) {
  return {(float) (c & 255u), (float) ((c >> 8) & 255u), (float) ((c >> 16) & 255u), (float) (c >> 24)};
}
static inline uint32_t pack(float r, float g, float b, float a) {
  return (uint32_t) to_u8(r) | ((uint32_t) to_u8(g) << 8) | ((uint32_t) to_u8(b) << 16) | ((uint32_t) to_u8(a) << 24);
}
// glm::mix on u8vec4 with a float factor, truncating back to u8
static inline uint32_t mixRGBA(uint32_t x, uint32_t y, float a) {
  RGBAf X = unpack(x), Y = unpack(y);
  float ia = 1.f - a;
  return pack(X.r * ia + Y.r * a, X.g * ia + Y.g * a, X.b * ia + Y.b * a, X.a * ia + Y.a * a);
}
static inline uint32_t mixF(uint32_t x, uint32_t y, float a) {
  float X, Y, R;
  memcpy(&X, &x, 4);
  memcpy(&Y, &y, 4);
  R = X * (1.f - a) + Y * a;
  uint32_t r;
  memcpy(&r, &R, 4);
  return r;
}

struct SamplerView {
  const std::vector<Level> *levels;   // of one layer
  int filter, wrap;
  uint32_t border;
  bool isFloat;
};

static inline uint32_t pixelWrap(const Level &L, int x, int y, int wrap, uint32_t border) {
  int w = L.w, h = L.h;
  switch (wrap) {
    case SGLC_WRAP_REPEAT:
      x = (x & ((w - 1) + w)) & (w - 1);   // CoordMod exactly as the macro expands (SamplerSoft.h:14)
      y = (y & ((h - 1) + h)) & (h - 1);
      break;
    case SGLC_WRAP_MIRRORED_REPEAT:
      x = (x & ((2 * w - 1) + 2 * w)) & (2 * w - 1);
      y = (y & ((2 * h - 1) + 2 * h)) & (2 * h - 1);
      x -= w;
      y -= h;
      x = x >= 0 ? x : (-1 - x);
      y = y >= 0 ? y : (-1 - y);
      x = w - 1 - x;
      y = h - 1 - y;
      break;
    case SGLC_WRAP_CLAMP_TO_EDGE:
      if (x < 0) x = 0;
      if (y < 0) y = 0;
      if (x >= w) x = w - 1;
      if (y >= h) y = h - 1;
      break;
    case SGLC_WRAP_CLAMP_TO_BORDER:
      if (x < 0 || x >= w) return border;
      if (y < 0 || y >= h) return border;
      break;
  }
  if ((size_t) x < (size_t) w && (size_t) y < (size_t) h) return L.data[(size_t) y * w + x];
  return 0;
}

static inline uint32_t sampleBilinearPx(const Level &L, float ux, float uy, int wrap, uint32_t border, bool isF) {
  float fx0 = ux - 0.5f, fy0 = uy - 0.5f;
  int x = (int) std::floor(fx0);
  int y = (int) std::floor(fy0);
  uint32_t s1 = pixelWrap(L, x, y, wrap, border);
  uint32_t s2 = pixelWrap(L, x + 1, y, wrap, border);
  uint32_t s3 = pixelWrap(L, x, y + 1, wrap, border);
  uint32_t s4 = pixelWrap(L, x + 1, y + 1, wrap, border);
  float fx = fx0 - std::floor(fx0);
  float fy = fy0 - std::floor(fy0);
  if (isF) return mixF(mixF(s1, s2, fx), mixF(s3, s4, fx), fy);
  return mixRGBA(mixRGBA(s1, s2, fx), mixRGBA(s3, s4, fx), fy);
}

static inline uint32_t sampleNearest(const Level &L, float u, float v, int wrap, uint32_t border) {
  float tx = u * (float) L.w, ty = v * (float) L.h;
  return pixelWrap(L, (int) std::floor(tx), (int) std::floor(ty), wrap, border);
}

static inline uint32_t sampleBilinear(const Level &L, float u, float v, int wrap, uint32_t border, bool isF) {
  float tx = u * (float) L.w, ty = v * (float) L.h;
  return sampleBilinearPx(L, tx, ty, wrap, border, isF);
}

static uint32_t textureImpl(const SamplerView &s, float u, float v, float lod) {
  const std::vector<Level> &lv = *s.levels;
  if (lv.empty()) return 0;
  if (s.filter == SGLC_FILTER_NEAREST) return sampleNearest(lv[0], u, v, s.wrap, s.border);
  if (s.filter == SGLC_FILTER_LINEAR) return sampleBilinear(lv[0], u, v, s.wrap, s.border, s.isFloat);
  int maxLevel = (int) lv.size() - 1;
  if (s.filter == SGLC_FILTER_NEAREST_MIPMAP_NEAREST || s.filter == SGLC_FILTER_LINEAR_MIPMAP_NEAREST) {
    int level = std::min(std::max((int) std::ceil(lod + 0.5f) - 1, 0), maxLevel);
    if (s.filter == SGLC_FILTER_NEAREST_MIPMAP_NEAREST) return sampleNearest(lv[level], u, v, s.wrap, s.border);
    return sampleBilinear(lv[level], u, v, s.wrap, s.border, s.isFloat);
  }
  if (s.filter == SGLC_FILTER_NEAREST_MIPMAP_LINEAR || s.filter == SGLC_FILTER_LINEAR_MIPMAP_LINEAR) {
    int hi = std::min(std::max((int) std::floor(lod), 0), maxLevel);
    int lo = std::min(std::max(hi + 1, 0), maxLevel);
    bool nearest = s.filter == SGLC_FILTER_NEAREST_MIPMAP_LINEAR;
    uint32_t th = nearest ? sampleNearest(lv[hi], u, v, s.wrap, s.border)
                          : sampleBilinear(lv[hi], u, v, s.wrap, s.border, s.isFloat);
    if (hi == lo) return th;
    uint32_t tl = nearest ? sampleNearest(lv[lo], u, v, s.wrap, s.border)
                          : sampleBilinear(lv[lo], u, v, s.wrap, s.border, s.isFloat);
    float f = lod - std::floor(lod);
    return s.isFloat ? mixF(th, tl, f) : mixRGBA(th, tl, f);
  }
  return 0;
}

// BaseSamplerCube::convertXYZ2UV (SamplerSoft.h:311-373), including its if-chain tie order
static inline void cubeUV(float x, float y, float z, int *index, float *u, float *v) {
  float ax = std::fabs(x), ay = std::fabs(y), az = std::fabs(z);
  bool px = x > 0, py = y > 0, pz = z > 0;
  float maxAxis = 0.f, uc = 0.f, vc = 0.f;
  *index = 0;
  if (px && ax >= ay && ax >= az) { maxAxis = ax; uc = -z; vc = y; *index = 0; }
  if (!px && ax >= ay && ax >= az) { maxAxis = ax; uc = z; vc = y; *index = 1; }
  if (py && ay >= ax && ay >= az) { maxAxis = ay; uc = x; vc = -z; *index = 2; }
  if (!py && ay >= ax && ay >= az) { maxAxis = ay; uc = x; vc = z; *index = 3; }
  if (pz && az >= ax && az >= ay) { maxAxis = az; uc = x; vc = y; *index = 4; }
  if (!pz && az >= ax && az >= ay) { maxAxis = az; uc = -x; vc = y; *index = 5; }
  vc = -vc;
  *u = 0.5f * (uc / maxAxis + 1.0f);
  *v = 0.5f * (vc / maxAxis + 1.0f);
}

// mip chain (SamplerSoft.h:89-115, 240-252)
static void generateMips(std::vector<Level> &levels, bool isF) {
  int w = levels[0].w, h = levels[0].h;
  uint32_t count = (uint32_t) std::floor(std::log2((double) std::max(w, h))) + 1;
  levels.resize(1);
  for (uint32_t l = 1; l < count; l++) {
    Level L;
    L.w = std::max(1, w >> l);
    L.h = std::max(1, h >> l);
    L.data.assign((size_t) L.w * L.h, 0);
    const Level &in = levels[l - 1];
    float rx = (float) in.w / (float) L.w, ry = (float) in.h / (float) L.h;
    float dx = 0.5f * rx, dy = 0.5f * ry;
    for (int y = 0; y < L.h; y++)
      for (int x = 0; x < L.w; x++) {
        float u = (float) x * rx + dx, v = (float) y * ry + dy;
        L.data[(size_t) y * L.w + x] = sampleBilinearPx(in, u, v, SGLC_WRAP_CLAMP_TO_EDGE, 0, isF);
      }
    levels.push_back(std::move(L));
  }
}

// ------------------------------------------------------------------------------------------------
// context and draw
// ------------------------------------------------------------------------------------------------
struct Viewport {
  float x = 0, y = 0, width = 0, height = 0, minDepth = 0, maxDepth = 1;
  V4 innerO{0, 0, 0, 0}, innerP{0, 0, 0, 1};
  float absMinDepth = 0, absMaxDepth = 1;
};

struct VertexH {
  const float *attr;          // raw attribute floats
  float *vary;                // varyings (aligned count)
  V4 clipPos, fragPos;
  int clipMask;
};

struct Prim {
  int idx[3];
  bool discard, frontFacing;
};

static const V4 kClipPlanes[6] = {{-1, 0, 0, 1}, {1, 0, 0, 1}, {0, -1, 0, 1},
                                  {0, 1, 0, 1},  {0, 0, -1, 1}, {0, 0, 1, 1}};

struct Ctx {
  std::map<int, Object> objects;
  int next = 1;
  std::string err;
  int threads = 1;
  bool earlyZ = true;
  Viewport vp;
  int fb = 0, vao = 0, prog = 0, states = 0;
  sglc_draw_stats stats{};

  Object *get(int h, int kind) {
    auto it = objects.find(h);
    if (it == objects.end() || it->second.kind != kind) return nullptr;
    return &it->second;
  }
  sglc_status fail(sglc_status s, const char *msg) {
    err = msg;
    return s;
  }
};

// Everything one draw needs, resolved from handles.
struct DrawState {
  const ShaderInfo *shader;
  const uint8_t *u;            // program uniform bytes
  const uint8_t *def;
  SamplerView samp[MAX_SAMPLERS][6];
  bool sampBound[MAX_SAMPLERS];
  int sampW[MAX_SAMPLERS], sampH[MAX_SAMPLERS];
  bool sampMip[MAX_SAMPLERS];
  const Level *shadowLevel0;
  const sglc_render_states *rs;
  Level *color;   // colour attachment level (may be null)
  Level *depth;
  int samples;
  Viewport vp;
  int varyCnt, varyAligned;
  bool earlyZ;
};

// uniform accessors (byte offsets of UniformsModel/Scene/Material inside ShaderUniforms)
static inline const float *U_MVP(const uint8_t *u) { return (const float *) (u + 80); }
static inline const float *U_MODEL(const uint8_t *u) { return (const float *) (u + 16); }
static inline const float *U_ITMODEL(const uint8_t *u) { return (const float *) (u + 144); }
static inline const float *U_SHADOWMVP(const uint8_t *u) { return (const float *) (u + 192); }
static inline int32_t U_REVERSEZ(const uint8_t *u) { return *(const int32_t *) (u + 0); }
static inline V3 U_AMBIENT(const uint8_t *u) { return load3((const float *) (u + 256)); }
static inline V3 U_CAMPOS(const uint8_t *u) { return load3((const float *) (u + 272)); }
static inline V3 U_LIGHTPOS(const uint8_t *u) { return load3((const float *) (u + 288)); }
static inline V3 U_LIGHTCOLOR(const uint8_t *u) { return load3((const float *) (u + 304)); }
static inline int32_t U_ENABLE_LIGHT(const uint8_t *u, int base) { return *(const int32_t *) (u + base + 0); }
static inline int32_t U_ENABLE_IBL(const uint8_t *u, int base) { return *(const int32_t *) (u + base + 4); }
static inline int32_t U_ENABLE_SHADOW(const uint8_t *u, int base) { return *(const int32_t *) (u + base + 8); }
static inline float U_KSPEC(const uint8_t *u, int base) { return *(const float *) (u + base + 16); }
static inline float U_POINTSIZE(const uint8_t *u, int base) { return *(const float *) (u + base + 12); }
static inline V4 U_BASECOLOR(const uint8_t *u, int base) {
  const float *p = (const float *) (u + base + 32);
  return {p[0], p[1], p[2], p[3]};
}

// ---- vertex shaders (BasicSoft.h:66-69, BlinnPhongSoft.h:185-203, PbrSoft.h:110-127) ----------
static void runVS(const DrawState &ds, const float *a, float *v, V4 *pos) {
  const uint8_t *u = ds.u;
  const uint8_t *def = ds.def;
  V4 position{a[0], a[1], a[2], 1.0f};
  *pos = mul44(U_MVP(u), position);
  switch (ds.shader->model) {
    case SGLC_SHADING_BASE_COLOR:
      break;
    case SGLC_SHADING_FXAA:   // FxaaSoft.h:60-63: the quad is already in clip space
      *pos = position;
      v[0] = a[4];
      v[1] = a[5];
      break;
    case SGLC_SHADING_SKYBOX:   // SkyboxSoft.h:67-76
      *pos = {pos->x, pos->y, pos->w, pos->w};
      if (U_REVERSEZ(u)) pos->z = 0.f;
      v[0] = a[0]; v[1] = a[1]; v[2] = a[2];
      break;
    case SGLC_SHADING_IBL_IRRADIANCE:   // IBLIrradianceSoft.h:62-67, IBLPrefilterSoft.h:67-72
    case SGLC_SHADING_IBL_PREFILTER:
      pos->z = pos->w;
      v[0] = a[0]; v[1] = a[1]; v[2] = a[2];
      break;
    case SGLC_SHADING_VERTEX_COLOR:
      v[0] = a[4];
      v[1] = a[5];
      v[2] = a[6];
      v[3] = a[7];
      break;
    case SGLC_SHADING_BLINN_PHONG:
    case SGLC_SHADING_BLINN_PHONG_DIR:
    case SGLC_SHADING_PBR: {
      bool bp = ds.shader->model != SGLC_SHADING_PBR;
      v[0] = a[4];
      v[1] = a[5];
      if (bp) {
        V4 s = mul44(U_SHADOWMVP(u), position);
        v[20] = s.x; v[21] = s.y; v[22] = s.z; v[23] = s.w;
      }
      V3 world = v3(mul44(U_MODEL(u), position));
      V3 nvec = mul33_of44(U_MODEL(u), load3(a + 8));
      V3 ldir = (ds.shader->model == SGLC_SHADING_BLINN_PHONG_DIR) ? U_LIGHTPOS(u) : U_LIGHTPOS(u) - world;
      V3 cdir = U_CAMPOS(u) - world;
      v[8] = world.x; v[9] = world.y; v[10] = world.z;
      v[4] = nvec.x; v[5] = nvec.y; v[6] = nvec.z;
      v[16] = ldir.x; v[17] = ldir.y; v[18] = ldir.z;
      v[12] = cdir.x; v[13] = cdir.y; v[14] = cdir.z;
      if (def[1]) {   // NORMAL_MAP
        V3 N = normalize3(mul33p(U_ITMODEL(u), load3(a + 8)));
        V3 T = normalize3(mul33p(U_ITMODEL(u), load3(a + 12)));
        V3 Tn = normalize3(T - dot3(T, N) * N);
        int o = bp ? 24 : 20;
        v[o] = N.x; v[o + 1] = N.y; v[o + 2] = N.z;
        v[o + 4] = Tn.x; v[o + 5] = Tn.y; v[o + 6] = Tn.z;
      }
      break;
    }
  }
}

static inline int clipMaskOf(V4 c) {
  int m = 0;
  if (c.w < c.x) m |= 1;
  if (c.w < -c.x) m |= 2;
  if (c.w < c.y) m |= 4;
  if (c.w < -c.y) m |= 8;
  if (c.w < c.z) m |= 16;
  if (c.w < -c.z) m |= 32;
  return m;
}

// ---- fragment shading -------------------------------------------------------------------------
struct FragIn {
  const float *v;      // interpolated varyings
  float dudx, dvdx, dudy, dvdy;   // texcoord differences across the quad (p1-p0, p2-p0)
};

static inline float lodOf(const DrawState &ds, int slot, const FragIn &f) {
  // ShaderSoft::getSampler2DLod (Render/Software/ShaderSoft.h:117-133)
  float tw = (float) ds.sampW[slot], th = (float) ds.sampH[slot];
  float dxx = f.dudx * tw, dxy = f.dvdx * th;
  float dyx = f.dudy * tw, dyy = f.dvdy * th;
  float d = gmax(dxx * dxx + dxy * dxy, dyx * dyx + dyy * dyy);
  return gmax(0.5f * std::log2(d), 0.0f);
}

static inline V4 tex2D(const DrawState &ds, int slot, float u, float v, const FragIn &f) {
  float lod = 0.f;
  if (ds.sampMip[slot]) lod += lodOf(ds, slot, f);
  RGBAf c = unpack(textureImpl(ds.samp[slot][0], u, v, lod));
  return {c.r / 255.f, c.g / 255.f, c.b / 255.f, c.a / 255.f};
}

static inline V4 texCube(const DrawState &ds, int slot, V3 d, float lod) {
  int face;
  float u, v;
  cubeUV(d.x, d.y, d.z, &face, &u, &v);
  RGBAf c = unpack(textureImpl(ds.samp[slot][face], u, v, lod));
  return {c.r / 255.f, c.g / 255.f, c.b / 255.f, c.a / 255.f};
}

static V3 normalFromMap(const DrawState &ds, const FragIn &f, int nOff, int tOff) {
  const float *v = f.v;
  if (ds.def[1]) {
    V3 N = normalize3(load3(v + nOff));
    V3 T = normalize3(load3(v + tOff));
    T = normalize3(T - dot3(T, N) * N);
    V3 B = cross3(T, N);
    V4 t = tex2D(ds, 1, v[0], v[1], f);
    V3 tn = {t.x * 2.0f - 1.0f, t.y * 2.0f - 1.0f, t.z * 2.0f - 1.0f};
    V3 r = {T.x * tn.x + B.x * tn.y + N.x * tn.z, T.y * tn.x + B.y * tn.y + N.y * tn.z,
            T.z * tn.x + B.z * tn.y + N.z * tn.z};
    return normalize3(r);
  }
  return normalize3(load3(v + 4));
}

static float shadowCalc(const DrawState &ds, const FragIn &f, V3 normal) {
  // BlinnPhongSoft.h:247-271
  const float *v = f.v;
  V4 fp{v[20], v[21], v[22], v[23]};
  V3 proj = {fp.x / fp.w, fp.y / fp.w, fp.z / fp.w};
  float cur = proj.z;
  if (cur < 0.f || cur > 1.f) return 0.0f;
  float bias = gmax(0.00025f * (1.0f - dot3(normal, normalize3(load3(v + 16)))), 0.00005f);
  float shadow = 0.0f;
  const Level *L0 = ds.shadowLevel0;
  float ox = 1.0f / (float) (L0 ? L0->w : 0), oy = 1.0f / (float) (L0 ? L0->h : 0);
  int reverseZ = U_REVERSEZ(ds.u);
  for (int x = -1; x <= 1; ++x)
    for (int y = -1; y <= 1; ++y) {
      float cu = proj.x + (float) x * ox, cv = proj.y + (float) y * oy;
      uint32_t bits = textureImpl(ds.samp[4][0], cu, cv, 0.f);
      float pcf;
      memcpy(&pcf, &bits, 4);
      if (reverseZ) shadow += cur + bias < pcf ? 1.0f : 0.0f;
      else shadow += cur - bias > pcf ? 1.0f : 0.0f;
    }
  shadow /= 9.0f;
  return shadow;
}

static V4 fsBlinnPhong(const DrawState &ds, const FragIn &f, bool directional) {
  // BlinnPhongSoft.h:273-324 (point) and the directional variant (oracle/ref/extra_shaders_soft.h)
  const uint8_t *u = ds.u;
  const float *v = f.v;
  const float specExp = directional ? 32.f : 128.f;
  const float rangeInv = 1.0f / 5.f;
  V4 base = ds.def[0] ? tex2D(ds, 0, v[0], v[1], f) : U_BASECOLOR(u, 320);
  V3 N = normalFromMap(ds, f, 24, 28);
  float ao = 1.f;
  if (ds.def[3]) ao = tex2D(ds, 3, v[0], v[1], f).x;
  V3 baseRgb = {base.x, base.y, base.z};
  V3 ambient = baseRgb * U_AMBIENT(u) * ao;
  V3 diffuseC{0, 0, 0}, specC{0, 0, 0}, emis{0, 0, 0};
  if (U_ENABLE_LIGHT(u, 320)) {
    V3 ldirRaw = load3(v + 16);
    float att = 1.0f;
    if (!directional) {
      V3 lDir = ldirRaw * rangeInv;
      att = gclamp(1.0f - dot3(lDir, lDir), 0.0f, 1.0f);
    }
    V3 L = normalize3(ldirRaw);
    float diffuse = gmax(dot3(N, L), 0.0f);
    diffuseC = directional ? U_LIGHTCOLOR(u) * baseRgb * diffuse : U_LIGHTCOLOR(u) * baseRgb * diffuse * att;
    V3 C = normalize3(load3(v + 12));
    V3 H = normalize3(L + C);
    float sa = gmax(dot3(N, H), 0.0f);
    float p = std::pow(sa, specExp);
    specC = U_KSPEC(u, 320) * V3{p, p, p};
    if (U_ENABLE_SHADOW(u, 320)) {
      float shadow = 1.0f - shadowCalc(ds, f, N);
      diffuseC = diffuseC * shadow;
      specC = specC * shadow;
    }
  }
  if (ds.def[2]) {
    V4 e = tex2D(ds, 2, v[0], v[1], f);
    emis = {e.x, e.y, e.z};
  }
  V3 c = ambient + diffuseC + specC + emis;
  return {c.x, c.y, c.z, base.w};
}

static V4 fsPbr(const DrawState &ds, const FragIn &f) {
  // PbrSoft.h:168-322
  const float PI = 3.14159265359f;
  const uint8_t *u = ds.u;
  const float *v = f.v;
  const float rangeInv = 1.0f / 5.f;
  V4 arg = ds.def[0] ? tex2D(ds, 0, v[0], v[1], f) : U_BASECOLOR(u, 320);
  V3 albedo = pow3({arg.x, arg.y, arg.z}, {2.2f, 2.2f, 2.2f});
  float metallic = 0.0f, roughness = 1.0f;
  if (ds.def[4]) {
    V4 mr = tex2D(ds, 4, v[0], v[1], f);
    metallic = mr.z;
    roughness = mr.y;
  }
  float ao = 1.f;
  if (ds.def[3]) ao = tex2D(ds, 3, v[0], v[1], f).x;
  V3 N = normalFromMap(ds, f, 20, 24);
  V3 V = normalize3(load3(v + 12));
  V3 mV = -V;
  V3 R = mV - N * dot3(N, mV) * 2.0f;
  V3 F0 = {0.04f, 0.04f, 0.04f};
  F0 = F0 * (1.0f - metallic) + albedo * metallic;
  V3 Lo{0, 0, 0};
  if (U_ENABLE_LIGHT(u, 320)) {
    V3 ldir = load3(v + 16);
    V3 L = normalize3(ldir);
    V3 H = normalize3(V + L);
    V3 lDir = ldir * rangeInv;
    float att = gclamp(1.0f - dot3(lDir, lDir), 0.0f, 1.0f);
    V3 radiance = U_LIGHTCOLOR(u) * att;
    // DistributionGGX
    float a = roughness * roughness;
    float a2 = a * a;
    float NdotH = gmax(dot3(N, H), 0.0f);
    float NdotH2 = NdotH * NdotH;
    float denom = (NdotH2 * (a2 - 1.0f) + 1.0f);
    denom = PI * denom * denom;
    float NDF = a2 / denom;
    // GeometrySmith
    float NdotV = gmax(dot3(N, V), 0.0f);
    float NdotL = gmax(dot3(N, L), 0.0f);
    float r1 = (roughness + 1.0f);
    float k = (r1 * r1) / 8.0f;
    float ggx2 = NdotV / (NdotV * (1.0f - k) + k);
    float ggx1 = NdotL / (NdotL * (1.0f - k) + k);
    float G = ggx1 * ggx2;
    // FresnelSchlick
    float ct = gmax(dot3(H, V), 0.0f);
    float p5 = std::pow(gclamp(1.0f - ct, 0.0f, 1.0f), 5.0f);
    V3 F = F0 + (1.0f - F0) * p5;
    V3 numerator = NDF * G * F;
    float denominator = 4.0f * gmax(dot3(N, V), 0.0f) * gmax(dot3(N, L), 0.0f) + 0.0001f;
    V3 specular = numerator / denominator;
    V3 kD = 1.0f - F;
    kD = kD * (1.0f - metallic);
    float NdL = gmax(dot3(N, L), 0.0f);
    Lo = Lo + (kD * albedo / PI + specular) * radiance * NdL;
  }
  V3 ambient{0, 0, 0};
  if (U_ENABLE_IBL(u, 320)) {
    float NdotV = gmax(dot3(N, V), 0.0f);
    float p5 = std::pow(gclamp(1.0f - NdotV, 0.0f, 1.0f), 5.0f);
    float omr = 1.0f - roughness;
    V3 F = F0 + (max3({omr, omr, omr}, F0) - F0) * p5;
    V3 kD = 1.0f - F;
    kD = kD * (1.0f - metallic);
    V4 irr = texCube(ds, 5, N, 0.f);
    V3 diffuse = V3{irr.x, irr.y, irr.z} * albedo;
    V4 pre = texCube(ds, 6, R, roughness * 4.0f);
    // EnvBRDFApprox (PbrSoft.h:209-223)
    V4 c0{-1.f, -0.0275f, -0.572f, 0.022f}, c1{1.f, 0.0425f, 1.04f, -0.04f};
    V4 r{roughness * c0.x + c1.x, roughness * c0.y + c1.y, roughness * c0.z + c1.z, roughness * c0.w + c1.w};
    float a004 = gmin(r.x * r.x, std::exp2(-9.28f * NdotV)) * r.x + r.y;
    float ABx = -1.04f * a004 + r.z;
    float ABy = 1.04f * a004 + r.w;
    ABy *= gmax(0.f, gmin(1.f, 50.0f * F.y));
    V3 env = F * ABx + ABy;
    V3 specular = V3{pre.x, pre.y, pre.z} * env;
    ambient = (kD * diffuse + specular) * ao;
  } else {
    ambient = U_AMBIENT(u) * albedo * ao;
  }
  V3 color = ambient + Lo;
  float g = 1.0f / 2.2f;
  color = pow3(color, {g, g, g});
  V3 emis{0, 0, 0};
  if (ds.def[2]) {
    V4 e = tex2D(ds, 2, v[0], v[1], f);
    emis = {e.x, e.y, e.z};
  }
  V3 c = color + emis;
  return {c.x, c.y, c.z, arg.w};
}

// ---- environment shaders drawn into cube faces by IBLGenerator (Environment.cpp:152-195) ---------
static V4 fsSkybox(const DrawState &ds, const FragIn &f) {
  // SkyboxSoft.h:84-103
  V3 wp = load3(f.v);
  if (ds.def[0]) {   // EQUIRECTANGULAR_MAP: SampleSphericalMap
    V3 dir = normalize3(wp);
    float u = std::atan2(dir.z, dir.x), v = std::asin(-dir.y);
    u = u * 0.1591f + 0.5f;
    v = v * 0.3183f + 0.5f;
    return tex2D(ds, 0, u, v, f);
  }
  return texCube(ds, 1, wp, 0.f);
}

static V4 fsIrradiance(const DrawState &ds, const FragIn &f) {
  // IBLIrradianceSoft.h:75-101
  const float PI = 3.14159265359f;
  V3 N = normalize3(load3(f.v));
  V3 irradiance{0.f, 0.f, 0.f};
  V3 up{0.0f, 1.0f, 0.0f};
  V3 right = normalize3(cross3(up, N));
  up = normalize3(cross3(N, right));
  const float sampleDelta = 0.025f;
  float nrSamples = 0.0f;
  for (float phi = 0.0f; phi < 2.0f * PI; phi += sampleDelta) {
    for (float theta = 0.0f; theta < 0.5f * PI; theta += sampleDelta) {
      V3 ts{std::sin(theta) * std::cos(phi), std::sin(theta) * std::sin(phi), std::cos(theta)};
      V3 sampleVec = ts.x * right + ts.y * up + ts.z * N;
      V4 c = texCube(ds, 0, sampleVec, 0.f);
      irradiance = irradiance + V3{c.x, c.y, c.z} * std::cos(theta) * std::sin(theta);
      nrSamples++;
    }
  }
  irradiance = PI * irradiance * (1.0f / nrSamples);
  return {irradiance.x, irradiance.y, irradiance.z, 1.0f};
}

static float radicalInverseVdC(uint32_t bits) {
  // IBLPrefilterSoft.h:93-100 (Hammersley point set, van der Corput radical inverse)
  bits = (bits << 16u) | (bits >> 16u);
  bits = ((bits & 0x55555555u) << 1u) | ((bits & 0xAAAAAAAAu) >> 1u);
  bits = ((bits & 0x33333333u) << 2u) | ((bits & 0xCCCCCCCCu) >> 2u);
  bits = ((bits & 0x0F0F0F0Fu) << 4u) | ((bits & 0xF0F0F0F0u) >> 4u);
  bits = ((bits & 0x00FF00FFu) << 8u) | ((bits & 0xFF00FF00u) >> 8u);
  return float(bits * 2.3283064365386963e-10);
}

static V4 fsPrefilter(const DrawState &ds, const FragIn &f) {
  // IBLPrefilterSoft.h:101-170
  const float PI = 3.14159265359f;
  const float srcResolution = *(const float *) (ds.u + 256), roughness = *(const float *) (ds.u + 260);
  V3 N = normalize3(load3(f.v));
  V3 V = N;
  const uint32_t SAMPLE_COUNT = 1024u;
  V3 color{0.f, 0.f, 0.f};
  float totalWeight = 0.0f;
  for (uint32_t i = 0u; i < SAMPLE_COUNT; ++i) {
    float xi0 = float(i) / float(SAMPLE_COUNT), xi1 = radicalInverseVdC(i);
    float a = roughness * roughness;
    float phi = 2.0f * PI * xi0;
    float cosTheta = std::sqrt((1.0f - xi1) / (1.0f + (a * a - 1.0f) * xi1));
    float sinTheta = std::sqrt(1.0f - cosTheta * cosTheta);
    V3 H{std::cos(phi) * sinTheta, std::sin(phi) * sinTheta, cosTheta};
    V3 upv = std::fabs(N.z) < 0.999 ? V3{0.0f, 0.0f, 1.0f} : V3{1.0f, 0.0f, 0.0f};
    V3 tangent = normalize3(cross3(upv, N));
    V3 bitangent = cross3(N, tangent);
    H = normalize3(tangent * H.x + bitangent * H.y + N * H.z);
    V3 L = normalize3(2.0f * dot3(V, H) * H - V);
    float NdotL = gmax(dot3(N, L), 0.0f);
    if (NdotL > 0.0f) {
      float a2 = a * a;
      float NdotH = gmax(dot3(N, H), 0.0f);
      float NdotH2 = NdotH * NdotH;
      float denom = (NdotH2 * (a2 - 1.0f) + 1.0f);
      denom = PI * denom * denom;
      float D = a2 / denom;
      float HdotV = gmax(dot3(H, V), 0.0f);
      float pdf = D * NdotH / (4.0f * HdotV) + 0.0001f;
      float saTexel = 4.0f * PI / (6.0f * srcResolution * srcResolution);
      float saSample = 1.0f / (float(SAMPLE_COUNT) * pdf + 0.0001f);
      float mipLevel = roughness == 0.0f ? 0.0f : 0.5f * std::log2(saSample / saTexel);
      V4 c = texCube(ds, 0, L, mipLevel);
      color = color + V3{c.x, c.y, c.z} * NdotL;
      totalWeight += NdotL;
    }
  }
  color = color / totalWeight;
  return {color.x, color.y, color.z, 1.0f};
}

// ---- FXAA screen pass (QuadFilter.cpp:12-112, FxaaSoft.h) -------------------------------------
static uint32_t textureOffsetImpl(const SamplerView &s, float u, float v, int ox, int oy) {
  // textureLodOffset at LOD 0 (SamplerSoft.h:117-165, 214-238)
  const std::vector<Level> &lv = *s.levels;
  if (lv.empty()) return 0;
  auto one = [&](const Level &L, bool nearest) -> uint32_t {
    float tx = u * (float) L.w, ty = v * (float) L.h;
    if (nearest) return pixelWrap(L, (int) std::floor(tx) + ox, (int) std::floor(ty) + oy, s.wrap, s.border);
    return sampleBilinearPx(L, tx + (float) ox, ty + (float) oy, s.wrap, s.border, s.isFloat);
  };
  bool nearest = s.filter == SGLC_FILTER_NEAREST || s.filter == SGLC_FILTER_NEAREST_MIPMAP_NEAREST ||
                 s.filter == SGLC_FILTER_NEAREST_MIPMAP_LINEAR;
  if (s.filter == SGLC_FILTER_NEAREST_MIPMAP_LINEAR || s.filter == SGLC_FILTER_LINEAR_MIPMAP_LINEAR) {
    uint32_t th = one(lv[0], nearest);
    if (lv.size() < 2) return th;
    uint32_t tl = one(lv[1], nearest);
    return s.isFloat ? mixF(th, tl, 0.f) : mixRGBA(th, tl, 0.f);
  }
  return one(lv[0], nearest);
}

static inline float fxaaQuality(float q) {   // QUALITY(q), FxaaSoft.h:74
  return q < 5.f ? 1.0f : (q > 5.f ? (q < 10.f ? 2.0f : (q < 11.f ? 4.0f : 8.0f)) : 1.5f);
}
static inline float rgb2luma(V3 c) { return dot3(c, V3{0.299f, 0.587f, 0.114f}); }
static inline float fxaaClamp01(float x) { return gclamp(x, 0.0f, 1.0f); }
static inline V3 fxaaTex(const DrawState &ds, float u, float v) {
  RGBAf c = unpack(textureImpl(ds.samp[0][0], u, v, 0.f));
  return {c.r / 255.f, c.g / 255.f, c.b / 255.f};
}
static inline V3 fxaaTexOff(const DrawState &ds, float u, float v, int ox, int oy) {
  RGBAf c = unpack(textureOffsetImpl(ds.samp[0][0], u, v, ox, oy));
  return {c.r / 255.f, c.g / 255.f, c.b / 255.f};
}

static V3 fxaaColor(const DrawState &ds, const FragIn &f) {
  // FxaaSoft.h:83-262 (FXAA 3.11-style edge walk: 12 iterations, subpixel quality 0.75)
  const float inv_x = 1.0f / *(const float *) (ds.u + 0), inv_y = 1.0f / *(const float *) (ds.u + 4);
  const float tu = f.v[0], tv = f.v[1];
  V3 colorCenter = fxaaTex(ds, tu, tv);
  float lumaCenter = rgb2luma(colorCenter);
  float lumaDown = rgb2luma(fxaaTexOff(ds, tu, tv, 0, -1));
  float lumaUp = rgb2luma(fxaaTexOff(ds, tu, tv, 0, 1));
  float lumaLeft = rgb2luma(fxaaTexOff(ds, tu, tv, -1, 0));
  float lumaRight = rgb2luma(fxaaTexOff(ds, tu, tv, 1, 0));
  float lumaMin = gmin(lumaCenter, gmin(gmin(lumaDown, lumaUp), gmin(lumaLeft, lumaRight)));
  float lumaMax = gmax(lumaCenter, gmax(gmax(lumaDown, lumaUp), gmax(lumaLeft, lumaRight)));
  float lumaRange = lumaMax - lumaMin;
  if (lumaRange < gmax(0.0312f, lumaMax * 0.125f)) return colorCenter;
  float lumaDownLeft = rgb2luma(fxaaTexOff(ds, tu, tv, -1, -1));
  float lumaUpRight = rgb2luma(fxaaTexOff(ds, tu, tv, 1, 1));
  float lumaUpLeft = rgb2luma(fxaaTexOff(ds, tu, tv, -1, 1));
  float lumaDownRight = rgb2luma(fxaaTexOff(ds, tu, tv, 1, -1));
  float lumaDownUp = lumaDown + lumaUp;
  float lumaLeftRight = lumaLeft + lumaRight;
  float lumaLeftCorners = lumaDownLeft + lumaUpLeft;
  float lumaDownCorners = lumaDownLeft + lumaDownRight;
  float lumaRightCorners = lumaDownRight + lumaUpRight;
  float lumaUpCorners = lumaUpRight + lumaUpLeft;
  float edgeHorizontal = std::fabs(-2.0f * lumaLeft + lumaLeftCorners) + std::fabs(-2.0f * lumaCenter + lumaDownUp) * 2.0f +
                         std::fabs(-2.0f * lumaRight + lumaRightCorners);
  float edgeVertical = std::fabs(-2.0f * lumaUp + lumaUpCorners) + std::fabs(-2.0f * lumaCenter + lumaLeftRight) * 2.0f +
                       std::fabs(-2.0f * lumaDown + lumaDownCorners);
  bool isHorizontal = (edgeHorizontal >= edgeVertical);
  float stepLength = isHorizontal ? inv_y : inv_x;
  float luma1 = isHorizontal ? lumaDown : lumaLeft;
  float luma2 = isHorizontal ? lumaUp : lumaRight;
  float gradient1 = luma1 - lumaCenter;
  float gradient2 = luma2 - lumaCenter;
  bool is1Steepest = std::fabs(gradient1) >= std::fabs(gradient2);
  float gradientScaled = 0.25f * gmax(std::fabs(gradient1), std::fabs(gradient2));
  float lumaLocalAverage = 0.0f;
  if (is1Steepest) {
    stepLength = -stepLength;
    lumaLocalAverage = 0.5f * (luma1 + lumaCenter);
  } else {
    lumaLocalAverage = 0.5f * (luma2 + lumaCenter);
  }
  float cu = tu, cv = tv;
  if (isHorizontal) cv += stepLength * 0.5f;
  else cu += stepLength * 0.5f;
  float offx = isHorizontal ? inv_x : 0.0f, offy = isHorizontal ? 0.0f : inv_y;
  float u1 = cu - offx * fxaaQuality(0.f), v1 = cv - offy * fxaaQuality(0.f);
  float u2 = cu + offx * fxaaQuality(0.f), v2 = cv + offy * fxaaQuality(0.f);
  float lumaEnd1 = 0.f, lumaEnd2 = 0.f;
  bool reached1 = false, reached2 = false, reachedBoth = false;
  for (int i = 1; i < 12; i++) {
    if (!reached1) {
      lumaEnd1 = rgb2luma(fxaaTex(ds, u1, v1));
      lumaEnd1 = lumaEnd1 - lumaLocalAverage;
      reached1 = std::fabs(lumaEnd1) >= gradientScaled;
    }
    if (!reached2) {
      lumaEnd2 = rgb2luma(fxaaTex(ds, u2, v2));
      lumaEnd2 = lumaEnd2 - lumaLocalAverage;
      reached2 = std::fabs(lumaEnd2) >= gradientScaled;
    }
    reachedBoth = reached1 && reached2;
    if (!reached1) {
      u1 -= offx * fxaaQuality((float) i);
      v1 -= offy * fxaaQuality((float) i);
    }
    if (!reached2) {
      u2 += offx * fxaaQuality((float) i);
      v2 += offy * fxaaQuality((float) i);
    }
    if (reachedBoth) break;
  }
  float distance1 = isHorizontal ? (tu - u1) : (tv - v1);
  float distance2 = isHorizontal ? (u2 - tu) : (v2 - tv);
  bool isDirection1 = distance1 < distance2;
  float distanceFinal = gmin(distance1, distance2);
  bool isLumaCenterSmaller = lumaCenter < lumaLocalAverage;
  bool correctVariation1 = (lumaEnd1 < 0.0f) != isLumaCenterSmaller;
  bool correctVariation2 = (lumaEnd2 < 0.0f) != isLumaCenterSmaller;
  bool correctVariation = isDirection1 ? correctVariation1 : correctVariation2;
  float edgeLength = (distance1 + distance2);
  float pixelOffset = -distanceFinal / edgeLength + 0.5f;
  float finalOffset = correctVariation ? pixelOffset : 0.0f;
  float lumaAverage = (1.0f / 12.0f) * (2.0f * (lumaDownUp + lumaLeftRight) + lumaLeftCorners + lumaRightCorners);
  float subPixelOffset1 = fxaaClamp01(std::fabs(lumaAverage - lumaCenter) / lumaRange);
  float subPixelOffset2 = (-2.0f * subPixelOffset1 + 3.0f) * subPixelOffset1 * subPixelOffset1;
  float subPixelOffsetFinal = subPixelOffset2 * subPixelOffset2 * 0.75f;
  finalOffset = gmax(finalOffset, subPixelOffsetFinal);
  float fu = tu, fv = tv;
  if (isHorizontal) fv += finalOffset * stepLength;
  else fu += finalOffset * stepLength;
  return fxaaTex(ds, fu, fv);
}

static V4 runFS(const DrawState &ds, const FragIn &f) {
  switch (ds.shader->model) {
    case SGLC_SHADING_BASE_COLOR: return U_BASECOLOR(ds.u, 256);
    case SGLC_SHADING_VERTEX_COLOR: return {f.v[0], f.v[1], f.v[2], f.v[3]};
    case SGLC_SHADING_BLINN_PHONG: return fsBlinnPhong(ds, f, false);
    case SGLC_SHADING_BLINN_PHONG_DIR: return fsBlinnPhong(ds, f, true);
    case SGLC_SHADING_PBR: return fsPbr(ds, f);
    case SGLC_SHADING_SKYBOX: return fsSkybox(ds, f);
    case SGLC_SHADING_IBL_IRRADIANCE: return fsIrradiance(ds, f);
    case SGLC_SHADING_IBL_PREFILTER: return fsPrefilter(ds, f);
    case SGLC_SHADING_FXAA: {
      V3 c = fxaaColor(ds, f);
      return {c.x, c.y, c.z, 1.f};
    }
  }
  return {0, 0, 0, 0};
}

// ---- per-sample operations (RendererSoft.cpp:358-407; BlendSoft.h; DepthSoft.h) -------------
static inline bool depthCmp(float a, float b, int func) {
  const float eps = 1.19209290e-07f;
  switch (func) {
    case SGLC_DEPTH_NEVER: return false;
    case SGLC_DEPTH_LESS: return a < b;
    case SGLC_DEPTH_EQUAL: return std::fabs(a - b) <= eps;
    case SGLC_DEPTH_LEQUAL: return a <= b;
    case SGLC_DEPTH_GREATER: return a > b;
    case SGLC_DEPTH_NOTEQUAL: return std::fabs(a - b) > eps;
    case SGLC_DEPTH_GEQUAL: return a >= b;
    case SGLC_DEPTH_ALWAYS: return true;
  }
  return a < b;
}

static inline float *depthPtr(DrawState &ds, int x, int y, int sample) {
  Level *d = ds.depth;
  if (!d || (size_t) x >= (size_t) d->w || (size_t) y >= (size_t) d->h) return nullptr;
  size_t p = (size_t) y * d->w + x;
  if (d->samples > 1) return reinterpret_cast<float *>(&d->data[p * 4 + sample]);
  return reinterpret_cast<float *>(&d->data[p]);
}

static inline uint32_t *colorPtr(DrawState &ds, int x, int y, int sample) {
  Level *c = ds.color;
  if (!c || (size_t) x >= (size_t) c->w || (size_t) y >= (size_t) c->h) return nullptr;
  size_t p = (size_t) y * c->w + x;
  if (c->samples > 1) return &c->data[p * 4 + sample];
  return &c->data[p];
}

static inline bool depthTest(DrawState &ds, int x, int y, float depth, int sample, bool skipWrite) {
  const sglc_render_states *rs = ds.rs;
  if (!rs->depth_test || !ds.depth) return true;
  depth = gclamp(depth, ds.vp.absMinDepth, ds.vp.absMaxDepth);
  float *z = depthPtr(ds, x, y, sample);
  if (z && depthCmp(depth, *z, rs->depth_func)) {
    if (!skipWrite && rs->depth_mask) *z = depth;
    return true;
  }
  return false;
}

static inline float blendFactorC(float src, float srcA, float dst, float dstA, int f) {
  switch (f) {
    case SGLC_BLEND_ZERO: return 0.f;
    case SGLC_BLEND_ONE: return 1.f;
    case SGLC_BLEND_SRC_COLOR: return src;
    case SGLC_BLEND_SRC_ALPHA: return srcA;
    case SGLC_BLEND_DST_COLOR: return dst;
    case SGLC_BLEND_DST_ALPHA: return dstA;
    case SGLC_BLEND_ONE_MINUS_SRC_COLOR: return 1.f - src;
    case SGLC_BLEND_ONE_MINUS_SRC_ALPHA: return 1.f - srcA;
    case SGLC_BLEND_ONE_MINUS_DST_COLOR: return 1.f - dst;
    case SGLC_BLEND_ONE_MINUS_DST_ALPHA: return 1.f - dstA;
  }
  return 0.f;
}

static inline float blendFunc(float s, float d, int fn) {
  switch (fn) {
    case SGLC_FUNC_ADD: return s + d;
    case SGLC_FUNC_SUBTRACT: return s - d;
    case SGLC_FUNC_REVERSE_SUBTRACT: return d - s;
    case SGLC_FUNC_MIN: return gmin(s, d);
    case SGLC_FUNC_MAX: return gmax(s, d);
  }
  return s + d;
}

static void perSample(DrawState &ds, int x, int y, float depth, V4 color, int sample) {
  if (!depthTest(ds, x, y, depth, sample, false)) return;
  if (!ds.color) return;
  const sglc_render_states *rs = ds.rs;
  float c[4] = {gmin(gmax(color.x, 0.f), 1.f), gmin(gmax(color.y, 0.f), 1.f), gmin(gmax(color.z, 0.f), 1.f),
                gmin(gmax(color.w, 0.f), 1.f)};
  uint32_t *ptr = colorPtr(ds, x, y, sample);
  if (rs->blend) {
    float d[4] = {0, 0, 0, 0};
    if (ptr) {
      RGBAf dc = unpack(*ptr);
      d[0] = dc.r / 255.f; d[1] = dc.g / 255.f; d[2] = dc.b / 255.f; d[3] = dc.a / 255.f;
    }
    float out[4];
    for (int i = 0; i < 3; i++) {
      float sf = blendFactorC(c[i], c[3], d[i], d[3], rs->blend_src_rgb);
      float df = blendFactorC(c[i], c[3], d[i], d[3], rs->blend_dst_rgb);
      out[i] = blendFunc(c[i] * sf, d[i] * df, rs->blend_func_rgb);
    }
    float sa = blendFactorC(c[3], c[3], d[3], d[3], rs->blend_src_alpha);
    float da = blendFactorC(c[3], c[3], d[3], d[3], rs->blend_dst_alpha);
    out[3] = blendFunc(c[3] * sa, d[3] * da, rs->blend_func_alpha);
    for (int i = 0; i < 4; i++) c[i] = out[i];
  }
  if (ptr) *ptr = pack(c[0] * 255.f, c[1] * 255.f, c[2] * 255.f, c[3] * 255.f);
}

// ---- raster -----------------------------------------------------------------------------------
static const float kSample4x[4][2] = {{0.375f, 0.875f}, {0.875f, 0.625f}, {0.125f, 0.375f}, {0.625f, 0.125f}};

struct Sample {
  bool inside;
  int fx, fy;
  V4 pos;   // x, y, z, w
  V4 bc;
};

struct Pixel {
  bool inside;
  int count;
  Sample s[5];
  int shading;   // index of the shading sample
  float *vary;
};

struct TriCtx {
  V4 vertPos[3];
  V4 flat0, flat1;          // vertPosFlat[0], [1]
  float vz[3][2];           // z, w of each vertex (the z/w pair interpolated together)
  V4 vertW;
  const float *vary[3];
  bool front;
};

// RendererSoft::barycentric, SSE path (RendererSoft.cpp:1021-1039, 1051-1055)
static inline bool bary(const TriCtx &t, float px, float py, V4 *bc) {
  const V4 &v0 = t.vertPos[0];
  float a0 = t.flat0.x - v0.x, a1 = t.flat0.y - v0.x, a2 = t.flat0.z - px;
  float b0 = t.flat1.x - v0.y, b1 = t.flat1.y - v0.y, b2 = t.flat1.z - py;
  float ux = a1 * b2 - a2 * b1;
  float uy = a2 * b0 - a0 * b2;
  float uz = a0 * b1 - a1 * b0;
  if (std::fabs(uz) < 1.19209290e-07f) return false;
  ux = ux / uz;
  uy = uy / uz;
  *bc = {1.f - (ux + uy), uy, ux, 0.f};
  if (bc->x < 0 || bc->y < 0 || bc->z < 0) return false;
  return true;
}

static inline void interpVary(float *out, const float *const in[3], int cnt, const V4 &bc) {
  // AVX2/FMA path: sum = v0*b0; sum = fma(v1, b1, sum); sum = fma(v2, b2, sum)
  for (int i = 0; i < cnt; i++) {
    float s = in[0][i] * bc.x;
    s = std::fma(in[1][i], bc.y, s);
    s = std::fma(in[2][i], bc.z, s);
    out[i] = s;
  }
}

static void rasterQuad(DrawState &ds, TriCtx &t, Pixel px[4], int band0, int band1, float *tmp) {
  int S = ds.samples;
  // barycentric + coverage + shading sample (RendererSoft.cpp:776-782; RendererInternal.h:97-124)
  for (int p = 0; p < 4; p++) {
    Pixel &P = px[p];
    int ns = S > 1 ? 5 : 1;
    for (int i = 0; i < ns; i++) P.s[i].inside = bary(t, P.s[i].pos.x, P.s[i].pos.y, &P.s[i].bc);
    if (S > 1) {
      int cov = 0;
      for (int i = 0; i < 4; i++) cov += P.s[i].inside;
      P.inside = cov > 0;
      P.shading = 4;
    } else {
      P.inside = P.s[0].inside;
      P.shading = 0;
    }
    if (!P.s[P.shading].inside) {
      for (int i = 0; i < ns; i++)
        if (P.s[i].inside) {
          P.shading = i;
          break;
        }
    }
  }
  if (!(px[0].inside || px[1].inside || px[2].inside || px[3].inside)) return;
  // z/w, depth-range clip, perspective correction (RendererSoft.cpp:787-804)
  for (int p = 0; p < 4; p++) {
    Pixel &P = px[p];
    int ns = S > 1 ? 5 : 1;
    for (int i = 0; i < ns; i++) {
      Sample &s = P.s[i];
      if (!s.inside) continue;
      s.pos.z = dot4(s.bc, V4{t.vz[0][0], t.vz[1][0], t.vz[2][0], 0.f});
      s.pos.w = dot4(s.bc, V4{t.vz[0][1], t.vz[1][1], t.vz[2][1], 0.f});
      if (s.pos.z < ds.vp.absMinDepth || s.pos.z > ds.vp.absMaxDepth) s.inside = false;
      float iw = 1.f / s.pos.w;
      s.bc = {s.bc.x * (iw * t.vertW.x), s.bc.y * (iw * t.vertW.y), s.bc.z * (iw * t.vertW.z),
              s.bc.w * (iw * t.vertW.w)};
    }
  }
  // pixels outside this thread's band take part only through their varyings (derivatives)
  bool own[4];
  for (int p = 0; p < 4; p++) own[p] = px[p].s[0].fy >= band0 && px[p].s[0].fy < band1;
  // early z (RendererSoft.cpp:806-811, 853-878)
  if (ds.earlyZ && ds.rs->depth_test) {
    bool any = false;
    for (int p = 0; p < 4; p++) {
      Pixel &P = px[p];
      if (!P.inside) continue;
      if (!own[p]) {
        any = true;
        continue;
      }
      if (S > 1) {
        bool in = false;
        for (int i = 0; i < 4; i++) {
          Sample &s = P.s[i];
          if (!s.inside) continue;
          s.inside = depthTest(ds, s.fx, s.fy, s.pos.z, i, true);
          if (s.inside) in = true;
        }
        P.inside = in;
      } else {
        Sample &s = P.s[P.shading];
        s.inside = depthTest(ds, s.fx, s.fy, s.pos.z, 0, true);
        P.inside = s.inside;
      }
      any = any || P.inside;
    }
    if (!any) return;
  }
  // varyings for all four pixels (derivatives need them)
  int vc = ds.varyCnt;
  for (int p = 0; p < 4; p++) interpVary(px[p].vary, t.vary, vc, px[p].s[px[p].shading].bc);
  (void) tmp;
  FragIn f;
  f.dudx = px[1].vary[0] - px[0].vary[0];
  f.dvdx = px[1].vary[1] - px[0].vary[1];
  f.dudy = px[2].vary[0] - px[0].vary[0];
  f.dvdy = px[2].vary[1] - px[0].vary[1];
  if (vc < 2) f.dudx = f.dvdx = f.dudy = f.dvdy = 0.f;
  for (int p = 0; p < 4; p++) {
    Pixel &P = px[p];
    if (!P.inside || !own[p]) continue;
    V4 color{0, 0, 0, 0};
    if (ds.color) {
      f.v = P.vary;
      color = runFS(ds, f);
    }
    if (S > 1) {
      for (int i = 0; i < 4; i++) {
        Sample &s = P.s[i];
        if (!s.inside) continue;
        perSample(ds, s.fx, s.fy, s.pos.z, color, i);
      }
    } else {
      Sample &s = P.s[P.shading];
      perSample(ds, s.fx, s.fy, s.pos.z, color, 0);
    }
  }
}

static void initPixel(Pixel &P, float x, float y, int S) {
  if (S > 1) {
    for (int i = 0; i < 4; i++) {
      P.s[i].fx = (int) x;
      P.s[i].fy = (int) y;
      P.s[i].pos = {kSample4x[i][0] + x, kSample4x[i][1] + y, 0.f, 0.f};
    }
    P.s[4].fx = (int) x;
    P.s[4].fy = (int) y;
    P.s[4].pos = {x + 0.5f, y + 0.5f, 0.f, 0.f};
  } else {
    P.s[0].fx = (int) x;
    P.s[0].fy = (int) y;
    P.s[0].pos = {x + 0.5f, y + 0.5f, 0.f, 0.f};
  }
}

// RendererSoft::rasterizationTriangle (RendererSoft.cpp:720-769) for one band of rows
static void rasterTriangle(DrawState &ds, const VertexH &a, const VertexH &b, const VertexH &c, bool front,
                           int band0, int band1, float *varyPool) {
  const VertexH *vert[3] = {&a, &b, &c};
  TriCtx t;
  for (int i = 0; i < 3; i++) {
    t.vertPos[i] = vert[i]->fragPos;
    t.vz[i][0] = vert[i]->fragPos.z;
    t.vz[i][1] = vert[i]->fragPos.w;
    t.vary[i] = vert[i]->vary;
  }
  t.vertW = {vert[0]->fragPos.w, vert[1]->fragPos.w, vert[2]->fragPos.w, 1.f};
  t.flat0 = {t.vertPos[2].x, t.vertPos[1].x, t.vertPos[0].x, 0.f};
  t.flat1 = {t.vertPos[2].y, t.vertPos[1].y, t.vertPos[0].y, 0.f};
  t.front = front;
  // triangleBoundingBox (RendererSoft.cpp:1005-1019), then min -= 1
  float minX = std::min(std::min(t.vertPos[0].x, t.vertPos[1].x), t.vertPos[2].x);
  float minY = std::min(std::min(t.vertPos[0].y, t.vertPos[1].y), t.vertPos[2].y);
  float maxX = std::max(std::max(t.vertPos[0].x, t.vertPos[1].x), t.vertPos[2].x);
  float maxY = std::max(std::max(t.vertPos[0].y, t.vertPos[1].y), t.vertPos[2].y);
  minX = std::max(minX - 0.5f, 0.f);
  minY = std::max(minY - 0.5f, 0.f);
  maxX = std::min(maxX + 0.5f, ds.vp.width - 1.f);
  maxY = std::min(maxY + 0.5f, ds.vp.height - 1.f);
  minX -= 1.f;
  minY -= 1.f;
  const int bs = 32;
  int bcx = (int) (((maxX - minX) + (float) bs - 1.f) / (float) bs);
  int bcy = (int) (((maxY - minY) + (float) bs - 1.f) / (float) bs);
  // rows this band can touch: quads start at y and cover y, y+1
  if ((int) maxY + 1 < band0 - 1 || (int) minY > band1 + 1) return;
  Pixel px[4];
  for (int p = 0; p < 4; p++) px[p].vary = varyPool + p * 32;
  for (int by = 0; by < bcy; by++) {
    int sy = (int) (minY + (float) (by * bs));
    if (sy + bs < band0 - 1 || sy > band1) continue;
    for (int bx = 0; bx < bcx; bx++) {
      int sx = (int) (minX + (float) (bx * bs));
      for (int y = sy + 1; y < sy + bs && (float) y <= maxY; y += 2) {
        if (y + 1 < band0 || y >= band1) continue;
        for (int x = sx + 1; x < sx + bs && (float) x <= maxX; x += 2) {
          initPixel(px[0], (float) x, (float) y, ds.samples);
          initPixel(px[1], (float) x + 1, (float) y, ds.samples);
          initPixel(px[2], (float) x, (float) y + 1, ds.samples);
          initPixel(px[3], (float) x + 1, (float) y + 1, ds.samples);
          rasterQuad(ds, t, px, band0, band1, nullptr);
        }
      }
    }
  }
}

// ---- points and lines (RendererSoft.cpp:636-712) -----------------------------------------------
static const int64_t kMaxLineSteps = 1 << 24;   // longer lines are refused (SGLC_ERR_OVERFLOW)

// float -> int as the reference's (int) casts compile on x86-64 (cvttss2si): truncation, and
// INT_MIN for NaN and for values outside the int range
static inline int truncI(float f) {
  if (!(f > -2147483904.f && f < 2147483648.f)) return INT32_MIN;
  return (int) f;
}

// rasterizationPoint (RendererSoft.cpp:636-661): a pointSize x pointSize stamp; every pixel runs
// the FS on the vertex's own varyings (no shader reads FragCoord, so one evaluation serves the
// stamp) and the per-sample operations on every sample. The reference walks the stamp with the
// vertex's fragPos as its loop variable, so a stamp that ran leaves fragPos.xy at its last pixel;
// a vertex drawn again starts from there.
static void rasterPoint(DrawState &ds, V4 &fragPos, const float *vary, float size) {
  if (!ds.color) return;
  float left = fragPos.x - size / 2.f + 0.5f;
  float right = left + size;
  float top = fragPos.y - size / 2.f + 0.5f;
  float bottom = top + size;
  int x0 = truncI(left), x1 = truncI(right), y0 = truncI(top), y1 = truncI(bottom);
  if (!(x0 < x1 && y0 < y1)) return;
  FragIn f;
  f.v = vary;
  f.dudx = f.dvdx = f.dudy = f.dvdy = 0.f;
  V4 color = runFS(ds, f);
  // pixels outside both attachments change nothing (getFrameColor / getFrameDepth return null)
  int W = std::max(ds.color->w, ds.depth ? ds.depth->w : 0), H = std::max(ds.color->h, ds.depth ? ds.depth->h : 0);
  for (int x = std::max(x0, 0); x < std::min(x1, W); x++)
    for (int y = std::max(y0, 0); y < std::min(y1, H); y++)
      for (int s = 0; s < ds.samples; s++) perSample(ds, x, y, fragPos.z, color, s);
  fragPos.x = (float) (x1 - 1);
  fragPos.y = (float) (y1 - 1);
}

// rasterizationLine (RendererSoft.cpp:663-712): Bresenham over the major axis; every step is a
// lineWidth stamp with z, w and the varyings lerped by t = (x - x0) / dx (glm::mix).
static sglc_status rasterLine(DrawState &ds, const VertexH &v0, const VertexH &v1, float width, float *tmp) {
  int64_t x0 = truncI(v0.fragPos.x), y0 = truncI(v0.fragPos.y);
  int64_t x1 = truncI(v1.fragPos.x), y1 = truncI(v1.fragPos.y);
  float z0 = v0.fragPos.z, z1 = v1.fragPos.z, w0 = v0.fragPos.w, w1 = v1.fragPos.w;
  bool steep = false;
  if (std::llabs(x0 - x1) < std::llabs(y0 - y1)) {
    std::swap(x0, y0);
    std::swap(x1, y1);
    steep = true;
  }
  const float *vin[2] = {v0.vary, v1.vary};
  if (x0 > x1) {
    std::swap(x0, x1);
    std::swap(y0, y1);
    std::swap(z0, z1);
    std::swap(w0, w1);
    std::swap(vin[0], vin[1]);
  }
  int64_t dx = x1 - x0, dy = y1 - y0;
  if (dx > kMaxLineSteps) return SGLC_ERR_OVERFLOW;
  int64_t error = 0, dError = 2 * std::llabs(dy), y = y0;
  for (int64_t x = x0; x <= x1; x++) {
    float t = (float) (x - x0) / (float) dx;
    V4 pos{(float) x, (float) y, z0 * (1.f - t) + z1 * t, w0 * (1.f - t) + w1 * t};
    if (steep) std::swap(pos.x, pos.y);
    for (int i = 0; i < ds.varyCnt; i++) tmp[i] = vin[0][i] * (1.f - t) + vin[1][i] * t;
    rasterPoint(ds, pos, tmp, width);
    error += dError;
    if (error > dx) {
      y += (y1 > y0 ? 1 : -1);
      error -= 2 * dx;
    }
  }
  return SGLC_OK;
}

static Level *attachmentLevel(Ctx *c, int texH, int layer, int level) {
  Object *t = c->get(texH, 2);
  if (!t) return nullptr;
  if (layer < 0 || layer >= t->tex.layers) return nullptr;
  auto &lv = t->tex.img[layer];
  if (level < 0 || level >= (int) lv.size()) return nullptr;
  return &lv[level];
}

// perspectiveDivideImpl + viewportTransformImpl (RendererSoft.cpp:981-992)
static inline V4 toScreen(const Viewport &vp, V4 f) {
  float invW = 1.f / f.w;
  f = {f.x * invW, f.y * invW, f.z * invW, f.w * invW};
  f.w = invW;
  f = {f.x * vp.innerP.x, f.y * vp.innerP.y, f.z * vp.innerP.z, f.w * vp.innerP.w};
  return {f.x + vp.innerO.x, f.y + vp.innerO.y, f.z + vp.innerO.z, f.w + vp.innerO.w};
}

// MSAA resolve after every draw (RendererSoft.cpp:161-163, 880-912)
static void resolveMsaa(DrawState &ds) {
  if (!ds.color || ds.color->samples <= 1) return;
  Level &L = *ds.color;
  L.resolved.assign((size_t) L.w * L.h, 0);
  for (size_t i = 0; i < (size_t) L.w * L.h; i++) {
    float s[4] = {0, 0, 0, 0};
    for (int k = 0; k < 4; k++) {
      RGBAf q = unpack(L.data[i * 4 + k]);
      s[0] += q.r; s[1] += q.g; s[2] += q.b; s[3] += q.a;
    }
    L.resolved[i] = pack(s[0] / 4.f, s[1] / 4.f, s[2] / 4.f, s[3] / 4.f);
  }
  L.hasResolved = true;
}

static sglc_status doDraw(Ctx *c) {
  Object *fbo = c->get(c->fb, 1), *vo = c->get(c->vao, 3), *po = c->get(c->prog, 4), *so = c->get(c->states, 5);
  if (!fbo || !vo || !po) return SGLC_OK;   // RendererSoft::draw is a silent no-op (RendererSoft.cpp:137-139)
  if (!so) return c->fail(SGLC_ERR_INVALID_VALUE, "draw: no pipeline states");
  ProgramObj &prog = po->prog;
  if (!prog.shader) return c->fail(SGLC_ERR_INVALID_VALUE, "draw: program has no shaders");
  const sglc_render_states *rs = &so->states;
  const int prim = rs->primitive_type;
  if (prim != SGLC_PRIMITIVE_POINT && prim != SGLC_PRIMITIVE_LINE && prim != SGLC_PRIMITIVE_TRIANGLE)
    return c->fail(SGLC_ERR_INVALID_VALUE, "draw: unknown primitive type");
  if (rs->polygon_mode != SGLC_POLYGON_POINT && rs->polygon_mode != SGLC_POLYGON_LINE &&
      rs->polygon_mode != SGLC_POLYGON_FILL)
    return c->fail(SGLC_ERR_INVALID_VALUE, "draw: unknown polygon mode");
  const bool fill = prim == SGLC_PRIMITIVE_TRIANGLE && rs->polygon_mode == SGLC_POLYGON_FILL;
  DrawState ds{};
  ds.shader = prog.shader;
  ds.u = prog.uniforms.data();
  ds.def = prog.defines;
  ds.rs = rs;
  ds.vp = c->vp;
  ds.color = fbo->fb.colorReady ? attachmentLevel(c, fbo->fb.colorTex, fbo->fb.colorLayer, fbo->fb.colorLevel) : nullptr;
  ds.depth = fbo->fb.depthReady ? attachmentLevel(c, fbo->fb.depthTex, 0, 0) : nullptr;
  ds.samples = ds.color ? ds.color->samples : (ds.depth ? ds.depth->samples : 1);
  ds.earlyZ = c->earlyZ;
  ds.varyCnt = prog.shader->varyingsCnt;
  ds.varyAligned = ((ds.varyCnt * 4 + 31) / 32) * 8;
  for (int s = 0; s < MAX_SAMPLERS; s++) {
    ds.sampBound[s] = false;
    Object *uso = c->get(prog.samplers[s], 7);
    if (!uso) continue;
    UniformSamplerObj &us = uso->us;
    Object *to = c->get(us.tex, 2);
    if (!to) continue;
    ds.sampBound[s] = true;
    ds.sampW[s] = us.width;
    ds.sampH[s] = us.height;
    // only samplers whose LOD callback the FS installs (setupSamplerDerivative: albedo, normal,
    // emissive, ao; BlinnPhongSoft.h:217-230, PbrSoft.h:138-151) get derivative-based LOD
    ds.sampMip[s] = us.useMipmaps && ((ds.shader->derivSlots >> s) & 1) && us.type == SGLC_TEXTURE_2D;
    for (int f = 0; f < 6; f++) {
      int layer = std::min(f, to->tex.layers - 1);
      ds.samp[s][f] = {&to->tex.img[layer], us.filter, us.wrap, us.border, us.format == SGLC_FORMAT_FLOAT32};
    }
    if (s == 4 && to->tex.img[0].size()) ds.shadowLevel0 = &to->tex.img[0][0];
  }
  // every sampler the shader may touch must be bound (the reference dereferences it)
  if (!fill) {
    // points and lines run the FS outside a pixel quad: the reference has no derivative context
    // there, so a derivative-LOD sampler in use has nothing to read
    for (int s = 0; s < 4; s++)
      if (ds.sampBound[s] && ds.sampMip[s] && ds.def[s])
        return c->fail(SGLC_ERR_UNSUPPORTED, "draw: points/lines with a derivative-LOD (mipmapped 2D) sampler");
  }
  VaoObj &vao = vo->vao;
  size_t nv = vao.vertexCnt;
  const int per = prim == SGLC_PRIMITIVE_POINT ? 1 : (prim == SGLC_PRIMITIVE_LINE ? 2 : 3);
  size_t ntri = vao.indices.size() / per;
  int strideF = (int) (vao.stride / 4);
  int va = std::max(ds.varyAligned, 1);
  // vertex stage (RendererSoft.cpp:170-190, 971-979, 994-1003)
  std::vector<VertexH> verts(nv);
  std::vector<float> vary(nv * va, 0.f);
  std::vector<std::vector<float>> extraAttr, extraVary;
  const float *attr = reinterpret_cast<const float *>(vao.vertexes.data());
  for (size_t i = 0; i < nv; i++) {
    VertexH &h = verts[i];
    h.attr = attr + i * strideF;
    h.vary = vary.data() + i * va;
    runVS(ds, h.attr, h.vary, &h.clipPos);
    h.clipMask = clipMaskOf(h.clipPos);
  }
  // primitive assembly (RendererSoft.cpp:409-437)
  std::vector<Prim> prims(ntri);
  for (size_t i = 0; i < ntri; i++) {
    prims[i].discard = false;
    prims[i].frontFacing = true;
    prims[i].idx[1] = prims[i].idx[2] = 0;
    for (int k = 0; k < per; k++) {
      int32_t ix = vao.indices[i * per + k];
      if (ix < 0 || (size_t) ix >= nv) prims[i].discard = true;
      prims[i].idx[k] = ix;
    }
  }
  // clipping (RendererSoft.cpp:206-257, 489-559, 956-969, 1058-1083)
  std::vector<std::unique_ptr<float[]>> keep;
  auto newVertex = [&](int i0, int i1, float tt, bool post = false) -> int {
    std::unique_ptr<float[]> a(new float[strideF]);
    std::unique_ptr<float[]> v(new float[va]());
    const float *A0 = verts[i0].attr, *A1 = verts[i1].attr;
    for (int k = 0; k < strideF; k++) a[k] = A0[k] * (1.f - tt) + A1[k] * tt;
    VertexH h;
    h.attr = a.get();
    h.vary = v.get();
    runVS(ds, h.attr, h.vary, &h.clipPos);
    h.clipMask = clipMaskOf(h.clipPos);
    if (post) h.fragPos = toScreen(ds.vp, h.clipPos);
    keep.push_back(std::move(a));
    keep.push_back(std::move(v));
    verts.push_back(h);
    return (int) verts.size() - 1;
  };
  // clippingLine (RendererSoft.cpp:443-487): parametric clip against the planes either end is
  // outside of; the far end is re-made from the already re-made near end (indices[0] is updated
  // before the second clippingNewVertex call)
  auto clipLine = [&](Prim &l, bool post) {
    const int m0 = verts[l.idx[0]].clipMask, m1 = verts[l.idx[1]].clipMask;
    const V4 c0 = verts[l.idx[0]].clipPos, c1 = verts[l.idx[1]].clipPos;
    float t0 = 0.f, t1 = 1.f;
    int mask = m0 | m1;
    for (int pl = 0; pl < 6 && mask; pl++) {
      if (!(mask & (1 << pl))) continue;
      float d0 = dot4(kClipPlanes[pl], c0), d1 = dot4(kClipPlanes[pl], c1);
      if (d0 < 0 && d1 < 0) {
        l.discard = true;
        return;
      } else if (d0 < 0) {
        float t = -d0 / (d1 - d0);
        t0 = (t0 < t) ? t : t0;   // std::max
      } else {
        float t = d0 / (d0 - d1);
        t1 = (t < t1) ? t : t1;   // std::min
      }
    }
    if (m0) l.idx[0] = newVertex(l.idx[0], l.idx[1], t0, post);
    if (m1) l.idx[1] = newVertex(l.idx[0], l.idx[1], t1, post);
  };
  size_t primCnt = prims.size();
  for (size_t pi = 0; pi < primCnt; pi++) {
    if (prims[pi].discard) continue;
    if (prim == SGLC_PRIMITIVE_POINT) {   // clippingPoint (RendererSoft.cpp:439-441)
      prims[pi].discard = verts[prims[pi].idx[0]].clipMask != 0;
      continue;
    }
    if (prim == SGLC_PRIMITIVE_LINE) {
      clipLine(prims[pi], false);
      continue;
    }
    if (!fill) continue;   // triangles drawn as points / lines are not clipped as triangles
    int mask = verts[prims[pi].idx[0]].clipMask | verts[prims[pi].idx[1]].clipMask | verts[prims[pi].idx[2]].clipMask;
    if (mask == 0) continue;
    std::vector<int> in = {prims[pi].idx[0], prims[pi].idx[1], prims[pi].idx[2]}, out;
    bool full = false;
    for (int pl = 0; pl < 6; pl++) {
      if (!(mask & (1 << pl))) continue;
      if (in.size() < 3) {
        full = true;
        break;
      }
      out.clear();
      int pre = in[0];
      float dPre = dot4(kClipPlanes[pl], verts[pre].clipPos);
      in.push_back(pre);
      for (size_t k = 1; k < in.size(); k++) {
        int cur = in[k];
        float d = dot4(kClipPlanes[pl], verts[cur].clipPos);
        if (dPre >= 0) out.push_back(pre);
        if (std::signbit(dPre) != std::signbit(d)) {
          float tt = d < 0 ? dPre / (dPre - d) : -dPre / (d - dPre);
          out.push_back(newVertex(pre, cur, tt));
        }
        pre = cur;
        dPre = d;
      }
      std::swap(in, out);
    }
    if (full || in.empty()) {
      prims[pi].discard = true;
      continue;
    }
    prims[pi].idx[0] = in[0];
    prims[pi].idx[1] = in[1];
    prims[pi].idx[2] = in[2];
    for (size_t k = 3; k < in.size(); k++) {
      Prim p;
      p.discard = false;
      p.frontFacing = prims[pi].frontFacing;
      p.idx[0] = in[0];
      p.idx[1] = in[k - 1];
      p.idx[2] = in[k];
      prims.push_back(p);
    }
  }
  c->stats.vertices_in = (int64_t) nv;
  c->stats.triangles_in = (int64_t) ntri;
  c->stats.clip_vertices = (int64_t) (verts.size() - nv);
  c->stats.primitives = (int64_t) prims.size();
  // perspective divide + viewport (RendererSoft.cpp:259-275, 981-992) for every referenced vertex
  std::vector<char> used(verts.size(), 0);
  for (auto &p : prims)
    if (!p.discard)
      for (int k = 0; k < per; k++) used[p.idx[k]] = 1;
  for (size_t i = 0; i < verts.size(); i++) {
    if (!used[i]) continue;
    verts[i].fragPos = toScreen(ds.vp, verts[i].clipPos);
  }
  // face culling (RendererSoft.cpp:277-299)
  for (auto &p : prims) {
    if (p.discard || prim != SGLC_PRIMITIVE_TRIANGLE) continue;
    V4 v0 = verts[p.idx[0]].fragPos, v1 = verts[p.idx[1]].fragPos, v2 = verts[p.idx[2]].fragPos;
    V3 e1 = {v1.x - v0.x, v1.y - v0.y, v1.z - v0.z}, e2 = {v2.x - v0.x, v2.y - v0.y, v2.z - v0.z};
    V3 n = cross3(e1, e2);
    float area = (n.x * 0.f + n.y * 0.f) + n.z * 1.f;
    p.frontFacing = area > 0;
    if (rs->cull_face) p.discard = !p.frontFacing;
  }
  if (!fill) {
    // points and lines, in primitive order (RendererSoft.cpp:301-321, 575-622)
    const float pointSize = ds.shader->model == SGLC_SHADING_BASE_COLOR ? U_POINTSIZE(ds.u, 256) : 1.f;
    std::vector<float> tmp(std::max(ds.varyCnt, 1));
    sglc_status st = SGLC_OK;
    for (size_t pi = 0; pi < prims.size() && st == SGLC_OK; pi++) {
      Prim &p = prims[pi];
      if (p.discard) continue;
      if (prim == SGLC_PRIMITIVE_POINT) {
        rasterPoint(ds, verts[p.idx[0]].fragPos, verts[p.idx[0]].vary, pointSize);
      } else if (prim == SGLC_PRIMITIVE_LINE) {
        st = rasterLine(ds, verts[p.idx[0]], verts[p.idx[1]], rs->line_width, tmp.data());
      } else if (rs->polygon_mode == SGLC_POLYGON_POINT) {
        for (int k = 0; k < 3; k++) {
          VertexH &h = verts[p.idx[k]];
          if (h.clipMask != 0) continue;
          rasterPoint(ds, h.fragPos, h.vary, pointSize);
        }
      } else {
        for (int k = 0; k < 3 && st == SGLC_OK; k++) {
          Prim l;
          l.discard = false;
          l.idx[0] = p.idx[k];
          l.idx[1] = p.idx[(k + 1) % 3];
          clipLine(l, true);
          if (l.discard) continue;
          st = rasterLine(ds, verts[l.idx[0]], verts[l.idx[1]], rs->line_width, tmp.data());
        }
      }
    }
    c->stats.clip_vertices = (int64_t) (verts.size() - nv);
    if (st != SGLC_OK) return c->fail(st, "draw: line longer than 2^24 steps");
    resolveMsaa(ds);
    return SGLC_OK;
  }
  // rasterization, row bands in parallel (each pixel sees the same ordered operations)
  int H = ds.color ? ds.color->h : (ds.depth ? ds.depth->h : 0);
  int nth = std::max(1, std::min(c->threads, H / 8 > 0 ? H / 8 : 1));
  auto work = [&](int band0, int band1) {
    std::vector<float> pool(4 * 32 + 8, 0.f);
    for (auto &p : prims) {
      if (p.discard) continue;
      rasterTriangle(ds, verts[p.idx[0]], verts[p.idx[1]], verts[p.idx[2]], p.frontFacing, band0, band1, pool.data());
    }
  };
  if (nth == 1) {
    work(-4, H + 4);
  } else {
    std::vector<std::thread> th;
    for (int k = 0; k < nth; k++) {
      int b0 = (int) ((int64_t) H * k / nth), b1 = (int) ((int64_t) H * (k + 1) / nth);
      if (k == 0) b0 = -4;
      if (k == nth - 1) b1 = H + 4;
      th.emplace_back(work, b0, b1);
    }
    for (auto &t : th) t.join();
  }
  resolveMsaa(ds);
  return SGLC_OK;
}

#define CTX Ctx *c = reinterpret_cast<Ctx *>(ctx)
#define GET(var, h, kind)                                                      \
  Object *var = c->get(h, kind);                                               \
  if (!var) return c->fail(SGLC_ERR_INVALID_HANDLE, "invalid handle");

static int addObject(Ctx *c, int kind) {
  int h = c->next++;
  c->objects[h].kind = kind;
  return h;
}

static void allocLevels(TextureObj &t, bool withMips) {
  t.img.assign(t.layers, {});
  for (int l = 0; l < t.layers; l++) {
    Level L;
    L.w = t.desc.width;
    L.h = t.desc.height;
    L.samples = t.desc.multi_sample ? 4 : 1;
    L.data.assign((size_t) L.w * L.h * L.samples, 0);
    t.img[l].push_back(std::move(L));
    if (withMips && t.desc.use_mipmaps) {
      int count = (int) std::floor(std::log2((double) std::max(t.desc.width, t.desc.height))) + 1;
      for (int lev = 1; lev < count; lev++) {
        Level M;
        M.w = std::max(1, t.desc.width >> lev);
        M.h = std::max(1, t.desc.height >> lev);
        M.data.assign((size_t) M.w * M.h, 0);
        t.img[l].push_back(std::move(M));
      }
    }
  }
}

// ---- texture files (TextureSoft::storeToFile / loadFromFile, TextureSoft.h:166-215) ------------
// Storage layout of a texture: attachments and multi-sample textures are Linear, others keep the
// layout of their description (the product's per-texture choice of the reference's compile-time
// Buffer layout).
static int storageLayout(const TextureObj &t) {
  bool attachment = (t.desc.usage & (4u | 8u)) != 0;
  if (attachment || t.desc.multi_sample) return SGLC_LAYOUT_LINEAR;
  return t.desc.layout;
}

// Buffer::initLayout + convertIndex (Buffer.h:26-33, 144-157, 175-202): the storage extent and the
// storage index of texel (x, y)
static size_t storageTexels(int layout, int w, int h) {
  if (layout == SGLC_LAYOUT_TILED) return (size_t) ((w + 3) / 4) * 4 * (size_t) ((h + 3) / 4) * 4;
  if (layout == SGLC_LAYOUT_MORTON) return (size_t) ((w + 31) / 32) * 32 * (size_t) ((h + 31) / 32) * 32;
  return (size_t) w * h;
}

static inline uint32_t spreadBits5(uint32_t v) {
  uint32_t r = 0;
  for (int b = 0; b < 5; b++) r |= ((v >> b) & 1u) << (2 * b);
  return r;
}

static size_t storageIndex(int layout, int w, int x, int y) {
  if (layout == SGLC_LAYOUT_TILED) {
    size_t tile = (size_t) (y >> 2) * (size_t) ((w + 3) / 4) + (size_t) (x >> 2);
    return (tile << 4) + ((size_t) (y & 3) << 2) + (size_t) (x & 3);
  }
  if (layout == SGLC_LAYOUT_MORTON) {
    size_t tile = (size_t) (y >> 5) * (size_t) ((w + 31) / 32) + (size_t) (x >> 5);
    return (tile << 10) + (spreadBits5((uint32_t) (x & 31)) | (spreadBits5((uint32_t) (y & 31)) << 1));
  }
  return (size_t) y * w + x;
}

}  // namespace

extern "C" {

sglc_status sglo_create(sglc_context **out, int32_t) {
  *out = reinterpret_cast<sglc_context *>(new Ctx());
  return SGLC_OK;
}
sglc_status sglo_destroy(sglc_context *ctx) {
  delete reinterpret_cast<Ctx *>(ctx);
  return SGLC_OK;
}
const char *sglo_last_error(sglc_context *ctx) { return reinterpret_cast<Ctx *>(ctx)->err.c_str(); }
sglc_status sglo_release(sglc_context *ctx, sglc_handle h) {
  CTX;
  return c->objects.erase(h) ? SGLC_OK : c->fail(SGLC_ERR_INVALID_HANDLE, "release: unknown handle");
}
/* oracle-only: worker threads of the raster stage (the CPU baseline uses all host cores) */
sglc_status sglo_set_threads(sglc_context *ctx, int32_t n) {
  CTX;
  c->threads = std::max(1, (int) n);
  return SGLC_OK;
}

sglc_status sglo_create_framebuffer(sglc_context *ctx, int32_t, sglc_handle *out) {
  CTX;
  *out = addObject(c, 1);
  return SGLC_OK;
}
sglc_status sglo_framebuffer_set_color_attachment(sglc_context *ctx, sglc_handle fb, sglc_handle tex, int32_t layer,
                                                  int32_t level) {
  CTX;
  GET(f, fb, 1);
  GET(t, tex, 2);
  f->fb.colorTex = tex;
  f->fb.colorLayer = t->tex.desc.type == SGLC_TEXTURE_CUBE ? layer : 0;
  f->fb.colorLevel = level;
  f->fb.colorReady = true;
  return SGLC_OK;
}
sglc_status sglo_framebuffer_set_depth_attachment(sglc_context *ctx, sglc_handle fb, sglc_handle tex) {
  CTX;
  GET(f, fb, 1);
  GET(t, tex, 2);
  (void) t;
  f->fb.depthTex = tex;
  f->fb.depthReady = true;
  return SGLC_OK;
}
sglc_status sglo_framebuffer_is_valid(sglc_context *ctx, sglc_handle fb, int32_t *valid) {
  CTX;
  GET(f, fb, 1);
  *valid = f->fb.colorReady || f->fb.depthReady;
  return SGLC_OK;
}

sglc_status sglo_create_texture(sglc_context *ctx, const sglc_texture_desc *d, sglc_handle *out) {
  CTX;
  if (d->format != SGLC_FORMAT_RGBA8 && d->format != SGLC_FORMAT_FLOAT32)
    return c->fail(SGLC_ERR_INVALID_VALUE, "createTexture: bad format");
  if (d->width <= 0 || d->height <= 0) return c->fail(SGLC_ERR_INVALID_VALUE, "createTexture: bad size");
  int h = addObject(c, 2);
  TextureObj &t = c->objects[h].tex;
  t.desc = *d;
  t.layers = d->type == SGLC_TEXTURE_CUBE ? 6 : 1;
  t.img.assign(t.layers, {});
  *out = h;
  return SGLC_OK;
}
sglc_status sglo_texture_set_sampler_desc(sglc_context *ctx, sglc_handle tex, const sglc_sampler_desc *s) {
  CTX;
  GET(t, tex, 2);
  t->tex.sampler = *s;
  return SGLC_OK;
}
sglc_status sglo_texture_init_image_data(sglc_context *ctx, sglc_handle tex) {
  CTX;
  GET(t, tex, 2);
  allocLevels(t->tex, true);
  return SGLC_OK;
}
sglc_status sglo_texture_set_image_data(sglc_context *ctx, sglc_handle tex, int32_t layer_count,
                                        const void *const *layers, size_t bytes_per_layer) {
  CTX;
  GET(t, tex, 2);
  TextureObj &T = t->tex;
  if (T.desc.multi_sample) return c->fail(SGLC_ERR_INVALID_VALUE, "setImageData: multi sample texture");
  size_t n = (size_t) T.desc.width * T.desc.height;
  if (layer_count < T.layers || bytes_per_layer < n * 4) return c->fail(SGLC_ERR_INVALID_VALUE, "setImageData: size");
  T.img.assign(T.layers, {});
  for (int l = 0; l < T.layers; l++) {
    Level L;
    L.w = T.desc.width;
    L.h = T.desc.height;
    L.data.resize(n);
    memcpy(L.data.data(), layers[l], n * 4);
    T.img[l].push_back(std::move(L));
    if (T.desc.use_mipmaps) generateMips(T.img[l], T.desc.format == SGLC_FORMAT_FLOAT32);
  }
  return SGLC_OK;
}
sglc_status sglo_texture_set_level_data(sglc_context *ctx, sglc_handle tex, int32_t layer, int32_t level,
                                        const void *data, size_t bytes) {
  CTX;
  GET(t, tex, 2);
  TextureObj &T = t->tex;
  if (layer < 0 || layer >= T.layers || level < 0 || level >= (int) T.img[layer].size())
    return c->fail(SGLC_ERR_INVALID_VALUE, "set_level_data: bad layer/level");
  Level &L = T.img[layer][level];
  if (L.samples != 1 || bytes < (size_t) L.w * L.h * 4) return c->fail(SGLC_ERR_INVALID_VALUE, "set_level_data: size");
  memcpy(L.data.data(), data, (size_t) L.w * L.h * 4);
  return SGLC_OK;
}
sglc_status sglo_texture_read_image(sglc_context *ctx, sglc_handle tex, int32_t layer, int32_t level,
                                    int32_t resolved, void *out, size_t bytes) {
  CTX;
  GET(t, tex, 2);
  TextureObj &T = t->tex;
  if (layer < 0 || layer >= T.layers || level < 0 || level >= (int) T.img[layer].size())
    return c->fail(SGLC_ERR_INVALID_VALUE, "read_image: bad layer/level");
  Level &L = T.img[layer][level];
  size_t n = (size_t) L.w * L.h;
  if (L.samples > 1 && resolved) {
    if (bytes < n * 4) return c->fail(SGLC_ERR_INVALID_VALUE, "read_image: size");
    if (L.hasResolved) memcpy(out, L.resolved.data(), n * 4);
    else memset(out, 0, n * 4);
    return SGLC_OK;
  }
  if (bytes < n * 4 * L.samples) return c->fail(SGLC_ERR_INVALID_VALUE, "read_image: size");
  memcpy(out, L.data.data(), n * 4 * L.samples);
  return SGLC_OK;
}

sglc_status sglo_texture_store_to_file(sglc_context *ctx, sglc_handle tex, const char *path) {
  CTX;
  GET(t, tex, 2);
  if (!path) return c->fail(SGLC_ERR_INVALID_VALUE, "store_to_file: null path");
  TextureObj &T = t->tex;
  const int layout = storageLayout(T);
  std::vector<uint32_t> raw;
  for (int layer = 0; layer < T.layers; layer++)
    for (const Level &L : T.img[layer]) {
      size_t base = raw.size();
      raw.resize(base + storageTexels(layout, L.w, L.h) * L.samples, 0u);
      for (int y = 0; y < L.h; y++)
        for (int x = 0; x < L.w; x++)
          for (int s = 0; s < L.samples; s++)
            raw[base + storageIndex(layout, L.w, x, y) * L.samples + s] = L.data[((size_t) y * L.w + x) * L.samples + s];
    }
  FILE *f = fopen(path, "wb");
  if (!f) return c->fail(SGLC_ERR_INVALID_VALUE, (std::string("store_to_file: failed to open file: ") + path).c_str());
  size_t wrote = raw.empty() ? 0 : fwrite(raw.data(), 4, raw.size(), f);
  int closed = fclose(f);
  if (wrote != raw.size() || closed != 0)
    return c->fail(SGLC_ERR_INVALID_VALUE, (std::string("store_to_file: failed to write file: ") + path).c_str());
  return SGLC_OK;
}

sglc_status sglo_texture_load_from_file(sglc_context *ctx, sglc_handle tex, const char *path) {
  CTX;
  GET(t, tex, 2);
  if (!path) return c->fail(SGLC_ERR_INVALID_VALUE, "load_from_file: null path");
  TextureObj &T = t->tex;
  const int layout = storageLayout(T);
  FILE *f = fopen(path, "rb");
  if (!f) return c->fail(SGLC_ERR_INVALID_VALUE, (std::string("load_from_file: failed to open file: ") + path).c_str());
  size_t total = 0;
  for (int layer = 0; layer < T.layers; layer++)
    for (const Level &L : T.img[layer]) total += storageTexels(layout, L.w, L.h) * L.samples;
  std::vector<uint32_t> raw(total);
  size_t got = total ? fread(raw.data(), 4, total, f) : 0;
  fclose(f);
  if (got != total) return c->fail(SGLC_ERR_INVALID_VALUE, (std::string("load_from_file: failed to read file: ") + path).c_str());
  size_t base = 0;
  for (int layer = 0; layer < T.layers; layer++)
    for (Level &L : T.img[layer]) {
      for (int y = 0; y < L.h; y++)
        for (int x = 0; x < L.w; x++)
          for (int s = 0; s < L.samples; s++)
            L.data[((size_t) y * L.w + x) * L.samples + s] = raw[base + storageIndex(layout, L.w, x, y) * L.samples + s];
      base += storageTexels(layout, L.w, L.h) * L.samples;
    }
  return SGLC_OK;
}

sglc_status sglo_create_vertex_array(sglc_context *ctx, const void *vertexes, size_t vlen, size_t stride,
                                     const int32_t *indices, size_t ilen, sglc_handle *out) {
  CTX;
  if (stride == 0 || stride % 4) return c->fail(SGLC_ERR_INVALID_VALUE, "vertex array: stride");
  int h = addObject(c, 3);
  VaoObj &v = c->objects[h].vao;
  v.stride = stride;
  v.vertexCnt = vlen / stride;
  v.vertexes.assign((const uint8_t *) vertexes, (const uint8_t *) vertexes + v.vertexCnt * stride);
  v.indices.assign(indices, indices + ilen / 4);
  *out = h;
  return SGLC_OK;
}
sglc_status sglo_vertex_array_update(sglc_context *ctx, sglc_handle vao, const void *data, size_t len) {
  CTX;
  GET(v, vao, 3);
  memcpy(v->vao.vertexes.data(), data, std::min(len, v->vao.vertexes.size()));
  return SGLC_OK;
}

sglc_status sglo_create_shader_program(sglc_context *ctx, sglc_handle *out) {
  CTX;
  *out = addObject(c, 4);
  return SGLC_OK;
}
sglc_status sglo_program_add_define(sglc_context *ctx, sglc_handle prog, const char *name) {
  CTX;
  GET(p, prog, 4);
  p->prog.defineNames.push_back(name);
  return SGLC_OK;
}
sglc_status sglo_program_set_shaders(sglc_context *ctx, sglc_handle prog, int32_t model) {
  CTX;
  GET(p, prog, 4);
  const ShaderInfo *s = findShader(model);
  if (!s) return c->fail(SGLC_ERR_UNSUPPORTED, "unknown shading model");
  ProgramObj &P = p->prog;
  P.shader = s;
  memset(P.defines, 0, sizeof(P.defines));
  for (auto &n : P.defineNames)
    for (size_t i = 0; i < s->defines.size(); i++)
      if (n == s->defines[i]) P.defines[i] = 1;
  P.uniforms.assign(s->uniformSize, 0);
  return SGLC_OK;
}

sglc_status sglo_create_pipeline_states(sglc_context *ctx, const sglc_render_states *s, sglc_handle *out) {
  CTX;
  int h = addObject(c, 5);
  c->objects[h].states = *s;
  *out = h;
  return SGLC_OK;
}

sglc_status sglo_create_uniform_block(sglc_context *ctx, const char *name, int32_t size, sglc_handle *out) {
  CTX;
  if (size < 0) return c->fail(SGLC_ERR_INVALID_VALUE, "uniform block size");
  int h = addObject(c, 6);
  c->objects[h].ub.name = name;
  c->objects[h].ub.data.assign(size, 0);
  *out = h;
  return SGLC_OK;
}
sglc_status sglo_uniform_block_set_sub_data(sglc_context *ctx, sglc_handle ub, const void *data, int32_t len,
                                            int32_t offset) {
  CTX;
  GET(u, ub, 6);
  if (offset < 0 || len < 0 || (size_t) offset + len > u->ub.data.size())
    return c->fail(SGLC_ERR_INVALID_VALUE, "uniform block: range");
  memcpy(u->ub.data.data() + offset, data, len);
  return SGLC_OK;
}
sglc_status sglo_uniform_block_set_data(sglc_context *ctx, sglc_handle ub, const void *data, int32_t len) {
  return sglo_uniform_block_set_sub_data(ctx, ub, data, len, 0);
}
sglc_status sglo_create_uniform_sampler(sglc_context *ctx, const char *name, int32_t type, int32_t format,
                                        sglc_handle *out) {
  CTX;
  int h = addObject(c, 7);
  c->objects[h].us.name = name;
  c->objects[h].us.type = type;
  c->objects[h].us.format = format;
  *out = h;
  return SGLC_OK;
}
sglc_status sglo_uniform_sampler_set_texture(sglc_context *ctx, sglc_handle us, sglc_handle tex) {
  CTX;
  GET(u, us, 7);
  GET(t, tex, 2);
  UniformSamplerObj &S = u->us;
  TextureObj &T = t->tex;
  S.tex = tex;
  S.filter = T.sampler.filter_min;
  S.wrap = T.sampler.wrap_s;
  if (S.format == SGLC_FORMAT_FLOAT32) {
    float b = T.sampler.border_color == SGLC_BORDER_WHITE ? 1.f : 0.f;
    memcpy(&S.border, &b, 4);
  } else {
    S.border = T.sampler.border_color == SGLC_BORDER_WHITE ? 0xFFFFFFFFu : 0u;
  }
  S.width = T.img.size() && T.img[0].size() ? T.img[0][0].w : 0;
  S.height = T.img.size() && T.img[0].size() ? T.img[0][0].h : 0;
  S.useMipmaps = S.filter > SGLC_FILTER_LINEAR;
  return SGLC_OK;
}
sglc_status sglo_create_shader_resources(sglc_context *ctx, sglc_handle *out) {
  CTX;
  *out = addObject(c, 8);
  return SGLC_OK;
}
sglc_status sglo_shader_resources_set_block(sglc_context *ctx, sglc_handle res, int32_t key, sglc_handle ub) {
  CTX;
  GET(r, res, 8);
  GET(u, ub, 6);
  (void) u;
  r->res.blocks[key] = ub;
  return SGLC_OK;
}
sglc_status sglo_shader_resources_set_sampler(sglc_context *ctx, sglc_handle res, int32_t key, sglc_handle us) {
  CTX;
  GET(r, res, 8);
  GET(u, us, 7);
  (void) u;
  r->res.samplers[key] = us;
  return SGLC_OK;
}

sglc_status sglo_begin_render_pass(sglc_context *ctx, sglc_handle fb, const sglc_clear_states *s) {
  CTX;
  GET(f, fb, 1);
  c->fb = fb;
  Level *col = f->fb.colorReady ? attachmentLevel(c, f->fb.colorTex, f->fb.colorLayer, f->fb.colorLevel) : nullptr;
  Level *dep = f->fb.depthReady ? attachmentLevel(c, f->fb.depthTex, 0, 0) : nullptr;
  if (s->color_flag && col) {
    uint32_t v = pack(s->clear_color[0] * 255, s->clear_color[1] * 255, s->clear_color[2] * 255,
                      s->clear_color[3] * 255);
    std::fill(col->data.begin(), col->data.end(), v);
  }
  if (s->depth_flag && dep) {
    uint32_t v;
    memcpy(&v, &s->clear_depth, 4);
    std::fill(dep->data.begin(), dep->data.end(), v);
  }
  return SGLC_OK;
}
sglc_status sglo_set_viewport(sglc_context *ctx, int32_t x, int32_t y, int32_t w, int32_t h) {
  CTX;
  Viewport &v = c->vp;
  v.x = (float) x;
  v.y = (float) y;
  v.width = (float) w;
  v.height = (float) h;
  v.minDepth = 0.f;
  v.maxDepth = 1.f;
  v.absMinDepth = std::min(v.minDepth, v.maxDepth);
  v.absMaxDepth = std::max(v.minDepth, v.maxDepth);
  v.innerO = {v.x + v.width / 2.f, v.y + v.height / 2.f, v.minDepth, 0.f};
  v.innerP = {v.width / 2.f, v.height / 2.f, v.maxDepth - v.minDepth, 1.f};
  return SGLC_OK;
}
sglc_status sglo_set_vertex_array(sglc_context *ctx, sglc_handle vao) {
  CTX;
  GET(v, vao, 3);
  (void) v;
  c->vao = vao;
  return SGLC_OK;
}
sglc_status sglo_set_shader_program(sglc_context *ctx, sglc_handle prog) {
  CTX;
  GET(p, prog, 4);
  (void) p;
  c->prog = prog;
  return SGLC_OK;
}
// ShaderProgram::bindResources (ShaderProgram.h:27-54) + UniformSoft.h:26-29,79-82: blocks are
// copied into the program's uniform buffer now; samplers are bound by reference.
sglc_status sglo_set_shader_resources(sglc_context *ctx, sglc_handle res) {
  CTX;
  GET(r, res, 8);
  Object *po = c->get(c->prog, 4);
  if (!po || !po->prog.shader) return SGLC_OK;
  ProgramObj &P = po->prog;
  for (auto &kv : r->res.blocks) {
    Object *u = c->get(kv.second, 6);
    if (!u) continue;
    for (auto &d : P.shader->uniforms) {
      if (d.samplerSlot >= 0 || u->ub.name != d.name) continue;
      size_t n = std::min(u->ub.data.size(), P.uniforms.size() - d.offset);
      memcpy(P.uniforms.data() + d.offset, u->ub.data.data(), n);
    }
  }
  for (auto &kv : r->res.samplers) {
    Object *u = c->get(kv.second, 7);
    if (!u) continue;
    for (auto &d : P.shader->uniforms)
      if (d.samplerSlot >= 0 && u->us.name == d.name) P.samplers[d.samplerSlot] = kv.second;
  }
  return SGLC_OK;
}
sglc_status sglo_set_pipeline_states(sglc_context *ctx, sglc_handle st) {
  CTX;
  GET(s, st, 5);
  (void) s;
  c->states = st;
  return SGLC_OK;
}
sglc_status sglo_draw(sglc_context *ctx) {
  CTX;
  return doDraw(c);
}
sglc_status sglo_end_render_pass(sglc_context *) { return SGLC_OK; }
// The batched draw is, by definition, the views drawn one after another in their own render passes.
sglc_status sglo_draw_views(sglc_context *ctx, const sglc_handle *fbs, const sglc_handle *res, int32_t count,
                            const sglc_clear_states *clear) {
  sglc_clear_states none{0, 0, {0.f, 0.f, 0.f, 0.f}, 1.f};
  for (int v = 0; v < count; v++) {
    sglc_status s = sglo_begin_render_pass(ctx, fbs[v], clear ? clear : &none);
    if (!s) s = sglo_set_shader_resources(ctx, res[v]);
    if (!s) s = sglo_draw(ctx);
    if (!s) s = sglo_end_render_pass(ctx);
    if (s) return s;
  }
  return SGLC_OK;
}
// The multi-scene draw restated as what it stands for: each scene in its own render pass with the
// viewport over its whole frame (the larger of its attachments) and its own vertex array.
sglc_status sglo_draw_scenes(sglc_context *ctx, const sglc_handle *vaos, const sglc_handle *fbs, const sglc_handle *res,
                             int32_t count, const sglc_clear_states *clear) {
  CTX;
  sglc_clear_states none{0, 0, {0.f, 0.f, 0.f, 0.f}, 1.f};
  for (int v = 0; v < count; v++) {
    GET(f, fbs[v], 1);
    Level *col = f->fb.colorReady ? attachmentLevel(c, f->fb.colorTex, f->fb.colorLayer, f->fb.colorLevel) : nullptr;
    Level *dep = f->fb.depthReady ? attachmentLevel(c, f->fb.depthTex, 0, 0) : nullptr;
    const int w = std::max(col ? col->w : 0, dep ? dep->w : 0), h = std::max(col ? col->h : 0, dep ? dep->h : 0);
    sglc_status s = sglo_begin_render_pass(ctx, fbs[v], clear ? clear : &none);
    if (!s) s = sglo_set_viewport(ctx, 0, 0, w, h);
    if (!s) s = sglo_set_vertex_array(ctx, vaos[v]);
    if (!s) s = sglo_set_shader_resources(ctx, res[v]);
    if (!s) s = sglo_draw(ctx);
    if (!s) s = sglo_end_render_pass(ctx);
    if (s) return s;
  }
  return SGLC_OK;
}
sglc_status sglo_wait_idle(sglc_context *) { return SGLC_OK; }
// Capacities only change how the GPU back-end sizes its working arrays; the CPU pipeline has no
// capacities and never overflows.
sglc_status sglo_set_capacity(sglc_context *, const sglc_capacity *) { return SGLC_OK; }
sglc_status sglo_get_peak_counts(sglc_context *, sglc_capacity *out) {
  if (out) *out = sglc_capacity{0, 0, 0, 0, 1};
  return SGLC_OK;
}
sglc_status sglo_get_overflow(sglc_context *, int32_t *flags) {
  if (flags) *flags = 0;
  return SGLC_OK;
}
sglc_status sglo_set_enable_early_z(sglc_context *ctx, int32_t e) {
  CTX;
  c->earlyZ = e != 0;
  return SGLC_OK;
}
sglc_status sglo_get_draw_stats(sglc_context *ctx, sglc_draw_stats *out) {
  CTX;
  *out = c->stats;
  return SGLC_OK;
}
sglc_status sglo_get_stream(sglc_context *, void **stream) {
  *stream = nullptr;
  return SGLC_OK;
}
sglc_status sglo_set_tile_size(sglc_context *, int32_t) { return SGLC_OK; }
sglc_status sglo_set_deferred_shading(sglc_context *, int32_t) { return SGLC_OK; }   // one raster path
sglc_status sglo_set_tma_store(sglc_context *, int32_t) { return SGLC_OK; }   // no tile write-back
sglc_status sglo_set_stats_level(sglc_context *, int32_t) { return SGLC_OK; }

}  // extern "C"
