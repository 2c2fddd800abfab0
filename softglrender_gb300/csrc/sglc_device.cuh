// Device-side data structures and per-fragment arithmetic of the sm_103a renderer.
//
// The arithmetic reproduces SoftGLRender's RendererSoft bit for bit where the reference's result
// is integer-like (coverage, depth, clip decisions): every kernel TU is compiled with
// --fmad=false so `a * b + c` is two rounded operations exactly as in the reference's
// -ffp-contract=off build, and __fmaf_rn is used only where the reference itself issues FMA
// (the AVX2 varying interpolation, RendererSoft.cpp:1134-1138). Evaluation orders follow GLM with
// aligned SIMD types (mat4*vec4: (m0v0+m1v1)+(m2v2+m3v3); dot(vec4): DPPS (p0+p1)+(p2+p3)).
#pragma once

#include <cstdint>
#include <utility>
#include <cuda.h>   // CUtensorMap (the TMA write-back's tensor maps)
#include <cuda_runtime.h>

namespace sglc {

constexpr int kMaxLevels = 16;

// Chained launches (programmatic dependent launch). The kernels of one draw form a chain in one
// stream; each is launched with programmatic stream serialisation, so its CTAs may be scheduled
// while the previous kernel's last CTAs are still running, instead of after that kernel has
// drained and the next launch has been processed. A chained kernel's first statement is
// chainEnter(): griddepcontrol.wait blocks until the previous grid has completed and its memory
// writes are visible (it returns at once for a kernel launched without the attribute), and
// griddepcontrol.launch_dependents lets the next kernel be scheduled once every CTA of this grid
// has started. Both are hardware-managed; no kernel spins on memory.
__device__ __forceinline__ void chainEnter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// launches `kernel` (whose first statement is chainEnter()) as the next link of the stream's chain.
// Only eager submissions are chained: in a captured CUDA graph the launch gaps are already short,
// and a graph of plain kernel nodes replays a GB300 frame slightly faster (0.491 against 0.498 ms
// for the 1080p PBR frame) than one with programmatic edges, while eager chaining gains 9 %.
template<typename... K, typename... A>
inline cudaError_t launchChained(void (*kernel)(K...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                 A &&...args) {
  cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(st, &capture) != cudaSuccess) capture = cudaStreamCaptureStatusActive;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = capture == cudaStreamCaptureStatusNone ? 1 : 0;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}
constexpr int kMaxSamplers = 8;
constexpr int kUniformBytes = 448;
constexpr int kBlock = 32;           // RendererSoft::rasterBlockSize_ (RendererSoft.h:128)

enum { LAYOUT_LINEAR = 0, LAYOUT_TILED = 1, LAYOUT_MORTON = 2 };
enum { FILTER_NEAREST = 0, FILTER_LINEAR, FILTER_NN, FILTER_LN, FILTER_NL, FILTER_LL };
enum { WRAP_REPEAT = 0, WRAP_MIRRORED, WRAP_EDGE, WRAP_BORDER };
// SH_PBR_CAPTURE: the plain PBR shader that also appends neural-shader training records (a separate
// instantiation, so the plain kernel carries no capture code); SH_PBR_NEURAL: the neural IBL variant
enum {
  SH_BASE = 1, SH_BLINN = 2, SH_PBR = 3, SH_SKYBOX = 4, SH_IBL_IRR = 5, SH_IBL_PRE = 6, SH_FXAA = 7,
  SH_BLINN_DIR = 100, SH_VCOLOR = 101, SH_PBR_NEURAL = 102, SH_PBR_CAPTURE = 103
};

// one texture as seen by a sampler: all layers x levels in one allocation
struct DevTex {
  const uint32_t *base;     // layer 0, level 0
  uint32_t layerStride;     // elements between layers (cube faces)
  int levels;
  int layout;
  uint32_t offset[kMaxLevels];   // element offset of each level inside a layer
  uint16_t w[kMaxLevels], h[kMaxLevels];
  uint16_t tilesW[kMaxLevels];   // tiles per row for Tiled (4x4) / Morton (32x32) layouts
};

// Sampler2DSoft / SamplerCubeSoft state captured by setTexture (SamplerSoft.h:388-436)
struct DevSampler {
  int valid;
  int filter, wrap;
  uint32_t border;
  int width, height;          // level-0 size captured at setTexture (used for the LOD)
  int lodFromDerivative;      // the FS installed its LOD callback on this sampler
  int isFloat;
  DevTex tex;
};

struct Viewport {
  float x, y, w, h;
  float oX, oY, oZ, oW;       // innerO (RendererSoft.cpp:104-107)
  float pX, pY, pZ, pW;       // innerP (RendererSoft.cpp:109-112)
  float absMin, absMax;
};

// per-triangle setup record read (broadcast) by every lane of the raster kernel
struct __align__(16) TriSetup {
  float v0x, v0y;                 // vertPos[0].xy
  float f0x, f0y, f0z;            // vertPosFlat[0] = (v2.x, v1.x, v0.x)
  float f1x, f1y, f1z;            // vertPosFlat[1] = (v2.y, v1.y, v0.y)
  float z0, z1, z2, w0, w1, w2;   // fragPos.z / fragPos.w per vertex
  float bminx, bminy, bmaxx, bmaxy;
  int bcx, bcy;                   // 32x32 block counts
  int vid0, vid1, vid2;           // varying rows
  int front;
  int rx0, rx1, ry0, ry1;         // pixel rectangle the quads can touch (inclusive)
  int view;                       // view of a batched draw (0 for a single draw)
  int pad;
};
static_assert(sizeof(TriSetup) == 128, "TriSetup is two 64-B lines");

// attachments of one view of a batched draw
struct ViewTarget {
  uint32_t *color;
  uint32_t *resolved;
  float *depth;
};

// one scene of a multi-scene draw (sglc_draw_scenes): its own vertex array, attachments and
// viewport; its vertices, triangles and raster tiles are consecutive ranges of the pass's
struct SceneRec {
  const float *attr;              // the scene's vertex rows
  const int *indices;
  int nv, ntri;                   // the scene's vertices and triangles
  int tilesX, tilesY;
  int cw, ch, dw, dh;             // colour / depth attachment sizes
  Viewport vp;
};

// everything a draw's kernels read; passed by value as a __grid_constant__ parameter
struct DrawParams {
  // shader
  int shading;
  int varyCnt;                    // floats interpolated (sizeof(ShaderVaryings)/4)
  int varyStride;                 // aligned row length in floats (multiple of 8)
  uint8_t def[8];
  alignas(16) uint8_t u[kUniformBytes];
  DevSampler samp[kMaxSamplers];
  // pipeline state
  int depthTest, depthMask, depthFunc, blend;
  int bFuncRgb, bSrcRgb, bDstRgb, bFuncA, bSrcA, bDstA;
  // branch-free blending (calcBlendFactor / calcBlendFunc, BlendSoft.h:13-56), set by the host:
  // factor f = c0 + c1 * x with x = {src, srcAlpha, dst, dstAlpha}[op]; result = s*ks + d*kd
  // (ADD/SUBTRACT/REVERSE_SUBTRACT) or min/max(s, d) when minmax is 1/2
  int bfOp[4];                    // srcRgb, dstRgb, srcAlpha, dstAlpha
  float bfC0[4], bfC1[4];
  float bKs[2], bKd[2];           // rgb, alpha
  int bMinMax[2];
  int cullFace, earlyZ;
  Viewport vp;
  // attachments (linear storage; multi-sample: 4 samples interleaved per pixel)
  uint32_t *color;
  uint32_t *resolved;
  float *depth;
  int cw, ch, cms;
  int dw, dh, dms;
  int samples;                    // raster samples
  int pendingClear;               // the pass's clear is fused into this draw's tile init
  uint32_t clearColor;
  float clearDepth;
  int clearColorFlag, clearDepthFlag;
  // geometry
  const float *attr;              // vertex attributes (stride floats per vertex)
  int strideF;
  int nv;
  const int32_t *indices;
  int ntri;
  // scratch
  float4 *vClip;                  // clip position per vertex (original + clip-generated)
  float4 *vFrag;                  // screen position, w = 1/w_clip
  uint8_t *vMask;
  float *vVary;                   // varyStride floats per vertex
  float *vAttrExtra;              // raw attributes of clip-generated vertices
  int vCap;                       // vertex capacity (original + generated)
  int4 *prims;                    // i0, i1, i2, flags (bit0 discard)
  int primCap;
  int *clipExtra;                 // per input triangle: fan triangles appended
  int *clipAppendOff;             // exclusive scan of clipExtra (+ total at [ntri])
  int4 *clipPoly;                 // per clipped triangle: up to 9 vertex ids (3 x int4), see kernels
  int *clipPolyTri;
  int clipPolyCap;
  int *counters;                  // [0] new vertices, [1] clipped polygons, [2] overflow flags
  TriSetup *tri;
  int *tileCount;                 // per primitive: tiles touched
  int *pairOff;                   // exclusive scan of tileCount (+ total)
  uint32_t *keyA, *keyB;          // (tile) sort keys
  int *valA, *valB;               // primitive ids
  int pairCap;
  int *tileStart, *tileEnd;
  int tile;                       // raster tile width in pixels (16)
  int tileH;                      // raster tile height in pixels: 16, or 8 (deferred raster only)
  int tilesX, tilesY;
  unsigned long long *fragCounter;   // FS invocations (instrumented runs only), else null
  int needDeriv;                  // the FS reads texcoord derivatives (a bound 2D sampler with a LOD callback)
  const int *tileOrder;           // raster CTA -> tile, heaviest tile lists first (null: identity)
  // neural IBL shader (sglc_nn.cuh): training-record capture by the plain PBR shader, and the
  // BF16 weight image read by the fused neural variant
  float *capRecords;              // null: no capture
  unsigned long long *capCount;
  long long capCap;
  int capStride;
  const uint8_t *nnImage;
  // neural shading (sglc_shade_neural.cu): hardware-sampled copies of the bound 2D RGBA8 textures
  // (0: none), the context's sticky flag word its bounded waits report to, and a test hook that
  // reports a timeout after every completed wait
  cudaTextureObject_t hwTex[kMaxSamplers];
  int *errFlags;
  int nnInjectTimeout;
  float4 *nnIn;                   // per dense record: the surface stage's 4 or 5 float4, in blocks of 32
                                  // records by float4 (sglc_shade_neural.cu nnRow)
  // TMA write-back of whole 16x16 tiles (single-view draws): tensor maps over this GPU's colour
  // (samples interleaved), resolved and depth attachments; tmaStore bit 0: colour and resolved by
  // k_rop, bit 1: depth by k_raster_cov; 0: per-thread stores
  CUtensorMap tmColor;
  CUtensorMap tmResolved;
  CUtensorMap tmDepth;
  int tmaStore;
  // batched views (sglc_draw_views): one pipeline pass over `views` copies of the draw that differ
  // only in uniforms and attachments. nv / ntri above count all views' vertices / triangles;
  // view v owns vertices [v * nvView, (v + 1) * nvView), triangles [v * ntriView, ...) and raster
  // tiles [v * tilesPerView, ...). A single draw is views = 1 with null per-view arrays.
  int views;
  int nvView, ntriView;
  int tilesPerView;
  const uint8_t *viewU;            // views x kUniformBytes, or null: DrawParams::u
  const ViewTarget *viewTarget;    // per-view attachments, or null: color / resolved / depth above
  // multi-scene draws: per scene its record and (views + 1 entries each) the first vertex, triangle
  // and raster tile of scene v; null for every other draw. The views then differ in geometry and
  // frame size, and nvView / ntriView / tilesPerView are unused.
  const SceneRec *scenes;
  const int *sceneVBase, *sceneTBase, *sceneTileBase;
  int numTiles;                    // raster tiles of the pass, all views
  // deferred shading (k_raster_cov -> k_shade -> k_rop in sglc_raster.cuh): fragment records in
  // chunks of kChunk, one linked chunk list per raster warp, in the warp's fragment order
  int4 *recA;                     // triangle, meta, px | py << 16, b0 bits
  float2 *recB;                   // b1, b2
  float4 *recColor;               // fragment shader output
  int *chunkNext, *chunkFill;     // per chunk: successor (-1: none), records in it
  int *warpHead;                  // per raster warp ((tile * kSplitParts + part) * warps + warp): first chunk, -1: none
  int *recDense;                  // record ids in append-round order, no gaps (-1: a dropped record)
  int chunkCap;
  // the heaviest tiles (the first heavySlots of the heavy-first order whose list is longer than
  // heavyMin) are split over 4 CTAs, each warp owning one 8-pixel row instead of an 8x4 block, or,
  // above heavyMin8, over 8 CTAs, each warp owning half a row
  int heavySlots, heavyMin, heavyMin8;   // split in 4 above heavyMin primitives, in 8 above heavyMin8
  // small steps folded into kernels that run anyway (each null / 0: not done there)
  int binZeroRanges;              // k_bin_emit zeroes tileStart / tileEnd of all tiles
  const int *binPairTotal;        // k_bin_emit sets counters[4] = min(*binPairTotal, pairCap)
  int *ropPeakChunks;             // k_rop: *ropPeakChunks = max(itself, counters[kCntChunks])
  int *ropSticky;                 // k_rop: *ropSticky |= counters[2] (overflow flags of the draw)
  int *clipScanSums;              // k_clip adds each scan tile's clipExtra total here (zeroed)
  int *tileScanSums;              // k_setup adds each scan tile's tileCount total here (zeroed)
};

constexpr int kChunk = 32;         // fragment records per chunk
constexpr int kSplitParts = 8;     // CTAs per split heavy tile of the deferred raster kernels
constexpr int kCntChunks = 5;      // DrawParams::counters[5]: chunks allocated
constexpr int kCntBound = 6;       // counters[6..7]: 64-bit upper bound on a draw's fragment records
constexpr int kCntDense = 8;       // counters[8]: entries of the dense record list
constexpr int kOvfFrags = 32;      // counters[2] flag: the fragment record pool ran out
constexpr int kFlagNeuralTimeout = 64;   // sticky flag: a tensor-core wait of the neural shader timed out

// Point and line draws (sglc_lines.cu; RendererSoft.cpp:301-321, 409-487, 575-712). Every input
// primitive owns three slots (a point draw uses one, a line draw one, a triangle drawn as points or
// as lines up to three), so slot order is the reference's drawing order. A slot becomes stamps (one
// for a point, one per Bresenham step for a line); a stamp becomes one fragment per covered pixel;
// the fragments are stably sorted by pixel and every pixel applies its own in stamp order.
enum { LP_POINTS = 0, LP_LINES = 1, LP_TRI_POINTS = 2, LP_TRI_LINES = 3 };
enum { LP_SLOT_NONE = 0, LP_SLOT_POINT = 1, LP_SLOT_LINE = 2 };
enum { LP_ERR_BADINDEX = 1, LP_ERR_LONGLINE = 2 };
constexpr int kMaxLineSteps = 1 << 24;   // longer lines are refused

struct LineParams {
  int mode;                       // LP_*
  int nIn;                        // input primitives (points, lines or triangles)
  float pointSize, lineWidth;
  int4 *slot;                     // [3 nIn] kind, vertex a, vertex b, 0
  float2 *pointOrigin;            // [3 nIn] fragPos.xy a point slot is stamped from
  int *stampCount, *stampOff;     // [3 nIn], [3 nIn + 1]
  float4 *stampGeo;               // x, y, z, size
  int *stampRow;                  // >= 0: row of stampVary; < 0: -(vertex + 1), a row of vVary
  float4 *stampColor;             // FS output
  float *stampVary;               // lerped varyings of line steps, varyStride floats per stamp
  int *fragCount, *fragOff;       // per stamp
  int fw, fh;                     // pixel grid: the larger of the attachments
  int *flags;                     // LP_ERR_*
  unsigned long long *totals;     // [0] stamps, [1] fragments (64-bit, overflow checks)
};

// (int) f as x86-64 converts it (cvttss2si): truncation; INT_MIN for NaN and out-of-range values
__device__ __forceinline__ int truncI(float f) {
  if (!(f > -2147483904.f && f < 2147483648.f)) return (int) 0x80000000u;
  return (int) f;
}

// TMA store of a 2D box from shared memory at element coordinates (x, y) of the tensor map (a
// __grid_constant__ parameter); x * 4 bytes is a multiple of 16 for every use here
__device__ __forceinline__ void tmaStore2d(const CUtensorMap *map, const void *smem, int x, int y) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"((uint32_t) __cvta_generic_to_shared(smem)), "r"(x), "r"(y)
               : "memory");
}
// commit the thread's bulk stores and wait until they have read shared memory (the CTA may then
// retire; the grid's completion, which the next chained kernel waits for, covers the writes)
__device__ __forceinline__ void tmaCommitWait() {
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
// this thread's shared-memory writes become visible to the async (TMA) proxy
__device__ __forceinline__ void fenceAsyncShared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// uniforms of view v
__device__ __forceinline__ const uint8_t *viewUniforms(const DrawParams &p, int view) {
  return p.viewU ? p.viewU + (size_t) view * kUniformBytes : p.u;
}

// the scene whose range [base[v], base[v + 1]) holds index i (base[0] = 0, n scenes)
__device__ __forceinline__ int sceneOf(const int *base, int n, int i) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(base + mid) <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// the viewport transform of view v
__device__ __forceinline__ const Viewport &viewViewport(const DrawParams &p, int view) {
  return p.scenes ? p.scenes[view].vp : p.vp;
}

// where raster tile `tile` of a pass lies: its view, tile coordinates, the view's attachment sizes
// and viewport extent, and its attachments
struct TileFrame {
  int view, tx, ty;
  int cW, cH, dW, dH;
  float vpW, vpH;
  uint32_t *color, *resolved;
  float *depth;
};

__device__ __forceinline__ TileFrame tileFrame(const DrawParams &p, int tile) {
  TileFrame f;
  int vtile, tilesX;
  if (p.scenes) {
    f.view = sceneOf(p.sceneTileBase, p.views, tile);
    const SceneRec &S = p.scenes[f.view];
    vtile = tile - p.sceneTileBase[f.view];
    tilesX = S.tilesX;
    f.cW = S.cw;
    f.cH = S.ch;
    f.dW = S.dw;
    f.dH = S.dh;
    f.vpW = S.vp.w;
    f.vpH = S.vp.h;
  } else {
    f.view = p.views > 1 ? tile / p.tilesPerView : 0;
    vtile = tile - f.view * p.tilesPerView;
    tilesX = p.tilesX;
    f.cW = p.cw;
    f.cH = p.ch;
    f.dW = p.dw;
    f.dH = p.dh;
    f.vpW = p.vp.w;
    f.vpH = p.vp.h;
  }
  f.tx = vtile % tilesX;
  f.ty = vtile / tilesX;
  f.color = p.viewTarget ? p.viewTarget[f.view].color : p.color;
  f.resolved = p.viewTarget ? p.viewTarget[f.view].resolved : p.resolved;
  f.depth = p.viewTarget ? p.viewTarget[f.view].depth : p.depth;
  return f;
}

// ------------------------------------------------------------------------------------------------
// exact helpers
// ------------------------------------------------------------------------------------------------
struct f3 { float x, y, z; };
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ f3 operator-(float s, f3 a) { return {s - a.x, s - a.y, s - a.z}; }
__device__ __forceinline__ f3 operator+(f3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float dot4(float4 a, float4 b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + a.w * b.w); }
__device__ __forceinline__ float gmax(float x, float y) { return (x < y) ? y : x; }
__device__ __forceinline__ float gmin(float x, float y) { return (y < x) ? y : x; }
__device__ __forceinline__ float gclamp(float x, float lo, float hi) { return gmin(gmax(x, lo), hi); }
__device__ __forceinline__ f3 normalize3(f3 v) { return v * (1.0f / sqrtf(dot3(v, v))); }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ f3 max3(f3 a, f3 b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
__device__ __forceinline__ f3 pow3(f3 a, float e) { return {powf(a.x, e), powf(a.y, e), powf(a.z, e)}; }
__device__ __forceinline__ f3 ld3(const uint8_t *p) {
  const float *f = reinterpret_cast<const float *>(p);
  return {f[0], f[1], f[2]};
}
// float -> u8 as `static_cast<uint8_t>(float)` compiles on the reference hosts (int32 then low byte)
__device__ __forceinline__ uint32_t u8of(float f) { return (uint32_t) ((int) f) & 255u; }
__device__ __forceinline__ uint32_t pack4(float r, float g, float b, float a) {
  return u8of(r) | (u8of(g) << 8) | (u8of(b) << 16) | (u8of(a) << 24);
}
__device__ __forceinline__ float4 unpack4(uint32_t c) {
  return make_float4((float) (c & 255u), (float) ((c >> 8) & 255u), (float) ((c >> 16) & 255u), (float) (c >> 24));
}
// x / 255 for an unpacked RGBA8 channel (x an integer 0..255), correctly rounded without a divide:
// the product with the rounded reciprocal, then one correction by the exact residual x - q*255
// (Markstein's FMA correction step). It equals the IEEE quotient for all 256 inputs, which
// tests/test_unit_division.py checks one by one.
__device__ __forceinline__ float div255(float x) {
  const float r = 1.f / 255.f;
  const float q = x * r;
  return __fmaf_rn(__fmaf_rn(-q, 255.f, x), r, q);
}
// the shaders' texel / 255 (ShaderSoft.h:80-103)
__device__ __forceinline__ float4 unpackUnit4(uint32_t c) {
  const float4 v = unpack4(c);
  return make_float4(div255(v.x), div255(v.y), div255(v.z), div255(v.w));
}

// column-major glm::mat4 * vec4 (type_mat4x4.inl:540-572)
__device__ __forceinline__ float4 mul44(const float *m, float4 v) {
  float4 r;
  r.x = (m[0] * v.x + m[4] * v.y) + (m[8] * v.z + m[12] * v.w);
  r.y = (m[1] * v.x + m[5] * v.y) + (m[9] * v.z + m[13] * v.w);
  r.z = (m[2] * v.x + m[6] * v.y) + (m[10] * v.z + m[14] * v.w);
  r.w = (m[3] * v.x + m[7] * v.y) + (m[11] * v.z + m[15] * v.w);
  return r;
}
// glm::mat3(mat4) * vec3 and a padded mat3 * vec3 (type_mat3x3.inl:468-474): same column stride
__device__ __forceinline__ f3 mul33(const float *m, f3 v) {
  return {m[0] * v.x + m[4] * v.y + m[8] * v.z, m[1] * v.x + m[5] * v.y + m[9] * v.z,
          m[2] * v.x + m[6] * v.y + m[10] * v.z};
}

// ------------------------------------------------------------------------------------------------
// texture addressing (Base/Buffer.h:20-227) and sampling (SamplerSoft.h:117-373)
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t spread5(uint32_t v) {
  return (v & 1u) | ((v & 2u) << 1) | ((v & 4u) << 2) | ((v & 8u) << 3) | ((v & 16u) << 4);
}

__device__ __forceinline__ uint32_t texIndex(const DevTex &t, int level, int x, int y) {
  if (t.layout == LAYOUT_LINEAR) return (uint32_t) x + (uint32_t) y * t.w[level];
  if (t.layout == LAYOUT_TILED) {
    uint32_t tile = (uint32_t) (y >> 2) * t.tilesW[level] + (uint32_t) (x >> 2);
    return (tile << 4) + ((uint32_t) (y & 3) << 2) + (uint32_t) (x & 3);
  }
  uint32_t tile = (uint32_t) (y >> 5) * t.tilesW[level] + (uint32_t) (x >> 5);
  return (tile << 10) + (spread5((uint32_t) (x & 31)) | (spread5((uint32_t) (y & 31)) << 1));
}

__device__ __forceinline__ uint32_t texel(const DevTex &t, int face, int level, int x, int y) {
  return __ldg(t.base + (size_t) face * t.layerStride + t.offset[level] + texIndex(t, level, x, y));
}

__device__ __forceinline__ int wrapCoord(int x, int n, int wrap) {
  if (wrap == WRAP_REPEAT) return (x & ((n - 1) + n)) & (n - 1);   // CoordMod as the macro expands (SamplerSoft.h:14)
  if (wrap == WRAP_EDGE) return x < 0 ? 0 : (x >= n ? n - 1 : x);
  if (wrap == WRAP_MIRRORED) {
    int m = (x & ((2 * n - 1) + 2 * n)) & (2 * n - 1);
    m -= n;
    m = m >= 0 ? m : (-1 - m);
    return n - 1 - m;
  }
  return x;   // CLAMP_TO_BORDER: range-checked by the caller
}

// storage index of (x, y) in one level (Buffer::convertIndex for the three layouts)
__device__ __forceinline__ uint32_t levelIndex(int layout, int x, int y, int w, int tilesW) {
  if (layout == LAYOUT_LINEAR) return (uint32_t) x + (uint32_t) y * (uint32_t) w;
  if (layout == LAYOUT_TILED)
    return ((((uint32_t) (y >> 2) * tilesW + (uint32_t) (x >> 2))) << 4) + ((uint32_t) (y & 3) << 2) + (uint32_t) (x & 3);
  return ((((uint32_t) (y >> 5) * tilesW + (uint32_t) (x >> 5))) << 10) +
         (spread5((uint32_t) (x & 31)) | (spread5((uint32_t) (y & 31)) << 1));
}

// BaseSampler::pixelWithWrapMode (SamplerSoft.h:170-213)
__device__ __forceinline__ uint32_t pixelWrap(const DevTex &t, int face, int level, int x, int y, int wrap,
                                              uint32_t border) {
  int w = t.w[level], h = t.h[level];
  int xx = wrapCoord(x, w, wrap), yy = wrapCoord(y, h, wrap);
  bool outside = (unsigned) xx >= (unsigned) w || (unsigned) yy >= (unsigned) h;
  if (outside) return wrap == WRAP_BORDER ? border : 0u;
  return texel(t, face, level, xx, yy);
}


__device__ __forceinline__ uint32_t mixTexel(uint32_t x, uint32_t y, float a, bool isF) {
  if (isF) {
    float r = __uint_as_float(x) * (1.f - a) + __uint_as_float(y) * a;
    return __float_as_uint(r);
  }
  float4 X = unpack4(x), Y = unpack4(y);
  float ia = 1.f - a;
  return pack4(X.x * ia + Y.x * a, X.y * ia + Y.y * a, X.z * ia + Y.z * a, X.w * ia + Y.w * a);
}

// BaseSampler::samplePixelBilinear (SamplerSoft.h:254-266): the 2x2 footprint's coordinates are
// wrapped once per axis and the level's base, size and layout are read once
__device__ __forceinline__ uint32_t bilinearPx(const DevTex &t, int face, int level, float ux, float uy, int wrap,
                                               uint32_t border, bool isF) {
  float fx0 = ux - 0.5f, fy0 = uy - 0.5f;
  float flx = floorf(fx0), fly = floorf(fy0);
  int x = (int) flx, y = (int) fly;
  const int w = t.w[level], h = t.h[level], tw = t.tilesW[level], layout = t.layout;
  const uint32_t *lv = t.base + (size_t) face * t.layerStride + t.offset[level];
  int xa = wrapCoord(x, w, wrap), xb = wrapCoord(x + 1, w, wrap);
  int ya = wrapCoord(y, h, wrap), yb = wrapCoord(y + 1, h, wrap);
  bool vxa = (unsigned) xa < (unsigned) w, vxb = (unsigned) xb < (unsigned) w;
  bool vya = (unsigned) ya < (unsigned) h, vyb = (unsigned) yb < (unsigned) h;
  uint32_t fill = wrap == WRAP_BORDER ? border : 0u;
  uint32_t s1 = (vxa && vya) ? __ldg(lv + levelIndex(layout, xa, ya, w, tw)) : fill;
  uint32_t s2 = (vxb && vya) ? __ldg(lv + levelIndex(layout, xb, ya, w, tw)) : fill;
  uint32_t s3 = (vxa && vyb) ? __ldg(lv + levelIndex(layout, xa, yb, w, tw)) : fill;
  uint32_t s4 = (vxb && vyb) ? __ldg(lv + levelIndex(layout, xb, yb, w, tw)) : fill;
  float fx = fx0 - flx, fy = fy0 - fly;
  return mixTexel(mixTexel(s1, s2, fx, isF), mixTexel(s3, s4, fx, isF), fy, isF);
}

__device__ __forceinline__ uint32_t nearestSample(const DevTex &t, int face, int level, float u, float v, int wrap,
                                                  uint32_t border) {
  float tx = u * (float) t.w[level], ty = v * (float) t.h[level];
  return pixelWrap(t, face, level, (int) floorf(tx), (int) floorf(ty), wrap, border);
}

__device__ __forceinline__ uint32_t bilinearSample(const DevTex &t, int face, int level, float u, float v, int wrap,
                                                   uint32_t border, bool isF) {
  return bilinearPx(t, face, level, u * (float) t.w[level], v * (float) t.h[level], wrap, border, isF);
}

static __device__ __forceinline__ uint32_t textureImpl(const DevSampler &s, int face, float u, float v, float lod) {
  const DevTex &t = s.tex;
  if (t.levels <= 0) return 0;
  const bool isF = s.isFloat;
  const int f = s.filter;
  const bool nearest = (f & 1) == 0;        // NEAREST, NEAREST_MIPMAP_NEAREST, NEAREST_MIPMAP_LINEAR
  const int maxLevel = t.levels - 1;
  int hi = 0, lo = 0;
  bool two = false;
  float frac = 0.f;
  if (f == FILTER_NN || f == FILTER_LN) {
    hi = min(max((int) ceilf(lod + 0.5f) - 1, 0), maxLevel);
  } else if (f >= FILTER_NL) {
    float fl = floorf(lod);
    hi = min(max((int) fl, 0), maxLevel);
    lo = min(max(hi + 1, 0), maxLevel);
    two = hi != lo;
    frac = lod - fl;
  }
  uint32_t th = nearest ? nearestSample(t, face, hi, u, v, s.wrap, s.border)
                        : bilinearSample(t, face, hi, u, v, s.wrap, s.border, isF);
  if (!two) return th;
  uint32_t tl = nearest ? nearestSample(t, face, lo, u, v, s.wrap, s.border)
                        : bilinearSample(t, face, lo, u, v, s.wrap, s.border, isF);
  return mixTexel(th, tl, frac, isF);
}

// RGBA8 lookups with the channels as floats. The reference mixes u8 texels in float and stores each
// mix back to u8 (glm::mix on u8vec4 truncates), so the bilinear and trilinear stages above pack and
// unpack between mixes. For weights in [0, 1] every mix lies in [0, 256), where that store equals
// truncf of the float mix: the float path keeps the channels as integer-valued floats from the texel
// loads to the shader's /255 and skips the packing. A weight outside [0, 1] (NaN or infinite
// coordinates, NaN LOD) sends the lookup through textureImpl instead, whose stores define it.
__device__ __forceinline__ float4 mixF4(float4 X, float4 Y, float a) {
  const float ia = 1.f - a;
  return make_float4(truncf(X.x * ia + Y.x * a), truncf(X.y * ia + Y.y * a), truncf(X.z * ia + Y.z * a),
                     truncf(X.w * ia + Y.w * a));
}

// bilinearPx as floats; false (nothing written) when a weight lies outside [0, 1]
__device__ __forceinline__ bool bilinearPxF(const DevTex &t, int face, int level, float ux, float uy, int wrap,
                                            uint32_t border, float4 &out) {
  float fx0 = ux - 0.5f, fy0 = uy - 0.5f;
  float flx = floorf(fx0), fly = floorf(fy0);
  const float fx = fx0 - flx, fy = fy0 - fly;
  if (!(fx >= 0.f && fx <= 1.f && fy >= 0.f && fy <= 1.f)) return false;
  int x = (int) flx, y = (int) fly;
  const int w = t.w[level], h = t.h[level], tw = t.tilesW[level], layout = t.layout;
  const uint32_t *lv = t.base + (size_t) face * t.layerStride + t.offset[level];
  int xa = wrapCoord(x, w, wrap), xb = wrapCoord(x + 1, w, wrap);
  int ya = wrapCoord(y, h, wrap), yb = wrapCoord(y + 1, h, wrap);
  bool vxa = (unsigned) xa < (unsigned) w, vxb = (unsigned) xb < (unsigned) w;
  bool vya = (unsigned) ya < (unsigned) h, vyb = (unsigned) yb < (unsigned) h;
  uint32_t fill = wrap == WRAP_BORDER ? border : 0u;
  uint32_t s1 = (vxa && vya) ? __ldg(lv + levelIndex(layout, xa, ya, w, tw)) : fill;
  uint32_t s2 = (vxb && vya) ? __ldg(lv + levelIndex(layout, xb, ya, w, tw)) : fill;
  uint32_t s3 = (vxa && vyb) ? __ldg(lv + levelIndex(layout, xa, yb, w, tw)) : fill;
  uint32_t s4 = (vxb && vyb) ? __ldg(lv + levelIndex(layout, xb, yb, w, tw)) : fill;
  out = mixF4(mixF4(unpack4(s1), unpack4(s2), fx), mixF4(unpack4(s3), unpack4(s4), fx), fy);
  return true;
}

static __device__ __noinline__ float4 textureRGBA8Packed(const DevSampler &s, int face, float u, float v, float lod) {
  return unpack4(textureImpl(s, face, u, v, lod));
}

// unpack4(textureImpl(s, face, u, v, lod)) for RGBA8 textures, computed as floats
static __device__ __forceinline__ float4 textureRGBA8(const DevSampler &s, int face, float u, float v, float lod) {
  const DevTex &t = s.tex;
  if (t.levels <= 0) return make_float4(0.f, 0.f, 0.f, 0.f);
  if (s.isFloat) return textureRGBA8Packed(s, face, u, v, lod);
  const int f = s.filter;
  const bool nearest = (f & 1) == 0;
  const int maxLevel = t.levels - 1;
  int hi = 0, lo = 0;
  bool two = false;
  float frac = 0.f;
  if (f == FILTER_NN || f == FILTER_LN) {
    hi = min(max((int) ceilf(lod + 0.5f) - 1, 0), maxLevel);
  } else if (f >= FILTER_NL) {
    float fl = floorf(lod);
    hi = min(max((int) fl, 0), maxLevel);
    lo = min(max(hi + 1, 0), maxLevel);
    two = hi != lo;
    frac = lod - fl;
  }
  if (two && !(frac >= 0.f && frac <= 1.f)) return textureRGBA8Packed(s, face, u, v, lod);
  // At a whole-number LOD (frac == 0) the level mix is trunc(th * 1 + tl * 0), which is th for the
  // finite, integer-valued channels of RGBA8 texels: the second level is not fetched.
  two = two && frac != 0.f;
  float4 th, tl;
  if (nearest) {
    th = unpack4(nearestSample(t, face, hi, u, v, s.wrap, s.border));
    if (!two) return th;
    tl = unpack4(nearestSample(t, face, lo, u, v, s.wrap, s.border));
  } else {
    if (!bilinearPxF(t, face, hi, u * (float) t.w[hi], v * (float) t.h[hi], s.wrap, s.border, th))
      return textureRGBA8Packed(s, face, u, v, lod);
    if (!two) return th;
    if (!bilinearPxF(t, face, lo, u * (float) t.w[lo], v * (float) t.h[lo], s.wrap, s.border, tl))
      return textureRGBA8Packed(s, face, u, v, lod);
  }
  return mixF4(th, tl, frac);
}

// textureLodOffset at LOD 0 (SamplerSoft.h:117-165, 214-238): integer texel offset added to the
// scaled coordinate (bilinear) or to the floored texel (nearest)
static __device__ __noinline__ uint32_t textureOffsetImpl(const DevSampler &s, float u, float v, int ox, int oy) {
  const DevTex &t = s.tex;
  if (t.levels <= 0) return 0;
  const bool isF = s.isFloat;
  const int f = s.filter;
  const bool nearest = (f & 1) == 0;
  const int maxLevel = t.levels - 1;
  int hi = 0, lo = 0;
  bool two = false;
  if (f == FILTER_NN || f == FILTER_LN) {
    hi = min(max((int) ceilf(0.f + 0.5f) - 1, 0), maxLevel);
  } else if (f >= FILTER_NL) {
    hi = 0;
    lo = min(1, maxLevel);
    two = hi != lo;
  }
  auto one = [&](int level) -> uint32_t {
    float tx = u * (float) t.w[level], ty = v * (float) t.h[level];
    if (nearest) return pixelWrap(t, 0, level, (int) floorf(tx) + ox, (int) floorf(ty) + oy, s.wrap, s.border);
    return bilinearPx(t, 0, level, tx + (float) ox, ty + (float) oy, s.wrap, s.border, isF);
  };
  uint32_t th = one(hi);
  if (!two) return th;
  return mixTexel(th, one(lo), 0.f, isF);
}

// BaseSamplerCube::convertXYZ2UV (SamplerSoft.h:311-373), if-chain order kept for ties
__device__ __forceinline__ void cubeUV(f3 d, int *face, float *u, float *v) {
  float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  bool px = d.x > 0, py = d.y > 0, pz = d.z > 0;
  float m = 0.f, uc = 0.f, vc = 0.f;
  int f = 0;
  if (px && ax >= ay && ax >= az) { m = ax; uc = -d.z; vc = d.y; f = 0; }
  if (!px && ax >= ay && ax >= az) { m = ax; uc = d.z; vc = d.y; f = 1; }
  if (py && ay >= ax && ay >= az) { m = ay; uc = d.x; vc = -d.z; f = 2; }
  if (!py && ay >= ax && ay >= az) { m = ay; uc = d.x; vc = d.z; f = 3; }
  if (pz && az >= ax && az >= ay) { m = az; uc = d.x; vc = d.y; f = 4; }
  if (!pz && az >= ax && az >= ay) { m = az; uc = -d.x; vc = d.y; f = 5; }
  vc = -vc;
  *face = f;
  *u = 0.5f * (uc / m + 1.0f);
  *v = 0.5f * (vc / m + 1.0f);
}

}  // namespace sglc
