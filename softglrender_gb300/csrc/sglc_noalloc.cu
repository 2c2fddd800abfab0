// sglc_draw_vertex_color_noalloc: one vertex-colour draw into caller-owned device buffers that
// allocates nothing. It exists for callers that cannot call cudaMalloc: code running inside a
// host framework that owns all device memory through its own pool, real-time render threads that
// must not enter the CUDA allocator (its calls can synchronise the device), and library code that
// must not grow the process's footprint behind the host's back. Such a caller cannot create a
// context either (sglc_create allocates a stream and buffers), so this entry point takes every
// input and output as a plain device pointer and keeps all of its own working memory in one
// file-scope device array of fixed size (kScratchBytes below), which every GPU that loads the
// library holds until the process exits.
//
// It runs the same kernels as sglc_draw (vertex, clip, setup, binning, tile raster) with a
// vertex-colour program, so its output equals sglc_draw's for the same inputs. Differences that
// follow from not allocating: fixed maximum sizes (checked up front), no host wait between the
// stages (every stage reads its element counts from device memory), and one stream synchronisation
// at the end to read the capacity flags.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include <cuda.h>

#include "softgl_cuda.h"
#include "sglc_device.cuh"
#include "sglc_kernels.h"

using namespace sglc;

namespace {

// limits of one call
constexpr int kMaxVertices = 65536;
constexpr int kMaxTriangles = 32768;
constexpr int kMaxClipVertices = 32768;    // vertices created by frustum clipping
constexpr int kMaxClipPolygons = 16384;    // clipped triangles that became polygons
constexpr int kMaxAppended = 16384;        // fan triangles appended by clipping
constexpr int kMaxSide = 1024;             // attachment width and height
constexpr int kMaxPairs = 262144;          // (tile, triangle) bin entries
constexpr int kTile = 16;
constexpr int kMaxTiles = (kMaxSide / kTile) * (kMaxSide / kTile);
constexpr int kVaryStride = 8;             // vertex colour: 4 varyings, row of 8 floats
constexpr int kAttrFloats = 8;             // position vec3 (padded) + RGBA colour
constexpr int kVCap = kMaxVertices + kMaxClipVertices;
constexpr int kPrimCap = kMaxTriangles + kMaxAppended;
constexpr int kSortBlocks = kMaxPairs / kSortTileSmall;   // the sort of up to kMaxPairs uses small blocks
static_assert(kMaxPairs % kSortTileSmall == 0 && kMaxPairs <= kSortSmallMax, "whole small sort blocks");

constexpr size_t align256(size_t n) { return (n + 255) & ~(size_t) 255; }
// byte offsets of every working buffer inside the scratch array
constexpr size_t oClip = 0;
constexpr size_t oFrag = oClip + align256(sizeof(float4) * kVCap);
constexpr size_t oMask = oFrag + align256(sizeof(float4) * kVCap);
constexpr size_t oVary = oMask + align256(kVCap);
constexpr size_t oAttrX = oVary + align256(sizeof(float) * kVCap * kVaryStride);
constexpr size_t oPrims = oAttrX + align256(sizeof(float) * kMaxClipVertices * kAttrFloats);
constexpr size_t oClipExtra = oPrims + align256(sizeof(int4) * kPrimCap);
constexpr size_t oClipOff = oClipExtra + align256(sizeof(int) * (kMaxTriangles + 1));
constexpr size_t oPoly = oClipOff + align256(sizeof(int) * (kMaxTriangles + 1));
constexpr size_t oPolyTri = oPoly + align256(sizeof(int4) * 3 * kMaxClipPolygons);
constexpr size_t oCounters = oPolyTri + align256(sizeof(int) * kMaxClipPolygons);
constexpr size_t oTri = oCounters + align256(sizeof(int) * 8);
constexpr size_t oTileCount = oTri + align256(sizeof(TriSetup) * kPrimCap);
constexpr size_t oPairOff = oTileCount + align256(sizeof(int) * kPrimCap);
constexpr size_t oKeyA = oPairOff + align256(sizeof(int) * (kPrimCap + 1));
constexpr size_t oKeyB = oKeyA + align256(sizeof(uint32_t) * kMaxPairs);
constexpr size_t oValA = oKeyB + align256(sizeof(uint32_t) * kMaxPairs);
constexpr size_t oValB = oValA + align256(sizeof(int) * kMaxPairs);
constexpr size_t oTileStart = oValB + align256(sizeof(int) * kMaxPairs);
constexpr size_t oTileEnd = oTileStart + align256(sizeof(int) * kMaxTiles);
constexpr size_t oTileOrder = oTileEnd + align256(sizeof(int) * kMaxTiles);
constexpr size_t oScan = oTileOrder + align256(sizeof(int) * kMaxTiles);
constexpr size_t oHist = oScan + align256(sizeof(int) * 8192);
constexpr size_t oHistScan = oHist + align256(sizeof(int) * (256 * kSortBlocks + 1));
constexpr size_t kScratchBytes = oHistScan + align256(sizeof(int) * (256 * kSortBlocks + 1));
static_assert(kScratchBytes <= (size_t) 24 << 20, "the no-allocation scratch must stay at most 24 MiB");

// The working memory of every call, shared by all calls on a device.
static __device__ __align__(256) unsigned char g_noallocScratch[kScratchBytes];

// number of bin entries the sort may read: min(total, capacity), kept on the device
__global__ void k_clamp_pairs(const int *total, int cap, int *out) { *out = min(*total, cap); }

// Address of g_noallocScratch as seen from one CUDA context, looked up once per (device, driver
// context) at set-up: host code cannot use the symbol itself as a device address. The array
// exists once per driver context that loads the library's module, so a host framework that runs
// its own driver-API context on a device gets its own copy and its own address. Contexts are told
// apart by cuCtxGetId, which is unique for the life of the process, so a device reset (a new
// primary context) is looked up afresh rather than served a stale address.
struct ScratchAddress {
  int device;
  unsigned long long contextId;
  unsigned char *ptr;
};
std::mutex g_lock;
std::vector<ScratchAddress> g_scratch;

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

// the current driver context's unique id; 0 when the driver entry points are unavailable (the
// cache then falls back to one entry per device)
unsigned long long currentContextId() {
  static CtxGetCurrentFn getCurrent = nullptr;
  static CtxGetIdFn getId = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      getCurrent = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      getId = reinterpret_cast<CtxGetIdFn>(f);
    cudaGetLastError();
  });
  CUcontext ctx = nullptr;
  unsigned long long id = 0;
  if (getCurrent && getId && getCurrent(&ctx) == CUDA_SUCCESS && ctx && getId(ctx, &id) == CUDA_SUCCESS) return id;
  return 0;
}

int fail(char *err, size_t errLen, int status, const char *msg) {
  if (err && errLen) {
    strncpy(err, msg, errLen - 1);
    err[errLen - 1] = 0;
  }
  return status;
}

}  // namespace

extern "C" SGLC_API sglc_status sglc_draw_vertex_color_noalloc(const sglc_noalloc_draw *d, void *stream) {
  if (!d) return SGLC_ERR_INVALID_VALUE;
  char *err = d->error;
  size_t errLen = d->error_len;
  if (d->vertex_count < 0 || d->vertex_count > kMaxVertices)
    return fail(err, errLen, SGLC_ERR_INVALID_VALUE, "noalloc draw: vertex_count outside [0, 65536]");
  if (d->triangle_count < 0 || d->triangle_count > kMaxTriangles)
    return fail(err, errLen, SGLC_ERR_INVALID_VALUE, "noalloc draw: triangle_count outside [0, 32768]");
  if (d->width < 1 || d->height < 1 || d->width > kMaxSide || d->height > kMaxSide)
    return fail(err, errLen, SGLC_ERR_INVALID_VALUE, "noalloc draw: width and height must lie in [1, 1024]");
  if (d->samples != 1 && d->samples != 4)
    return fail(err, errLen, SGLC_ERR_INVALID_VALUE, "noalloc draw: samples must be 1 or 4");
  if (d->stride != 32) return fail(err, errLen, SGLC_ERR_INVALID_VALUE, "noalloc draw: stride must be 32 bytes");
  if ((d->vertex_count && !d->vertexes) || (d->triangle_count && !d->indices) || !d->color || !d->depth ||
      !d->uniforms_model || !d->uniforms_material || (d->samples == 4 && !d->resolved))
    return fail(err, errLen, SGLC_ERR_INVALID_VALUE, "noalloc draw: null buffer");
  const sglc_render_states &rs = d->states;
  if (rs.primitive_type != SGLC_PRIMITIVE_TRIANGLE || rs.polygon_mode != SGLC_POLYGON_FILL)
    return fail(err, errLen, SGLC_ERR_UNSUPPORTED, "noalloc draw: only filled triangles");
  if (rs.depth_func < 0 || rs.depth_func > 7 || rs.blend_func_rgb < 0 || rs.blend_func_rgb > 4 ||
      rs.blend_func_alpha < 0 || rs.blend_func_alpha > 4 || rs.blend_src_rgb < 0 || rs.blend_src_rgb > 9 ||
      rs.blend_dst_rgb < 0 || rs.blend_dst_rgb > 9 || rs.blend_src_alpha < 0 || rs.blend_src_alpha > 9 ||
      rs.blend_dst_alpha < 0 || rs.blend_dst_alpha > 9)
    return fail(err, errLen, SGLC_ERR_INVALID_VALUE, "noalloc draw: render state enum out of range");

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) {
    cudaGetLastError();
    return fail(err, errLen, SGLC_ERR_NO_DEVICE, "noalloc draw: no current CUDA device");
  }
  unsigned char *scratch = nullptr;
  {
    std::lock_guard<std::mutex> g(g_lock);
    const unsigned long long ctxId = currentContextId();
    for (const ScratchAddress &a : g_scratch)
      if (a.device == dev && a.contextId == ctxId) scratch = a.ptr;
    if (!scratch) {
      // first call on this device and context: resolve the array's device address (make this
      // call before any stream capture)
      void *ptr = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&ptr, g_noallocScratch);
      if (e != cudaSuccess || !ptr) {
        cudaGetLastError();
        return fail(err, errLen, SGLC_ERR_DEVICE, "noalloc draw: cudaGetSymbolAddress of the scratch array failed");
      }
      scratch = reinterpret_cast<unsigned char *>(ptr);
      g_scratch.push_back({dev, ctxId, scratch});
    }
  }
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

  DrawParams p;
  memset(&p, 0, sizeof(p));
  p.shading = SH_VCOLOR;
  p.varyCnt = 4;
  p.varyStride = kVaryStride;
  memcpy(p.u, d->uniforms_model, 256);          // UniformsModel at 0 (ShaderVertexColor layout)
  memcpy(p.u + 256, d->uniforms_material, 48);  // UniformsMaterial at 256
  p.depthTest = rs.depth_test;
  p.depthMask = rs.depth_mask;
  p.depthFunc = rs.depth_func;
  p.blend = rs.blend;
  const int facs[4] = {rs.blend_src_rgb, rs.blend_dst_rgb, rs.blend_src_alpha, rs.blend_dst_alpha};
  for (int k = 0; k < 4; k++) {   // factor = c0 + c1 * operand, as sglc_draw sets it up
    int f = facs[k];
    static const int op[10] = {0, 0, 0, 1, 2, 3, 0, 1, 2, 3};
    static const float c0[10] = {0.f, 1.f, 0.f, 0.f, 0.f, 0.f, 1.f, 1.f, 1.f, 1.f};
    static const float c1[10] = {0.f, 0.f, 1.f, 1.f, 1.f, 1.f, -1.f, -1.f, -1.f, -1.f};
    p.bfOp[k] = op[f];
    p.bfC0[k] = c0[f];
    p.bfC1[k] = c1[f];
  }
  const int fns[2] = {rs.blend_func_rgb, rs.blend_func_alpha};
  for (int k = 0; k < 2; k++) {
    p.bKs[k] = fns[k] == SGLC_FUNC_REVERSE_SUBTRACT ? -1.f : 1.f;
    p.bKd[k] = fns[k] == SGLC_FUNC_SUBTRACT ? -1.f : 1.f;
    p.bMinMax[k] = fns[k] == SGLC_FUNC_MIN ? 1 : (fns[k] == SGLC_FUNC_MAX ? 2 : 0);
  }
  p.cullFace = rs.cull_face;
  p.earlyZ = d->early_z;
  // viewport (0, 0, width, height) as RendererSoft::setViewPort (RendererSoft.cpp:92-113)
  Viewport &v = p.vp;
  v.x = 0.f;
  v.y = 0.f;
  v.w = (float) d->width;
  v.h = (float) d->height;
  v.absMin = 0.f;
  v.absMax = 1.f;
  v.oX = v.x + v.w / 2.f;
  v.oY = v.y + v.h / 2.f;
  v.oZ = 0.f;
  v.oW = 0.f;
  v.pX = v.w / 2.f;
  v.pY = v.h / 2.f;
  v.pZ = 1.f;
  v.pW = 1.f;
  p.color = d->color;
  p.resolved = d->samples == 4 ? d->resolved : nullptr;
  p.depth = d->depth;
  p.cw = p.dw = d->width;
  p.ch = p.dh = d->height;
  p.cms = p.dms = d->samples == 4;
  p.samples = d->samples;
  p.attr = reinterpret_cast<const float *>(d->vertexes);
  p.strideF = kAttrFloats;
  p.nv = d->vertex_count;
  p.indices = d->indices;
  p.ntri = d->triangle_count;
  p.vClip = reinterpret_cast<float4 *>(scratch + oClip);
  p.vFrag = reinterpret_cast<float4 *>(scratch + oFrag);
  p.vMask = scratch + oMask;
  p.vVary = reinterpret_cast<float *>(scratch + oVary);
  p.vAttrExtra = reinterpret_cast<float *>(scratch + oAttrX);
  p.vCap = p.nv + kMaxClipVertices;
  p.prims = reinterpret_cast<int4 *>(scratch + oPrims);
  p.primCap = p.ntri + kMaxAppended;
  p.clipExtra = reinterpret_cast<int *>(scratch + oClipExtra);
  p.clipAppendOff = reinterpret_cast<int *>(scratch + oClipOff);
  p.clipPoly = reinterpret_cast<int4 *>(scratch + oPoly);
  p.clipPolyTri = reinterpret_cast<int *>(scratch + oPolyTri);
  p.clipPolyCap = kMaxClipPolygons;
  p.counters = reinterpret_cast<int *>(scratch + oCounters);
  p.tri = reinterpret_cast<TriSetup *>(scratch + oTri);
  p.tileCount = reinterpret_cast<int *>(scratch + oTileCount);
  p.pairOff = reinterpret_cast<int *>(scratch + oPairOff);
  p.keyA = reinterpret_cast<uint32_t *>(scratch + oKeyA);
  p.keyB = reinterpret_cast<uint32_t *>(scratch + oKeyB);
  p.valA = reinterpret_cast<int *>(scratch + oValA);
  p.valB = reinterpret_cast<int *>(scratch + oValB);
  p.pairCap = kMaxPairs;
  p.tileStart = reinterpret_cast<int *>(scratch + oTileStart);
  p.tileEnd = reinterpret_cast<int *>(scratch + oTileEnd);
  p.tile = kTile;
  p.tileH = kTile;
  p.tilesX = (d->width + kTile - 1) / kTile;
  p.tilesY = (d->height + kTile - 1) / kTile;
  int numTiles = p.tilesX * p.tilesY;
  p.views = 1;
  p.nvView = p.nv;
  p.ntriView = p.ntri;
  p.tilesPerView = numTiles;
  p.numTiles = numTiles;
  int *scan = reinterpret_cast<int *>(scratch + oScan);
  int *hist = reinterpret_cast<int *>(scratch + oHist);
  int *histScan = reinterpret_cast<int *>(scratch + oHistScan);

  // what must start at zero: the counters and the tile ranges (the array keeps the last call's data)
  if (cudaMemsetAsync(p.counters, 0, sizeof(int) * 8, st) != cudaSuccess ||
      cudaMemsetAsync(p.tileStart, 0, sizeof(int) * numTiles, st) != cudaSuccess ||
      cudaMemsetAsync(p.tileEnd, 0, sizeof(int) * numTiles, st) != cudaSuccess)
    return fail(err, errLen, SGLC_ERR_DEVICE, "noalloc draw: cudaMemsetAsync failed");
  launchVertexAndClip(p, st);
  scanExclusive(p.clipExtra, p.clipAppendOff, nullptr, std::max(p.ntri, 1), scan, st);
  launchClipAppend(p, st);
  launchSetup(p, p.primCap, st);
  scanExclusive(p.tileCount, p.pairOff, p.counters + 3, p.primCap, scan, st);
  k_clamp_pairs<<<1, 1, 0, st>>>(p.pairOff + p.primCap, kMaxPairs, p.counters + 4);
  launchBinEmit(p, p.primCap, st);
  int keyBits = 1;
  while ((1 << keyBits) < numTiles) keyBits++;
  sortPairs(p, kMaxPairs, p.counters + 4, keyBits, hist, histScan, scan, st, false, 8);   // 256-bucket digits
  launchTileRanges(p, kMaxPairs, p.counters + 4, st);
  launchTileOrder(p, reinterpret_cast<int *>(scratch + oTileOrder), st);
  p.tileOrder = reinterpret_cast<int *>(scratch + oTileOrder);
  launchRaster(p, true, true, st);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(err, errLen, SGLC_ERR_DEVICE, cudaGetErrorString(e));
  // capacity flags (clip vertices / polygons / appended triangles / bin entries / bad indices)
  int flags = 0;
  if (cudaMemcpyAsync(&flags, p.counters + 2, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return fail(err, errLen, SGLC_ERR_DEVICE, "noalloc draw: reading the capacity flags failed");
  if (flags & 16) return fail(err, errLen, SGLC_ERR_INVALID_VALUE, "noalloc draw: index out of range");
  if (flags) return fail(err, errLen, SGLC_ERR_OVERFLOW, "noalloc draw: a fixed capacity was exceeded");
  return SGLC_OK;
}
