// sm_103a geometry-side kernels of one draw (RendererSoft::draw, RendererSoft.cpp:136-164):
//
//   k_vertex      vertex shader + clip mask + perspective divide + viewport   (:170-190, 971-1003)
//   k_clip        primitive assembly + Sutherland-Hodgman clipping; new vertices re-run the VS on
//                 lerped raw attributes; fan triangles are appended after all input triangles in
//                 input order via a scan of per-triangle counts                (:192-257, 489-559)
//   k_setup       face culling + bounding box + block/quad anchoring + tile range (:277-299, 720-729)
//   k_bin_*       (tile, primitive) pairs in primitive order, stably sorted by tile (LSD radix),
//                 so every tile list is in the reference's primitive order
//   k_scan_*      exclusive scans whose element counts live in device memory
//   k_fill32, k_mip_level, k_swizzle_*   clears, mip chains (SamplerSoft.h:89-115), texture layouts
//
// The raster kernels are in sglc_raster.cuh, instantiated per shading model in sglc_raster_*.cu.
// Every kernel is compiled with --fmad=false (see sglc_device.cuh).
#include <cstdio>

#include "sglc_device.cuh"
#include "sglc_kernels.h"
#include "sglc_shaders.cuh"  // VS bodies

namespace sglc {

enum { CNT_NEWVERT = 0, CNT_POLY = 1, CNT_FLAGS = 2 };
enum { OVF_VERTS = 1, OVF_POLYS = 2, OVF_PRIMS = 4, OVF_PAIRS = 8, OVF_BADINDEX = 16 };

__constant__ float4 kPlanes[6] = {{-1, 0, 0, 1}, {1, 0, 0, 1}, {0, -1, 0, 1}, {0, 1, 0, 1}, {0, 0, -1, 1}, {0, 0, 1, 1}};


__device__ __forceinline__ int clipMaskOf(float4 c) {
  int m = 0;
  if (c.w < c.x) m |= 1;
  if (c.w < -c.x) m |= 2;
  if (c.w < c.y) m |= 4;
  if (c.w < -c.y) m |= 8;
  if (c.w < c.z) m |= 16;
  if (c.w < -c.z) m |= 32;
  return m;
}

// perspectiveDivideImpl + viewportTransformImpl (RendererSoft.cpp:981-992)
__device__ __forceinline__ float4 toScreen(const Viewport &vp, float4 c) {
  float invW = 1.f / c.w;
  float4 f = make_float4(c.x * invW, c.y * invW, c.z * invW, c.w * invW);
  f.w = invW;
  f = make_float4(f.x * vp.pX, f.y * vp.pY, f.z * vp.pZ, f.w * vp.pW);
  return make_float4(f.x + vp.oX, f.y + vp.oY, f.z + vp.oZ, f.w + vp.oW);
}

// ------------------------------------------------------------------------------------------------
// vertex stage
// ------------------------------------------------------------------------------------------------
template<int SH>
__global__ void __launch_bounds__(256) k_vertex(const __grid_constant__ DrawParams p) {
  chainEnter();
  // The warp's 32 attribute rows (the caller's AoS vertex layout) are contiguous in memory unless
  // they straddle two views: they are then read with coalesced 16-byte loads into shared memory
  // (rows at an odd float stride, so the threads' reads of their own rows do not collide) and each
  // thread runs the vertex shader on its row from there. Each warp's 32 varying rows are contiguous
  // too: they are staged in the same buffer and written as one contiguous run of 16-byte stores
  // (varyStride <= 32 floats for every model).
  __shared__ float4 stage[8][32 * 8];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = p.varyStride / 4;
  const int sf = p.strideF;
  const int i0 = i - lane;
  const int rows = min(32, p.nv - i0);
  float *sa = reinterpret_cast<float *>(stage[warp]);
  bool staged = false;
  if (rows > 0 && (sf & 3) == 0 && sf <= 28) {   // 32 rows of sf + 1 floats fit the warp's buffer
    int v0 = 0, v1 = 0;
    const float *src;
    if (p.scenes) {
      v0 = sceneOf(p.sceneVBase, p.views, i0);
      v1 = sceneOf(p.sceneVBase, p.views, i0 + rows - 1);
      src = p.scenes[v0].attr + (size_t) (i0 - p.sceneVBase[v0]) * sf;
    } else if (p.views > 1) {
      v0 = i0 / p.nvView;
      v1 = (i0 + rows - 1) / p.nvView;
      src = p.attr + (size_t) (i0 - v0 * p.nvView) * sf;
    } else {
      src = p.attr + (size_t) i0 * sf;
    }
    if (v0 == v1) {   // warp-uniform
      const int q4 = sf >> 2;
      const float4 *s4 = reinterpret_cast<const float4 *>(src);   // rows are multiples of 16 bytes
      for (int e = lane; e < rows * q4; e += 32) {
        const float4 f = __ldg(s4 + e);
        const int r = e / q4;
        float *d = sa + r * (sf + 1) + 4 * (e - r * q4);
        d[0] = f.x;
        d[1] = f.y;
        d[2] = f.z;
        d[3] = f.w;
      }
      __syncwarp();
      staged = true;
    }
  }
  float v[32];
#pragma unroll
  for (int k = 0; k < 32; k++) v[k] = 0.f;
  if (i < p.nv) {
    int view;
    const float *a;
    if (p.scenes) {   // a multi-scene draw: the scene's own vertex rows
      view = sceneOf(p.sceneVBase, p.views, i);
      a = p.scenes[view].attr + (size_t) (i - p.sceneVBase[view]) * sf;
    } else {
      view = p.views > 1 ? i / p.nvView : 0;
      a = p.attr + (size_t) (i - view * p.nvView) * sf;
    }
    if (staged) a = sa + lane * (sf + 1);
    float4 c = runVS<SH>(p, viewUniforms(p, view), a, v);
    p.vClip[i] = c;
    p.vMask[i] = (uint8_t) clipMaskOf(c);
    p.vFrag[i] = toScreen(viewViewport(p, view), c);
  }
  float4 *st = stage[warp];
  __syncwarp();   // every lane has read its attribute row from the buffer
#pragma unroll
  for (int k = 0; k < 8; k++)
    if (k < q) st[lane * q + k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
  __syncwarp();
  if (rows > 0) {
    float4 *dst = reinterpret_cast<float4 *>(p.vVary + (size_t) i0 * p.varyStride);
    for (int e = lane; e < rows * q; e += 32) dst[e] = st[e];
  }
}

// ------------------------------------------------------------------------------------------------
// assembly + clipping
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ const float *attrOf(const DrawParams &p, int idx) {
  if (idx >= p.nv) return p.vAttrExtra + (size_t) (idx - p.nv) * p.strideF;
  if (p.scenes) {
    const int v = sceneOf(p.sceneVBase, p.views, idx);
    return p.scenes[v].attr + (size_t) (idx - p.sceneVBase[v]) * p.strideF;
  }
  return p.attr + (size_t) (idx % p.nvView) * p.strideF;
}

template<int SH>
__device__ int newClipVertex(const DrawParams &p, int view, int i0, int i1, float t) {
  int k = atomicAdd(&p.counters[CNT_NEWVERT], 1);
  int idx = p.nv + k;
  if (idx >= p.vCap) {
    atomicOr(&p.counters[CNT_FLAGS], OVF_VERTS);
    return -1;
  }
  const float *A0 = attrOf(p, i0), *A1 = attrOf(p, i1);
  float *dst = p.vAttrExtra + (size_t) k * p.strideF;
  for (int j = 0; j < p.strideF; j++) dst[j] = A0[j] * (1.f - t) + A1[j] * t;   // glm::mix
  float *v = p.vVary + (size_t) idx * p.varyStride;
  float4 c = runVS<SH>(p, viewUniforms(p, view), dst, v);
  p.vClip[idx] = c;
  p.vMask[idx] = (uint8_t) clipMaskOf(c);
  p.vFrag[idx] = toScreen(viewViewport(p, view), c);
  return idx;
}

// exclusive scans: tiles of kScanTile elements, kScanThreads threads per tile
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

template<int SH>
__global__ void __launch_bounds__(128) k_clip(const __grid_constant__ DrawParams p) {
  chainEnter();
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= p.ntri) return;
  int view, lt, nvView, vBase;
  const int *indices;
  if (p.scenes) {   // a multi-scene draw: the scene's own indices into its own vertex rows
    view = sceneOf(p.sceneTBase, p.views, t);
    lt = t - p.sceneTBase[view];
    indices = p.scenes[view].indices;
    nvView = p.scenes[view].nv;
    vBase = p.sceneVBase[view];
  } else {
    view = p.views > 1 ? t / p.ntriView : 0;
    lt = t - view * p.ntriView;
    indices = p.indices;
    nvView = p.nvView;
    vBase = view * p.nvView;
  }
  const int viewBits = view << 8;   // primitive flags: bit 0 discard, bits 8+ view
  int i0 = indices[3 * lt], i1 = indices[3 * lt + 1], i2 = indices[3 * lt + 2];
  p.clipExtra[t] = 0;
  if ((unsigned) i0 >= (unsigned) nvView || (unsigned) i1 >= (unsigned) nvView || (unsigned) i2 >= (unsigned) nvView) {
    atomicOr(&p.counters[CNT_FLAGS], OVF_BADINDEX);
    p.prims[t] = make_int4(0, 0, 0, 1);
    return;
  }
  i0 += vBase;
  i1 += vBase;
  i2 += vBase;
  int mask = p.vMask[i0] | p.vMask[i1] | p.vMask[i2];
  if (mask == 0) {
    p.prims[t] = make_int4(i0, i1, i2, viewBits);
    return;
  }
  // Sutherland-Hodgman over the flagged planes (RendererSoft.cpp:489-559)
  int in[12], out[12];
  int nin = 3, nout;
  in[0] = i0; in[1] = i1; in[2] = i2;
  bool full = false;
  for (int pl = 0; pl < 6; pl++) {
    if (!(mask & (1 << pl))) continue;
    if (nin < 3) {
      full = true;
      break;
    }
    nout = 0;
    if (nin > 10) {
      atomicOr(&p.counters[CNT_FLAGS], OVF_POLYS);
      p.prims[t] = make_int4(0, 0, 0, 1);
      return;
    }
    float4 P = kPlanes[pl];
    int pre = in[0];
    float dPre = dot4(P, p.vClip[pre]);
    in[nin] = pre;
    for (int k = 1; k <= nin; k++) {
      int cur = in[k];
      float d = dot4(P, p.vClip[cur]);
      if (nout > 9) {   // a convex clip adds at most one vertex per plane; more means degenerate input
        atomicOr(&p.counters[CNT_FLAGS], OVF_POLYS);
        p.prims[t] = make_int4(0, 0, 0, 1);
        return;
      }
      if (dPre >= 0) out[nout++] = pre;
      if (signbit(dPre) != signbit(d)) {
        float tt = d < 0 ? dPre / (dPre - d) : -dPre / (d - dPre);
        int nvid = newClipVertex<SH>(p, view, pre, cur, tt);
        if (nvid < 0) {
          p.prims[t] = make_int4(0, 0, 0, 1);
          return;
        }
        out[nout++] = nvid;
      }
      pre = cur;
      dPre = d;
    }
    for (int k = 0; k < nout; k++) in[k] = out[k];
    nin = nout;
  }
  if (full || nin == 0) {
    p.prims[t] = make_int4(0, 0, 0, 1);
    return;
  }
  if (nin > 11) {
    atomicOr(&p.counters[CNT_FLAGS], OVF_POLYS);
    p.prims[t] = make_int4(0, 0, 0, 1);
    return;
  }
  p.prims[t] = make_int4(in[0], in[1], in[2], viewBits);
  if (nin > 3) {
    int slot = atomicAdd(&p.counters[CNT_POLY], 1);
    if (slot >= p.clipPolyCap) {
      atomicOr(&p.counters[CNT_FLAGS], OVF_POLYS);
      return;
    }
    int4 *dst = p.clipPoly + (size_t) slot * 3;
    dst[0] = make_int4(nin, in[0], in[1], in[2]);
    dst[1] = make_int4(nin > 3 ? in[3] : 0, nin > 4 ? in[4] : 0, nin > 5 ? in[5] : 0, nin > 6 ? in[6] : 0);
    dst[2] = make_int4(nin > 7 ? in[7] : 0, nin > 8 ? in[8] : 0, nin > 9 ? in[9] : 0, nin > 10 ? in[10] : 0);
    p.clipPolyTri[slot] = t;
    p.clipExtra[t] = nin - 3;
    // the reduce step of the scan of clipExtra (scan tile totals); clipped triangles are few
    if (p.clipScanSums && nin > 3) atomicAdd(&p.clipScanSums[t / kScanTile], nin - 3);
  }
}

// number of primitives after clipping, kept on the device for the count-driven kernels
__global__ void k_clip_append(const __grid_constant__ DrawParams p) {
  chainEnter();
  int slot = blockIdx.x * blockDim.x + threadIdx.x;
  // the draw's primitive count: input triangles plus the appended fan triangles
  if (slot == 0) p.counters[3] = min(p.ntri + p.clipAppendOff[p.ntri], p.primCap);
  int n = min(p.counters[CNT_POLY], p.clipPolyCap);
  if (slot >= n) return;
  int t = p.clipPolyTri[slot];
  const int4 *src = p.clipPoly + (size_t) slot * 3;
  int4 a = src[0], b = src[1], c = src[2];
  int ids[11] = {a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w};
  int nin = a.x;
  int base = p.ntri + p.clipAppendOff[t];
  const int viewBits = (p.scenes ? sceneOf(p.sceneTBase, p.views, t) : (p.views > 1 ? t / p.ntriView : 0)) << 8;
  for (int k = 3; k < nin; k++) {
    int dst = base + k - 3;
    if (dst >= p.primCap) {
      atomicOr(&p.counters[CNT_FLAGS], OVF_PRIMS);
      return;
    }
    p.prims[dst] = make_int4(ids[0], ids[k - 1], ids[k], viewBits);
  }
}

// ------------------------------------------------------------------------------------------------
// setup: culling, bounding box, block anchoring, tile range
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }   // std::min
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }   // std::max

// A triangle that can cover no sample point is not binned (its fragments and depth writes are
// none either way):
// * |uz| below FLT_EPSILON: the reference's barycentric() rejects it at every point
//   (RendererSoft.cpp:1035-1037; uz as it computes it, from the vertices' differences);
// * a small, well-shaped triangle (bounding-box extent L in [1/256, 1] pixel, |uz| >= 0.01 L^2)
//   whose bounding box grown by m = 1/32 pixel holds none of the draw's sample points (the pixel
//   centre, or the four 4x MSAA positions). A point outside the box by m has a barycentric at most
//   -m / (2 L) (the negative ones sum to at least m / L), while the rounding of the reference's
//   edge functions there (exact vertex differences, products of magnitude <= 3 px^2) moves a
//   barycentric by at most ~6e-7 / |uz| + 3e-5 |b|, far less for these triangles: the test cannot
//   accept the point. Dense meshes at low resolution are mostly such sub-pixel triangles.
__device__ __forceinline__ bool coversNoSample(const DrawParams &p, float4 a, float4 b, float4 c) {
  const float a0 = c.x - a.x, a1 = b.x - a.x, c0 = c.y - a.y, c1 = b.y - a.y;   // v2 - v0, v1 - v0
  const float uz = a0 * c1 - a1 * c0;
  if (fabsf(uz) < 1.19209290e-07f) return true;
  const float x0 = smin(smin(a.x, b.x), c.x), x1 = smax(smax(a.x, b.x), c.x);
  const float y0 = smin(smin(a.y, b.y), c.y), y1 = smax(smax(a.y, b.y), c.y);
  const float L = smax(x1 - x0, y1 - y0);
  if (!(L >= 1.f / 256.f && L <= 1.f && fabsf(uz) >= 0.01f * L * L)) return false;
  const float m = 1.f / 32.f;
  const int n = p.samples == 4 ? 4 : 1;
  // 4x MSAA sample positions inside a pixel (RendererInternal.h), else the pixel centre
  const float sx4[4] = {0.375f, 0.875f, 0.125f, 0.625f}, sy4[4] = {0.875f, 0.625f, 0.375f, 0.125f};
  for (int i = 0; i < n; i++) {
    const float ox = n == 4 ? sx4[i] : 0.5f, oy = n == 4 ? sy4[i] : 0.5f;
    // the smallest sample coordinate k + o >= lo, for both axes; a sample lies in the box if both fit
    const float sx = ceilf(x0 - m - ox) + ox, sy = ceilf(y0 - m - oy) + oy;
    if (sx <= x1 + m && sy <= y1 + m) return false;
  }
  return true;
}

// one primitive's setup; returns its upper bound on emitted fragments
__device__ __forceinline__ unsigned long long setupPrim(const DrawParams &p, int i) {
  int4 pr = p.prims[i];
  TriSetup T;
  int cnt = 0;
  T.rx0 = 1;
  T.rx1 = 0;
  T.ry0 = 1;
  T.ry1 = 0;
  if (!(pr.w & 1)) {
    float4 a = p.vFrag[pr.x], b = p.vFrag[pr.y], c = p.vFrag[pr.z];
    // processFaceCulling (RendererSoft.cpp:287-297)
    f3 e1 = mk3(b.x - a.x, b.y - a.y, b.z - a.z), e2 = mk3(c.x - a.x, c.y - a.y, c.z - a.z);
    f3 n = cross3(e1, e2);
    float area = (n.x * 0.f + n.y * 0.f) + n.z * 1.f;
    bool front = area > 0;
    bool discard = p.cullFace && !front;
    // triangleBoundingBox (RendererSoft.cpp:1005-1019) then bounds.min -= 1 (:725)
    float minX = smin(smin(a.x, b.x), c.x), minY = smin(smin(a.y, b.y), c.y);
    float maxX = smax(smax(a.x, b.x), c.x), maxY = smax(smax(a.y, b.y), c.y);
    minX = smax(minX - 0.5f, 0.f);
    minY = smax(minY - 0.5f, 0.f);
    const Viewport &vp = viewViewport(p, pr.w >> 8);
    maxX = smin(maxX + 0.5f, vp.w - 1.f);
    maxY = smin(maxY + 0.5f, vp.h - 1.f);
    minX -= 1.f;
    minY -= 1.f;
    if (!(isfinite(minX) && isfinite(minY) && isfinite(maxX) && isfinite(maxY))) discard = true;
    if (!discard && coversNoSample(p, a, b, c)) discard = true;
    if (!discard) {
      int bcx = (int) (((maxX - minX) + (float) kBlock - 1.f) / (float) kBlock);
      int bcy = (int) (((maxY - minY) + (float) kBlock - 1.f) / (float) kBlock);
      T.v0x = a.x; T.v0y = a.y;
      T.f0x = c.x; T.f0y = b.x; T.f0z = a.x;
      T.f1x = c.y; T.f1y = b.y; T.f1z = a.y;
      T.z0 = a.z; T.z1 = b.z; T.z2 = c.z;
      T.w0 = a.w; T.w1 = b.w; T.w2 = c.w;
      T.bminx = minX; T.bminy = minY; T.bmaxx = maxX; T.bmaxy = maxY;
      T.bcx = bcx; T.bcy = bcy;
      T.vid0 = pr.x; T.vid1 = pr.y; T.vid2 = pr.z;
      T.front = front;
      T.view = pr.w >> 8;
      if (bcx > 0 && bcy > 0) {
        int bsx0 = (int) (minX + 0.f), bsy0 = (int) (minY + 0.f);
        int bsxL = (int) (minX + (float) ((bcx - 1) * kBlock)), bsyL = (int) (minY + (float) ((bcy - 1) * kBlock));
        int fw = max(p.cw, p.dw), fh = max(p.ch, p.dh);
        if (p.scenes) {
          const SceneRec &S = p.scenes[T.view];
          fw = max(S.cw, S.dw);
          fh = max(S.ch, S.dh);
        }
        T.rx0 = max(bsx0 + 1, 0);
        T.ry0 = max(bsy0 + 1, 0);
        T.rx1 = min(min((int) floorf(maxX) + 1, bsxL + kBlock), fw - 1);
        T.ry1 = min(min((int) floorf(maxY) + 1, bsyL + kBlock), fh - 1);
        if (T.rx1 >= T.rx0 && T.ry1 >= T.ry0) {
          int tx0 = T.rx0 / p.tile, tx1 = T.rx1 / p.tile, ty0 = T.ry0 / p.tileH, ty1 = T.ry1 / p.tileH;
          cnt = (tx1 - tx0 + 1) * (ty1 - ty0 + 1);
        }
      }
    }
  }
  if (cnt) p.tri[i] = T;   // only binned primitives are read again (bin emission, raster)
  p.tileCount[i] = cnt;
  // upper bound on the fragments the raster can emit for this primitive: each pixel of its quad
  // rectangle once, plus one more per row / column where two adjacent 32x32 blocks overlap
  return cnt ? (unsigned long long) (T.rx1 - T.rx0 + T.bcx) * (unsigned long long) (T.ry1 - T.ry0 + T.bcy) : 0ull;
}

__global__ void __launch_bounds__(256) k_setup(const __grid_constant__ DrawParams p) {
  chainEnter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int np = min(p.ntri + p.clipAppendOff[p.ntri], p.primCap);
  unsigned long long bound = i < np ? setupPrim(p, i) : 0ull;
  if (p.tileScanSums) {   // the reduce step of the scan of tileCount: a warp's primitives share a scan tile
    int cnt = i < np ? p.tileCount[i] : 0;
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&p.tileScanSums[i / kScanTile], cnt);
  }
  for (int o = 16; o > 0; o >>= 1) bound += __shfl_down_sync(0xffffffffu, bound, o);
  if ((threadIdx.x & 31) == 0 && bound)
    atomicAdd(reinterpret_cast<unsigned long long *>(p.counters + kCntBound), bound);
}

__global__ void __launch_bounds__(256) k_bin_emit(const __grid_constant__ DrawParams p) {
  chainEnter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  // two set-up steps that would otherwise be launches of their own: clearing the tile ranges
  // (k_tile_ranges fills the non-empty ones) and the bin-entry count clamped to the capacity
  if (p.binZeroRanges)
    for (int t = i; t < p.numTiles; t += gridDim.x * blockDim.x) p.tileStart[t] = p.tileEnd[t] = 0;
  if (p.binPairTotal && i == 0) p.counters[4] = min(*p.binPairTotal, p.pairCap);
  int np = min(p.ntri + p.clipAppendOff[p.ntri], p.primCap);
  if (i >= np || p.tileCount[i] == 0) return;
  const TriSetup &T = p.tri[i];
  int off = p.pairOff[i];
  const uint32_t viewBase =
      p.scenes ? (uint32_t) p.sceneTileBase[T.view] : (uint32_t) T.view * (uint32_t) p.tilesPerView;
  const int tilesX = p.scenes ? p.scenes[T.view].tilesX : p.tilesX;
  int tx0 = T.rx0 / p.tile, tx1 = T.rx1 / p.tile, ty0 = T.ry0 / p.tileH, ty1 = T.ry1 / p.tileH;
  for (int ty = ty0; ty <= ty1; ty++)
    for (int tx = tx0; tx <= tx1; tx++) {
      if (off >= p.pairCap) {
        atomicOr(&p.counters[CNT_FLAGS], OVF_PAIRS);
        return;
      }
      p.keyA[off] = viewBase + (uint32_t) (ty * tilesX + tx);
      p.valA[off] = i;
      off++;
    }
}

// ------------------------------------------------------------------------------------------------
// stable LSD radix sort of (tile, primitive) pairs by tile, 8-bit digits
// ------------------------------------------------------------------------------------------------

template<int ITEMS>
__global__ void __launch_bounds__(kSortThreads) k_radix_hist(const uint32_t *keys, const int *nPtr, int shift,
                                                             int bits, int *hist, int numBlocks) {
  constexpr int TILE = kSortThreads * ITEMS;
  chainEnter();
  __shared__ int h[1 << kMaxDigitBits];
  const int buckets = 1 << bits;
  const uint32_t mask = (uint32_t) buckets - 1u;
  int n = *nPtr;
  for (int d = threadIdx.x; d < buckets; d += blockDim.x) h[d] = 0;
  __syncthreads();
  int base = blockIdx.x * TILE;
  for (int k = 0; k < ITEMS; k++) {
    int i = base + k * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & mask], 1);
  }
  __syncthreads();
  for (int d = threadIdx.x; d < buckets; d += blockDim.x) hist[d * numBlocks + blockIdx.x] = h[d];
}

// Items of a CTA are split into 8 contiguous warp ranges of 32 ITEMS; each warp ranks its range in
// order (match.any + popc), then warp prefixes per digit make the scatter stable.
template<int ITEMS>
__global__ void __launch_bounds__(kSortThreads) k_radix_scatter(const uint32_t *keysIn, const int *valsIn,
                                                                uint32_t *keysOut, int *valsOut, const int *nPtr,
                                                                int shift, int bits, const int *histOff,
                                                                int numBlocks) {
  chainEnter();
  __shared__ int wcount[8][1 << kMaxDigitBits];
  const int buckets = 1 << bits;
  const uint32_t mask = (uint32_t) buckets - 1u;
  int n = *nPtr;
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int d = lane; d < buckets; d += 32) wcount[warp][d] = 0;
  __syncwarp();
  constexpr int TILE = kSortThreads * ITEMS;
  int base = blockIdx.x * TILE + warp * (TILE / 8);
  uint32_t myKey[ITEMS];
  int myVal[ITEMS], myPos[ITEMS], myDig[ITEMS];
  unsigned lt = (1u << lane) - 1u;
  for (int k = 0; k < ITEMS; k++) {
    int i = base + k * 32 + lane;
    bool valid = i < n;
    uint32_t key = valid ? keysIn[i] : 0u;
    int dig = valid ? (int) ((key >> shift) & mask) : buckets;
    unsigned peers = __match_any_sync(0xffffffffu, dig);
    int rank = __popc(peers & lt);
    int before = dig < buckets ? wcount[warp][dig] : 0;
    __syncwarp();
    if (dig < buckets && rank == 0) wcount[warp][dig] = before + __popc(peers);
    __syncwarp();
    myKey[k] = key;
    myVal[k] = valid ? valsIn[i] : 0;
    myDig[k] = dig;
    myPos[k] = before + rank;
  }
  __syncthreads();
  // exclusive prefix over warps for each digit
  for (int d = threadIdx.x; d < buckets; d += blockDim.x) {
    int s = 0;
    for (int w = 0; w < 8; w++) {
      int c = wcount[w][d];
      wcount[w][d] = s;
      s += c;
    }
  }
  __syncthreads();
  for (int k = 0; k < ITEMS; k++) {
    int d = myDig[k];
    if (d >= buckets) continue;
    int pos = histOff[d * numBlocks + blockIdx.x] + wcount[warp][d] + myPos[k];
    keysOut[pos] = myKey[k];
    valsOut[pos] = myVal[k];
  }
}

__global__ void k_tile_ranges(const uint32_t *keys, const int *nPtr, int *tileStart, int *tileEnd) {
  chainEnter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int n = *nPtr;
  if (i >= n) return;
  uint32_t k = keys[i];
  if (i == 0 || keys[i - 1] != k) tileStart[k] = i;
  if (i == n - 1 || keys[i + 1] != k) tileEnd[k] = i + 1;
}

// bucket of tile t in the heavy-first order: log2 of its list length (0: empty), 33: no tile
__device__ __forceinline__ int orderBucket(const int *tileStart, const int *tileEnd, int numTiles, int t) {
  if (t >= numTiles) return 33;
  const int len = tileEnd[t] - tileStart[t];
  return len > 0 ? 32 - __clz(len) : 0;
}

// Raster CTA order: tiles bucketed by log2 of their list length, longest first, so the tiles that
// take longest start first and do not form the tail of the launch. One CTA; order within a bucket
// is arbitrary (tiles are independent). Most tiles of a frame fall in a few buckets (the empty one
// above all), so each warp adds its lanes of one bucket with one shared-memory atomic; each thread
// issues the loads of K tiles before it uses them.
__global__ void __launch_bounds__(1024) k_tile_order(const int *tileStart, const int *tileEnd, int numTiles,
                                                     int *order) {
  chainEnter();
  constexpr int K = 8;   // tiles per thread and sweep, their loads issued together
  __shared__ int cnt[33], off[33];
  const int lane = threadIdx.x & 31;
  if (threadIdx.x < 33) cnt[threadIdx.x] = 0;
  __syncthreads();
  const int sweep = K * blockDim.x;
  for (int base = 0; base < numTiles; base += sweep) {   // uniform bounds: whole warps every round
    int b[K];
#pragma unroll
    for (int k = 0; k < K; k++) b[k] = orderBucket(tileStart, tileEnd, numTiles, base + k * blockDim.x + threadIdx.x);
#pragma unroll
    for (int k = 0; k < K; k++) {
      const unsigned peers = __match_any_sync(0xffffffffu, b[k]);
      if (b[k] < 33 && lane == __ffs(peers) - 1) atomicAdd(&cnt[b[k]], __popc(peers));
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int b = 32; b >= 0; b--) {
      off[b] = s;
      s += cnt[b];
    }
  }
  __syncthreads();
  for (int base = 0; base < numTiles; base += sweep) {
    int b[K];
#pragma unroll
    for (int k = 0; k < K; k++) b[k] = orderBucket(tileStart, tileEnd, numTiles, base + k * blockDim.x + threadIdx.x);
#pragma unroll
    for (int k = 0; k < K; k++) {
      const int t = base + k * blockDim.x + threadIdx.x;
      const unsigned peers = __match_any_sync(0xffffffffu, b[k]);
      const int leader = __ffs(peers) - 1;
      int first = 0;
      if (b[k] < 33 && lane == leader) first = atomicAdd(&off[b[k]], __popc(peers));
      first = __shfl_sync(0xffffffffu, first, leader);
      if (b[k] < 33) order[first + __popc(peers & ((1u << lane) - 1u))] = t;
    }
  }
}

// ------------------------------------------------------------------------------------------------
// exclusive scan (three phases), counts read from device memory
// ------------------------------------------------------------------------------------------------

__device__ __forceinline__ int blockExclusiveScan(int v, int *total) {
  __shared__ int warpSums[32];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warpSums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int nw = blockDim.x >> 5;
    int s = lane < nw ? warpSums[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) warpSums[lane] = s;
  }
  __syncthreads();
  int warpPrefix = warp > 0 ? warpSums[warp - 1] : 0;
  *total = warpSums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warpPrefix + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_local(const int *in, int *out, const int *nPtr, int nMax,
                                                             int *blockSums) {
  chainEnter();
  int n = nPtr ? min(*nPtr, nMax) : nMax;
  int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems], s = 0;
  for (int k = 0; k < kScanItems; k++) {
    int i = base + k;
    v[k] = i < n ? in[i] : 0;
    s += v[k];
  }
  int total;
  int pre = blockExclusiveScan(s, &total);
  for (int k = 0; k < kScanItems; k++) {
    int i = base + k;
    if (i < nMax) out[i] = pre;
    pre += v[k];
  }
  if (threadIdx.x == 0) blockSums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int *blockSums, int numBlocks) {
  chainEnter();
  // single CTA: exclusive scan of up to kScanTile block sums, in place; total at [numBlocks]
  int base = threadIdx.x * kScanItems;
  int v[kScanItems], s = 0;
  for (int k = 0; k < kScanItems; k++) {
    int i = base + k;
    v[k] = i < numBlocks ? blockSums[i] : 0;
    s += v[k];
  }
  int total;
  int pre = blockExclusiveScan(s, &total);
  for (int k = 0; k < kScanItems; k++) {
    int i = base + k;
    if (i < numBlocks) blockSums[i] = pre;
    pre += v[k];
  }
  if (threadIdx.x == 0) blockSums[numBlocks] = total;
}

__global__ void k_scan_add(int *out, const int *nPtr, int nMax, const int *blockSums, int numBlocks) {
  chainEnter();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  int n = nPtr ? min(*nPtr, nMax) : nMax;
  if (i < nMax) out[i] += blockSums[i / kScanTile];
  if (i == 0) out[nMax] = blockSums[numBlocks];
  (void) n;
}

// Two-launch exclusive scan (reduce, then apply): the apply kernel sums the tile totals before its
// own tile itself instead of reading them from a third launch's scan. Tiles of kScanTile elements;
// at most kScanTile tiles, as for the three-launch form.
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const int *in, const int *nPtr, int nMax,
                                                              int *blockSums) {
  chainEnter();
  const int n = nPtr ? min(*nPtr, nMax) : nMax;
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int s = 0;
  for (int k = 0; k < kScanItems; k++) s += base + k < n ? in[base + k] : 0;
  int total;
  blockExclusiveScan(s, &total);
  if (threadIdx.x == 0) blockSums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const int *in, int *out, const int *nPtr, int nMax,
                                                             const int *blockSums) {
  chainEnter();
  const int n = nPtr ? min(*nPtr, nMax) : nMax;
  int before = 0;
  for (int j = threadIdx.x; j < (int) blockIdx.x; j += blockDim.x) before += blockSums[j];
  int prefix;
  blockExclusiveScan(before, &prefix);
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  int v[kScanItems], s = 0;
  for (int k = 0; k < kScanItems; k++) {
    v[k] = base + k < n ? in[base + k] : 0;
    s += v[k];
  }
  int total;
  int pre = prefix + blockExclusiveScan(s, &total);
  for (int k = 0; k < kScanItems; k++) {
    if (base + k < nMax) out[base + k] = pre;
    pre += v[k];
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[nMax] = prefix + total;
}

// ------------------------------------------------------------------------------------------------
// clear, mip generation
// ------------------------------------------------------------------------------------------------
__global__ void k_fill32(uint32_t *dst, uint32_t value, size_t n) {
  size_t i = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
  size_t stride = (size_t) gridDim.x * blockDim.x;
  for (; i < n; i += stride) dst[i] = value;
}

// BaseSampler::sampleBufferBilinear (SamplerSoft.h:240-252): level l from level l-1
__global__ void k_mip_level(DevTex t, int face, int level, int isFloat) {
  int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  int w = t.w[level], h = t.h[level];
  if (x >= w || y >= h) return;
  float rx = (float) t.w[level - 1] / (float) w, ry = (float) t.h[level - 1] / (float) h;
  float dx = 0.5f * rx, dy = 0.5f * ry;
  float u = (float) x * rx + dx, v = (float) y * ry + dy;
  uint32_t c = bilinearPx(t, face, level - 1, u, v, WRAP_EDGE, 0u, isFloat != 0);
  uint32_t *dst = const_cast<uint32_t *>(t.base) + (size_t) face * t.layerStride + t.offset[level] + texIndex(t, level, x, y);
  *dst = c;
}

// linear host image -> the texture's storage layout
__global__ void k_swizzle_in(DevTex t, int face, int level, const uint32_t *src) {
  int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  int w = t.w[level], h = t.h[level];
  if (x >= w || y >= h) return;
  uint32_t *dst = const_cast<uint32_t *>(t.base) + (size_t) face * t.layerStride + t.offset[level] + texIndex(t, level, x, y);
  *dst = src[(size_t) y * w + x];
}

__global__ void k_swizzle_out(DevTex t, int face, int level, uint32_t *dst) {
  int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
  int w = t.w[level], h = t.h[level];
  if (x >= w || y >= h) return;
  dst[(size_t) y * w + x] = texel(t, face, level, x, y);
}

// ------------------------------------------------------------------------------------------------
// host-side launchers
// ------------------------------------------------------------------------------------------------
static inline int cdiv(long a, long b) { return (int) ((a + b - 1) / b); }

void scanExclusive(const int *in, int *out, const int *nPtr, int nMax, int *blockSums, cudaStream_t st) {
  int nb = max(1, cdiv(nMax, kScanTile));
  launchChained(k_scan_local, dim3(nb), dim3(kScanThreads), 0, st, in, out, nPtr, nMax, blockSums);
  launchChained(k_scan_sums, dim3(1), dim3(kScanThreads), 0, st, blockSums, nb);
  launchChained(k_scan_add, dim3(max(1, cdiv(nMax, 256))), dim3(256), 0, st, out, nPtr, nMax, blockSums, nb);
}

int scanScratchInts(int nMax) { return max(1, cdiv(nMax, kScanTile)) + 1; }

void scanApply(const int *in, int *out, const int *nPtr, int nMax, const int *blockSums, cudaStream_t st) {
  int nb = max(1, cdiv(nMax, kScanTile));
  launchChained(k_scan_apply, dim3(nb), dim3(kScanThreads), 0, st, in, out, nPtr, nMax, blockSums);
}

int scanTiles(int nMax) { return max(1, cdiv(nMax, kScanTile)); }

void scanExclusive2(const int *in, int *out, const int *nPtr, int nMax, int *blockSums, cudaStream_t st) {
  int nb = max(1, cdiv(nMax, kScanTile));
  launchChained(k_scan_reduce, dim3(nb), dim3(kScanThreads), 0, st, in, nPtr, nMax, blockSums);
  launchChained(k_scan_apply, dim3(nb), dim3(kScanThreads), 0, st, in, out, nPtr, nMax, (const int *) blockSums);
}

// ------------------------------------------------------------------------------------------------
// points and lines: assembly, clipping and culling into drawing-order slots
// ------------------------------------------------------------------------------------------------
// clippingLine (RendererSoft.cpp:443-487): parametric clip against the planes either end is outside
// of; the far end is re-made from the already re-made near end, as the reference updates
// indices[0] before its second clippingNewVertex call. Returns false when the line is culled (or
// the vertex capacity ran out, flagged).
template<int SH>
__device__ bool clipLine(const DrawParams &p, int &a, int &b) {
  const int m0 = p.vMask[a], m1 = p.vMask[b];
  const float4 c0 = p.vClip[a], c1 = p.vClip[b];
  float t0 = 0.f, t1 = 1.f;
  const int mask = m0 | m1;
  for (int pl = 0; pl < 6 && mask; pl++) {
    if (!(mask & (1 << pl))) continue;
    float d0 = dot4(kPlanes[pl], c0), d1 = dot4(kPlanes[pl], c1);
    if (d0 < 0 && d1 < 0) return false;
    if (d0 < 0) {
      float t = -d0 / (d1 - d0);
      t0 = (t0 < t) ? t : t0;   // std::max
    } else {
      float t = d0 / (d0 - d1);
      t1 = (t < t1) ? t : t1;   // std::min
    }
  }
  if (m0) {
    a = newClipVertex<SH>(p, 0, a, b, t0);
    if (a < 0) return false;
  }
  if (m1) {
    b = newClipVertex<SH>(p, 0, a, b, t1);
    if (b < 0) return false;
  }
  return true;
}

// One thread per input primitive: processPointAssembly / processLineAssembly /
// processPolygonAssembly (:409-437), clippingPoint / clippingLine (:439-487), face culling of
// triangles (:277-299) and the per-triangle point / edge loops of rasterizationPolygonsPoint /
// rasterizationPolygonsLine (:575-622). Triangles drawn as points or lines are not clipped as
// triangles; their edges are clipped as lines, their corners as points.
template<int SH>
__global__ void __launch_bounds__(128) k_lp_assemble(const __grid_constant__ DrawParams p,
                                                     const __grid_constant__ LineParams lp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= lp.nIn) return;
  int4 *out = lp.slot + (size_t) 3 * i;
  int4 s[3] = {make_int4(0, 0, 0, 0), make_int4(0, 0, 0, 0), make_int4(0, 0, 0, 0)};
  const int per = lp.mode == LP_POINTS ? 1 : (lp.mode == LP_LINES ? 2 : 3);
  int idx[3] = {0, 0, 0};
  bool ok = true;
  for (int k = 0; k < per; k++) {
    idx[k] = p.indices[(size_t) per * i + k];
    if ((unsigned) idx[k] >= (unsigned) p.nv) ok = false;
  }
  if (!ok) {
    atomicOr(lp.flags, LP_ERR_BADINDEX);
  } else if (lp.mode == LP_POINTS) {
    if (p.vMask[idx[0]] == 0) s[0] = make_int4(LP_SLOT_POINT, idx[0], 0, 0);
  } else if (lp.mode == LP_LINES) {
    int a = idx[0], b = idx[1];
    if (clipLine<SH>(p, a, b)) s[0] = make_int4(LP_SLOT_LINE, a, b, 0);
  } else {
    float4 a = p.vFrag[idx[0]], b = p.vFrag[idx[1]], c = p.vFrag[idx[2]];
    f3 e1 = mk3(b.x - a.x, b.y - a.y, b.z - a.z), e2 = mk3(c.x - a.x, c.y - a.y, c.z - a.z);
    f3 n = cross3(e1, e2);
    float area = (n.x * 0.f + n.y * 0.f) + n.z * 1.f;
    if (!(p.cullFace && !(area > 0))) {
      for (int k = 0; k < 3; k++) {
        if (lp.mode == LP_TRI_POINTS) {
          if (p.vMask[idx[k]] == 0) s[k] = make_int4(LP_SLOT_POINT, idx[k], 0, 0);
        } else {
          int va = idx[k], vb = idx[(k + 1) % 3];
          if (clipLine<SH>(p, va, vb)) s[k] = make_int4(LP_SLOT_LINE, va, vb, 0);
        }
      }
    }
  }
  out[0] = s[0];
  out[1] = s[1];
  out[2] = s[2];
}

template<int SH>
static void launchGeometry(const DrawParams &p, cudaStream_t st) {
  if (p.nv > 0) launchChained(k_vertex<SH>, dim3(cdiv(p.nv, 256)), dim3(256), 0, st, p);
  if (p.ntri > 0) launchChained(k_clip<SH>, dim3(cdiv(p.ntri, 128)), dim3(128), 0, st, p);
}

template<int SH>
static void pointsLinesGeometry(const DrawParams &p, const LineParams &lp, cudaStream_t st) {
  if (p.nv > 0) launchChained(k_vertex<SH>, dim3(cdiv(p.nv, 256)), dim3(256), 0, st, p);
  if (lp.nIn > 0) k_lp_assemble<SH><<<cdiv(lp.nIn, 128), 128, 0, st>>>(p, lp);
}

#define SGLC_GEOMETRY_SWITCH(FN, ...)                                 \
  switch (p.shading) {                                                \
    case SH_BASE: FN<SH_BASE>(__VA_ARGS__); break;                    \
    case SH_BLINN: FN<SH_BLINN>(__VA_ARGS__); break;                  \
    case SH_BLINN_DIR: FN<SH_BLINN_DIR>(__VA_ARGS__); break;          \
    case SH_PBR:                                                      \
    case SH_PBR_CAPTURE:                                              \
    case SH_PBR_NEURAL: FN<SH_PBR>(__VA_ARGS__); break;               \
    case SH_SKYBOX: FN<SH_SKYBOX>(__VA_ARGS__); break;                \
    case SH_FXAA: FN<SH_FXAA>(__VA_ARGS__); break;                    \
    case SH_IBL_IRR:                                                  \
    case SH_IBL_PRE: FN<SH_IBL_IRR>(__VA_ARGS__); break;              \
    case SH_VCOLOR: FN<SH_VCOLOR>(__VA_ARGS__); break;                \
  }

void launchVertexAndClip(const DrawParams &p, cudaStream_t st) { SGLC_GEOMETRY_SWITCH(launchGeometry, p, st) }

void launchPointsLinesGeometry(const DrawParams &p, const LineParams &lp, cudaStream_t st) {
  SGLC_GEOMETRY_SWITCH(pointsLinesGeometry, p, lp, st)
}

void launchClipAppend(const DrawParams &p, cudaStream_t st) {
  launchChained(k_clip_append, dim3(max(1, cdiv(p.clipPolyCap, 256))), dim3(256), 0, st, p);
}

void launchSetup(const DrawParams &p, int primCount, cudaStream_t st) {
  if (primCount > 0) launchChained(k_setup, dim3(cdiv(primCount, 256)), dim3(256), 0, st, p);
}

void launchBinEmit(const DrawParams &p, int primCount, cudaStream_t st) {
  if (primCount > 0) launchChained(k_bin_emit, dim3(cdiv(primCount, 256)), dim3(256), 0, st, p);
}

int sortScratchInts(int nPairs) { return (1 << kMaxDigitBits) * max(1, cdiv(nPairs, kSortTileSmall)) + 1; }
int sortPassCount(int keyBits, int maxDigitBits) {
  maxDigitBits = min(max(maxDigitBits, 1), kMaxDigitBits);
  return max(1, cdiv(max(keyBits, 1), maxDigitBits));
}

// sorts (keyA,valA) by key, result back in (keyA,valA); hist needs sortScratchInts ints plus a
// scan scratch of scanScratchInts(2^digit bits * blocks)
void sortPairs(const DrawParams &p, int nPairs, const int *nPtr, int keyBits, int *hist, int *histScan,
               int *scanScratch, cudaStream_t st, bool twoLaunchScan, int maxDigitBits) {
  if (nPairs <= 0) return;
  // small sorts in blocks of 512 pairs (more CTAs in flight), large ones in blocks of 2,048 (a
  // quarter of the histogram entries to scan): 1080p binning 0.047 -> 0.039 ms with 512, the 256-view
  // batch slower with it
  const bool small = nPairs <= kSortSmallMax;
  const int nb = cdiv(nPairs, small ? kSortTileSmall : kSortTileLarge);
  uint32_t *kin = p.keyA, *kout = p.keyB;
  int *vin = p.valA, *vout = p.valB;
  // as few passes as digits of at most maxDigitBits bits allow, the key bits spread evenly over them
  const int passes = sortPassCount(keyBits, maxDigitBits);
  const int bits = cdiv(max(keyBits, 1), passes);
  for (int pass = 0; pass < passes; pass++) {
    int shift = pass * bits;
    if (small) launchChained(k_radix_hist<kSortItemsSmall>, dim3(nb), dim3(kSortThreads), 0, st, kin, nPtr, shift, bits, hist, nb);
    else launchChained(k_radix_hist<kSortItemsLarge>, dim3(nb), dim3(kSortThreads), 0, st, kin, nPtr, shift, bits, hist, nb);
    if (twoLaunchScan) scanExclusive2(hist, histScan, nullptr, (1 << bits) * nb, scanScratch, st);
    else scanExclusive(hist, histScan, nullptr, (1 << bits) * nb, scanScratch, st);
    if (small)
      launchChained(k_radix_scatter<kSortItemsSmall>, dim3(nb), dim3(kSortThreads), 0, st, kin, vin, kout, vout, nPtr,
                    shift, bits, histScan, nb);
    else
      launchChained(k_radix_scatter<kSortItemsLarge>, dim3(nb), dim3(kSortThreads), 0, st, kin, vin, kout, vout, nPtr,
                    shift, bits, histScan, nb);
    uint32_t *tk = kin; kin = kout; kout = tk;
    int *tv = vin; vin = vout; vout = tv;
  }
  if (passes & 1) {   // result must land in A
    cudaMemcpyAsync(p.keyA, p.keyB, sizeof(uint32_t) * (size_t) nPairs, cudaMemcpyDeviceToDevice, st);
    cudaMemcpyAsync(p.valA, p.valB, sizeof(int) * (size_t) nPairs, cudaMemcpyDeviceToDevice, st);
  }
}

void launchTileRanges(const DrawParams &p, int nPairs, const int *nPtr, cudaStream_t st) {
  if (nPairs > 0) launchChained(k_tile_ranges, dim3(cdiv(nPairs, 256)), dim3(256), 0, st, p.keyA, nPtr, p.tileStart, p.tileEnd);
}

void launchTileOrder(const DrawParams &p, int *order, cudaStream_t st) {
  launchChained(k_tile_order, dim3(1), dim3(1024), 0, st, p.tileStart, p.tileEnd, p.numTiles, order);
}

__global__ void k_accumulate_flags(const int *flags, int *sticky) {
  chainEnter();
  *sticky |= *flags;
}

void launchAccumulateFlags(const int *flags, int *sticky, cudaStream_t st) {
  launchChained(k_accumulate_flags, dim3(1), dim3(1), 0, st, flags, sticky);
}

void launchFill32(uint32_t *dst, uint32_t value, size_t n, cudaStream_t st) {
  if (n == 0) return;
  int grid = (int) min((size_t) 152 * 8, (n + 255) / 256);
  k_fill32<<<grid, 256, 0, st>>>(dst, value, n);
}

void launchMipLevel(const DevTex &t, int face, int level, int isFloat, cudaStream_t st) {
  dim3 b(16, 16), g(cdiv(t.w[level], 16), cdiv(t.h[level], 16));
  k_mip_level<<<g, b, 0, st>>>(t, face, level, isFloat);
}

void launchSwizzleIn(const DevTex &t, int face, int level, const uint32_t *src, cudaStream_t st) {
  dim3 b(16, 16), g(cdiv(t.w[level], 16), cdiv(t.h[level], 16));
  k_swizzle_in<<<g, b, 0, st>>>(t, face, level, src);
}

void launchSwizzleOut(const DevTex &t, int face, int level, uint32_t *dst, cudaStream_t st) {
  dim3 b(16, 16), g(cdiv(t.w[level], 16), cdiv(t.h[level], 16));
  k_swizzle_out<<<g, b, 0, st>>>(t, face, level, dst);
}

}  // namespace sglc
