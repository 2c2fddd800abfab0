// Tile raster kernel (RendererSoft::rasterizationTriangle / rasterizationPixelQuad / earlyZTest /
// processPerSampleOperations / multiSampleResolve, RendererSoft.cpp:720-912).
//
// One CTA per 16x16 screen tile, 8 warps of 8x4 pixels. Each thread owns one pixel for the whole
// draw: its colour and depth samples live in registers, loaded once (or taken from the pass's clear
// values, fusing the clear) and stored once with 128-bit accesses, with the MSAA resolve fused
// into the store. Because a pixel is touched by exactly one thread, and that thread walks the
// tile's primitive list in primitive order, every pixel sees the reference's sequence of depth
// tests and blends without any inter-thread ordering.
//
// RendererSoft rasterises each triangle in 32x32 blocks anchored at its own bounding box and in
// 2x2 quads anchored at odd offsets inside each block (:727-763); the quad decides which pixels
// share derivatives and, when blocks overlap, a pixel can be visited twice. quadCandsF() finds, for
// one pixel, exactly the quads the reference visits, in the reference's order; neighbourBC()
// recomputes the quad neighbours' shading-sample barycentrics for dFdx/dFdy.
#pragma once

#include "sglc_device.cuh"
#include "sglc_host_util.h"
#include "sglc_shaders.cuh"

namespace sglc {

__constant__ float2 kLoc4xR[4] = {{0.375f, 0.875f}, {0.875f, 0.625f}, {0.125f, 0.375f}, {0.625f, 0.125f}};

// the part of a triangle's setup that coverage, depth and perspective correction read
struct TriCov {
  float v0x, v0y, f0x, f0y, f0z, f1x, f1y, f1z;
  float z0, z1, z2, w0, w1, w2;
};

struct Tri : TriCov {
  float bminx, bminy, bmaxx, bmaxy;
  int bcx, bcy, vid0, vid1, vid2;
};

__device__ __forceinline__ TriCov loadTriCov(const TriSetup *t) {
  const float4 *q = reinterpret_cast<const float4 *>(t);
  float4 a = __ldg(q + 0), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3);
  TriCov T;
  T.v0x = a.x; T.v0y = a.y; T.f0x = a.z; T.f0y = a.w;
  T.f0z = b.x; T.f1x = b.y; T.f1y = b.z; T.f1z = b.w;
  T.z0 = c.x; T.z1 = c.y; T.z2 = c.z; T.w0 = c.w;
  T.w1 = d.x; T.w2 = d.y;
  return T;
}


__device__ __forceinline__ Tri loadTri(const TriSetup *t) {
  const float4 *q = reinterpret_cast<const float4 *>(t);
  float4 a = __ldg(q + 0), b = __ldg(q + 1), c = __ldg(q + 2), d = __ldg(q + 3), e = __ldg(q + 4);
  int4 f = __ldg(reinterpret_cast<const int4 *>(q + 5));
  Tri T;
  T.v0x = a.x; T.v0y = a.y; T.f0x = a.z; T.f0y = a.w;
  T.f0z = b.x; T.f1x = b.y; T.f1y = b.z; T.f1z = b.w;
  T.z0 = c.x; T.z1 = c.y; T.z2 = c.z; T.w0 = c.w;
  T.w1 = d.x; T.w2 = d.y; T.bminx = d.z; T.bminy = d.w;
  T.bmaxx = e.x; T.bmaxy = e.y;
  T.bcx = __float_as_int(e.z); T.bcy = __float_as_int(e.w);
  T.vid0 = f.x; T.vid1 = f.y; T.vid2 = f.z;
  return T;
}

// RendererSoft::barycentric, SSE lane order (RendererSoft.cpp:1025-1039, 1051-1055)
__device__ __forceinline__ bool bary(const TriCov &t, float px, float py, float &b0, float &b1, float &b2) {
  float a0 = t.f0x - t.v0x, a1 = t.f0y - t.v0x, a2 = t.f0z - px;
  float c0 = t.f1x - t.v0y, c1 = t.f1y - t.v0y, c2 = t.f1z - py;
  float ux = a1 * c2 - a2 * c1;
  float uy = a2 * c0 - a0 * c2;
  float uz = a0 * c1 - a1 * c0;
  if (fabsf(uz) < 1.19209290e-07f) return false;
  ux = ux / uz;
  uy = uy / uz;
  b0 = 1.f - (ux + uy);
  b1 = uy;
  b2 = ux;
  return !(b0 < 0 || b1 < 0 || b2 < 0);
}

// Same result as bary() when it returns true. Samples whose barycentrics are clearly negative are
// rejected first with a reciprocal estimate (its error is far below the 1e-4 margin, so every
// rejected sample is also rejected by the exact division); the rest take the exact path.
__device__ __forceinline__ bool baryCover(const TriCov &t, float px, float py, float &b0, float &b1, float &b2) {
  float a0 = t.f0x - t.v0x, a1 = t.f0y - t.v0x, a2 = t.f0z - px;
  float c0 = t.f1x - t.v0y, c1 = t.f1y - t.v0y, c2 = t.f1z - py;
  float ux = a1 * c2 - a2 * c1;
  float uy = a2 * c0 - a0 * c2;
  float uz = a0 * c1 - a1 * c0;
  if (fabsf(uz) < 1.19209290e-07f) return false;
  float r = __fdividef(1.f, uz);
  float ex = ux * r, ey = uy * r;
  if (ex < -1e-4f || ey < -1e-4f || 1.f - (ex + ey) < -1e-4f) return false;
  ux = ux / uz;
  uy = uy / uz;
  b0 = 1.f - (ux + uy);
  b1 = uy;
  b2 = ux;
  return !(b0 < 0 || b1 < 0 || b2 < 0);
}

// glm::dot(bc, vec4(v0, v1, v2, 0)) with DPPS order (z and w of a sample)
__device__ __forceinline__ float interpZW(float b0, float b1, float b2, float v0, float v1, float v2) {
  return (b0 * v0 + b1 * v1) + (b2 * v2 + 0.f * 0.f);
}

// barycentric *= (1 / w * vertW) (RendererSoft.cpp:802)
__device__ __forceinline__ void correct(const TriCov &t, float &b0, float &b1, float &b2) {
  float w = interpZW(b0, b1, b2, t.w0, t.w1, t.w2);
  float iw = 1.f / w;
  b0 = b0 * (iw * t.w0);
  b1 = b1 * (iw * t.w1);
  b2 = b2 * (iw * t.w2);
}

// shading-sample barycentrics of a quad neighbour (RendererInternal.h:97-124 + :787-804)
template<int S>
__device__ __forceinline__ void neighbourBC(const TriCov &t, int fx, int fy, float &b0, float &b1, float &b2) {
  const float x = (float) fx, y = (float) fy;
  float c0 = 0.f, c1 = 0.f, c2 = 0.f;
  bool cin = bary(t, x + 0.5f, y + 0.5f, c0, c1, c2);
  if (S == 1 || cin) {
    if (cin) correct(t, c0, c1, c2);
    b0 = c0; b1 = c1; b2 = c2;
    return;
  }
#pragma unroll
  for (int i = 0; i < 4; i++) {
    float s0, s1, s2;
    if (bary(t, kLoc4xR[i].x + x, kLoc4xR[i].y + y, s0, s1, s2)) {
      correct(t, s0, s1, s2);
      b0 = s0; b1 = s1; b2 = s2;
      return;
    }
  }
  b0 = c0; b1 = c1; b2 = c2;
}

// quads of one triangle that contain coordinate `pos` along one axis, in block order (<= 2)
__device__ __forceinline__ int quadCandsF(float bmin, float bmax, int bc, int pos, int &q0, int &q1) {
  int n = 0;
  int kEst = (int) floorf(((float) (pos - 1) - bmin) * (1.f / (float) kBlock));
#pragma unroll
  for (int dk = -1; dk <= 1; dk++) {
    int k = kEst + dk;
    if (k < 0 || k >= bc) continue;
    int bs = (int) (bmin + (float) (k * kBlock));
    if (pos < bs + 1 || pos > bs + kBlock) continue;
    int q = bs + 1 + ((pos - bs - 1) & ~1);
    if ((float) q > bmax) continue;
    if (n == 0) q0 = q;
    else q1 = q;
    n++;
  }
  return n;
}

// quads of triangle `t` containing pixel (px, py): block bounds from the setup record
__device__ __forceinline__ int quadsOf(const TriSetup *t, int px, int py, int &x0, int &x1, int &y0, int &y1, int &nx) {
  const float4 *q = reinterpret_cast<const float4 *>(t);
  float4 d = __ldg(q + 3), e = __ldg(q + 4);
  nx = quadCandsF(d.z, e.x, __float_as_int(e.z), px, x0, x1);
  int ny = nx ? quadCandsF(d.w, e.y, __float_as_int(e.w), py, y0, y1) : 0;
  return nx * ny;
}

// DepthTest (DepthSoft.h:13-25) as an 8-entry truth table indexed by the depth function
__device__ __forceinline__ bool depthCmp(float a, float b, int func) {
  bool lt = a < b, gt = a > b, le = a <= b, ge = a >= b, eq = fabsf(a - b) <= 1.19209290e-07f;
  uint32_t bits = 0x80u | ((uint32_t) lt << 1) | ((uint32_t) eq << 2) | ((uint32_t) le << 3) | ((uint32_t) gt << 4) |
                  ((uint32_t) !eq << 5) | ((uint32_t) ge << 6);
  return (bits >> func) & 1u;
}

// DepthFunction values (RenderStates.h:13-22), each the index of its bit in depthCmp
constexpr int DEPTH_LESS = 1, DEPTH_LEQUAL = 3, DEPTH_GREATER = 4, DEPTH_GEQUAL = 6;

// The depth a sample keeps when a fragment of clamped depth b meets stored depth a, for the four
// functions whose depth write keeps a running extremum: b if it passes the test against a, else a.
// On non-NaN values it is associative (the earliest minimum for LESS, the latest for LEQUAL, and
// likewise for the maximum), which is what lets pass 2 evaluate a pixel's fragments as a scan.
__device__ __forceinline__ float depthKeep(float a, float b, int func) {
  const bool take = func == DEPTH_LESS ? b < a : (func == DEPTH_LEQUAL ? b <= a : (func == DEPTH_GREATER ? b > a : b >= a));
  return take ? b : a;
}

// calcBlendFactor: one of {0, 1, x, 1 - x}, x chosen among the four blend operands
__device__ __forceinline__ float blendFactor(const DrawParams &p, int k, float src, float srcA, float dst, float dstA) {
  int op = p.bfOp[k];
  float x = op == 0 ? src : (op == 1 ? srcA : (op == 2 ? dst : dstA));
  return p.bfC0[k] + p.bfC1[k] * x;
}

// calcBlendFunc: s + d, s - d, d - s exactly as s*ks + d*kd with ks, kd = +-1; or min / max
__device__ __forceinline__ float blendFn(const DrawParams &p, int k, float s, float d) {
  float r = s * p.bKs[k] + d * p.bKd[k];
  int mm = p.bMinMax[k];
  float mn = gmin(s, d), mx = gmax(s, d);
  return mm == 0 ? r : (mm == 1 ? mn : mx);
}

// glm::clamp(vec4, 0, 1) on the SSE path: minps(maxps(x, 0), 1)
__device__ __forceinline__ float sseClamp01(float x) {
  float t = (x > 0.f) ? x : 0.f;
  return (t < 1.f) ? t : 1.f;
}

// processPerSampleOperations (RendererSoft.cpp:358-407) on one register-resident sample
template<bool HAS_COLOR, bool HAS_DEPTH>
__device__ __forceinline__ void perSample(const DrawParams &p, bool inC, bool inD, uint32_t &col, float &dep, float z,
                                          float4 color) {
  if (p.depthTest && HAS_DEPTH) {
    float d = gclamp(z, p.vp.absMin, p.vp.absMax);
    if (!inD || !depthCmp(d, dep, p.depthFunc)) return;
    if (p.depthMask) dep = d;
  }
  if (!HAS_COLOR) return;
  float c0 = sseClamp01(color.x), c1 = sseClamp01(color.y), c2 = sseClamp01(color.z), c3 = sseClamp01(color.w);
  if (p.blend) {
    float4 d = make_float4(0.f, 0.f, 0.f, 0.f);
    if (inC) {
      d = unpackUnit4(col);
    }
    float r0 = blendFn(p, 0, c0 * blendFactor(p, 0, c0, c3, d.x, d.w), d.x * blendFactor(p, 1, c0, c3, d.x, d.w));
    float r1 = blendFn(p, 0, c1 * blendFactor(p, 0, c1, c3, d.y, d.w), d.y * blendFactor(p, 1, c1, c3, d.y, d.w));
    float r2 = blendFn(p, 0, c2 * blendFactor(p, 0, c2, c3, d.z, d.w), d.z * blendFactor(p, 1, c2, c3, d.z, d.w));
    float r3 = blendFn(p, 1, c3 * blendFactor(p, 2, c3, c3, d.w, d.w), d.w * blendFactor(p, 3, c3, c3, d.w, d.w));
    c0 = r0; c1 = r1; c2 = r2; c3 = r3;
  }
  if (inC) col = pack4(c0 * 255.f, c1 * 255.f, c2 * 255.f, c3 * 255.f);
}

struct Samples4 {
  uint32_t c0, c1, c2, c3;
  float d0, d1, d2, d3;
};

// Hierarchical depth rejection for the four ordered depth functions. A sample's depth is the
// interpolation (b0 z0 + b1 z1) + b2 z2 with barycentrics in [0, 1] summing to 1 within rounding,
// so every covered sample of a triangle lies in [min z_i, max z_i] up to a few ulps; clamping to the
// depth range keeps that order. If the triangle's whole range fails the test against the most
// permissive depth stored in a set of samples (the minimum for GREATER / GEQUAL, the maximum for
// LESS / LEQUAL), none of its samples there can pass, now or later in the draw (with depth writes
// the stored depth only moves further in the test's direction), so the triangle is skipped for
// them. kHizMargin covers the rounding of the interpolation.
enum { HIZ_NONE = 0, HIZ_GREATER, HIZ_GEQUAL, HIZ_LESS, HIZ_LEQUAL };
constexpr float kHizMargin = 1e-6f;

__device__ __forceinline__ int hizMode(const DrawParams &p, bool hasDepth) {
  if (!(p.depthTest && hasDepth)) return HIZ_NONE;
  switch (p.depthFunc) {
    case DEPTH_GREATER: return HIZ_GREATER;
    case DEPTH_GEQUAL: return HIZ_GEQUAL;
    case DEPTH_LESS: return HIZ_LESS;
    case DEPTH_LEQUAL: return HIZ_LEQUAL;
  }
  return HIZ_NONE;
}

// the most permissive stored depth of one pixel's samples for the mode (NaN samples pass nothing
// under an ordered test: they are left out)
template<int S>
__device__ __forceinline__ float hizPixelBound(int mode, const Samples4 &fb, bool inD) {
  const float inf = __int_as_float(0x7f800000);
  const bool lower = mode == HIZ_GREATER || mode == HIZ_GEQUAL;
  float b = lower ? inf : -inf;
  if (!inD || mode == HIZ_NONE) return b;
  const float d[4] = {fb.d0, fb.d1, fb.d2, fb.d3};
#pragma unroll
  for (int q = 0; q < S; q++)
    if (d[q] == d[q]) b = lower ? fminf(b, d[q]) : fmaxf(b, d[q]);
  return b;
}

// true: a triangle whose depths lie in [zmin, zmax] passes the test at no sample with stored depth
// bound `bound` (hizPixelBound, or its minimum / maximum over several pixels)
__device__ __forceinline__ bool hizReject(int mode, float zmin, float zmax, float bound) {
  switch (mode) {
    case HIZ_GREATER: return zmax + kHizMargin * (fabsf(zmax) + 1.f) <= bound;
    case HIZ_GEQUAL: return zmax + kHizMargin * (fabsf(zmax) + 1.f) < bound;
    case HIZ_LESS: return zmin - kHizMargin * (fabsf(zmin) + 1.f) >= bound;
    case HIZ_LEQUAL: return zmin - kHizMargin * (fabsf(zmin) + 1.f) > bound;
  }
  return false;
}

// per-warp fragment queue in shared memory (phase A appends, phase B shades, phase C applies)
constexpr int kQueue = 64;
struct FragQueue {
  int tri[kQueue];
  uint32_t meta[kQueue];   // bits 0-4 lane, 5-8 sample mask, 9 pixel is right of quad origin, 10 below
  float b0[kQueue], b1[kQueue], b2[kQueue];
  float4 col[kQueue];
};

__device__ __forceinline__ bool depthPass(const DrawParams &p, float z, float dep) {
  return depthCmp(gclamp(z, p.vp.absMin, p.vp.absMax), dep, p.depthFunc);
}

// Phase B for one fragment: quad derivatives of the texture coordinates, then the FS. Inlined into
// the deferred shading kernel (no call, no spills around it: 0.156 -> 0.137 ms at 1080p MSAA4 PBR);
// the fused raster kernel calls it through shadeFragment below, which keeps that kernel's code small.
template<int SH, int S>
__device__ __forceinline__ float4 shadeFragmentInl(const DrawParams &p, const uint8_t *U, int tri, int qx, int qy,
                                                   int px, int py, float sb0, float sb1, float sb2) {
  Tri t = loadTri(p.tri + tri);
  const float *r0 = p.vVary + (size_t) t.vid0 * p.varyStride;
  const float *r1 = p.vVary + (size_t) t.vid1 * p.varyStride;
  const float *r2 = p.vVary + (size_t) t.vid2 * p.varyStride;
  FragIn f;
  f.U = U;
  f.v = Vary{r0, r1, r2, sb0, sb1, sb2};
  f.dudx = f.dvdx = f.dudy = f.dvdy = 0.f;
  if (p.needDeriv) {
    // p0 = (qx, qy), p1 = (qx+1, qy), p2 = (qx, qy+1): varyings at each pixel's shading sample
    // (RendererSoft.cpp:815-820; ShaderSoft.h:117-133)
    float u[3], v[3];
    for (int k = 0; k < 3; k++) {
      int nx = qx + (k == 1), ny = qy + (k == 2);
      float c0 = sb0, c1 = sb1, c2 = sb2;
      if (nx != px || ny != py) neighbourBC<S>(t, nx, ny, c0, c1, c2);
      Vary vk{r0, r1, r2, c0, c1, c2};
      u[k] = vk[0];
      v[k] = vk[1];
    }
    f.dudx = u[1] - u[0];
    f.dvdx = v[1] - v[0];
    f.dudy = u[2] - u[0];
    f.dvdy = v[2] - v[0];
  }
  return runFS<SH>(p, f);
}

template<int SH, int S>
__device__ __noinline__ float4 shadeFragment(const DrawParams &p, const uint8_t *U, int tri, int qx, int qy, int px,
                                             int py, float sb0, float sb1, float sb2) {
  return shadeFragmentInl<SH, S>(p, U, tri, qx, qy, px, py, sb0, sb1, sb2);
}

template<int SH, int S, bool HAS_DEPTH>
__device__ __forceinline__ void flushQueue(const DrawParams &p, const uint8_t *U, FragQueue &q, int &count,
                                           unsigned long long &mine, int lane, int rx0, int ry0, bool inC, Samples4 &fb) {
  __syncwarp();
  // phase B: shade the queued fragments 32 at a time
  for (int base = 0; base < count; base += 32) {
    int e = base + lane;
    if (e < count) {
      uint32_t m = q.meta[e];
      int l = m & 31;
      int px = rx0 + (l & 7), py = ry0 + (l >> 3);
      int qx = px - ((m >> 9) & 1), qy = py - ((m >> 10) & 1);
      q.col[e] = shadeFragment<SH, S>(p, U, q.tri[e], qx, qy, px, py, q.b0[e], q.b1[e], q.b2[e]);
    }
  }
  __syncwarp();
  if (p.fragCounter && lane == 0) atomicAdd(p.fragCounter, (unsigned long long) count);
  // phase C: every pixel applies its own fragments' colour operations in queue (= primitive) order;
  // the lanes walk their own entries concurrently
  while (mine) {
    int e = __ffsll(mine) - 1;
    mine &= mine - 1;
    float4 color = q.col[e];
    uint32_t mask = (q.meta[e] >> 5) & 15u;
    if (mask & 1u) perSample<true, false>(p, inC, true, fb.c0, fb.d0, 0.f, color);
    if (S == 4) {
      if (mask & 2u) perSample<true, false>(p, inC, true, fb.c1, fb.d1, 0.f, color);
      if (mask & 4u) perSample<true, false>(p, inC, true, fb.c2, fb.d2, 0.f, color);
      if (mask & 8u) perSample<true, false>(p, inC, true, fb.c3, fb.d3, 0.f, color);
    }
  }
  __syncwarp();
  count = 0;
}

// Coverage of pixel (px, py) by one triangle: a pure function of the two (RendererSoft.cpp:776-804).
// mask bit i = sample i covered and inside the depth range (S=1: bit 0 = centre covered; its depth
// range clip has no effect, RendererSoft.cpp:797-799 vs :846-849, :872-874); z per sample; the
// perspective-corrected barycentrics of the shading sample (RendererInternal.h:114-124).
struct Cover {
  uint32_t mask;
  float z0, z1, z2, z3;
  float b0, b1, b2;
};

template<int S>
__device__ __forceinline__ Cover coverSamples(const DrawParams &p, const TriCov &t, int px, int py) {
  Cover c;
  c.mask = 0u;
  c.z0 = c.z1 = c.z2 = c.z3 = 0.f;
  c.b0 = c.b1 = c.b2 = 0.f;
  const float fx = (float) px, fy = (float) py;
  if (S == 1) {
    if (!baryCover(t, fx + 0.5f, fy + 0.5f, c.b0, c.b1, c.b2)) return c;
    c.z0 = interpZW(c.b0, c.b1, c.b2, t.z0, t.z1, t.z2);
    correct(t, c.b0, c.b1, c.b2);
    c.mask = 1u;
    return c;
  }
  float a0, a1, a2, b0, b1, b2, d0, d1, d2, e0, e1, e2, m0, m1, m2;
  bool s0 = baryCover(t, kLoc4xR[0].x + fx, kLoc4xR[0].y + fy, a0, a1, a2);
  bool s1 = baryCover(t, kLoc4xR[1].x + fx, kLoc4xR[1].y + fy, b0, b1, b2);
  bool s2 = baryCover(t, kLoc4xR[2].x + fx, kLoc4xR[2].y + fy, d0, d1, d2);
  bool s3 = baryCover(t, kLoc4xR[3].x + fx, kLoc4xR[3].y + fy, e0, e1, e2);
  if (!(s0 || s1 || s2 || s3)) return c;
  bool sc = baryCover(t, fx + 0.5f, fy + 0.5f, m0, m1, m2);
  // InitShadingSample: the centre if covered, else the first covered sample
  if (sc) { c.b0 = m0; c.b1 = m1; c.b2 = m2; }
  else if (s0) { c.b0 = a0; c.b1 = a1; c.b2 = a2; }
  else if (s1) { c.b0 = b0; c.b1 = b1; c.b2 = b2; }
  else if (s2) { c.b0 = d0; c.b1 = d1; c.b2 = d2; }
  else { c.b0 = e0; c.b1 = e1; c.b2 = e2; }
  if (s0) { c.z0 = interpZW(a0, a1, a2, t.z0, t.z1, t.z2); if (!(c.z0 < p.vp.absMin || c.z0 > p.vp.absMax)) c.mask |= 1u; }
  if (s1) { c.z1 = interpZW(b0, b1, b2, t.z0, t.z1, t.z2); if (!(c.z1 < p.vp.absMin || c.z1 > p.vp.absMax)) c.mask |= 2u; }
  if (s2) { c.z2 = interpZW(d0, d1, d2, t.z0, t.z1, t.z2); if (!(c.z2 < p.vp.absMin || c.z2 > p.vp.absMax)) c.mask |= 4u; }
  if (s3) { c.z3 = interpZW(e0, e1, e2, t.z0, t.z1, t.z2); if (!(c.z3 < p.vp.absMin || c.z3 > p.vp.absMax)) c.mask |= 8u; }
  correct(t, c.b0, c.b1, c.b2);
  c.mask |= 16u;   // the pixel is covered (its fragment runs even if every sample is depth-clipped)
  return c;
}

// early-Z (RendererSoft.cpp:853-878), then the per-sample depth test + write in sample order
// (processPerSampleOperations, :838-849). Returns the samples whose colour operation follows.
template<int S, bool HAS_DEPTH>
__device__ __forceinline__ uint32_t depthOps(const DrawParams &p, const Cover &c, bool inD, Samples4 &fb) {
  const bool testDepth = p.depthTest && HAS_DEPTH;
  if (S == 1) {
    if (!c.mask) return 0u;
    if (!testDepth) return 1u;
    if (!(inD && depthPass(p, c.z0, fb.d0))) return 0u;   // early-Z and the per-sample test agree
    if (p.depthMask) fb.d0 = gclamp(c.z0, p.vp.absMin, p.vp.absMax);
    return 1u;
  }
  if (!(c.mask & 16u)) return 0u;
  bool i0 = c.mask & 1u, i1 = c.mask & 2u, i2 = c.mask & 4u, i3 = c.mask & 8u;
  if (!testDepth) return c.mask & 15u;
  if (p.earlyZ) {
    if (i0) i0 = inD && depthPass(p, c.z0, fb.d0);
    if (i1) i1 = inD && depthPass(p, c.z1, fb.d1);
    if (i2) i2 = inD && depthPass(p, c.z2, fb.d2);
    if (i3) i3 = inD && depthPass(p, c.z3, fb.d3);
    if (!(i0 || i1 || i2 || i3)) return 0u;
  }
  if (i0) { i0 = inD && depthPass(p, c.z0, fb.d0); if (i0 && p.depthMask) fb.d0 = gclamp(c.z0, p.vp.absMin, p.vp.absMax); }
  if (i1) { i1 = inD && depthPass(p, c.z1, fb.d1); if (i1 && p.depthMask) fb.d1 = gclamp(c.z1, p.vp.absMin, p.vp.absMax); }
  if (i2) { i2 = inD && depthPass(p, c.z2, fb.d2); if (i2 && p.depthMask) fb.d2 = gclamp(c.z2, p.vp.absMin, p.vp.absMax); }
  if (i3) { i3 = inD && depthPass(p, c.z3, fb.d3); if (i3 && p.depthMask) fb.d3 = gclamp(c.z3, p.vp.absMin, p.vp.absMax); }
  return (i0 ? 1u : 0u) | (i1 ? 2u : 0u) | (i2 ? 4u : 0u) | (i3 ? 8u : 0u);
}

// Lane r holds row r of a 32x32 bit matrix (bit c = column c); returns column `lane` (bit r = row r).
// Each step swaps the off-diagonal s x s blocks of every 2s x 2s block, for s = 16, 8, 4, 2, 1.
__device__ __forceinline__ unsigned transposeBits(unsigned x, int lane) {
  const unsigned lowCols[5] = {0x0000ffffu, 0x00ff00ffu, 0x0f0f0f0fu, 0x33333333u, 0x55555555u};
#pragma unroll
  for (int i = 0; i < 5; i++) {
    const int s = 16 >> i;
    const unsigned m = lowCols[i];
    const unsigned y = __shfl_xor_sync(0xffffffffu, x, s);
    x = (lane & s) ? ((x & ~m) | ((y & ~m) >> s)) : ((x & m) | ((y & m) << s));
  }
  return x;
}

// Pass 1 of a batch of up to 32 tile primitives (lane = primitive): a conservative edge-function
// test of each triangle against the sample box of every pixel of the warp's 8x4 rectangle, and for
// 4x MSAA against each of the four sample points of a pixel whose box passes (a triangle covering
// no sample point cannot cover the pixel; slivers that cross a pixel between its samples are
// dropped here rather than in the exact per-pixel test). Returns this lane's pixel's candidate mask
// (bit = batch index); `prim` = this lane's primitive id.
template<int S>
__device__ __forceinline__ unsigned pass1Prim(const DrawParams &p, int prim, int lane, int rx0, int ry0, float lo, float hi,
                                              float vpExtent, int rh = 4, int hiz = HIZ_NONE,
                                              float hizBound = 0.f) {
  bool hit = false;
  int4 r = make_int4(0, -1, 0, -1);
  float ea[3] = {0.f, 0.f, 0.f}, eb[3] = {0.f, 0.f, 0.f}, ek[3] = {0.f, 0.f, 0.f}, et[3] = {0.f, 0.f, 0.f};
  float es[3][4] = {};   // 4x MSAA: edge value at each sample offset, less a px + b py
  bool anyPix = false;
  if (prim >= 0) {
    const TriSetup *tp = p.tri + prim;
    r = __ldg(reinterpret_cast<const int4 *>(&tp->rx0));
    hit = !(r.y < rx0 || r.x > rx0 + 7 || r.w < ry0 || r.z > ry0 + rh - 1);
    float4 q0 = make_float4(0.f, 0.f, 0.f, 0.f), q1 = q0;
    float uz = 0.f;
    if (hit) {
      q0 = __ldg(reinterpret_cast<const float4 *>(tp));        // v0x v0y v2x v1x
      q1 = __ldg(reinterpret_cast<const float4 *>(tp) + 1);    // v0x v2y v1y v0y
      // the barycentric denominator does not depend on the point (baryCover): a triangle whose
      // |uz| is below FLT_EPSILON covers nothing (RendererSoft.cpp:1035-1037)
      uz = (q0.z - q0.x) * (q1.z - q0.y) - (q0.w - q0.x) * (q1.y - q0.y);
      if (fabsf(uz) < 1.19209290e-07f) hit = false;
    }
    if (hit && hiz != HIZ_NONE) {   // the whole triangle fails the depth test at every warp pixel
      const float4 q2 = __ldg(reinterpret_cast<const float4 *>(tp) + 2);   // z0 z1 z2 w0
      if (hizReject(hiz, fminf(q2.x, fminf(q2.y, q2.z)), fmaxf(q2.x, fmaxf(q2.y, q2.z)), hizBound)) hit = false;
    }
    if (hit) {
      float X[3] = {q0.x, q0.w, q0.z}, Y[3] = {q0.y, q1.z, q1.y};     // v0, v1, v2
      float mag = fabsf(X[1] - X[0]) + fabsf(Y[1] - Y[0]) + fabsf(X[2] - X[0]) + fabsf(Y[2] - Y[0]);
      anyPix = !(fabsf(uz) > 1e-6f * mag * mag + 1e-6f);   // near-degenerate: skip the edge pre-test
      // orientation from the reference's own denominator: its coverage signs are ux/uz, uy/uz and
      // 1 - (ux + uy)/uz, so the edge functions take the sign uz was computed with (uz is twice the
      // signed area with the opposite sign of (v1 - v0) x (v2 - v0))
      float o = uz > 0.f ? -1.f : 1.f;
#pragma unroll
      for (int e = 0; e < 3; e++) {
        // E(x, y) = a x + b y + c >= 0 inside; its maximum over a pixel's sample box is at the
        // corner picked by the signs of a, b: E_max(px, py) = a px + b py + k
        float sx = X[e], sy = Y[e], dx = X[(e + 1) % 3] - sx, dy = Y[(e + 1) % 3] - sy;
        float a = -o * dy, b = o * dx, c = o * (dy * sx - dx * sy);
        ea[e] = a;
        eb[e] = b;
        ek[e] = a * (a > 0.f ? hi : lo) + b * (b > 0.f ? hi : lo) + c;
        et[e] = 1e-5f * ((fabsf(a) + fabsf(b)) * (vpExtent + fabsf(sx) + fabsf(sy)) + fabsf(c) + 1.f);
        if (S == 4) {
#pragma unroll
          for (int k = 0; k < 4; k++) es[e][k] = a * kLoc4xR[k].x + b * kLoc4xR[k].y + c;
        }
      }
    }
  }
  const int x0 = max(r.x, rx0), x1 = min(r.y, rx0 + 7), y0 = max(r.z, ry0), y1 = min(r.w, ry0 + rh - 1);
  const int w = hit && x1 >= x0 && y1 >= y0 ? x1 - x0 + 1 : 0;
  const int n = w ? w * (y1 - y0 + 1) : 0;
  const int nMax = __reduce_max_sync(0xffffffffu, n);
  auto test = [&](int px, int py) -> bool {
    if (anyPix) return true;
    float fx = (float) px, fy = (float) py;
    float g0 = ea[0] * fx + eb[0] * fy, g1 = ea[1] * fx + eb[1] * fy, g2 = ea[2] * fx + eb[2] * fy;
    bool c = (g0 + ek[0] >= -et[0]) && (g1 + ek[1] >= -et[1]) && (g2 + ek[2] >= -et[2]);
    if (S == 4 && c) {
      bool any = false;
#pragma unroll
      for (int q = 0; q < 4; q++)
        any = any || ((g0 + es[0][q] >= -et[0]) && (g1 + es[1][q] >= -et[1]) && (g2 + es[2][q] >= -et[2]));
      c = any;
    }
    return c;
  };
  if (nMax > 12) {
    // large primitives: every pixel of the rectangle in turn, one ballot per pixel
    unsigned cand = 0;
#pragma unroll 4
    for (int pp = 0; pp < 32; pp++) {
      int px = rx0 + (pp & 7), py = ry0 + (pp >> 3);   // rows beyond rh fall outside [y0, y1]
      bool c = px >= x0 && px <= x1 && py >= y0 && py <= y1 && w && test(px, py);
      unsigned mm = __ballot_sync(0xffffffffu, c);
      if (lane == pp) cand = mm;
    }
    return cand;
  }
  // small primitives: each lane (primitive) visits only the pixels of the warp's 8x4 rectangle inside
  // its own pixel rectangle and collects the ones that pass in a row (bit = pixel); transposing the
  // warp's 32x32 bit matrix gives each lane its pixel's candidate mask (bit = batch index)
  unsigned row = 0u;
  int cx = x0, cy = y0;
  for (int k = 0; k < n; k++) {
    if (test(cx, cy)) row |= 1u << ((cy - ry0) * 8 + (cx - rx0));
    if (++cx > x1) {
      cx = x0;
      cy++;
    }
  }
  return transposeBits(row, lane);
}

// pass 1 for the batch of tile-list entries [base, base + 32): lane i tests entry base + i
template<int S>
__device__ __forceinline__ unsigned pass1Candidates(const DrawParams &p, int base, int end, int lane, int rx0, int ry0,
                                                    float lo, float hi, float vpExtent, int &prim) {
  int i = base + lane;
  prim = i < end ? __ldg(p.valA + i) : -1;
  return pass1Prim<S>(p, prim, lane, rx0, ry0, lo, hi, vpExtent);
}

// does a tile-list primitive's pixel rectangle touch the warp's 8x4 rectangle
__device__ __forceinline__ bool touchesRect(const DrawParams &p, int prim, int rx0, int ry0, int rh = 4) {
  int4 r = __ldg(reinterpret_cast<const int4 *>(&p.tri[prim].rx0));
  return !(r.y < rx0 || r.x > rx0 + 7 || r.w < ry0 || r.z > ry0 + rh - 1);
}

template<int SH, int S, bool HAS_COLOR, bool HAS_DEPTH>
__global__ void __launch_bounds__(256, 2) k_raster(const __grid_constant__ DrawParams p) {
  chainEnter();
  __shared__ FragQueue queues[HAS_COLOR ? 8 : 1];
  const int tile = p.tileOrder ? p.tileOrder[blockIdx.x] : blockIdx.x;
  const TileFrame fr = tileFrame(p, tile);
  const int view = fr.view;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rx0 = fr.tx * 16 + (warp & 1) * 8, ry0 = fr.ty * 16 + (warp >> 1) * 4;
  const int px = rx0 + (lane & 7), py = ry0 + (lane >> 3);
  const bool inC = HAS_COLOR && px < fr.cW && py < fr.cH;
  const bool inD = HAS_DEPTH && px < fr.dW && py < fr.dH;
  FragQueue &q = queues[HAS_COLOR ? warp : 0];
  const uint8_t *U = viewUniforms(p, view);
  uint32_t *colorBuf = fr.color;
  uint32_t *resolvedBuf = fr.resolved;
  float *depthBuf = fr.depth;
  int count = 0;
  unsigned long long mine = 0ull;   // queue entries of this lane's pixel
  const unsigned lt = (1u << lane) - 1u;
  Samples4 fb = {0u, 0u, 0u, 0u, 0.f, 0.f, 0.f, 0.f};
  if (inC) {
    size_t pix = (size_t) py * fr.cW + px;
    if (p.pendingClear && p.clearColorFlag) {
      fb.c0 = fb.c1 = fb.c2 = fb.c3 = p.clearColor;
    } else if (S == 4) {
      uint4 v = *reinterpret_cast<const uint4 *>(colorBuf + pix * 4);
      fb.c0 = v.x; fb.c1 = v.y; fb.c2 = v.z; fb.c3 = v.w;
    } else {
      fb.c0 = colorBuf[pix];
    }
  }
  if (inD) {
    size_t pix = (size_t) py * fr.dW + px;
    if (p.pendingClear && p.clearDepthFlag) {
      fb.d0 = fb.d1 = fb.d2 = fb.d3 = p.clearDepth;
    } else if (S == 4) {
      float4 v = *reinterpret_cast<const float4 *>(depthBuf + pix * 4);
      fb.d0 = v.x; fb.d1 = v.y; fb.d2 = v.z; fb.d3 = v.w;
    } else {
      fb.d0 = depthBuf[pix];
    }
  }
  const int start = p.tileStart[tile], end = p.tileEnd[tile];
  // sample box offsets inside a pixel: 4x MSAA samples span [1/8, 7/8], one sample sits at 1/2
  const float lo = S == 4 ? 0.125f : 0.5f, hi = S == 4 ? 0.875f : 0.5f;
  const float vpExtent = fabsf(fr.vpW) + fabsf(fr.vpH) + 2.f * (float) (rx0 + ry0) + 64.f;
  for (int base = start; base < end; base += 32) {
    int prim;
    unsigned cand = pass1Candidates<S>(p, base, end, lane, rx0, ry0, lo, hi, vpExtent, prim);
    if (!(inC || inD)) cand = 0;
    // ---- pass 2 (lane = pixel): exact coverage and depth for each candidate, in primitive order
    int nIter = __reduce_max_sync(0xffffffffu, __popc(cand));
    for (int it = 0; it < nIter; it++) {
      int j = cand ? __ffs(cand) - 1 : -1;
      if (cand) cand &= cand - 1;
      int pr = __shfl_sync(0xffffffffu, prim, j < 0 ? 0 : j);
      int x0 = 0, x1 = 0, y0 = 0, y1 = 0, nx = 0, nq = 0;
      Cover cv;
      cv.mask = 0u;
      if (j >= 0) {
        const TriSetup *tp = p.tri + pr;
        nq = quadsOf(tp, px, py, x0, x1, y0, y1, nx);
        if (nq) cv = coverSamples<S>(p, loadTriCov(tp), px, py);
        if (!cv.mask) nq = 0;
      }
      int nqMax = __reduce_max_sync(0xffffffffu, nq);
      for (int k = 0; k < nqMax; k++) {   // a pixel can lie in two overlapping blocks' quads
        uint32_t mask = 0;
        int qx = 0, qy = 0;
        if (k < nq) {
          qy = (k / nx) ? y1 : y0;
          qx = (k % nx) ? x1 : x0;
          mask = depthOps<S, HAS_DEPTH>(p, cv, inD, fb);
        }
        if (HAS_COLOR) {
          if (count + 32 > kQueue) flushQueue<SH, S, HAS_DEPTH>(p, U, q, count, mine, lane, rx0, ry0, inC, fb);
          unsigned want = __ballot_sync(0xffffffffu, mask != 0);
          if (mask) {
            int e = count + __popc(want & lt);
            q.tri[e] = pr;
            q.meta[e] = (uint32_t) lane | (mask << 5) | ((uint32_t) (px - qx) << 9) | ((uint32_t) (py - qy) << 10);
            q.b0[e] = cv.b0;
            q.b1[e] = cv.b1;
            q.b2[e] = cv.b2;
            mine |= 1ull << e;
          }
          count += __popc(want);
        }
      }
    }
  }
  if (HAS_COLOR && count > 0) flushQueue<SH, S, HAS_DEPTH>(p, U, q, count, mine, lane, rx0, ry0, inC, fb);
  if (inC) {
    size_t pix = (size_t) py * fr.cW + px;
    if (S == 4) {
      *reinterpret_cast<uint4 *>(colorBuf + pix * 4) = make_uint4(fb.c0, fb.c1, fb.c2, fb.c3);
      // multiSampleResolve (RendererSoft.cpp:880-912): mean of four u8 samples, truncated
      uint32_t rsv = 0;
#pragma unroll
      for (int ch = 0; ch < 4; ch++) {
        uint32_t sum = ((fb.c0 >> (8 * ch)) & 255u) + ((fb.c1 >> (8 * ch)) & 255u) + ((fb.c2 >> (8 * ch)) & 255u) +
                       ((fb.c3 >> (8 * ch)) & 255u);
        rsv |= ((sum >> 2) & 255u) << (8 * ch);
      }
      resolvedBuf[pix] = rsv;
    } else {
      colorBuf[pix] = fb.c0;
    }
  }
  if (inD) {
    size_t pix = (size_t) py * fr.dW + px;
    if (S == 4) {
      *reinterpret_cast<float4 *>(depthBuf + pix * 4) = make_float4(fb.d0, fb.d1, fb.d2, fb.d3);
    } else {
      depthBuf[pix] = fb.d0;
    }
  }
}

template<int SH>
void launchRasterModel(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st) {
  int grid = p.numTiles;
  if (p.samples == 4) {
    if (hasDepth) launchChained(k_raster<SH, 4, true, true>, dim3(grid), dim3(256), 0, st, p);
    else launchChained(k_raster<SH, 4, true, false>, dim3(grid), dim3(256), 0, st, p);
  } else {
    if (hasDepth) launchChained(k_raster<SH, 1, true, true>, dim3(grid), dim3(256), 0, st, p);
    else launchChained(k_raster<SH, 1, true, false>, dim3(grid), dim3(256), 0, st, p);
  }
  (void) hasColor;
}

// ------------------------------------------------------------------------------------------------
// Deferred shading: the per-pixel sequence of k_raster split over three kernels, so that the large
// fragment shader runs in a kernel of its own (full SIMD width, one code path per SM, no coverage
// code competing for the instruction cache) and the coverage kernel carries no shader registers.
//
//   k_raster_cov  coverage, early-Z and depth exactly as k_raster; each fragment that reaches the
//                 colour stage is appended, in the warp's order, to the warp's chunk list
//   k_shade       the fragment shader once per record (any order: it is a pure function)
//   k_rop         every warp walks its chunk list and applies each record's colour operations to
//                 its pixel in list order, then stores colour and the MSAA resolve
//
// A pixel belongs to one warp in both k_raster_cov and k_rop, and that warp's list keeps the
// pixel's fragments in the order k_raster would apply them, so the result is the same bit for bit.
// ------------------------------------------------------------------------------------------------

// meta of a record: lane | sample mask << 5 | (px - qx) << 9 | (py - qy) << 10 | view << 11
__device__ __forceinline__ int allocChunk(const DrawParams &p, int lane) {
  int c = 0;
  if (lane == 0) {
    c = atomicAdd(&p.counters[kCntChunks], 1);
    if (c >= p.chunkCap) {
      atomicOr(&p.counters[2], kOvfFrags);
      c = -1;
    } else {
      p.chunkNext[c] = -1;
    }
  }
  return __shfl_sync(0xffffffffu, c, 0);
}

// The tile (and part) a coverage / ROP CTA works on. CTAs [0, 4 H) take the first H tiles of the
// heavy-first order, four per tile: a tile with more than heavyMin primitives is split by rows (part
// p = row p of every warp's 8x4 block, so each warp owns 8 pixels); a lighter one is done whole by its
// first CTA. CTAs [4 H, tiles + 3 H) take the rest of the order one tile each.
struct TileJob {
  int tile, part, rows;   // rows of each warp's block: 4 (whole tile) or 1 (split)
  bool skip;
  int halves;             // a split tile: 1 (four parts, a whole row per warp) or 2 (eight, half rows)
};


__device__ __forceinline__ TileJob tileJob(const DrawParams &p) {
  const int H = p.tileOrder ? p.heavySlots : 0;
  const int nTiles = p.numTiles;
  const int b = blockIdx.x;
  if (b < kSplitParts * H) {
    const int slot = b / kSplitParts, part = b % kSplitParts;
    if (slot >= nTiles) return {0, 0, 4, true, 1};
    const int tile = p.tileOrder[slot];
    const int len = p.tileEnd[tile] - p.tileStart[tile];
    if (len > p.heavyMin8) return {tile, part, 1, false, 2};                 // eight parts
    if (len > p.heavyMin) return {tile, part & 3, 1, part >= 4, 1};        // four parts
    return {tile, 0, 4, part != 0, 1};
  }
  const int k = b - (kSplitParts - 1) * H;
  return {p.tileOrder ? p.tileOrder[k] : k, 0, 4, false, 1};
}

// Pixels of a job: a whole tile gives each warp its 8x4 block (every lane owns a pixel); part q of a
// split tile gives each warp row q % 4 of its block, and in eight parts only the half of that row
// numbered q / 4 (lanes 0-3 or 4-7 own a pixel). The 8-pixel row stays the warp's rectangle for the
// list compaction and pass 1; lanes that own no pixel take part in the load-balanced pass 2 only.
__device__ __forceinline__ int jobRow(const TileJob &job) { return job.rows == 4 ? 0 : job.part & 3; }
__device__ __forceinline__ bool jobOwns(const TileJob &job, int lane) {
  if (job.rows == 4) return true;
  return (lane >> 3) == 0 && (job.halves == 1 || ((lane & 7) >> 2) == (job.part >> 2));
}
// the record-list head of warp `warp` of a job
__device__ __forceinline__ int warpSlot(const TileJob &job, int W, int warp) {
  return (job.tile * kSplitParts + job.part) * W + warp;
}

// one evaluated (pixel, candidate) pair of the load-balanced pass 2
struct CovSlot {
  Cover cv;
  int x0, x1, y0, y1, nx, nq;
  int prim;
};

template<int S, bool HAS_DEPTH, int W>
__global__ void __launch_bounds__(32 * W, (S == 4 ? 2 : 4) * 8 / W) k_raster_cov(const __grid_constant__ DrawParams p) {
  constexpr int TH = 2 * W;   // tile height in pixels (width 16): W warps of 8x4 pixels, two per row
  chainEnter();
  __shared__ CovSlot covSlots[W][32];
  __shared__ int covQueue[W][64];
  const TileJob job = tileJob(p);
  if (job.skip) return;
  const int tile = job.tile, rh = job.rows;
  const TileFrame fr = tileFrame(p, tile);
  const int view = fr.view, tx = fr.tx, ty = fr.ty;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rx0 = tx * 16 + (warp & 1) * 8, ry0 = ty * TH + (warp >> 1) * 4 + jobRow(job);
  const int px = rx0 + (lane & 7), py = ry0 + (lane >> 3);
  const bool own = jobOwns(job, lane);   // this lane has a pixel (all 32 in a whole tile, 4 or 8 in a split one)
  const bool inD = HAS_DEPTH && own && px < fr.dW && py < fr.dH;
  float *depthBuf = fr.depth;
  const unsigned lt = (1u << lane) - 1u;
  const int start = p.tileStart[tile], end = p.tileEnd[tile];
  if (start >= end) {
    // an empty list (most tiles of a frame): no records, so no part in the dense list (the whole
    // CTA leaves here); only the warps' empty record lists and, on a pass's first draw, the
    // cleared depth
    if (lane == 0) p.warpHead[warpSlot(job, W, warp)] = -1;
    if (inD && p.pendingClear && p.clearDepthFlag) {
      const size_t pix = (size_t) py * fr.dW + px;
      if (S == 4) {
        *reinterpret_cast<float4 *>(depthBuf + pix * 4) = make_float4(p.clearDepth, p.clearDepth, p.clearDepth,
                                                                      p.clearDepth);
      } else {
        depthBuf[pix] = p.clearDepth;
      }
    }
    return;
  }
  Samples4 fb = {0u, 0u, 0u, 0u, 0.f, 0.f, 0.f, 0.f};
  if (inD) {
    size_t pix = (size_t) py * fr.dW + px;
    if (p.pendingClear && p.clearDepthFlag) {
      fb.d0 = fb.d1 = fb.d2 = fb.d3 = p.clearDepth;
    } else if (S == 4) {
      float4 v = *reinterpret_cast<const float4 *>(depthBuf + pix * 4);
      fb.d0 = v.x; fb.d1 = v.y; fb.d2 = v.z; fb.d3 = v.w;
    } else {
      fb.d0 = depthBuf[pix];
    }
  }
  const bool inPix = (own && px < fr.cW && py < fr.cH) || inD;
  const uint32_t pixWord = (uint32_t) px | ((uint32_t) py << 16);
  int head = -1, ch = -1, cnt = 0;
  bool dead = false;
  unsigned long long total = 0;
  const float lo = S == 4 ? 0.125f : 0.5f, hi = S == 4 ? 0.875f : 0.5f;
  const float vpExtent = fabsf(fr.vpW) + fabsf(fr.vpH) + 2.f * (float) (rx0 + ry0) + 64.f;
  CovSlot *slots = covSlots[warp];
  int *queue = covQueue[warp];
  int qn = 0;
  // the depth functions whose depth write keeps a running minimum or maximum (or no depth write)
  // take the scanned depth path of pass 2; EQUAL, NOTEQUAL, ALWAYS and NEVER with depth writes run
  // each pixel's pairs in order on its owner lane
  const bool testDepth = p.depthTest && HAS_DEPTH;
  const int df = p.depthFunc;
  const bool scanDepth = !testDepth || !p.depthMask || df == DEPTH_LESS || df == DEPTH_LEQUAL ||
                         df == DEPTH_GREATER || df == DEPTH_GEQUAL;
  const float keepId = (df == DEPTH_LESS || df == DEPTH_LEQUAL) ? __int_as_float(0x7f800000) : __int_as_float(0xff800000);
  const int hiz = hizMode(p, HAS_DEPTH);
  // appends one record per lane with a non-zero sample mask, in lane order, to this warp's list
  auto appendRecords = [&](uint32_t mask, uint32_t meta, int prim, uint32_t pixw, float b0, float b1, float b2) {
    const unsigned want = __ballot_sync(0xffffffffu, mask != 0);
    if (!want || dead) return;
    const int n = __popc(want);
    if (head < 0) {
      ch = head = allocChunk(p, lane);
      cnt = 0;
      if (ch < 0) {
        dead = true;
        return;
      }
    }
    int nch = -1;
    if (cnt + n > kChunk) nch = allocChunk(p, lane);
    if (mask) {
      const int ei = cnt + __popc(want & lt);
      const int c2 = ei < kChunk ? ch : nch;
      if (c2 >= 0) {
        const size_t r = (size_t) c2 * kChunk + (ei < kChunk ? ei : ei - kChunk);
        p.recA[r] = make_int4(prim, (int) meta, (int) pixw, __float_as_int(b0));
        p.recB[r] = make_float2(b1, b2);
      }
    }
    total += (unsigned long long) n;
    if (cnt + n > kChunk) {
      if (lane == 0) {
        p.chunkFill[ch] = kChunk;
        if (nch >= 0) p.chunkNext[ch] = nch;
      }
      cnt = cnt + n - kChunk;
      ch = nch;
      if (nch < 0) dead = true;
    } else {
      cnt += n;
    }
  };
  for (int base = start; base < end || qn > 0;) {
    // dense batches: the tile-list primitives whose rectangle touches this warp's pixels, in list
    // order, 32 at a time (most of a tile's list misses any one 8x4 rectangle)
    while (qn < 32 && base < end) {
      const int i = base + lane;
      const int pr0 = i < end ? __ldg(p.valA + i) : -1;
      const bool t = pr0 >= 0 && touchesRect(p, pr0, rx0, ry0, rh);
      const unsigned bm = __ballot_sync(0xffffffffu, t);
      if (t) queue[qn + __popc(bm & lt)] = pr0;
      qn += __popc(bm);
      base += 32;
    }
    __syncwarp();
    const int nb = min(qn, 32);
    const int prim = lane < nb ? queue[lane] : -1;
    const int rest = qn - nb;
    const int keep = lane < rest ? queue[nb + lane] : 0;
    __syncwarp();
    if (lane < rest) queue[lane] = keep;
    qn = rest;
    __syncwarp();
    // depth bounds of this lane's pixel and of the warp's pixels at the start of the batch
    const float pixBound = hizPixelBound<S>(hiz, fb, inD);
    float warpBound = pixBound;
    if (hiz != HIZ_NONE) {
      const bool lower = hiz == HIZ_GREATER || hiz == HIZ_GEQUAL;
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        const float v = __shfl_xor_sync(0xffffffffu, warpBound, o);
        warpBound = lower ? fminf(warpBound, v) : fmaxf(warpBound, v);
      }
    }
    unsigned cand = pass1Prim<S>(p, prim, lane, rx0, ry0, lo, hi, vpExtent, rh, hiz, warpBound);
    if (!inPix) cand = 0;
    // pass 2, load-balanced: the (pixel, candidate) pairs of the batch, pixel-major in candidate
    // order, are evaluated 32 at a time by all lanes (coverage does not depend on the depth buffer);
    // then each pixel's owner lane runs the depth operations of its pairs in order
    const int cnum = __popc(cand);
    int off = cnum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int v = __shfl_up_sync(0xffffffffu, off, o);
      if (lane >= o) off += v;
    }
    const int pairs = __shfl_sync(0xffffffffu, off, 31);
    off -= cnum;   // exclusive
    for (int r0 = 0; r0 < pairs; r0 += 32) {
      const int kk = r0 + lane;
      // owner pixel of pair kk: the last lane whose offset is <= kk
      int L = 0;
#pragma unroll
      for (int step = 16; step; step >>= 1) {
        int o2 = __shfl_sync(0xffffffffu, off, (L + step) & 31);
        if (L + step < 32 && o2 <= kk) L += step;
      }
      const unsigned candL = __shfl_sync(0xffffffffu, cand, L);
      const int offL = __shfl_sync(0xffffffffu, off, L);
      // the (kk - offL)-th candidate of pixel L
      int nth = kk - offL, pos = 0;
      unsigned m = candL;
#pragma unroll
      for (int w = 16; w; w >>= 1) {
        int c1 = __popc(m & ((1u << w) - 1u));
        if (nth >= c1) {
          nth -= c1;
          m >>= w;
          pos += w;
        }
      }
      const int pr = __shfl_sync(0xffffffffu, prim, pos & 31);
      const float boundL = __shfl_sync(0xffffffffu, pixBound, L);
      CovSlot sl;
      sl.nq = 0;
      if (kk < pairs) {
        const int lpx = rx0 + (L & 7), lpy = ry0 + (L >> 3);
        const TriSetup *tp = p.tri + pr;
        int x0 = 0, x1 = 0, y0 = 0, y1 = 0, nx = 0;
        bool culled = false;
        if (hiz != HIZ_NONE) {   // the triangle fails the depth test at every sample of pixel L
          const float4 q2 = __ldg(reinterpret_cast<const float4 *>(tp) + 2);
          culled = hizReject(hiz, fminf(q2.x, fminf(q2.y, q2.z)), fmaxf(q2.x, fmaxf(q2.y, q2.z)), boundL);
        }
        int nq = culled ? 0 : quadsOf(tp, lpx, lpy, x0, x1, y0, y1, nx);
        Cover cv;
        cv.mask = 0u;
        if (nq) cv = coverSamples<S>(p, loadTriCov(tp), lpx, lpy);
        if (!cv.mask) nq = 0;
        sl.cv = cv;
        sl.x0 = x0; sl.x1 = x1; sl.y0 = y0; sl.y1 = y1;
        sl.nx = nx;
        sl.nq = nq;
        sl.prim = pr;
      }
      const int s0 = max(off, r0) - r0, s1 = min(off + cnum, r0 + 32) - r0;   // this lane's pixel's pairs
      const int nOwn = max(0, s1 - s0);
      if (scanDepth && !__any_sync(0xffffffffu, sl.nq > 1)) {
        // every pair at once: a pixel's pairs occupy consecutive lanes in candidate order, so the
        // depth each one is tested against is a segmented scan over the lanes (depthKeep), seeded
        // with the pixel's depth; the segment's last lane holds the pixel's new depth
        const bool has = kk < pairs && sl.nq > 0;
        uint32_t cov = 0u;
        if (has) cov = S == 4 ? ((sl.cv.mask & 16u) ? (sl.cv.mask & 15u) : 0u) : (sl.cv.mask & 1u);
        uint32_t pass = cov;
        if (testDepth) {
          const int segStart = max(offL, r0) - r0;
          // the longest segment of the round: scan steps at or beyond it combine no two lanes of
          // one segment (lane - d < segStart for every lane of it), so they are skipped
          const int segMax = __reduce_max_sync(0xffffffffu, nOwn);
          const bool inDL = __shfl_sync(0xffffffffu, inD, L);
          const float zs[4] = {sl.cv.z0, sl.cv.z1, sl.cv.z2, sl.cv.z3};
          const float fbd[4] = {fb.d0, fb.d1, fb.d2, fb.d3};
          float last[4] = {0.f, 0.f, 0.f, 0.f};
          float cz[4], cur[4], x[4];
#pragma unroll
          for (int q = 0; q < S; q++) {
            cz[q] = gclamp(zs[q], p.vp.absMin, p.vp.absMax);
            cur[q] = __shfl_sync(0xffffffffu, fbd[q], L);
            x[q] = ((cov >> q) & 1u) && cz[q] == cz[q] ? cz[q] : keepId;
          }
          if (p.depthMask) {
            // the samples' scans step together (independent chains, one branch per step)
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
              if (d >= segMax) break;
              const bool take = lane - d >= segStart;
#pragma unroll
              for (int q = 0; q < S; q++) {
                const float y = __shfl_up_sync(0xffffffffu, x[q], d);
                if (take) x[q] = depthKeep(y, x[q], p.depthFunc);
              }
            }
#pragma unroll
            for (int q = 0; q < S; q++) {
              const float ex = __shfl_up_sync(0xffffffffu, x[q], 1);
              if (lane > segStart) cur[q] = depthKeep(cur[q], ex, p.depthFunc);
              last[q] = __shfl_sync(0xffffffffu, x[q], nOwn > 0 ? s1 - 1 : lane);
            }
          }
          pass = 0u;
#pragma unroll
          for (int q = 0; q < S; q++)
            if (((cov >> q) & 1u) && inDL && depthCmp(cz[q], cur[q], p.depthFunc)) pass |= 1u << q;
          if (p.depthMask && inD && nOwn > 0) {
            fb.d0 = depthKeep(fb.d0, last[0], p.depthFunc);
            if (S == 4) {
              fb.d1 = depthKeep(fb.d1, last[1], p.depthFunc);
              fb.d2 = depthKeep(fb.d2, last[2], p.depthFunc);
              fb.d3 = depthKeep(fb.d3, last[3], p.depthFunc);
            }
          }
        }
        const int lpx = rx0 + (L & 7), lpy = ry0 + (L >> 3);
        appendRecords(pass, (uint32_t) L | (pass << 5) | ((uint32_t) (lpx - sl.x0) << 9) |
                                ((uint32_t) (lpy - sl.y0) << 10) | ((uint32_t) view << 11),
                      sl.prim, (uint32_t) lpx | ((uint32_t) lpy << 16), sl.cv.b0, sl.cv.b1, sl.cv.b2);
        continue;
      }
      slots[lane] = sl;
      __syncwarp();
      // owner phase: this lane's pairs of the round, in order
      const int maxOwn = __reduce_max_sync(0xffffffffu, nOwn);
      for (int q = 0; q < maxOwn; q++) {
        const CovSlot *e = q < nOwn ? &slots[s0 + q] : nullptr;
        const int nq = e ? e->nq : 0;
        const int nqMax = __reduce_max_sync(0xffffffffu, nq);
        for (int k = 0; k < nqMax; k++) {   // a pixel can lie in two overlapping blocks' quads
          uint32_t mask = 0;
          int qx = 0, qy = 0;
          if (k < nq) {
            qy = (k / e->nx) ? e->y1 : e->y0;
            qx = (k % e->nx) ? e->x1 : e->x0;
            mask = depthOps<S, HAS_DEPTH>(p, e->cv, inD, fb);
          }
          appendRecords(mask, (uint32_t) lane | (mask << 5) | ((uint32_t) (px - qx) << 9) |
                                  ((uint32_t) (py - qy) << 10) | ((uint32_t) view << 11),
                        e ? e->prim : 0, pixWord, e ? e->cv.b0 : 0.f, e ? e->cv.b1 : 0.f, e ? e->cv.b2 : 0.f);
        }
      }
      __syncwarp();
    }
  }
  if (lane == 0) {
    p.warpHead[warpSlot(job, W, warp)] = head;
    if (ch >= 0) p.chunkFill[ch] = cnt;
    if (p.fragCounter && total) atomicAdd(p.fragCounter, total);
  }
  // the dense record list: one contiguous run per CTA (one atomic), each warp's records in its
  // list order inside it, so the shading kernel reads no unfilled chunk slots and keeps each warp's
  // records together
  __shared__ int wRecs[W], ctaBase;
  int recs = 0;
  for (int c = head; c >= 0;) {   // this warp's chunks: every one full but the last
    const int f = c == ch ? cnt : kChunk;
    recs += f;
    c = c == ch ? -1 : p.chunkNext[c];
  }
  if (lane == 0) wRecs[warp] = recs;
  __syncthreads();
  if (threadIdx.x == 0) {
    int sum = 0;
    for (int w = 0; w < W; w++) sum += wRecs[w];
    ctaBase = sum ? atomicAdd(&p.counters[kCntDense], sum) : 0;
  }
  __syncthreads();
  int d = ctaBase;
  for (int w = 0; w < warp; w++) d += wRecs[w];
  for (int c = head; c >= 0;) {
    const int f = c == ch ? cnt : kChunk;
    if (lane < f && d + lane < p.chunkCap * kChunk) p.recDense[d + lane] = c * kChunk + lane;
    d += f;
    c = c == ch ? -1 : p.chunkNext[c];
  }
  if ((p.tmaStore & 2) && rh == 4) {
    // whole tile: its depth samples through shared memory and one TMA bulk store
    __shared__ alignas(128) float sDep[16 * TH * S];
    const int li = (py - ty * TH) * 16 + (px - tx * 16);
    sDep[li * S] = fb.d0;
    if (S == 4) {
      sDep[li * 4 + 1] = fb.d1;
      sDep[li * 4 + 2] = fb.d2;
      sDep[li * 4 + 3] = fb.d3;
    }
    fenceAsyncShared();
    __syncthreads();
    if (threadIdx.x == 0) {
      tmaStore2d(&p.tmDepth, sDep, tx * 16 * S, ty * TH);
      tmaCommitWait();
    }
    return;
  }
  if (inD) {
    size_t pix = (size_t) py * fr.dW + px;
    if (S == 4) {
      *reinterpret_cast<float4 *>(depthBuf + pix * 4) = make_float4(fb.d0, fb.d1, fb.d2, fb.d3);
    } else {
      depthBuf[pix] = fb.d0;
    }
  }
}

// the fragment shader over every record (grid-stride over the dense record list, so no lane idles
// on the unfilled tail of a warp's last chunk); 8 CTAs of 4 warps per SM: the sampler is inlined
// and latency-bound, more warps beat a few spills
template<int SH, int S>
__global__ void __launch_bounds__(128, 8) k_shade(const __grid_constant__ DrawParams p) {
  chainEnter();
  const int n = min(p.counters[kCntDense], p.chunkCap * kChunk);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int r = p.recDense[i];
    if (r < 0) continue;
    const int4 a = p.recA[r];
    const float2 b = p.recB[r];
    const uint32_t meta = (uint32_t) a.y;
    const int px = a.z & 0xffff, py = (int) ((uint32_t) a.z >> 16);
    const int qx = px - (int) ((meta >> 9) & 1u), qy = py - (int) ((meta >> 10) & 1u);
    p.recColor[r] = shadeFragmentInl<SH, S>(p, viewUniforms(p, (int) (meta >> 11)), a.x, qx, qy, px, py,
                                            __int_as_float(a.w), b.x, b.y);
  }
}

// colour operations in each warp's list order, then colour store and MSAA resolve
template<int S, int W>
__global__ void __launch_bounds__(32 * W) k_rop(const __grid_constant__ DrawParams p) {
  constexpr int TH = 2 * W;   // tile height in pixels (width 16)
  chainEnter();
  __shared__ float4 scol[W][kChunk];
  __shared__ uint32_t smeta[W][kChunk];
  __shared__ uint32_t sown[W][kChunk];
  if (blockIdx.x == 0 && threadIdx.x == 0) {   // the draw's last kernel: its peak chunk use and flags
    if (p.ropPeakChunks) *p.ropPeakChunks = max(*p.ropPeakChunks, p.counters[kCntChunks]);
    if (p.ropSticky) *p.ropSticky |= p.counters[2];
  }
  const TileJob job = tileJob(p);
  if (job.skip) return;
  const int tile = job.tile;
  const TileFrame fr = tileFrame(p, tile);
  const int tx = fr.tx, ty = fr.ty;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rx0 = tx * 16 + (warp & 1) * 8, ry0 = ty * TH + (warp >> 1) * 4 + jobRow(job);
  const int px = rx0 + (lane & 7), py = ry0 + (lane >> 3);
  const bool inC = jobOwns(job, lane) && px < fr.cW && py < fr.cH;
  uint32_t *colorBuf = fr.color;
  uint32_t *resolvedBuf = fr.resolved;
  Samples4 fb = {0u, 0u, 0u, 0u, 0.f, 0.f, 0.f, 0.f};
  const size_t pix = (size_t) py * fr.cW + px;
  if (inC) {
    if (p.pendingClear && p.clearColorFlag) {
      fb.c0 = fb.c1 = fb.c2 = fb.c3 = p.clearColor;
    } else if (S == 4) {
      uint4 v = *reinterpret_cast<const uint4 *>(colorBuf + pix * 4);
      fb.c0 = v.x; fb.c1 = v.y; fb.c2 = v.z; fb.c3 = v.w;
    } else {
      fb.c0 = colorBuf[pix];
    }
  }
  int ch = p.warpHead[warpSlot(job, W, warp)];
  while (ch >= 0) {
    const int fill = p.chunkFill[ch];
    const size_t r = (size_t) ch * kChunk + lane;
    uint32_t meta = 0u;
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
    if (lane < fill) {
      meta = (uint32_t) p.recA[r].y;
      c = p.recColor[r];
    }
    sown[warp][lane] = 0u;
    __syncwarp();
    if (lane < fill) atomicOr(&sown[warp][meta & 31u], 1u << lane);
    smeta[warp][lane] = meta;
    scol[warp][lane] = c;
    __syncwarp();
    unsigned mine = sown[warp][lane];
    while (mine) {
      const int e = __ffs(mine) - 1;
      mine &= mine - 1;
      const float4 color = scol[warp][e];
      const uint32_t mask = (smeta[warp][e] >> 5) & 15u;
      if (mask & 1u) perSample<true, false>(p, inC, true, fb.c0, fb.d0, 0.f, color);
      if (S == 4) {
        if (mask & 2u) perSample<true, false>(p, inC, true, fb.c1, fb.d1, 0.f, color);
        if (mask & 4u) perSample<true, false>(p, inC, true, fb.c2, fb.d2, 0.f, color);
        if (mask & 8u) perSample<true, false>(p, inC, true, fb.c3, fb.d3, 0.f, color);
      }
    }
    const int next = fill == kChunk ? p.chunkNext[ch] : -1;
    __syncwarp();
    ch = next;
  }
  // multiSampleResolve (RendererSoft.cpp:880-912): mean of four u8 samples, truncated
  uint32_t rsv = 0;
  if (S == 4) {
#pragma unroll
    for (int k = 0; k < 4; k++) {
      uint32_t sum = ((fb.c0 >> (8 * k)) & 255u) + ((fb.c1 >> (8 * k)) & 255u) + ((fb.c2 >> (8 * k)) & 255u) +
                     ((fb.c3 >> (8 * k)) & 255u);
      rsv |= ((sum >> 2) & 255u) << (8 * k);
    }
  }
  if ((p.tmaStore & 1) && job.rows == 4) {
    // whole tile: stage its colour samples and resolved pixels in shared memory in the
    // attachments' own order and write each with one TMA bulk store (pixels outside the
    // attachment are clipped by the copy)
    __shared__ alignas(128) uint32_t sCol[16 * TH * S];
    __shared__ alignas(128) uint32_t sRes[S == 4 ? 16 * TH : 1];
    const int li = (py - ty * TH) * 16 + (px - tx * 16);
    sCol[li * S] = fb.c0;
    if (S == 4) {
      sCol[li * 4 + 1] = fb.c1;
      sCol[li * 4 + 2] = fb.c2;
      sCol[li * 4 + 3] = fb.c3;
      sRes[li] = rsv;
    }
    fenceAsyncShared();
    __syncthreads();
    if (threadIdx.x == 0) {
      tmaStore2d(&p.tmColor, sCol, tx * 16 * S, ty * TH);
      if (S == 4) tmaStore2d(&p.tmResolved, sRes, tx * 16, ty * TH);
      tmaCommitWait();
    }
    return;
  }
  if (inC) {
    if (S == 4) {
      *reinterpret_cast<uint4 *>(colorBuf + pix * 4) = make_uint4(fb.c0, fb.c1, fb.c2, fb.c3);
      resolvedBuf[pix] = rsv;
    } else {
      colorBuf[pix] = fb.c0;
    }
  }
}

// the shading kernel of one model; the coverage and ROP kernels are model-independent
template<int SH>
void launchShadeModel(const DrawParams &p, cudaStream_t st) {
  // 32 CTAs of 128 threads per SM, grid-stride over the dense record list (at 1080p MSAA4, 708,939
  // records: about 1.1 per thread; 0.135 -> 0.129 ms against 16 per SM, equal at 64 per SM)
  const int grid = currentSmCount() * 32;
  if (p.samples == 4) launchChained(k_shade<SH, 4>, dim3(grid), dim3(128), 0, st, p);
  else launchChained(k_shade<SH, 1>, dim3(grid), dim3(128), 0, st, p);
}

}  // namespace sglc
