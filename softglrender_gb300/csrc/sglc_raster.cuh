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
// share derivatives and, when blocks overlap, a pixel can be visited twice. quadCands() finds, for
// one pixel, exactly the quads the reference visits, in the reference's order; neighbourBC()
// recomputes the quad neighbours' shading-sample barycentrics for dFdx/dFdy.
#pragma once

#include "sglc_device.cuh"
#include "sglc_shaders.cuh"

namespace sglc {

__constant__ float2 kLoc4xR[4] = {{0.375f, 0.875f}, {0.875f, 0.625f}, {0.125f, 0.375f}, {0.625f, 0.125f}};

struct Tri {
  float v0x, v0y, f0x, f0y, f0z, f1x, f1y, f1z;
  float z0, z1, z2, w0, w1, w2;
  float bminx, bminy, bmaxx, bmaxy;
  int bcx, bcy, vid0, vid1, vid2;
};

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
__device__ __forceinline__ bool bary(const Tri &t, float px, float py, float &b0, float &b1, float &b2) {
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

// glm::dot(bc, vec4(v0, v1, v2, 0)) with DPPS order (z and w of a sample)
__device__ __forceinline__ float interpZW(float b0, float b1, float b2, float v0, float v1, float v2) {
  return (b0 * v0 + b1 * v1) + (b2 * v2 + 0.f * 0.f);
}

// barycentric *= (1 / w * vertW) (RendererSoft.cpp:802)
__device__ __forceinline__ void correct(const Tri &t, float &b0, float &b1, float &b2) {
  float w = interpZW(b0, b1, b2, t.w0, t.w1, t.w2);
  float iw = 1.f / w;
  b0 = b0 * (iw * t.w0);
  b1 = b1 * (iw * t.w1);
  b2 = b2 * (iw * t.w2);
}

// shading-sample barycentrics of a quad neighbour (RendererInternal.h:97-124 + :787-804)
template<int S>
__device__ __forceinline__ void neighbourBC(const Tri &t, int fx, int fy, float &b0, float &b1, float &b2) {
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
__device__ __forceinline__ int quadCands(float bmin, float bmax, int bc, int pos, int &q0, int &q1) {
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

__device__ __forceinline__ bool depthCmp(float a, float b, int func) {
  switch (func) {
    case 0: return false;
    case 1: return a < b;
    case 2: return fabsf(a - b) <= 1.19209290e-07f;
    case 3: return a <= b;
    case 4: return a > b;
    case 5: return fabsf(a - b) > 1.19209290e-07f;
    case 6: return a >= b;
    case 7: return true;
  }
  return a < b;
}

__device__ __forceinline__ float blendFactor(float src, float srcA, float dst, float dstA, int f) {
  switch (f) {
    case 0: return 0.f;
    case 1: return 1.f;
    case 2: return src;
    case 3: return srcA;
    case 4: return dst;
    case 5: return dstA;
    case 6: return 1.f - src;
    case 7: return 1.f - srcA;
    case 8: return 1.f - dst;
    case 9: return 1.f - dstA;
  }
  return 0.f;
}

__device__ __forceinline__ float blendFn(float s, float d, int fn) {
  switch (fn) {
    case 0: return s + d;
    case 1: return s - d;
    case 2: return d - s;
    case 3: return gmin(s, d);
    case 4: return gmax(s, d);
  }
  return s + d;
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
      float4 q = unpack4(col);
      d = make_float4(q.x / 255.f, q.y / 255.f, q.z / 255.f, q.w / 255.f);
    }
    float r0 = blendFn(c0 * blendFactor(c0, c3, d.x, d.w, p.bSrcRgb), d.x * blendFactor(c0, c3, d.x, d.w, p.bDstRgb),
                       p.bFuncRgb);
    float r1 = blendFn(c1 * blendFactor(c1, c3, d.y, d.w, p.bSrcRgb), d.y * blendFactor(c1, c3, d.y, d.w, p.bDstRgb),
                       p.bFuncRgb);
    float r2 = blendFn(c2 * blendFactor(c2, c3, d.z, d.w, p.bSrcRgb), d.z * blendFactor(c2, c3, d.z, d.w, p.bDstRgb),
                       p.bFuncRgb);
    float r3 = blendFn(c3 * blendFactor(c3, c3, d.w, d.w, p.bSrcA), d.w * blendFactor(c3, c3, d.w, d.w, p.bDstA),
                       p.bFuncA);
    c0 = r0; c1 = r1; c2 = r2; c3 = r3;
  }
  if (inC) col = pack4(c0 * 255.f, c1 * 255.f, c2 * 255.f, c3 * 255.f);
}

struct Samples4 {
  uint32_t c0, c1, c2, c3;
  float d0, d1, d2, d3;
};

// One quad of one triangle, seen from the pixel (px, py) it contains.
template<int SH, int S, bool HAS_COLOR, bool HAS_DEPTH>
__device__ __forceinline__ void rasterQuadPixel(const DrawParams &p, const Tri &t, int qx, int qy, int px, int py,
                                                bool inC, bool inD, bool needDeriv, Samples4 &fb) {
  const float fx = (float) px, fy = (float) py;
  float sb0, sb1, sb2;   // shading-sample barycentrics
  float z0 = 0.f, z1 = 0.f, z2 = 0.f, z3 = 0.f;
  bool i0 = false, i1 = false, i2 = false, i3 = false;
  if (S == 1) {
    if (!bary(t, fx + 0.5f, fy + 0.5f, sb0, sb1, sb2)) return;
    z0 = interpZW(sb0, sb1, sb2, t.z0, t.z1, t.z2);
    correct(t, sb0, sb1, sb2);
    // the S=1 depth-range clip has no effect: early-Z overwrites it and the per-sample path
    // does not read it (RendererSoft.cpp:797-799 vs :846-849, :872-874)
    if (p.earlyZ && p.depthTest && HAS_DEPTH) {
      float d = gclamp(z0, p.vp.absMin, p.vp.absMax);
      if (!inD || !depthCmp(d, fb.d0, p.depthFunc)) return;
    }
    i0 = true;
  } else {
    float a0, a1, a2, b0, b1, b2, c0, c1, c2, e0, e1, e2, m0, m1, m2;
    bool s0 = bary(t, kLoc4xR[0].x + fx, kLoc4xR[0].y + fy, a0, a1, a2);
    bool s1 = bary(t, kLoc4xR[1].x + fx, kLoc4xR[1].y + fy, b0, b1, b2);
    bool s2 = bary(t, kLoc4xR[2].x + fx, kLoc4xR[2].y + fy, c0, c1, c2);
    bool s3 = bary(t, kLoc4xR[3].x + fx, kLoc4xR[3].y + fy, e0, e1, e2);
    if (!(s0 || s1 || s2 || s3)) return;
    bool sc = bary(t, fx + 0.5f, fy + 0.5f, m0, m1, m2);
    // InitShadingSample: the centre if covered, else the first covered sample
    if (sc) { sb0 = m0; sb1 = m1; sb2 = m2; }
    else if (s0) { sb0 = a0; sb1 = a1; sb2 = a2; }
    else if (s1) { sb0 = b0; sb1 = b1; sb2 = b2; }
    else if (s2) { sb0 = c0; sb1 = c1; sb2 = c2; }
    else { sb0 = e0; sb1 = e1; sb2 = e2; }
    if (s0) { z0 = interpZW(a0, a1, a2, t.z0, t.z1, t.z2); i0 = !(z0 < p.vp.absMin || z0 > p.vp.absMax); }
    if (s1) { z1 = interpZW(b0, b1, b2, t.z0, t.z1, t.z2); i1 = !(z1 < p.vp.absMin || z1 > p.vp.absMax); }
    if (s2) { z2 = interpZW(c0, c1, c2, t.z0, t.z1, t.z2); i2 = !(z2 < p.vp.absMin || z2 > p.vp.absMax); }
    if (s3) { z3 = interpZW(e0, e1, e2, t.z0, t.z1, t.z2); i3 = !(z3 < p.vp.absMin || z3 > p.vp.absMax); }
    correct(t, sb0, sb1, sb2);
    if (p.earlyZ && p.depthTest && HAS_DEPTH) {
      if (i0) i0 = inD && depthCmp(gclamp(z0, p.vp.absMin, p.vp.absMax), fb.d0, p.depthFunc);
      if (i1) i1 = inD && depthCmp(gclamp(z1, p.vp.absMin, p.vp.absMax), fb.d1, p.depthFunc);
      if (i2) i2 = inD && depthCmp(gclamp(z2, p.vp.absMin, p.vp.absMax), fb.d2, p.depthFunc);
      if (i3) i3 = inD && depthCmp(gclamp(z3, p.vp.absMin, p.vp.absMax), fb.d3, p.depthFunc);
      if (!(i0 || i1 || i2 || i3)) return;
    }
  }
  float4 color = make_float4(0.f, 0.f, 0.f, 0.f);
  if (HAS_COLOR) {
    const float *r0 = p.vVary + (size_t) t.vid0 * p.varyStride;
    const float *r1 = p.vVary + (size_t) t.vid1 * p.varyStride;
    const float *r2 = p.vVary + (size_t) t.vid2 * p.varyStride;
    FragIn f;
    f.v = Vary{r0, r1, r2, sb0, sb1, sb2};
    f.dudx = f.dvdx = f.dudy = f.dvdy = 0.f;
    if (needDeriv) {
      float u0, v0, u1, v1, u2, v2;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        int nx = qx + (k == 1), ny = qy + (k == 2);
        float c0, c1, c2;
        if (nx == px && ny == py) {
          c0 = sb0; c1 = sb1; c2 = sb2;
        } else {
          neighbourBC<S>(t, nx, ny, c0, c1, c2);
        }
        Vary vk{r0, r1, r2, c0, c1, c2};
        float uu = vk[0], vv = vk[1];
        if (k == 0) { u0 = uu; v0 = vv; }
        else if (k == 1) { u1 = uu; v1 = vv; }
        else { u2 = uu; v2 = vv; }
      }
      f.dudx = u1 - u0;
      f.dvdx = v1 - v0;
      f.dudy = u2 - u0;
      f.dvdy = v2 - v0;
    }
    color = runFS<SH>(p, f);
    if (p.fragCounter) atomicAdd(p.fragCounter, 1ull);
  }
  if (i0) perSample<HAS_COLOR, HAS_DEPTH>(p, inC, inD, fb.c0, fb.d0, z0, color);
  if (S == 4) {
    if (i1) perSample<HAS_COLOR, HAS_DEPTH>(p, inC, inD, fb.c1, fb.d1, z1, color);
    if (i2) perSample<HAS_COLOR, HAS_DEPTH>(p, inC, inD, fb.c2, fb.d2, z2, color);
    if (i3) perSample<HAS_COLOR, HAS_DEPTH>(p, inC, inD, fb.c3, fb.d3, z3, color);
  }
}

template<int SH, int S, bool HAS_COLOR, bool HAS_DEPTH>
__global__ void __launch_bounds__(256) k_raster(const __grid_constant__ DrawParams p) {
  const int tile = blockIdx.x;
  const int tx = tile % p.tilesX, ty = tile / p.tilesX;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rx0 = tx * 16 + (warp & 1) * 8, ry0 = ty * 16 + (warp >> 1) * 4;
  const int px = rx0 + (lane & 7), py = ry0 + (lane >> 3);
  const bool inC = HAS_COLOR && px < p.cw && py < p.ch;
  const bool inD = HAS_DEPTH && px < p.dw && py < p.dh;
  Samples4 fb = {0u, 0u, 0u, 0u, 0.f, 0.f, 0.f, 0.f};
  if (inC) {
    size_t pix = (size_t) py * p.cw + px;
    if (p.pendingClear && p.clearColorFlag) {
      fb.c0 = fb.c1 = fb.c2 = fb.c3 = p.clearColor;
    } else if (S == 4) {
      uint4 q = *reinterpret_cast<const uint4 *>(p.color + pix * 4);
      fb.c0 = q.x; fb.c1 = q.y; fb.c2 = q.z; fb.c3 = q.w;
    } else {
      fb.c0 = p.color[pix];
    }
  }
  if (inD) {
    size_t pix = (size_t) py * p.dw + px;
    if (p.pendingClear && p.clearDepthFlag) {
      fb.d0 = fb.d1 = fb.d2 = fb.d3 = p.clearDepth;
    } else if (S == 4) {
      float4 q = *reinterpret_cast<const float4 *>(p.depth + pix * 4);
      fb.d0 = q.x; fb.d1 = q.y; fb.d2 = q.z; fb.d3 = q.w;
    } else {
      fb.d0 = p.depth[pix];
    }
  }
  const bool needDeriv = HAS_COLOR && needsDerivatives(p);
  const int start = p.tileStart[tile], end = p.tileEnd[tile];
  for (int base = start; base < end; base += 32) {
    int i = base + lane;
    int prim = -1;
    bool hit = false;
    if (i < end) {
      prim = __ldg(p.valA + i);
      int4 r = __ldg(reinterpret_cast<const int4 *>(&p.tri[prim].rx0));
      hit = !(r.y < rx0 || r.x > rx0 + 7 || r.w < ry0 || r.z > ry0 + 3);
    }
    unsigned m = __ballot_sync(0xffffffffu, hit);
    while (m) {
      int j = __ffs(m) - 1;
      m &= m - 1;
      int pr = __shfl_sync(0xffffffffu, prim, j);
      const TriSetup *ts = p.tri + pr;
      int4 r = __ldg(reinterpret_cast<const int4 *>(&ts->rx0));
      if (px < r.x || px > r.y || py < r.z || py > r.w || !(inC || inD)) continue;
      Tri t = loadTri(ts);
      int x0 = 0, x1 = 0, y0 = 0, y1 = 0;
      int nx = quadCands(t.bminx, t.bmaxx, t.bcx, px, x0, x1);
      if (nx == 0) continue;
      int ny = quadCands(t.bminy, t.bmaxy, t.bcy, py, y0, y1);
      for (int iy = 0; iy < ny; iy++) {
        int qy = iy ? y1 : y0;
        for (int ix = 0; ix < nx; ix++) {
          int qx = ix ? x1 : x0;
          rasterQuadPixel<SH, S, HAS_COLOR, HAS_DEPTH>(p, t, qx, qy, px, py, inC, inD, needDeriv, fb);
        }
      }
    }
  }
  if (inC) {
    size_t pix = (size_t) py * p.cw + px;
    if (S == 4) {
      *reinterpret_cast<uint4 *>(p.color + pix * 4) = make_uint4(fb.c0, fb.c1, fb.c2, fb.c3);
      // multiSampleResolve (RendererSoft.cpp:880-912): mean of four u8 samples, truncated
      uint32_t r = 0;
#pragma unroll
      for (int ch = 0; ch < 4; ch++) {
        uint32_t s = ((fb.c0 >> (8 * ch)) & 255u) + ((fb.c1 >> (8 * ch)) & 255u) + ((fb.c2 >> (8 * ch)) & 255u) +
                     ((fb.c3 >> (8 * ch)) & 255u);
        r |= ((s >> 2) & 255u) << (8 * ch);
      }
      p.resolved[pix] = r;
    } else {
      p.color[pix] = fb.c0;
    }
  }
  if (inD) {
    size_t pix = (size_t) py * p.dw + px;
    if (S == 4) {
      *reinterpret_cast<float4 *>(p.depth + pix * 4) = make_float4(fb.d0, fb.d1, fb.d2, fb.d3);
    } else {
      p.depth[pix] = fb.d0;
    }
  }
}

template<int SH>
void launchRasterModel(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st) {
  int grid = p.tilesX * p.tilesY;
  if (p.samples == 4) {
    if (hasDepth) k_raster<SH, 4, true, true><<<grid, 256, 0, st>>>(p);
    else k_raster<SH, 4, true, false><<<grid, 256, 0, st>>>(p);
  } else {
    if (hasDepth) k_raster<SH, 1, true, true><<<grid, 256, 0, st>>>(p);
    else k_raster<SH, 1, true, false><<<grid, 256, 0, st>>>(p);
  }
  (void) hasColor;
}

}  // namespace sglc
