// sm_103a kernels of point and line draws: Primitive_POINT, Primitive_LINE and triangles drawn in
// PolygonMode_POINT / PolygonMode_LINE (RendererSoft.cpp:301-321, 575-712). The reference draws
// them one primitive after another on one thread; here every stage is data-parallel and the
// reference's order survives as slot / stamp order:
//
//   k_lp_assemble (sglc_geom.cu)   input primitive -> three drawing-order slots (clip, cull)
//   k_lp_point_keys + radix sort + k_lp_point_chain
//                                  rasterizationPoint moves the vertex to the last pixel of its
//                                  stamp (it loops on fragPos itself), so a vertex stamped again
//                                  starts from there: per vertex, its point slots are walked in
//                                  order to find every stamp's origin
//   k_lp_stamp_count + scan        stamps per slot: 1 for a point, dx + 1 Bresenham steps for a line
//   k_lp_stamp_emit                stamp position, z and (lines) lerped varyings
//   k_lp_stamp_shade (sglc_lines_shade.cu)  fragment shader once per stamp (no shader reads
//                                  FragCoord, so every pixel of a stamp gets the same colour)
//   k_lp_frag_count + scan, k_lp_frag_emit   one (pixel, stamp) pair per covered pixel
//   radix sort by pixel (stable: stamp order survives within a pixel)
//   k_lp_frag_apply                every pixel applies its fragments' per-sample operations in
//                                  stamp order (processPerSampleOperations on every sample)
//   k_lp_resolve                   multiSampleResolve of the whole attachment after the draw
#include "sglc_device.cuh"
#include "sglc_kernels.h"
#include "sglc_raster.cuh"   // perSample

namespace sglc {

namespace {

inline int cdiv(long a, long b) { return (int) ((a + b - 1) / b); }

__device__ __forceinline__ long long llabs_(long long v) { return v < 0 ? -v : v; }

// the integer set-up of rasterizationLine (RendererSoft.cpp:663-688)
struct LineSetup {
  long long x0, y0, x1, y1;
  float z0, z1;
  bool steep, swapped;
};

__device__ __forceinline__ LineSetup lineSetup(const DrawParams &p, int a, int b) {
  float4 f0 = p.vFrag[a], f1 = p.vFrag[b];
  LineSetup L;
  L.x0 = truncI(f0.x);
  L.y0 = truncI(f0.y);
  L.x1 = truncI(f1.x);
  L.y1 = truncI(f1.y);
  L.z0 = f0.z;
  L.z1 = f1.z;
  L.steep = false;
  L.swapped = false;
  if (llabs_(L.x0 - L.x1) < llabs_(L.y0 - L.y1)) {
    long long t = L.x0; L.x0 = L.y0; L.y0 = t;
    t = L.x1; L.x1 = L.y1; L.y1 = t;
    L.steep = true;
  }
  if (L.x0 > L.x1) {
    long long t = L.x0; L.x0 = L.x1; L.x1 = t;
    t = L.y0; L.y0 = L.y1; L.y1 = t;
    float f = L.z0; L.z0 = L.z1; L.z1 = f;
    L.swapped = true;
  }
  return L;
}

// the pixel rectangle [x0, x1) x [y0, y1) a stamp's loops visit (RendererSoft.cpp:641-648)
struct StampRect {
  int x0, x1, y0, y1;
};

__device__ __forceinline__ StampRect stampRect(float x, float y, float size) {
  float left = x - size / 2.f + 0.5f;
  float right = left + size;
  float top = y - size / 2.f + 0.5f;
  float bottom = top + size;
  return {truncI(left), truncI(right), truncI(top), truncI(bottom)};
}

__device__ __forceinline__ void addTotal(unsigned long long *total, long long v) {
  // one atomic per warp
  unsigned long long s = (unsigned long long) v;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(total, s);
}

__global__ void __launch_bounds__(256) k_lp_point_keys(const __grid_constant__ LineParams lp, uint32_t *keys, int *vals,
                                                       int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int4 s = lp.slot[i];
  keys[i] = s.x == LP_SLOT_POINT ? (uint32_t) (s.y + 1) : 0u;
  vals[i] = i;
}

// keys: vertex + 1 of each point slot (0: not a point), stably sorted; vals: slot ids
__global__ void __launch_bounds__(256) k_lp_point_chain(const __grid_constant__ DrawParams p,
                                                        const __grid_constant__ LineParams lp, const uint32_t *keys,
                                                        const int *vals, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t k = keys[i];
  if (k == 0u || (i > 0 && keys[i - 1] == k)) return;
  float4 f = p.vFrag[k - 1];
  float x = f.x, y = f.y;
  for (int j = i; j < n && keys[j] == k; j++) {
    lp.pointOrigin[vals[j]] = make_float2(x, y);
    StampRect r = stampRect(x, y, lp.pointSize);
    if (r.x0 < r.x1 && r.y0 < r.y1) {   // the loops ran: fragPos is left at the last pixel
      x = (float) (r.x1 - 1);
      y = (float) (r.y1 - 1);
    }
  }
}

__global__ void __launch_bounds__(256) k_lp_stamp_count(const __grid_constant__ DrawParams p,
                                                        const __grid_constant__ LineParams lp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  long long cnt = 0;
  if (i < 3 * lp.nIn) {
    int4 s = lp.slot[i];
    if (s.x == LP_SLOT_POINT) {
      cnt = 1;
    } else if (s.x == LP_SLOT_LINE) {
      LineSetup L = lineSetup(p, s.y, s.z);
      cnt = L.x1 - L.x0 + 1;
      if (cnt > kMaxLineSteps) {
        atomicOr(lp.flags, LP_ERR_LONGLINE);
        cnt = 0;
      }
    }
    lp.stampCount[i] = (int) cnt;
  }
  addTotal(&lp.totals[0], cnt);
}

__global__ void __launch_bounds__(256) k_lp_stamp_emit(const __grid_constant__ DrawParams p,
                                                       const __grid_constant__ LineParams lp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * lp.nIn) return;
  int4 s = lp.slot[i];
  if (s.x == LP_SLOT_NONE) return;
  const int off = lp.stampOff[i];
  if (s.x == LP_SLOT_POINT) {
    float2 o = lp.pointOrigin[i];
    lp.stampGeo[off] = make_float4(o.x, o.y, p.vFrag[s.y].z, lp.pointSize);
    lp.stampRow[off] = -(s.y + 1);
    return;
  }
  // rasterizationLine (RendererSoft.cpp:663-712)
  LineSetup L = lineSetup(p, s.y, s.z);
  if (L.x1 - L.x0 + 1 > kMaxLineSteps) return;
  const float *vin0 = p.vVary + (size_t) (L.swapped ? s.z : s.y) * p.varyStride;
  const float *vin1 = p.vVary + (size_t) (L.swapped ? s.y : s.z) * p.varyStride;
  const long long dx = L.x1 - L.x0, dy = L.y1 - L.y0;
  const long long dError = 2 * llabs_(dy);
  long long error = 0, y = L.y0;
  int k = off;
  for (long long x = L.x0; x <= L.x1; x++, k++) {
    float t = (float) (x - L.x0) / (float) dx;
    float px = (float) x, py = (float) y;
    float z = L.z0 * (1.f - t) + L.z1 * t;   // glm::mix
    if (L.steep) {
      float q = px; px = py; py = q;
    }
    lp.stampGeo[k] = make_float4(px, py, z, lp.lineWidth);
    lp.stampRow[k] = k;
    if (p.varyCnt > 0) {   // interpolateLinear
      float *dst = lp.stampVary + (size_t) k * p.varyStride;
      for (int v = 0; v < p.varyCnt; v++) dst[v] = vin0[v] * (1.f - t) + vin1[v] * t;
    }
    error += dError;
    if (error > dx) {
      y += (L.y1 > L.y0 ? 1 : -1);
      error -= 2 * dx;
    }
  }
}

__global__ void __launch_bounds__(256) k_lp_frag_count(const __grid_constant__ LineParams lp, int nStamps) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  long long cnt = 0;
  if (i < nStamps) {
    float4 g = lp.stampGeo[i];
    StampRect r = stampRect(g.x, g.y, g.w);
    if (r.x0 < r.x1 && r.y0 < r.y1) {
      long long w = (long long) min(r.x1, lp.fw) - max(r.x0, 0), h = (long long) min(r.y1, lp.fh) - max(r.y0, 0);
      cnt = w > 0 && h > 0 ? w * h : 0;
    }
    lp.fragCount[i] = (int) min(cnt, (long long) 0x7fffffff);
  }
  addTotal(&lp.totals[1], cnt);
}

__global__ void __launch_bounds__(256) k_lp_frag_emit(const __grid_constant__ LineParams lp, int nStamps,
                                                      uint32_t *keys, int *vals) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nStamps || lp.fragCount[i] == 0) return;
  float4 g = lp.stampGeo[i];
  StampRect r = stampRect(g.x, g.y, g.w);
  int o = lp.fragOff[i];
  for (int x = max(r.x0, 0); x < min(r.x1, lp.fw); x++)
    for (int y = max(r.y0, 0); y < min(r.y1, lp.fh); y++, o++) {
      keys[o] = (uint32_t) y * (uint32_t) lp.fw + (uint32_t) x;
      vals[o] = i;
    }
}

// one thread per pixel run of the pixel-sorted fragments
template<int S, bool HAS_DEPTH>
__global__ void __launch_bounds__(256) k_lp_frag_apply(const __grid_constant__ DrawParams p,
                                                       const __grid_constant__ LineParams lp, const uint32_t *keys,
                                                       const int *vals, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t key = keys[i];
  if (i > 0 && keys[i - 1] == key) return;
  const int x = (int) (key % (uint32_t) lp.fw), y = (int) (key / (uint32_t) lp.fw);
  const bool inC = x < p.cw && y < p.ch;
  const bool inD = HAS_DEPTH && x < p.dw && y < p.dh;
  uint32_t col[S];
  float dep[S];
  const size_t pc = (size_t) y * p.cw + x, pd = (size_t) y * p.dw + x;
  for (int s = 0; s < S; s++) {
    col[s] = inC ? p.color[pc * S + s] : 0u;
    dep[s] = inD ? p.depth[pd * S + s] : 0.f;
  }
  for (int j = i; j < n && keys[j] == key; j++) {
    const int st = vals[j];
    const float z = lp.stampGeo[st].z;
    const float4 color = lp.stampColor[st];
    for (int s = 0; s < S; s++) perSample<true, HAS_DEPTH>(p, inC, inD, col[s], dep[s], z, color);
  }
  for (int s = 0; s < S; s++) {
    if (inC) p.color[pc * S + s] = col[s];
    if (inD) p.depth[pd * S + s] = dep[s];
  }
}

// multiSampleResolve (RendererSoft.cpp:880-912): mean of the four u8 samples, truncated
__global__ void __launch_bounds__(256) k_lp_resolve(const uint4 *color, uint32_t *resolved, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint4 c = color[i];
  uint32_t r = 0;
#pragma unroll
  for (int ch = 0; ch < 4; ch++) {
    uint32_t sum = ((c.x >> (8 * ch)) & 255u) + ((c.y >> (8 * ch)) & 255u) + ((c.z >> (8 * ch)) & 255u) +
                   ((c.w >> (8 * ch)) & 255u);
    r |= ((sum >> 2) & 255u) << (8 * ch);
  }
  resolved[i] = r;
}

}  // namespace

void launchPointKeys(const LineParams &lp, uint32_t *keys, int *vals, int n, cudaStream_t st) {
  if (n > 0) k_lp_point_keys<<<cdiv(n, 256), 256, 0, st>>>(lp, keys, vals, n);
}

void launchPointChain(const DrawParams &p, const LineParams &lp, const uint32_t *keys, const int *vals, int n,
                      cudaStream_t st) {
  if (n > 0) k_lp_point_chain<<<cdiv(n, 256), 256, 0, st>>>(p, lp, keys, vals, n);
}

void launchStampCount(const DrawParams &p, const LineParams &lp, cudaStream_t st) {
  if (lp.nIn > 0) k_lp_stamp_count<<<cdiv(3 * lp.nIn, 256), 256, 0, st>>>(p, lp);
}

void launchStampEmit(const DrawParams &p, const LineParams &lp, cudaStream_t st) {
  if (lp.nIn > 0) k_lp_stamp_emit<<<cdiv(3 * lp.nIn, 256), 256, 0, st>>>(p, lp);
}

void launchFragCount(const LineParams &lp, int nStamps, cudaStream_t st) {
  if (nStamps > 0) k_lp_frag_count<<<cdiv(nStamps, 256), 256, 0, st>>>(lp, nStamps);
}

void launchFragEmit(const LineParams &lp, int nStamps, uint32_t *keys, int *vals, cudaStream_t st) {
  if (nStamps > 0) k_lp_frag_emit<<<cdiv(nStamps, 256), 256, 0, st>>>(lp, nStamps, keys, vals);
}

void launchFragApply(const DrawParams &p, const LineParams &lp, const uint32_t *keys, const int *vals, int n,
                     bool hasDepth, cudaStream_t st) {
  if (n <= 0) return;
  int grid = cdiv(n, 256);
  if (p.samples == 4) {
    if (hasDepth) k_lp_frag_apply<4, true><<<grid, 256, 0, st>>>(p, lp, keys, vals, n);
    else k_lp_frag_apply<4, false><<<grid, 256, 0, st>>>(p, lp, keys, vals, n);
  } else {
    if (hasDepth) k_lp_frag_apply<1, true><<<grid, 256, 0, st>>>(p, lp, keys, vals, n);
    else k_lp_frag_apply<1, false><<<grid, 256, 0, st>>>(p, lp, keys, vals, n);
  }
}

void launchResolve(const DrawParams &p, cudaStream_t st) {
  int n = p.cw * p.ch;
  if (n > 0 && p.samples == 4 && p.resolved)
    k_lp_resolve<<<cdiv(n, 256), 256, 0, st>>>(reinterpret_cast<const uint4 *>(p.color), p.resolved, n);
}

}  // namespace sglc
