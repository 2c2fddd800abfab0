// Raster variant with the neural IBL shader fused into the fragment stage (PBR programs with a
// bound network, sglc_program_set_neural_shader).
//
// Coverage, depth and the per-pixel order of colour operations are exactly those of k_raster
// (same pass 1 / pass 2 code, same fragment queues, same phase C). What changes is phase B: the
// CTA's 8 warps shade their queued fragments together, 32 per warp per chunk, so that each
// warpgroup (4 warps = 128 fragments) forms one M = 128 tile for the tensor cores:
//   1. every lane evaluates the surface terms of its fragment (material texels, normal map, direct
//      light, emissive: pbrSurface) and encodes the network inputs into its warpgroup's tile;
//   2. thread 0 issues the MMA chains of both warpgroups (layer 1 in two K halves of 80 features,
//      so the input tile is 20 KB; then layers 2 and 3 on the hidden tiles written back into the
//      same buffer by the epilogues), accumulators in TMEM (128 columns per warpgroup);
//   3. each lane reads its own TMEM lane back (tcgen05.ld), squares the output into the IBL term
//      and finishes the colour (ambient occlusion, gamma, emissive).
// Because the warps of a CTA must meet for every chunk, pass 2 runs in CTA-wide steps here: one
// candidate per lane per step, with a CTA-wide vote before each step on whether any queue must be
// flushed first.
#include "sglc_raster.cuh"
#include "sglc_host_util.h"
#include "sglc_nn.cuh"

namespace sglc {

using namespace nn;

constexpr int kQueueN = 96;

struct FragQueueN {
  int tri[kQueueN];
  uint32_t meta[kQueueN];
  float b0[kQueueN], b1[kQueueN], b2[kQueueN];
  float4 col[kQueueN];
};

// dynamic shared memory (from a 1024-aligned base)
constexpr int kRnQueues = 0;
constexpr int kRnX = ((8 * (int) sizeof(FragQueueN) + 1023) / 1024) * 1024;   // 2 x [128][80] BF16
constexpr int kRnImg = kRnX + 2 * 128 * 80 * 2;
constexpr int kRnBar = kRnImg + kImgBytes;
constexpr int kRnTmem = kRnBar + 8;
constexpr int kRnChunks = kRnTmem + 4;
constexpr int kRnBytes = kRnChunks + 4 + 1024;   // + alignment slack
static_assert(kRnBytes * 2 <= 227 * 1024, "two CTAs per SM");

// surface terms and network inputs of one queued fragment
struct NeuralPre {
  float x[kIn];
  float lo0, lo1, lo2, alpha, ao, e0, e1, e2;
};

template<int S>
__device__ __noinline__ NeuralPre neuralPre(const DrawParams &p, const uint8_t *U, int tri, int qx, int qy, int px,
                                            int py, float sb0, float sb1, float sb2) {
  Tri t = loadTri(p.tri + tri);
  const float *r0 = p.vVary + (size_t) t.vid0 * p.varyStride;
  const float *r1 = p.vVary + (size_t) t.vid1 * p.varyStride;
  const float *r2 = p.vVary + (size_t) t.vid2 * p.varyStride;
  FragIn f;
  f.U = U;
  f.v = Vary{r0, r1, r2, sb0, sb1, sb2};
  f.dudx = f.dvdx = f.dudy = f.dvdy = 0.f;
  if (p.needDeriv) {
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
  PbrSurface s = pbrSurface<true>(p, f);
  NeuralPre o;
  o.x[0] = s.N.x; o.x[1] = s.N.y; o.x[2] = s.N.z;
  o.x[3] = s.V.x; o.x[4] = s.V.y; o.x[5] = s.V.z;
  o.x[6] = s.roughness; o.x[7] = s.metallic;
  o.x[8] = s.arg.x; o.x[9] = s.arg.y; o.x[10] = s.arg.z;
  o.x[11] = gmax(dot3(s.N, s.V), 0.0f);
  o.lo0 = s.Lo.x; o.lo1 = s.Lo.y; o.lo2 = s.Lo.z;
  o.alpha = s.arg.w;
  o.ao = s.ao;
  o.e0 = s.emissive.x; o.e1 = s.emissive.y; o.e2 = s.emissive.z;
  return o;
}

struct NeuralCta {
  uint8_t *xTile;       // this warp's warpgroup tile
  uint32_t sX[2];       // both warpgroups' tiles (shared addresses)
  uint32_t sW1, sW2, sW3;
  const float *bias;
  uint64_t *bar;
  uint32_t tmem;        // TMEM base of the CTA
  uint32_t lanes;       // this thread's TMEM lane (+ its warpgroup's column base)
  int *chunks;
  const uint8_t *U;     // uniforms of the CTA's view
  uint32_t phase;
  int row;              // row of this thread in its warpgroup tile
};

__device__ __forceinline__ void ntHandOff() {
  tc::fenceProxyAsync();
  tc::fenceBefore();
  __syncthreads();
}

// bounded wait; a timeout (or the injected one of a test) leaves this chunk's colours unspecified
// and is reported through the draw's device error flag
__device__ __forceinline__ void ntWait(const DrawParams &p, NeuralCta &n) {
  const bool ok = tc::barWait(n.bar, n.phase);
  if ((!ok || p.nnInjectTimeout) && p.errFlags) atomicOr(p.errFlags, kFlagNeuralTimeout);
  n.phase ^= 1u;
  tc::fenceAfter();
}

// Phase B + C for the whole CTA (every thread calls it together).
template<int S, bool HAS_DEPTH>
__device__ __forceinline__ void neuralFlush(const DrawParams &p, NeuralCta &n, FragQueueN &q, int &count,
                                            unsigned long long &mine0, unsigned long long &mine1, int lane, int rx0,
                                            int ry0, bool inC, Samples4 &fb) {
  // CTA-wide number of 32-entry chunks
  __syncthreads();
  if (lane == 0 && count > 0) atomicMax(n.chunks, (count + 31) >> 5);
  __syncthreads();
  const int nch = *n.chunks;
  __syncthreads();
  if (threadIdx.x == 0) *n.chunks = 0;
  for (int ch = 0; ch < nch; ch++) {
    const int e = ch * 32 + lane;
    const bool valid = e < count;
    NeuralPre pre;
    if (valid) {
      uint32_t m = q.meta[e];
      int l = m & 31;
      int px = rx0 + (l & 7), py = ry0 + (l >> 3);
      int qx = px - ((m >> 9) & 1), qy = py - ((m >> 10) & 1);
      pre = neuralPre<S>(p, n.U, q.tri[e], qx, qy, px, py, q.b0[e], q.b1[e], q.b2[e]);
    } else {
#pragma unroll
      for (int i = 0; i < kIn; i++) pre.x[i] = 0.f;
      pre.lo0 = pre.lo1 = pre.lo2 = pre.alpha = pre.ao = pre.e0 = pre.e1 = pre.e2 = 0.f;
    }
    // layer 1, features 0-79
    encodeChunks<0, 10, true>(pre.x, n.xTile, n.row, 80, false);
    ntHandOff();
    if (threadIdx.x == 0) {
      tc::fenceAfter();
      for (int w = 0; w < 2; w++) issueKMajor(n.tmem + 128 * w, n.sX[w], 80, 0, n.sW1, kK1, 0, 64, 80, false);
      tc::commit(n.bar);
    }
    ntWait(p, n);
    // layer 1, features 80-159 (the tile is free again)
    encodeChunks<10, 20, true>(pre.x, n.xTile, n.row, 80, false);
    ntHandOff();
    if (threadIdx.x == 0) {
      tc::fenceAfter();
      for (int w = 0; w < 2; w++) issueKMajor(n.tmem + 128 * w, n.sX[w], 80, 0, n.sW1, kK1, 80, 64, 80, true);
      tc::commit(n.bar);
    }
    ntWait(p, n);
    hiddenEpilogue(n.lanes, n.bias, n.xTile, n.row, 64, 0);
    ntHandOff();
    if (threadIdx.x == 0) {
      tc::fenceAfter();
      for (int w = 0; w < 2; w++) issueKMajor(n.tmem + 128 * w + 64, n.sX[w], 64, 0, n.sW2, 64, 0, 64, 64, false);
      tc::commit(n.bar);
    }
    ntWait(p, n);
    hiddenEpilogue(n.lanes + 64, n.bias + 64, n.xTile, n.row, 64, 0);
    ntHandOff();
    if (threadIdx.x == 0) {
      tc::fenceAfter();
      for (int w = 0; w < 2; w++) issueKMajor(n.tmem + 128 * w, n.sX[w], 64, 0, n.sW3, 64, 0, 16, 64, false);
      tc::commit(n.bar);
    }
    ntWait(p, n);
    float y[16];
    tc::ld16(n.lanes, y);
    tc::ldWait();
    tc::fenceBefore();
    if (valid) {
      float a0 = gmax(y[0] + n.bias[128], 0.f), a1 = gmax(y[1] + n.bias[129], 0.f), a2 = gmax(y[2] + n.bias[130], 0.f);
      f3 ambient = mk3(a0 * a0, a1 * a1, a2 * a2) * pre.ao;
      q.col[e] = pbrFinish(p, ambient, mk3(pre.lo0, pre.lo1, pre.lo2), mk3(pre.e0, pre.e1, pre.e2), pre.alpha);
    }
  }
  __syncwarp();
  if (p.fragCounter && lane == 0) atomicAdd(p.fragCounter, (unsigned long long) count);
  // phase C: each pixel's own fragments in queue (= primitive) order
  for (int half = 0; half < 2; half++) {
    unsigned long long mine = half ? mine1 : mine0;
    while (mine) {
      int e = __ffsll(mine) - 1 + 64 * half;
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
  }
  __syncwarp();
  count = 0;
  mine0 = mine1 = 0ull;
}

template<int S, bool HAS_DEPTH>
__global__ void __launch_bounds__(256, 2) k_raster_neural(const __grid_constant__ DrawParams p) {
  extern __shared__ __align__(1024) uint8_t smraw[];
  uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t) 1023);
  FragQueueN *queues = reinterpret_cast<FragQueueN *>(sm + kRnQueues);
  const int tile = p.tileOrder ? p.tileOrder[blockIdx.x] : blockIdx.x;
  const TileFrame fr = tileFrame(p, tile);
  const int view = fr.view;
  uint32_t *colorBuf = fr.color;
  uint32_t *resolvedBuf = fr.resolved;
  float *depthBuf = fr.depth;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rx0 = fr.tx * 16 + (warp & 1) * 8, ry0 = fr.ty * 16 + (warp >> 1) * 4;
  const int px = rx0 + (lane & 7), py = ry0 + (lane >> 3);
  const bool inC = px < fr.cW && py < fr.cH;
  const bool inD = HAS_DEPTH && px < fr.dW && py < fr.dH;
  FragQueueN &q = queues[warp];

  NeuralCta n;
  n.xTile = sm + kRnX + (warp >> 2) * 128 * 80 * 2;
  n.sX[0] = tc::smemAddr(sm + kRnX);
  n.sX[1] = tc::smemAddr(sm + kRnX + 128 * 80 * 2);
  uint8_t *img = sm + kRnImg;
  n.sW1 = tc::smemAddr(img + kImgW1);
  n.sW2 = tc::smemAddr(img + kImgW2);
  n.sW3 = tc::smemAddr(img + kImgW3);
  n.bias = reinterpret_cast<const float *>(img + kImgBias);
  n.bar = reinterpret_cast<uint64_t *>(sm + kRnBar);
  n.chunks = reinterpret_cast<int *>(sm + kRnChunks);
  n.phase = 0;
  n.U = viewUniforms(p, view);
  n.row = (warp & 3) * 32 + lane;
  uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(sm + kRnTmem);
  for (int i = threadIdx.x; i < kImgBytes / 16; i += 256)
    reinterpret_cast<uint4 *>(img)[i] = __ldg(reinterpret_cast<const uint4 *>(p.nnImage) + i);
  if (threadIdx.x == 0) {
    tc::barInit(n.bar, 1);
    *n.chunks = 0;
  }
  if (warp == 0) tc::tmemAlloc(tmemSlot, 256);
  tc::fenceBefore();
  __syncthreads();
  tc::fenceAfter();
  n.tmem = *tmemSlot;
  n.lanes = n.tmem + ((uint32_t) ((warp & 3) * 32) << 16) + 128u * (uint32_t) (warp >> 2);

  int count = 0;
  unsigned long long mine0 = 0ull, mine1 = 0ull;   // queue entries 0-63 / 64-95 of this lane's pixel
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
  const float lo = S == 4 ? 0.125f : 0.5f, hi = S == 4 ? 0.875f : 0.5f;
  const float vpExtent = fabsf(fr.vpW) + fabsf(fr.vpH) + 2.f * (float) (rx0 + ry0) + 64.f;
  for (int base = start; base < end; base += 32) {
    int prim;
    unsigned cand = pass1Candidates<S>(p, base, end, lane, rx0, ry0, lo, hi, vpExtent, prim);
    if (!(inC || inD)) cand = 0;
    // pass 2 in CTA-wide steps: one candidate per lane per step (up to 2 quads = 64 queue entries)
    while (__syncthreads_or(cand != 0u)) {
      if (__syncthreads_or(count > kQueueN - 64))
        neuralFlush<S, HAS_DEPTH>(p, n, q, count, mine0, mine1, lane, rx0, ry0, inC, fb);
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
      for (int k = 0; k < nqMax; k++) {
        uint32_t mask = 0;
        int qx = 0, qy = 0;
        if (k < nq) {
          qy = (k / nx) ? y1 : y0;
          qx = (k % nx) ? x1 : x0;
          mask = depthOps<S, HAS_DEPTH>(p, cv, inD, fb);
        }
        unsigned want = __ballot_sync(0xffffffffu, mask != 0);
        if (mask) {
          int e = count + __popc(want & lt);
          q.tri[e] = pr;
          q.meta[e] = (uint32_t) lane | (mask << 5) | ((uint32_t) (px - qx) << 9) | ((uint32_t) (py - qy) << 10);
          q.b0[e] = cv.b0;
          q.b1[e] = cv.b1;
          q.b2[e] = cv.b2;
          if (e < 64) mine0 |= 1ull << e;
          else mine1 |= 1ull << (e - 64);
        }
        count += __popc(want);
      }
    }
  }
  if (__syncthreads_or(count > 0)) neuralFlush<S, HAS_DEPTH>(p, n, q, count, mine0, mine1, lane, rx0, ry0, inC, fb);
  if (inC) {
    size_t pix = (size_t) py * fr.cW + px;
    if (S == 4) {
      *reinterpret_cast<uint4 *>(colorBuf + pix * 4) = make_uint4(fb.c0, fb.c1, fb.c2, fb.c3);
      uint32_t rsv = 0;
#pragma unroll
      for (int c = 0; c < 4; c++) {
        uint32_t sum = ((fb.c0 >> (8 * c)) & 255u) + ((fb.c1 >> (8 * c)) & 255u) + ((fb.c2 >> (8 * c)) & 255u) +
                       ((fb.c3 >> (8 * c)) & 255u);
        rsv |= ((sum >> 2) & 255u) << (8 * c);
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
  tc::fenceBefore();
  __syncthreads();
  tc::fenceAfter();
  if (warp == 0) tc::tmemFree(n.tmem, 256);
}

// A failed attribute set makes the launch after it fail; the draw reports that launch error.
template<int S, bool D>
static void launchNeural(const DrawParams &p, int grid, cudaStream_t st) {
  static PerDeviceAttr attr;
  setDynamicSmemOnce(attr, k_raster_neural<S, D>, kRnBytes);
  k_raster_neural<S, D><<<grid, 256, kRnBytes, st>>>(p);
}

void launchRasterNeural(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st) {
  int grid = p.numTiles;
  (void) hasColor;   // the neural shader writes colour; depth-only draws never select it
  if (p.samples == 4) {
    if (hasDepth) launchNeural<4, true>(p, grid, st);
    else launchNeural<4, false>(p, grid, st);
  } else {
    if (hasDepth) launchNeural<1, true>(p, grid, st);
    else launchNeural<1, false>(p, grid, st);
  }
}

}  // namespace sglc
