// Training and evaluation of the neural IBL shader (sglc_nn.cuh) on the tensor cores.
//
// k_nn_tile runs the network over 128-row tiles of fragment records, one warpgroup per CTA (thread
// t owns row t and TMEM lane t), persistent over tiles. Every layer is a chain of
// tcgen05.mma.kind::f16 (BF16 operands in shared memory, FP32 accumulators in TMEM) issued by thread
// 0 and completed through one mbarrier; the other threads run the encoding and the epilogues
// (tcgen05.ld, bias, ReLU, BF16). In training mode the backward pass follows on the same tile:
//   dY  = 2 (y - t) / B                                   (epilogue of layer 3)
//   dH2 = (dY W3) * relu'(H2)      MMA, W3 read MN-major  (K = 16)
//   dH1 = (dH2 W2) * relu'(H1)     MMA, W2 read MN-major  (K = 64)
//   dW1^T  += X^T dH1              MMA, X and dH1 read MN-major, two M = 128 halves (features 0-127, 32-159)
//   [dW2^T | dW3^T] += [H1 | H2]^T [dH2 | dY]   one MMA chain, diagonal blocks used
//   [db2 | db3] += 1^T [dH2 | dY]  MMA with an all-ones A operand; db1 = row 156 of dW1^T
// The weight-gradient accumulators stay in TMEM across the CTA's tiles and are written once per
// launch as a per-CTA partial, summed in a fixed order by k_nn_adam / k_nn_sum: gradients are
// deterministic run to run.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "softgl_cuda.h"
#include "sglc_nn.cuh"
#include "sglc_host_util.h"
#include "sglc_nn_host.h"

namespace sglc {
namespace nn {

// shared memory of k_nn_tile (bytes from a 1024-aligned base)
constexpr int kSmX = 0;                       // [128][160] encoded inputs
constexpr int kSmHH = kSmX + 128 * kK1 * 2;   // [128][128] H1 | H2
constexpr int kSmD2 = kSmHH + 128 * 128 * 2;  // [128][80]  dH2 | dY
constexpr int kSmDH1 = kSmD2 + 128 * 80 * 2;  // [128][64]  dH1
constexpr int kSmImg = kSmDH1 + 128 * 64 * 2; // weight image
constexpr int kSmOnes = kSmImg + kImgBytes;   // one 8x8 core matrix of ones
constexpr int kSmRed = kSmOnes + 128;         // 4 floats: per-warp loss
constexpr int kSmBar = kSmRed + 16;           // mbarrier
constexpr int kSmTmem = kSmBar + 8;           // TMEM base address
// Every descriptor's reach stays below this size under either reading of the LBO/SBO fields.
constexpr int kSmBytes = 153600;
static_assert(kSmTmem + 4 <= kSmBytes, "shared memory layout");
static_assert(kSmImg + kImgW3 + 7 * 1024 + 2 * 128 <= kSmBytes, "MN-major W3 reach");

// TMEM columns
constexpr uint32_t kTm1 = 0, kTm2 = 64, kTm3 = 128, kTmBias = 144, kTmW1a = 256, kTmW1b = 320, kTmW23 = 384;
constexpr uint32_t kTmCols = 512;

enum { MODE_INFER = 0, MODE_GRAD = 1, MODE_TRAIN = 2 };

// Descriptor of an MN-major SWIZZLE_NONE operand: the leading byte offset is the stride between
// 8-row groups along K, the stride byte offset the stride between 8-element core matrices along M
// (or N) (the canonical MN-major layout ((8,1,m),(8,k)) : ((1,8,SBO),(8,LBO)) in elements).
__device__ __forceinline__ uint64_t mnDesc(uint32_t addr, uint32_t mnStride, uint32_t kStride) {
  return tc::smemDesc(addr, kStride, mnStride);
}

struct TileArgs {
  const float *records;
  long long nRecords;
  long long first;
  long long rows;          // rows of this launch (batch size or evaluated records)
  int mode;
  int step;
  unsigned long long seed;
  const uint8_t *image;
  float *partials;         // [gridDim.x][kPartialStride]
  float *out;              // MODE_INFER: 3 floats per row
  float invBatch;
  int *error;
};

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ __forceinline__ long long recordIndex(const TileArgs &a, long long g) {
  if (a.mode == MODE_TRAIN)
    return (long long) (mix64(a.seed ^ ((unsigned long long) (unsigned) a.step << 32) ^ (unsigned long long) g) %
                        (unsigned long long) a.nRecords);
  return a.first + g;
}

__global__ void __launch_bounds__(128, 1) k_nn_tile(const TileArgs a) {
  extern __shared__ __align__(1024) uint8_t smraw[];
  uint8_t *sm = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smraw) + 1023) & ~(uintptr_t) 1023);
  uint8_t *X = sm + kSmX, *HH = sm + kSmHH, *D2 = sm + kSmD2, *DH1 = sm + kSmDH1, *IMG = sm + kSmImg;
  const float *bias = reinterpret_cast<const float *>(IMG + kImgBias);
  float *red = reinterpret_cast<float *>(sm + kSmRed);
  uint64_t *bar = reinterpret_cast<uint64_t *>(sm + kSmBar);
  uint32_t *tmemSlot = reinterpret_cast<uint32_t *>(sm + kSmTmem);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const bool train = a.mode != MODE_INFER;

  // weight image and the ones core matrix
  for (int i = t; i < kImgBytes / 16; i += 128)
    reinterpret_cast<uint4 *>(IMG)[i] = __ldg(reinterpret_cast<const uint4 *>(a.image) + i);
  if (t < 8) reinterpret_cast<uint4 *>(sm + kSmOnes)[t] = make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
  if (t == 0) tc::barInit(bar, 1);
  if (warp == 0) tc::tmemAlloc(tmemSlot, kTmCols);
  tc::fenceBefore();
  __syncthreads();
  tc::fenceAfter();
  const uint32_t tmem = *tmemSlot;
  const uint32_t lanes = tmem + ((uint32_t) (warp * 32) << 16);
  const uint32_t sX = tc::smemAddr(X), sHH = tc::smemAddr(HH), sD2 = tc::smemAddr(D2), sDH1 = tc::smemAddr(DH1);
  const uint32_t sW1 = tc::smemAddr(IMG + kImgW1), sW2 = tc::smemAddr(IMG + kImgW2), sW3 = tc::smemAddr(IMG + kImgW3);
  const uint32_t sOnes = tc::smemAddr(sm + kSmOnes);
  uint32_t phase = 0;
  bool ok = true;
  float lossAcc = 0.f;
  bool firstTile = true;
  const long long nTiles = (a.rows + 127) / 128;

  auto waitMma = [&]() {
    if (!tc::barWait(bar, phase)) {
      ok = false;
      if (a.error) atomicExch(a.error, 1);
    }
    phase ^= 1u;
    tc::fenceAfter();
  };
  auto handOff = [&]() {   // operand writes -> MMA issue
    tc::fenceProxyAsync();
    tc::fenceBefore();
    __syncthreads();
  };

  for (long long tile = blockIdx.x; tile < nTiles; tile += gridDim.x) {
    const long long g = tile * 128 + t;
    const bool valid = g < a.rows;
    float x[kIn], tgt[3] = {0.f, 0.f, 0.f};
    if (valid) {
      const float4 *rp = reinterpret_cast<const float4 *>(a.records + (size_t) recordIndex(a, g) * kRecordFloats);
      float4 r0 = __ldg(rp), r1 = __ldg(rp + 1), r2 = __ldg(rp + 2), r3 = __ldg(rp + 3);
      x[0] = r0.x; x[1] = r0.y; x[2] = r0.z; x[3] = r0.w;
      x[4] = r1.x; x[5] = r1.y; x[6] = r1.z; x[7] = r1.w;
      x[8] = r2.x; x[9] = r2.y; x[10] = r2.z; x[11] = r2.w;
      tgt[0] = r3.x; tgt[1] = r3.y; tgt[2] = r3.z;
    } else {
#pragma unroll
      for (int i = 0; i < kIn; i++) x[i] = 0.f;
    }
    encodeRow(x, X, t, train);
    handOff();
    // ---- layer 1: [128 x 160] x [160 x 64]
    if (t == 0) {
      tc::fenceAfter();
      issueKMajor(tmem + kTm1, sX, kK1, 0, sW1, kK1, 0, 64, kK1, false);
      tc::commit(bar);
    }
    waitMma();
    unsigned long long m1 = hiddenEpilogue(lanes + kTm1, bias, HH, t, 128, 0);
    handOff();
    // ---- layer 2
    if (t == 0) {
      tc::fenceAfter();
      issueKMajor(tmem + kTm2, sHH, 128, 0, sW2, 64, 0, 64, 64, false);
      tc::commit(bar);
    }
    waitMma();
    unsigned long long m2 = hiddenEpilogue(lanes + kTm2, bias + 64, HH, t, 128, 64);
    handOff();
    // ---- layer 3 (N = 16, outputs 0-2 used)
    if (t == 0) {
      tc::fenceAfter();
      issueKMajor(tmem + kTm3, sHH, 128, 64, sW3, 64, 0, 16, 64, false);
      tc::commit(bar);
    }
    waitMma();
    float y[16];
    tc::ld16(lanes + kTm3, y);
    tc::ldWait();
#pragma unroll
    for (int c = 0; c < 3; c++) y[c] += bias[128 + c];
    if (!train) {
      if (valid) {
        float *o = a.out + (size_t) g * 3;
        o[0] = y[0]; o[1] = y[1]; o[2] = y[2];
      }
      tc::fenceBefore();
      if (!__syncthreads_and(ok)) break;   // X / HH are rewritten by the next tile
      continue;
    }
    // ---- loss and dY (BF16 into D2 columns 64-79)
    float dy[3];
#pragma unroll
    for (int c = 0; c < 3; c++) {
      float e = valid ? y[c] - tgt[c] : 0.f;
      lossAcc += e * e;
      dy[c] = 2.0f * e * a.invBatch;
    }
    *reinterpret_cast<uint4 *>(D2 + tc::tileOffset(t, 64, 80)) =
        make_uint4(tc::packBf16(dy[0], dy[1]), tc::packBf16(dy[2], 0.f), 0u, 0u);
    *reinterpret_cast<uint4 *>(D2 + tc::tileOffset(t, 72, 80)) = make_uint4(0u, 0u, 0u, 0u);
    handOff();
    // ---- dH2 = dY W3: A = dY [128 x 16] K-major, B = W3 tile [16 out][64 hid] read MN-major (N = hid)
    if (t == 0) {
      tc::fenceAfter();
      tc::mma(tmem + kTm2, tc::smemDesc(sD2 + tc::tileOffset(0, 64, 80), 128, 10 * 128),
              mnDesc(sW3, 128, 8 * 128), tc::instrDesc(128, 64, false, true), false);
      tc::commit(bar);
    }
    waitMma();
#pragma unroll
    for (int h = 0; h < 4; h++) {
      float v[16];
      tc::ld16(lanes + kTm2 + 16 * h, v);
      tc::ldWait();
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = ((m2 >> (16 * h + j)) & 1ull) ? v[j] : 0.f;
#pragma unroll
      for (int q = 0; q < 2; q++)
        *reinterpret_cast<uint4 *>(D2 + tc::tileOffset(t, 16 * h + 8 * q, 80)) =
            make_uint4(tc::packBf16(v[8 * q], v[8 * q + 1]), tc::packBf16(v[8 * q + 2], v[8 * q + 3]),
                       tc::packBf16(v[8 * q + 4], v[8 * q + 5]), tc::packBf16(v[8 * q + 6], v[8 * q + 7]));
    }
    handOff();
    // ---- dH1 = dH2 W2: A = dH2 (D2 columns 0-63) K-major, B = W2 tile [64 out][64 in] read MN-major
    if (t == 0) {
      tc::fenceAfter();
      const uint32_t idesc = tc::instrDesc(128, 64, false, true);
      for (int k = 0; k < 64; k += 16)
        tc::mma(tmem + kTm1, tc::smemDesc(sD2 + tc::tileOffset(0, k, 80), 128, 10 * 128),
                mnDesc(sW2 + tc::tileOffset(k, 0, 64), 128, 8 * 128), idesc, k > 0);
      tc::commit(bar);
    }
    waitMma();
#pragma unroll
    for (int h = 0; h < 4; h++) {
      float v[16];
      tc::ld16(lanes + kTm1 + 16 * h, v);
      tc::ldWait();
#pragma unroll
      for (int j = 0; j < 16; j++) v[j] = ((m1 >> (16 * h + j)) & 1ull) ? v[j] : 0.f;
#pragma unroll
      for (int q = 0; q < 2; q++)
        *reinterpret_cast<uint4 *>(DH1 + tc::tileOffset(t, 16 * h + 8 * q, 64)) =
            make_uint4(tc::packBf16(v[8 * q], v[8 * q + 1]), tc::packBf16(v[8 * q + 2], v[8 * q + 3]),
                       tc::packBf16(v[8 * q + 4], v[8 * q + 5]), tc::packBf16(v[8 * q + 6], v[8 * q + 7]));
    }
    handOff();
    // ---- weight gradients, accumulated in TMEM over the CTA's tiles (K = the tile's 128 rows)
    if (t == 0) {
      tc::fenceAfter();
      const uint32_t iW1 = tc::instrDesc(128, 64, true, true);
      const uint32_t iW23 = tc::instrDesc(128, 80, true, true);
      const uint32_t iB = tc::instrDesc(128, 80, false, true);
      for (int k = 0; k < 128; k += 16) {
        bool acc = !firstTile || k > 0;
        uint64_t bDH1 = mnDesc(sDH1 + tc::tileOffset(k, 0, 64), 128, 8 * 128);
        uint64_t bD2 = mnDesc(sD2 + tc::tileOffset(k, 0, 80), 128, 10 * 128);
        tc::mma(tmem + kTmW1a, mnDesc(sX + tc::tileOffset(k, 0, kK1), 128, 20 * 128), bDH1, iW1, acc);
        tc::mma(tmem + kTmW1b, mnDesc(sX + tc::tileOffset(k, 32, kK1), 128, 20 * 128), bDH1, iW1, acc);
        tc::mma(tmem + kTmW23, mnDesc(sHH + tc::tileOffset(k, 0, 128), 128, 16 * 128), bD2, iW23, acc);
        tc::mma(tmem + kTmBias, tc::smemDesc(sOnes, 0, 0), bD2, iB, acc);
      }
      tc::commit(bar);
    }
    waitMma();   // the next tile overwrites X, HH, D2 and DH1
    tc::fenceBefore();
    firstTile = false;
    if (!__syncthreads_and(ok)) break;   // a timed-out wait ends the launch on every thread
  }

  if (train) {
    float *part = a.partials + (size_t) blockIdx.x * kPartialStride;
    if (firstTile) {   // no tile: zero partial
      for (int i = t; i < kPartialStride; i += 128) part[i] = 0.f;
    } else {
      float v[16];
      for (int h = 0; h < 4; h++) {   // dW1^T rows 0-127 (features), columns = outputs
        tc::ld16(lanes + kTmW1a + 16 * h, v);
        tc::ldWait();
        for (int j = 0; j < 16; j++) part[kW1 + (16 * h + j) * kFeat + t] = v[j];
      }
      const int f = 32 + t;
      for (int h = 0; h < 4; h++) {   // features 32-159: keep 128-155, row 156 = db1
        tc::ld16(lanes + kTmW1b + 16 * h, v);
        tc::ldWait();
        for (int j = 0; j < 16; j++) {
          if (f >= 128 && f < kFeat) part[kW1 + (16 * h + j) * kFeat + f] = v[j];
          if (f == kOneFeature) part[kB1 + 16 * h + j] = v[j];
        }
      }
      for (int h = 0; h < 5; h++) {   // [dW2^T | dW3^T]
        tc::ld16(lanes + kTmW23 + 16 * h, v);
        tc::ldWait();
        for (int j = 0; j < 16; j++) {
          int col = 16 * h + j;
          if (t < 64 && col < 64) part[kW2 + col * 64 + t] = v[j];
          if (t >= 64 && col >= 64 && col < 67) part[kW3 + (col - 64) * 64 + (t - 64)] = v[j];
        }
      }
      for (int h = 0; h < 5; h++) {   // [db2 | db3]: every lane holds the same row
        tc::ld16(lanes + kTmBias + 16 * h, v);
        tc::ldWait();
        if (t == 0)
          for (int j = 0; j < 16; j++) {
            int col = 16 * h + j;
            if (col < 64) part[kB2 + col] = v[j];
            else if (col < 67) part[kB3 + col - 64] = v[j];
          }
      }
      float l = lossAcc;
      for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
      if (lane == 0) red[warp] = l;
      __syncthreads();
      if (t == 0) part[kParams] = ((red[0] + red[1]) + (red[2] + red[3])) * a.invBatch;
    }
  }
  tc::fenceBefore();
  __syncthreads();
  tc::fenceAfter();
  if (warp == 0) tc::tmemFree(tmem, kTmCols);
}

// the inference image's copy of parameter i (layout in sglc_nn.cuh); a bias goes in as two BF16
// values whose sum carries 16 significant bits
__device__ __forceinline__ void writeInferImage(uint8_t *img, int i, float w) {
  uint8_t *im = img + kInferOffset;
  auto put = [&](int base, int r, int c, int C, float v) {
    *reinterpret_cast<__nv_bfloat16 *>(im + base + tc::tileOffset(r, c, C)) = __float2bfloat16_rn(v);
  };
  auto putBias = [&](int base, int r, int c, int C) {
    const float hi = __bfloat162float(__float2bfloat16_rn(w));
    put(base, r, c, C, w);
    put(base, r, c + 1, C, w - hi);
  };
  if (i < kB1) put(kIW1, i / kFeat, inferColumn(i % kFeat), kK1, w);
  else if (i < kW2) putBias(kIW1, i - kB1, 158, kK1);
  else if (i < kB2) put(kIW2, (i - kW2) / 64, (i - kW2) % 64, 80, w);
  else if (i < kW3) putBias(kIW2, i - kB2, 64, 80);
  else if (i < kB3) put(kIW3, (i - kW3) / 64, (i - kW3) % 64, 80, w);
  else if (i < kParams) putBias(kIW3, i - kB3, 64, 80);
}

__device__ __forceinline__ void writeImage(uint8_t *img, int i, float w) {
  writeInferImage(img, i, w);
  if (i < kB1) {
    *reinterpret_cast<__nv_bfloat16 *>(img + kImgW1 + tc::tileOffset(i / kFeat, i % kFeat, kK1)) = __float2bfloat16_rn(w);
  } else if (i < kW2) {
    reinterpret_cast<float *>(img + kImgBias)[i - kB1] = w;
  } else if (i < kB2) {
    int j = i - kW2;
    *reinterpret_cast<__nv_bfloat16 *>(img + kImgW2 + tc::tileOffset(j / 64, j % 64, 64)) = __float2bfloat16_rn(w);
  } else if (i < kW3) {
    reinterpret_cast<float *>(img + kImgBias)[64 + i - kB2] = w;
  } else if (i < kB3) {
    int j = i - kW3;
    *reinterpret_cast<__nv_bfloat16 *>(img + kImgW3 + tc::tileOffset(j / 64, j % 64, 64)) = __float2bfloat16_rn(w);
  } else if (i < kParams) {
    reinterpret_cast<float *>(img + kImgBias)[128 + i - kB3] = w;
  }
}

__global__ void k_nn_image(const float *params, uint8_t *img) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kParams) writeImage(img, i, params[i]);
}

// Adam step (Kingma & Ba 2015) on the summed per-CTA gradient partials, then the BF16 image.
__global__ void k_nn_adam(float *params, float *m, float *v, const float *partials, int nParts, float lr, float b1,
                          float b2, float eps, float bc1, float bc2, uint8_t *img, float *lossOut) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < kParams) {
    float g = 0.f;
    for (int q = 0; q < nParts; q++) g += partials[(size_t) q * kPartialStride + i];
    float mi = b1 * m[i] + (1.0f - b1) * g;
    float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    float w = params[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    params[i] = w;
    writeImage(img, i, w);
  } else if (i == kParams && lossOut) {
    float l = 0.f;
    for (int q = 0; q < nParts; q++) l += partials[(size_t) q * kPartialStride + kParams];
    *lossOut = l;
  }
}

__global__ void k_nn_sum(const float *partials, int nParts, float *out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= kParams) {
    float g = 0.f;
    for (int q = 0; q < nParts; q++) g += partials[(size_t) q * kPartialStride + i];
    out[i] = g;
  }
}

}  // namespace nn
}  // namespace sglc

// ------------------------------------------------------------------------------------------------
// host side
// ------------------------------------------------------------------------------------------------
using namespace sglc;
using namespace sglc::nn;

struct sglc_neural {
  sglc_context *ctx = nullptr;
  int device = 0;
  int sms = 0;
  float *params = nullptr, *m = nullptr, *v = nullptr;
  uint8_t *image = nullptr;
  float *records = nullptr;
  long long recCap = 0, nRec = 0;
  unsigned long long *capCount = nullptr;
  long long captureCap = 0;
  int captureStride = 1;
  float *partials = nullptr;
  int partialRows = 0;
  float *scratch = nullptr;   // gradients / loss (kPartialStride floats)
  float *out = nullptr;
  long long outCap = 0;
  int *error = nullptr;
  int step = 0;
};

namespace {

PerDeviceAttr gTileAttr;   // k_nn_tile's dynamic shared-memory limit, per device

sglc_status nnFail(sglc_neural *n, sglc_status s, const std::string &msg) {
  ctxSetError(n ? n->ctx : nullptr, msg.c_str());
  return s;
}

#define NCK(call)                                                                                      \
  do {                                                                                                 \
    cudaError_t e_ = (call);                                                                           \
    if (e_ != cudaSuccess)                                                                             \
      return nnFail(n, e_ == cudaErrorMemoryAllocation ? SGLC_ERR_OUT_OF_MEMORY : SGLC_ERR_DEVICE,     \
                    std::string(#call) + ": " + cudaGetErrorString(e_));                               \
  } while (0)

cudaError_t ensure(float **p, long long *cap, long long need) {
  if (need <= *cap) return cudaSuccess;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc(p, (size_t) need * sizeof(float));
  if (e == cudaSuccess) *cap = need;
  return e;
}

unsigned long long splitmix(unsigned long long &s) {
  unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

sglc_status runTiles(sglc_neural *n, int mode, long long first, long long rows, int step, unsigned long long seed,
                     float invBatch, float *out) {
  NCK(setDynamicSmemOnce(gTileAttr, k_nn_tile, kSmBytes + 1024));
  long long tiles = (rows + 127) / 128;
  int grid = (int) std::min<long long>(tiles, n->sms);
  if (grid <= 0) return SGLC_OK;
  if (mode != MODE_INFER && grid > n->partialRows) {
    if (n->partials) cudaFree(n->partials);
    n->partials = nullptr;
    n->partialRows = 0;
    NCK(cudaMalloc(&n->partials, (size_t) grid * kPartialStride * sizeof(float)));
    n->partialRows = grid;
  }
  TileArgs a;
  a.records = n->records;
  a.nRecords = n->nRec;
  a.first = first;
  a.rows = rows;
  a.mode = mode;
  a.step = step;
  a.seed = seed;
  a.image = n->image;
  a.partials = n->partials;
  a.out = out;
  a.invBatch = invBatch;
  a.error = n->error;
  k_nn_tile<<<grid, 128, kSmBytes + 1024, ctxStream(n->ctx)>>>(a);
  NCK(cudaGetLastError());
  return SGLC_OK;
}

sglc_status checkError(sglc_neural *n) {
  int err = 0;
  NCK(cudaMemcpyAsync(&err, n->error, sizeof(int), cudaMemcpyDeviceToHost, ctxStream(n->ctx)));
  NCK(cudaStreamSynchronize(ctxStream(n->ctx)));
  if (err) return nnFail(n, SGLC_ERR_DEVICE, "neural shader: tensor-core completion wait timed out");
  return SGLC_OK;
}

}  // namespace

extern "C" {

SGLC_API sglc_status sglc_neural_create(sglc_context *ctx, uint64_t seed, sglc_neural **out) {
  if (!ctx || !out) return SGLC_ERR_INVALID_VALUE;
  *out = nullptr;
  sglc_neural *n = new sglc_neural();
  n->ctx = ctx;
  n->device = ctxDevice(ctx);
  DeviceGuard deviceGuard(n->device);
  cudaDeviceGetAttribute(&n->sms, cudaDevAttrMultiProcessorCount, n->device);
  auto fail = [&](cudaError_t e) {
    sglc_neural_destroy(n);
    ctxSetError(ctx, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? SGLC_ERR_OUT_OF_MEMORY : SGLC_ERR_DEVICE;
  };
  cudaError_t e;
  if ((e = cudaMalloc(&n->params, kParams * sizeof(float))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&n->m, kParams * sizeof(float))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&n->v, kParams * sizeof(float))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&n->image, kImageAllocBytes)) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&n->capCount, sizeof(unsigned long long))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&n->scratch, kPartialStride * sizeof(float))) != cudaSuccess) return fail(e);
  if ((e = cudaMalloc(&n->error, sizeof(int))) != cudaSuccess) return fail(e);
  cudaStream_t st = ctxStream(ctx);
  cudaMemsetAsync(n->image, 0, kImageAllocBytes, st);
  cudaMemsetAsync(n->error, 0, sizeof(int), st);
  cudaMemsetAsync(n->capCount, 0, sizeof(unsigned long long), st);
  // He-uniform initialisation from the seed (biases zero)
  std::vector<float> w(kParams, 0.f);
  unsigned long long s = seed;
  auto uni = [&](float bound) { return (float) ((double) (splitmix(s) >> 11) * 0x1.0p-53 * 2.0 - 1.0) * bound; };
  for (int i = kW1; i < kB1; i++) w[i] = uni(std::sqrt(6.0f / kFeat));
  for (int i = kW2; i < kB2; i++) w[i] = uni(std::sqrt(6.0f / kHid));
  for (int i = kW3; i < kB3; i++) w[i] = uni(std::sqrt(6.0f / kHid));
  sglc_status r = sglc_neural_set_params(n, w.data(), kParams);
  if (r != SGLC_OK) {
    sglc_neural_destroy(n);
    return r;
  }
  *out = n;
  return SGLC_OK;
}

SGLC_API sglc_status sglc_neural_destroy(sglc_neural *n) {
  if (!n) return SGLC_ERR_INVALID_VALUE;
  DeviceGuard deviceGuard(n->device);
  if (n->ctx) {
    cudaStreamSynchronize(ctxStream(n->ctx));
    ctxDetachNeural(n->ctx, n);
  }
  for (void *p : {(void *) n->params, (void *) n->m, (void *) n->v, (void *) n->image, (void *) n->records,
                  (void *) n->capCount, (void *) n->partials, (void *) n->scratch, (void *) n->out, (void *) n->error})
    if (p) cudaFree(p);
  delete n;
  return SGLC_OK;
}

SGLC_API int64_t sglc_neural_param_count(void) { return kParams; }

SGLC_API sglc_status sglc_neural_set_params(sglc_neural *n, const float *in, int64_t count) {
  if (!n || !in) return SGLC_ERR_INVALID_VALUE;
  if (count != kParams) return nnFail(n, SGLC_ERR_INVALID_VALUE, "neural shader: parameter count mismatch");
  DeviceGuard deviceGuard(n->device);
  cudaStream_t st = ctxStream(n->ctx);
  NCK(cudaMemcpyAsync(n->params, in, kParams * sizeof(float), cudaMemcpyHostToDevice, st));
  NCK(cudaMemsetAsync(n->m, 0, kParams * sizeof(float), st));
  NCK(cudaMemsetAsync(n->v, 0, kParams * sizeof(float), st));
  k_nn_image<<<(kParams + 255) / 256, 256, 0, st>>>(n->params, n->image);
  NCK(cudaGetLastError());
  NCK(cudaStreamSynchronize(st));
  n->step = 0;
  return SGLC_OK;
}

SGLC_API sglc_status sglc_neural_get_params(sglc_neural *n, float *out, int64_t count) {
  if (!n || !out) return SGLC_ERR_INVALID_VALUE;
  if (count != kParams) return nnFail(n, SGLC_ERR_INVALID_VALUE, "neural shader: parameter count mismatch");
  DeviceGuard deviceGuard(n->device);
  cudaStream_t st = ctxStream(n->ctx);
  NCK(cudaMemcpyAsync(out, n->params, kParams * sizeof(float), cudaMemcpyDeviceToHost, st));
  NCK(cudaStreamSynchronize(st));
  return SGLC_OK;
}

SGLC_API sglc_status sglc_neural_set_records(sglc_neural *n, const float *records, int64_t count) {
  if (!n || (count > 0 && !records) || count < 0) return SGLC_ERR_INVALID_VALUE;
  DeviceGuard deviceGuard(n->device);
  NCK(ensure(&n->records, &n->recCap, count * kRecordFloats));
  cudaStream_t st = ctxStream(n->ctx);
  if (count > 0)
    NCK(cudaMemcpyAsync(n->records, records, (size_t) count * kRecordFloats * sizeof(float), cudaMemcpyHostToDevice,
                        st));
  NCK(cudaStreamSynchronize(st));
  n->recCap = std::max(n->recCap, (long long) count * kRecordFloats);
  n->nRec = count;
  return SGLC_OK;
}

SGLC_API sglc_status sglc_neural_get_records(sglc_neural *n, float *out, int64_t first, int64_t count) {
  if (!n || !out || first < 0 || count < 0) return SGLC_ERR_INVALID_VALUE;
  if (first + count > n->nRec) return nnFail(n, SGLC_ERR_INVALID_VALUE, "neural shader: record range out of bounds");
  DeviceGuard deviceGuard(n->device);
  cudaStream_t st = ctxStream(n->ctx);
  if (count > 0)
    NCK(cudaMemcpyAsync(out, n->records + (size_t) first * kRecordFloats, (size_t) count * kRecordFloats * sizeof(float),
                        cudaMemcpyDeviceToHost, st));
  NCK(cudaStreamSynchronize(st));
  return SGLC_OK;
}

SGLC_API sglc_status sglc_neural_capture(sglc_context *ctx, sglc_neural *n, int64_t capacity, int32_t stride) {
  if (!ctx || !n || capacity < 0 || stride < 1) return SGLC_ERR_INVALID_VALUE;
  DeviceGuard deviceGuard(n->device);
  cudaStream_t st = ctxStream(ctx);
  if (capacity == 0) {
    ctxSetCapture(ctx, nullptr, nullptr, 0, 1);
    return SGLC_OK;
  }
  NCK(ensure(&n->records, &n->recCap, capacity * kRecordFloats));
  NCK(cudaMemsetAsync(n->capCount, 0, sizeof(unsigned long long), st));
  n->captureCap = capacity;
  n->captureStride = stride;
  n->nRec = 0;
  ctxSetCapture(ctx, n->records, n->capCount, capacity, stride);
  return SGLC_OK;
}

SGLC_API sglc_status sglc_neural_record_count(sglc_neural *n, int64_t *count) {
  if (!n || !count) return SGLC_ERR_INVALID_VALUE;
  DeviceGuard deviceGuard(n->device);
  cudaStream_t st = ctxStream(n->ctx);
  if (n->captureCap > 0) {
    unsigned long long c = 0;
    NCK(cudaMemcpyAsync(&c, n->capCount, sizeof(c), cudaMemcpyDeviceToHost, st));
    NCK(cudaStreamSynchronize(st));
    unsigned long long kept = (c + (unsigned long long) n->captureStride - 1) / (unsigned long long) n->captureStride;
    n->nRec = (long long) std::min<unsigned long long>(kept, (unsigned long long) n->captureCap);
  }
  *count = n->nRec;
  return SGLC_OK;
}

SGLC_API sglc_status sglc_neural_train(sglc_neural *n, const sglc_neural_train_params *p, float *loss) {
  if (!n || !p || p->steps < 0 || p->batch <= 0) return SGLC_ERR_INVALID_VALUE;
  if (n->nRec <= 0) return nnFail(n, SGLC_ERR_INVALID_VALUE, "neural shader: no training records");
  DeviceGuard deviceGuard(n->device);
  cudaStream_t st = ctxStream(n->ctx);
  n->captureCap = 0;
  NCK(cudaMemsetAsync(n->error, 0, sizeof(int), st));
  long long tiles = (p->batch + 127) / 128;
  int parts = (int) std::min<long long>(tiles, n->sms);
  for (int s = 0; s < p->steps; s++) {
    sglc_status r = runTiles(n, MODE_TRAIN, 0, p->batch, n->step, p->seed, 1.0f / (float) p->batch, nullptr);
    if (r != SGLC_OK) return r;
    n->step++;
    float bc1 = (float) (1.0 - std::pow((double) p->beta1, n->step));
    float bc2 = (float) (1.0 - std::pow((double) p->beta2, n->step));
    k_nn_adam<<<(kParams + 256) / 256, 256, 0, st>>>(n->params, n->m, n->v, n->partials, parts, p->lr, p->beta1,
                                                      p->beta2, p->eps, bc1, bc2, n->image, n->scratch + kParams);
    NCK(cudaGetLastError());
  }
  sglc_status r = checkError(n);
  if (r != SGLC_OK) return r;
  if (loss) {
    NCK(cudaMemcpyAsync(loss, n->scratch + kParams, sizeof(float), cudaMemcpyDeviceToHost, st));
    NCK(cudaStreamSynchronize(st));
  }
  return SGLC_OK;
}

SGLC_API sglc_status sglc_neural_gradients(sglc_neural *n, int64_t first, int64_t count, float *grads, float *loss) {
  if (!n || !grads || first < 0 || count <= 0) return SGLC_ERR_INVALID_VALUE;
  if (first + count > n->nRec) return nnFail(n, SGLC_ERR_INVALID_VALUE, "neural shader: record range out of bounds");
  DeviceGuard deviceGuard(n->device);
  cudaStream_t st = ctxStream(n->ctx);
  NCK(cudaMemsetAsync(n->error, 0, sizeof(int), st));
  sglc_status r = runTiles(n, MODE_GRAD, first, count, 0, 0, 1.0f / (float) count, nullptr);
  if (r != SGLC_OK) return r;
  int parts = (int) std::min<long long>((count + 127) / 128, n->sms);
  k_nn_sum<<<(kParams + 256) / 256, 256, 0, st>>>(n->partials, parts, n->scratch);
  NCK(cudaGetLastError());
  r = checkError(n);
  if (r != SGLC_OK) return r;
  NCK(cudaMemcpyAsync(grads, n->scratch, kParams * sizeof(float), cudaMemcpyDeviceToHost, st));
  float l = 0.f;
  NCK(cudaMemcpyAsync(&l, n->scratch + kParams, sizeof(float), cudaMemcpyDeviceToHost, st));
  NCK(cudaStreamSynchronize(st));
  if (loss) *loss = l;
  return SGLC_OK;
}

SGLC_API sglc_status sglc_neural_infer(sglc_neural *n, int64_t first, int64_t count, float *out) {
  if (!n || !out || first < 0 || count < 0) return SGLC_ERR_INVALID_VALUE;
  if (first + count > n->nRec) return nnFail(n, SGLC_ERR_INVALID_VALUE, "neural shader: record range out of bounds");
  if (count == 0) return SGLC_OK;
  DeviceGuard deviceGuard(n->device);
  cudaStream_t st = ctxStream(n->ctx);
  NCK(ensure(&n->out, &n->outCap, count * 3));
  NCK(cudaMemsetAsync(n->error, 0, sizeof(int), st));
  sglc_status r = runTiles(n, MODE_INFER, first, count, 0, 0, 0.f, n->out);
  if (r != SGLC_OK) return r;
  r = checkError(n);
  if (r != SGLC_OK) return r;
  NCK(cudaMemcpyAsync(out, n->out, (size_t) count * 3 * sizeof(float), cudaMemcpyDeviceToHost, st));
  NCK(cudaStreamSynchronize(st));
  return SGLC_OK;
}

}  // extern "C"

namespace sglc {
const uint8_t *neuralImage(const sglc_neural *n) { return n ? n->image : nullptr; }
}  // namespace sglc
