// The neural IBL shader: a small MLP that stands in for the image-based-lighting term of the PBR
// fragment shader (PbrSoft.h:296-309: irradiance fetch, prefiltered-cube fetch at a roughness
// LOD, FresnelSchlickRoughness and EnvBRDFApprox). The direct point light, gamma and emissive stay
// analytic. Shared by the training / inference kernels (sglc_nn.cu) and the fused raster variant.
//
// Network: 12 inputs -> frequency encoding (156 features, padded to 160) -> 64 ReLU -> 64 ReLU -> 3.
// Inputs: normal N (3), view direction V (3), roughness, metallic, albedo texel (3, sRGB as
// sampled), max(dot(N, V), 0). Output: sqrt of the IBL ambient term before the ambient-occlusion
// factor; the shader squares it back (ambient = max(y, 0)^2).
// Encoding of input x_i: for k = 0..5 feature 24k + 2i = sin(2^k pi x_i), 24k + 2i + 1 =
// cos(2^k pi x_i), computed from sincospi(x_i) by the double-angle recurrences t = 2 s, s' = t c,
// c' = 1 - t s (fused, one rounding); feature 144 + i = x_i. Feature 156 is the constant 1 on training tiles (its weight
// column stays zero, so the forward pass ignores it, and the weight gradient's row 156 is the first
// layer's bias gradient); features 157-159 are zero.
//
// Parameters (FP32 master copy, flat order): W1[64][156], b1[64], W2[64][64], b2[64], W3[3][64],
// b3[3]. The device keeps a BF16 "image" of the weights in the core-matrix tile layout of
// sglc_tc.cuh, ready to copy into shared memory: W1 as a [64][160] tile, W2 [64][64], W3 [16][64]
// (rows 3-15 zero), followed by the FP32 biases b1 (64), b2 (64), b3 (3) and one zero.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>
#include "sglc_tc.cuh"

namespace sglc {
namespace nn {

constexpr int kIn = 12;
constexpr int kFreq = 6;
constexpr int kFeat = kIn * (1 + 2 * kFreq);   // 156
constexpr int kK1 = 160;                       // padded first-layer K
constexpr int kHid = 64;
constexpr int kOut = 3;
constexpr int kOutPad = 16;
constexpr int kOneFeature = 156;

// offsets into the flat parameter vector
constexpr int kW1 = 0;
constexpr int kB1 = kW1 + kHid * kFeat;        // 9984
constexpr int kW2 = kB1 + kHid;
constexpr int kB2 = kW2 + kHid * kHid;
constexpr int kW3 = kB2 + kHid;
constexpr int kB3 = kW3 + kOut * kHid;
constexpr int kParams = kB3 + kOut;            // 14403
constexpr int kPartialStride = 14408;          // per-CTA gradient partial: params, loss, pad

// weight image (bytes)
constexpr int kImgW1 = 0;
constexpr int kImgW2 = kImgW1 + kHid * kK1 * 2;          // 20480
constexpr int kImgW3 = kImgW2 + kHid * kHid * 2;         // 28672
constexpr int kImgBias = kImgW3 + kOutPad * kHid * 2;    // 30720
constexpr int kImgBytes = kImgBias + (64 + 64 + 4) * 4;  // 31248
static_assert(kImgBytes % 16 == 0, "image copies in 16-byte pieces");

// Inference image (follows the training image in the same allocation, at kInferOffset): the same
// network laid out for the deferred shading kernel, which encodes a fragment in two halves of 80
// features (inputs 0-5, then inputs 6-11) and folds every bias into its layer's MMA:
//   W1 [64][160]: half H (columns 80H..80H+79) holds inputs 6H+j, j = 0..5: column 80H + 12k + 2j
//                 = sin(2^k pi x), + 1 = cos, k = 0..5; column 80H + 72 + j = x; columns 158 and
//                 159 hold b1 split into a BF16 high part and the BF16 rounding of its remainder
//                 (the encoder puts 1 in both input columns), 78 and 79 stay zero;
//   W2 [64][80], W3 [16][80]: columns 0-63 the weights, 64 and 65 the bias split the same way
//                 (the hidden tiles carry ones there), the rest zero.
constexpr int kIW1 = 0;
constexpr int kIW2 = kIW1 + kHid * kK1 * 2;               // 20480
constexpr int kIW3 = kIW2 + kHid * 80 * 2;                // 30720
constexpr int kInferBytes = kIW3 + kOutPad * 80 * 2;      // 33280
constexpr int kInferOffset = kImgBytes;                   // 16-byte aligned
constexpr int kImageAllocBytes = kInferOffset + kInferBytes;

// inference-image column of canonical first-layer feature f (0..155)
__host__ __device__ constexpr int inferColumn(int f) {
  return f < 144 ? 80 * (((f % 24) / 2) / 6) + 12 * (f / 24) + 2 * (((f % 24) / 2) % 6) + (f & 1)
                 : 80 * ((f - 144) / 6) + 72 + (f - 144) % 6;
}

// training record: 12 inputs, 3 targets (sqrt of the ambient term), 1 pad
constexpr int kRecordFloats = 16;

// Encode one fragment's 12 inputs into row `row` of a core-matrix tile (BF16), one 16-byte store per
// 8 features: the 8-feature chunks [C0, C1) go to tile columns 8 * (chunk - C0) of a tile with
// `tileC` columns (the whole row: C0 = 0, C1 = 20, tileC = 160).
// FAST (the shading kernels, judged by PSNR): sin / cos of pi x from the special-function unit
// (__sincosf; the inputs lie in [-1, 1], where its error is below 1e-6, which can move a feature
// across a BF16 rounding boundary, one BF16 ulp); otherwise sincospi (training and the inference
// entry point, which the oracle checks).
template<int C0, int C1, bool FAST = false>
__device__ __forceinline__ void encodeChunks(const float *x, uint8_t *tile, int row, int tileC, bool oneFeature) {
  float s[kIn], c[kIn];
#pragma unroll
  for (int i = 0; i < kIn; i++) {
    if (FAST) __sincosf(3.14159265358979f * x[i], &s[i], &c[i]);
    else sincospif(x[i], &s[i], &c[i]);
  }
#pragma unroll
  for (int k = 0; k < kFreq; k++) {
#pragma unroll
    for (int q = 0; q < 3; q++) {   // features 24k + 8q .. +7 = inputs 4q .. 4q+3, (sin, cos) pairs
      const int chunk = 3 * k + q;
      if (chunk >= C0 && chunk < C1) {
        uint4 v = make_uint4(tc::packBf16(s[4 * q], c[4 * q]), tc::packBf16(s[4 * q + 1], c[4 * q + 1]),
                             tc::packBf16(s[4 * q + 2], c[4 * q + 2]), tc::packBf16(s[4 * q + 3], c[4 * q + 3]));
        *reinterpret_cast<uint4 *>(tile + tc::tileOffset(row, 8 * (chunk - C0), tileC)) = v;
      }
    }
    if (k + 1 < kFreq) {
#pragma unroll
      for (int i = 0; i < kIn; i++) {   // double angle: t = 2 s, s' = t c, c' = 1 - t s (one rounding)
        const float t = s[i] + s[i];
        const float c2 = __fmaf_rn(-t, s[i], 1.0f);
        s[i] = t * c[i];
        c[i] = c2;
      }
    }
  }
  if (18 >= C0 && 18 < C1) {
    uint4 a = make_uint4(tc::packBf16(x[0], x[1]), tc::packBf16(x[2], x[3]), tc::packBf16(x[4], x[5]),
                         tc::packBf16(x[6], x[7]));
    *reinterpret_cast<uint4 *>(tile + tc::tileOffset(row, 8 * (18 - C0), tileC)) = a;
  }
  if (19 >= C0 && 19 < C1) {
    uint4 b = make_uint4(tc::packBf16(x[8], x[9]), tc::packBf16(x[10], x[11]),
                         tc::packBf16(oneFeature ? 1.f : 0.f, 0.f), 0u);
    *reinterpret_cast<uint4 *>(tile + tc::tileOffset(row, 8 * (19 - C0), tileC)) = b;
  }
}

template<bool FAST = false>
__device__ __forceinline__ void encodeRow(const float *x, uint8_t *tile, int row, bool oneFeature) {
  encodeChunks<0, 20, FAST>(x, tile, row, kK1, oneFeature);
}

// Epilogue of a hidden layer for one row: 64 accumulator columns from TMEM (this thread's lane),
// + bias, ReLU, BF16 into row `row` of `out` (a tile with `outC` columns, starting at column
// `outCol`). Returns the ReLU mask (bit j: unit j active).
__device__ __forceinline__ unsigned long long hiddenEpilogue(uint32_t taddr, const float *bias, uint8_t *out,
                                                             int row, int outC, int outCol) {
  unsigned long long mask = 0ull;
#pragma unroll
  for (int h = 0; h < 4; h++) {
    float a[16];
    tc::ld16(taddr + 16 * h, a);
    tc::ldWait();
#pragma unroll
    for (int j = 0; j < 16; j++) {
      float v = a[j] + bias[16 * h + j];
      v = v > 0.f ? v : 0.f;
      if (v > 0.f) mask |= 1ull << (16 * h + j);
      a[j] = v;
    }
#pragma unroll
    for (int q = 0; q < 2; q++) {
      uint4 v = make_uint4(tc::packBf16(a[8 * q], a[8 * q + 1]), tc::packBf16(a[8 * q + 2], a[8 * q + 3]),
                           tc::packBf16(a[8 * q + 4], a[8 * q + 5]), tc::packBf16(a[8 * q + 6], a[8 * q + 7]));
      *reinterpret_cast<uint4 *>(out + tc::tileOffset(row, outCol + 16 * h + 8 * q, outC)) = v;
    }
  }
  return mask;
}

// MMA issue helper (one thread). Descriptors follow the tile layout of sglc_tc.cuh.
// D[128 x N] (+)= A[128 x K] * B[K x N]: A = K columns of a tile with aC columns starting at column
// aCol (K-major); B = a weight tile [N][bC] (K-major) from column bCol.
// Each K step of 16 advances both operands by two core matrices (256 bytes), which is 16 in the
// descriptor's address field (addresses >> 4; shared-memory addresses stay far below its 18-bit
// range), so the descriptors are built once and stepped by an add.
__device__ __forceinline__ void issueKMajor(uint32_t dTmem, uint32_t aBase, int aC, int aCol, uint32_t bBase, int bC,
                                            int bCol, int N, int K, bool accumulate) {
  const uint32_t idesc = tc::instrDesc(128, N, false, false);
  uint64_t ad = tc::smemDesc(aBase + tc::tileOffset(0, aCol, aC), 128, (uint32_t) aC / 8 * 128);
  uint64_t bd = tc::smemDesc(bBase + tc::tileOffset(0, bCol, bC), 128, (uint32_t) bC / 8 * 128);
#pragma unroll 1
  for (int k = 0; k < K; k += 16) {
    tc::mma(dTmem, ad, bd, idesc, accumulate || k > 0);
    ad += 16;
    bd += 16;
  }
}

}  // namespace nn
}  // namespace sglc
