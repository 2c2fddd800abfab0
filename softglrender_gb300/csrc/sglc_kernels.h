// Host-side launchers of the draw kernels (defined in sglc_geom.cu, sglc_raster_*.cu, sglc_lines*.cu).
#pragma once

#include <cuda_runtime.h>

#include "sglc_device.cuh"

namespace sglc {

void scanExclusive(const int *in, int *out, const int *nPtr, int nMax, int *blockSums, cudaStream_t st);
void scanExclusive2(const int *in, int *out, const int *nPtr, int nMax, int *blockSums, cudaStream_t st);
// the apply step alone, when the producer of `in` already summed each scan tile into blockSums
// (zeroed beforehand); scanTiles(nMax) tiles
void scanApply(const int *in, int *out, const int *nPtr, int nMax, const int *blockSums, cudaStream_t st);
int scanTiles(int nMax);
int scanScratchInts(int nMax);
void launchVertexAndClip(const DrawParams &p, cudaStream_t st);
void launchClipAppend(const DrawParams &p, cudaStream_t st);
void launchSetup(const DrawParams &p, int primCount, cudaStream_t st);
void launchBinEmit(const DrawParams &p, int primCount, cudaStream_t st);
// stable LSD radix sort of (keyA, valA) by the low keyBits bits of the key, in as few passes as
// digits of at most maxDigitBits (<= kMaxDigitBits) bits allow; hist and histScan hold
// sortScratchInts(nPairs) ints (2^maxDigitBits buckets per block of 2048 pairs are used)
constexpr int kMaxDigitBits = 10;
constexpr int kSortThreads = 256;
constexpr int kSortItemsSmall = 2, kSortItemsLarge = 8;          // items per thread
constexpr int kSortTileSmall = kSortThreads * kSortItemsSmall;   // 512 items per CTA
constexpr int kSortTileLarge = kSortThreads * kSortItemsLarge;   // 2,048 items per CTA
constexpr int kSortSmallMax = 1 << 20;                           // sorts up to this size use the small blocks
int sortScratchInts(int nPairs);
int sortPassCount(int keyBits, int maxDigitBits = kMaxDigitBits);
void sortPairs(const DrawParams &p, int nPairs, const int *nPtr, int keyBits, int *hist, int *histScan,
               int *scanScratch, cudaStream_t st, bool twoLaunchScan = false, int maxDigitBits = kMaxDigitBits);
void launchTileRanges(const DrawParams &p, int nPairs, const int *nPtr, cudaStream_t st);
void launchTileOrder(const DrawParams &p, int *order, cudaStream_t st);
void launchRaster(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st);
// deferred shading (coverage -> shade -> ROP) for the shading models it is built for
bool deferredShadingModel(int shading);
// evCov / evShade (may be null) are recorded after the coverage and the shading kernel
void launchRasterDeferred(const DrawParams &p, bool hasDepth, cudaStream_t st, cudaEvent_t evCov = nullptr,
                          cudaEvent_t evShade = nullptr);
void launchFill32(uint32_t *dst, uint32_t value, size_t n, cudaStream_t st);
// *sticky |= *flags
void launchAccumulateFlags(const int *flags, int *sticky, cudaStream_t st);
void launchMipLevel(const DevTex &t, int face, int level, int isFloat, cudaStream_t st);
void launchSwizzleIn(const DevTex &t, int face, int level, const uint32_t *src, cudaStream_t st);
void launchSwizzleOut(const DevTex &t, int face, int level, uint32_t *dst, cudaStream_t st);

// point and line draws (sglc_lines.cu, sglc_lines_shade.cu, k_lp_assemble in sglc_geom.cu)
void launchPointsLinesGeometry(const DrawParams &p, const LineParams &lp, cudaStream_t st);
void launchPointKeys(const LineParams &lp, uint32_t *keys, int *vals, int n, cudaStream_t st);
void launchPointChain(const DrawParams &p, const LineParams &lp, const uint32_t *keys, const int *vals, int n,
                      cudaStream_t st);
void launchStampCount(const DrawParams &p, const LineParams &lp, cudaStream_t st);
void launchStampEmit(const DrawParams &p, const LineParams &lp, cudaStream_t st);
void launchStampShade(const DrawParams &p, const LineParams &lp, int nStamps, cudaStream_t st);
void launchFragCount(const LineParams &lp, int nStamps, cudaStream_t st);
void launchFragEmit(const LineParams &lp, int nStamps, uint32_t *keys, int *vals, cudaStream_t st);
void launchFragApply(const DrawParams &p, const LineParams &lp, const uint32_t *keys, const int *vals, int n,
                     bool hasDepth, cudaStream_t st);
void launchResolve(const DrawParams &p, cudaStream_t st);

}  // namespace sglc
