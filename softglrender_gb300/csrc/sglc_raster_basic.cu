// Raster instantiations: base colour, vertex colour and depth-only passes, plus the dispatcher.
#include "sglc_kernels.h"
#include "sglc_raster.cuh"

namespace sglc {

void launchRasterBlinn(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st);
void launchRasterPbr(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st);
void launchRasterNeural(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st);
void launchRasterPbrCapture(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st);
void launchRasterEnvironment(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st);
void launchShadeBlinn(const DrawParams &p, cudaStream_t st);
void launchShadePbr(const DrawParams &p, cudaStream_t st);
void launchShadePbrCapture(const DrawParams &p, cudaStream_t st);
void launchShadeEnvironment(const DrawParams &p, cudaStream_t st);
void launchShadeNeural(const DrawParams &p, cudaStream_t st);

bool deferredShadingModel(int shading) {
  switch (shading) {
    case SH_VCOLOR:   // cheap shader, but the coverage kernel's balanced pass 2 pays off on dense soups
    case SH_BLINN:
    case SH_BLINN_DIR:
    case SH_PBR:
    case SH_PBR_CAPTURE:
    case SH_SKYBOX:
    case SH_IBL_IRR:
    case SH_IBL_PRE:
    case SH_FXAA:
    case SH_PBR_NEURAL: return true;
  }
  return false;   // base / vertex colour: the shader is a load
}

// the coverage kernel for the tile shape: 16 x 16 pixels (8 warps) or 16 x 8 (4 warps)
template<int W>
static void launchCoverage(const DrawParams &p, bool hasDepth, int grid, cudaStream_t st) {
  if (p.samples == 4) {
    if (hasDepth) launchChained(k_raster_cov<4, true, W>, dim3(grid), dim3(32 * W), 0, st, p);
    else launchChained(k_raster_cov<4, false, W>, dim3(grid), dim3(32 * W), 0, st, p);
  } else {
    if (hasDepth) launchChained(k_raster_cov<1, true, W>, dim3(grid), dim3(32 * W), 0, st, p);
    else launchChained(k_raster_cov<1, false, W>, dim3(grid), dim3(32 * W), 0, st, p);
  }
}

template<int W>
static void launchRop(const DrawParams &p, int grid, cudaStream_t st) {
  if (p.samples == 4) launchChained(k_rop<4, W>, dim3(grid), dim3(32 * W), 0, st, p);
  else launchChained(k_rop<1, W>, dim3(grid), dim3(32 * W), 0, st, p);
}

void launchRasterDeferred(const DrawParams &p, bool hasDepth, cudaStream_t st, cudaEvent_t evCov, cudaEvent_t evShade) {
  const int grid = p.numTiles + (kSplitParts - 1) * (p.tileOrder ? p.heavySlots : 0);   // see tileJob
  if (p.tileH == 8) launchCoverage<4>(p, hasDepth, grid, st);
  else launchCoverage<8>(p, hasDepth, grid, st);
  if (evCov) cudaEventRecord(evCov, st);
  switch (p.shading) {
    case SH_VCOLOR: launchShadeModel<SH_VCOLOR>(p, st); break;
    case SH_BLINN:
    case SH_BLINN_DIR: launchShadeBlinn(p, st); break;
    case SH_PBR: launchShadePbr(p, st); break;
    case SH_PBR_CAPTURE: launchShadePbrCapture(p, st); break;
    case SH_PBR_NEURAL: launchShadeNeural(p, st); break;
    case SH_SKYBOX:
    case SH_IBL_IRR:
    case SH_IBL_PRE:
    case SH_FXAA: launchShadeEnvironment(p, st); break;
  }
  if (evShade) cudaEventRecord(evShade, st);
  if (p.tileH == 8) launchRop<4>(p, grid, st);
  else launchRop<8>(p, grid, st);
}

void launchRaster(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st) {
  int grid = p.numTiles;
  if (!hasColor) {   // depth-only pass: the fragment shader is skipped (RendererSoft.cpp:346-348)
    if (!hasDepth) return;
    if (p.samples == 4) launchChained(k_raster<SH_BASE, 4, false, true>, dim3(grid), dim3(256), 0, st, p);
    else launchChained(k_raster<SH_BASE, 1, false, true>, dim3(grid), dim3(256), 0, st, p);
    return;
  }
  switch (p.shading) {
    case SH_BASE: launchRasterModel<SH_BASE>(p, hasColor, hasDepth, st); break;
    case SH_VCOLOR: launchRasterModel<SH_VCOLOR>(p, hasColor, hasDepth, st); break;
    case SH_BLINN:
    case SH_BLINN_DIR: launchRasterBlinn(p, hasColor, hasDepth, st); break;
    case SH_PBR: launchRasterPbr(p, hasColor, hasDepth, st); break;
    case SH_PBR_NEURAL: launchRasterNeural(p, hasColor, hasDepth, st); break;
    case SH_PBR_CAPTURE: launchRasterPbrCapture(p, hasColor, hasDepth, st); break;
    case SH_SKYBOX:
    case SH_IBL_IRR:
    case SH_IBL_PRE:
    case SH_FXAA: launchRasterEnvironment(p, hasColor, hasDepth, st); break;
  }
}

}  // namespace sglc
