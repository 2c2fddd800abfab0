// Raster instantiations: base colour, vertex colour and depth-only passes, plus the dispatcher.
#include "sglc_kernels.h"
#include "sglc_raster.cuh"

namespace sglc {

void launchRasterBlinn(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st);
void launchRasterPbr(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st);
void launchRasterNeural(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st);
void launchRasterPbrCapture(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st);
void launchRasterEnvironment(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st);

void launchRaster(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st) {
  int grid = p.views * p.tilesPerView;
  if (!hasColor) {   // depth-only pass: the fragment shader is skipped (RendererSoft.cpp:346-348)
    if (!hasDepth) return;
    if (p.samples == 4) k_raster<SH_BASE, 4, false, true><<<grid, 256, 0, st>>>(p);
    else k_raster<SH_BASE, 1, false, true><<<grid, 256, 0, st>>>(p);
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
