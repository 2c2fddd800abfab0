// Raster instantiations: the environment passes (skybox / equirectangular-to-cube, irradiance and
// prefiltered-specular convolution) that IBLGenerator draws into cube-map faces, and the FXAA
// screen pass that QuadFilter draws.
#include "sglc_raster.cuh"

namespace sglc {

void launchRasterEnvironment(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st) {
  switch (p.shading) {
    case SH_SKYBOX: launchRasterModel<SH_SKYBOX>(p, hasColor, hasDepth, st); break;
    case SH_IBL_IRR: launchRasterModel<SH_IBL_IRR>(p, hasColor, hasDepth, st); break;
    case SH_IBL_PRE: launchRasterModel<SH_IBL_PRE>(p, hasColor, hasDepth, st); break;
    case SH_FXAA: launchRasterModel<SH_FXAA>(p, hasColor, hasDepth, st); break;
  }
}

void launchShadeEnvironment(const DrawParams &p, cudaStream_t st) {
  switch (p.shading) {
    case SH_SKYBOX: launchShadeModel<SH_SKYBOX>(p, st); break;
    case SH_IBL_IRR: launchShadeModel<SH_IBL_IRR>(p, st); break;
    case SH_IBL_PRE: launchShadeModel<SH_IBL_PRE>(p, st); break;
    case SH_FXAA: launchShadeModel<SH_FXAA>(p, st); break;
  }
}

}  // namespace sglc
