// Raster instantiations: Blinn-Phong (point light) and Blinn-Phong (directional light).
#include "sglc_raster.cuh"

namespace sglc {

void launchRasterBlinn(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st) {
  if (p.shading == SH_BLINN) launchRasterModel<SH_BLINN>(p, hasColor, hasDepth, st);
  else launchRasterModel<SH_BLINN_DIR>(p, hasColor, hasDepth, st);
}

void launchShadeBlinn(const DrawParams &p, cudaStream_t st) {
  if (p.shading == SH_BLINN) launchShadeModel<SH_BLINN>(p, st);
  else launchShadeModel<SH_BLINN_DIR>(p, st);
}

}  // namespace sglc
