// Raster instantiations: PBR + IBL that also captures neural-shader training records.
#include "sglc_raster.cuh"

namespace sglc {

void launchRasterPbrCapture(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st) {
  launchRasterModel<SH_PBR_CAPTURE>(p, hasColor, hasDepth, st);
}

void launchShadePbrCapture(const DrawParams &p, cudaStream_t st) { launchShadeModel<SH_PBR_CAPTURE>(p, st); }

}  // namespace sglc
