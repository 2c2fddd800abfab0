// Raster instantiations: PBR + IBL.
#include "sglc_raster.cuh"

namespace sglc {

void launchRasterPbr(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st) {
  launchRasterModel<SH_PBR>(p, hasColor, hasDepth, st);
}

void launchShadePbr(const DrawParams &p, cudaStream_t st) { launchShadeModel<SH_PBR>(p, st); }

}  // namespace sglc
