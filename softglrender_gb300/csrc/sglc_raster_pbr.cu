// Raster instantiations: PBR + IBL.
#include "sglc_raster.cuh"

namespace sglc {

void launchRasterPbr(const DrawParams &p, bool hasColor, bool hasDepth, cudaStream_t st) {
  launchRasterModel<SH_PBR>(p, hasColor, hasDepth, st);
}

}  // namespace sglc
