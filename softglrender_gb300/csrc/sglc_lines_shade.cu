// The fragment shader of point and line stamps (rasterizationPoint, RendererSoft.cpp:650-653): one
// evaluation per stamp on the stamp's varyings (a point's own vertex row, or a line step's lerped
// row), without derivatives (the reference has no quad there; draws whose shader would need them
// are refused on the host). Instantiated for every shading model the renderer has.
#include "sglc_device.cuh"
#include "sglc_kernels.h"
#include "sglc_shaders.cuh"

namespace sglc {

namespace {

template<int SH>
__global__ void __launch_bounds__(128) k_lp_stamp_shade(const __grid_constant__ DrawParams p,
                                                        const __grid_constant__ LineParams lp, int nStamps) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nStamps) return;
  const int r = lp.stampRow[i];
  const float *row = r >= 0 ? lp.stampVary + (size_t) r * p.varyStride : p.vVary + (size_t) (-r - 1) * p.varyStride;
  FragIn f;
  f.U = p.u;
  // weights (1, 0, 0) over three copies of the row reproduce it exactly for finite varyings
  f.v = Vary{row, row, row, 1.f, 0.f, 0.f};
  f.dudx = f.dvdx = f.dudy = f.dvdy = 0.f;
  lp.stampColor[i] = runFS<SH>(p, f);
}

}  // namespace

void launchStampShade(const DrawParams &p, const LineParams &lp, int nStamps, cudaStream_t st) {
  if (nStamps <= 0) return;
  const int grid = (nStamps + 127) / 128;
  switch (p.shading) {
    case SH_BASE: k_lp_stamp_shade<SH_BASE><<<grid, 128, 0, st>>>(p, lp, nStamps); break;
    case SH_VCOLOR: k_lp_stamp_shade<SH_VCOLOR><<<grid, 128, 0, st>>>(p, lp, nStamps); break;
    case SH_BLINN: k_lp_stamp_shade<SH_BLINN><<<grid, 128, 0, st>>>(p, lp, nStamps); break;
    case SH_BLINN_DIR: k_lp_stamp_shade<SH_BLINN_DIR><<<grid, 128, 0, st>>>(p, lp, nStamps); break;
    case SH_PBR: k_lp_stamp_shade<SH_PBR><<<grid, 128, 0, st>>>(p, lp, nStamps); break;
    case SH_SKYBOX: k_lp_stamp_shade<SH_SKYBOX><<<grid, 128, 0, st>>>(p, lp, nStamps); break;
    case SH_IBL_IRR: k_lp_stamp_shade<SH_IBL_IRR><<<grid, 128, 0, st>>>(p, lp, nStamps); break;
    case SH_IBL_PRE: k_lp_stamp_shade<SH_IBL_PRE><<<grid, 128, 0, st>>>(p, lp, nStamps); break;
    case SH_FXAA: k_lp_stamp_shade<SH_FXAA><<<grid, 128, 0, st>>>(p, lp, nStamps); break;
  }
}

}  // namespace sglc
