// sph_pair32.cu -- mixed-precision pair passes (FP32 pair arithmetic on
// cell-relative positions, FP64 accumulation).
#include "sph_launch.h"
#include "sphgpu.h"

namespace sphgpu {

cudaError_t launch_pair_mixed(const LaunchCtx&, const State&, const Geometry&, const Consts&,
                              const BinScratch&, int, int, int, int, int) {
  return cudaErrorNotSupported;
}

}  // namespace sphgpu
