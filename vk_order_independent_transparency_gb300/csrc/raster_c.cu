// Tile raster instantiations: Spinlock/Interlock and weighted blended OIT.
#include "raster.cuh"

namespace oit {
cudaError_t launch_raster_c(Alg alg, const RasterParams& p, cudaStream_t s) {
  switch (alg) {
    case Alg::Spinlock:
    case Alg::Interlock: return oitd::launch_transparent<oitd::LockPolicy>(p, s);
    case Alg::Weighted: return oitd::launch_transparent<oitd::WeightedPolicy>(p, s);
    default: return cudaErrorInvalidValue;
  }
}
cudaError_t launch_raster_mv_c(Alg alg, const MvRaster& mv, cudaStream_t s) {
  switch (alg) {
    case Alg::Spinlock:
    case Alg::Interlock: return oitd::launch_transparent_mv<oitd::LockPolicy>(mv, s);
    case Alg::Weighted: return oitd::launch_transparent_mv<oitd::WeightedPolicy>(mv, s);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace oit
