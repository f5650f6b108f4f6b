// Tile raster instantiations: Loop32 and Loop64 k-buffers.
#include "raster.cuh"

namespace oit {
cudaError_t launch_raster_b(Alg alg, const RasterParams& p, cudaStream_t s) {
  switch (alg) {
    case Alg::Loop: return oitd::launch_transparent<oitd::LoopPolicy>(p, s);
    case Alg::Loop64: return oitd::launch_transparent<oitd::Loop64Policy>(p, s);
    default: return cudaErrorInvalidValue;
  }
}
cudaError_t launch_raster_mv_b(Alg alg, const MvRaster& mv, cudaStream_t s) {
  switch (alg) {
    case Alg::Loop: return oitd::launch_transparent_mv<oitd::LoopPolicy>(mv, s);
    case Alg::Loop64: return oitd::launch_transparent_mv<oitd::Loop64Policy>(mv, s);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace oit
