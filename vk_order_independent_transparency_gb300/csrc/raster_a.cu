// Tile raster instantiations: Simple, Linked List and the opaque pass.
#include "raster.cuh"

namespace oit {
cudaError_t launch_raster_a(Alg alg, const RasterParams& p, cudaStream_t s) {
  switch (alg) {
    case Alg::Simple: return oitd::launch_transparent<oitd::SimplePolicy>(p, s);
    case Alg::LinkedList: return oitd::launch_transparent<oitd::LinkedListPolicy>(p, s);
    case Alg::Opaque: return oitd::launch_opaque(p, s);
    default: return cudaErrorInvalidValue;
  }
}
cudaError_t launch_raster_mv_a(Alg alg, const MvRaster& mv, cudaStream_t s) {
  switch (alg) {
    case Alg::Simple: return oitd::launch_transparent_mv<oitd::SimplePolicy>(mv, s);
    case Alg::LinkedList: return oitd::launch_transparent_mv<oitd::LinkedListPolicy>(mv, s);
    case Alg::Opaque: return oitd::launch_opaque_mv(mv, s);
    default: return cudaErrorInvalidValue;
  }
}
}  // namespace oit
