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
}  // namespace oit
