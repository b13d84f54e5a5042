// Kernel instantiations for grid shapes: 16,16,64 32,32,256 64,64,512 (Nx,Ny,Nt).
#include "mpc_shapes.cuh"

namespace mpc {
extern const ShapeOps* const shape_list_a[];
const ShapeOps* const shape_list_a[] = {
    Shape<16,16,64>::ops(),
    Shape<32,32,256>::ops(),
    Shape<64,64,512>::ops(),
    Shape<64,64,512,1,256>::ops(),      // plane 256 threads x 2 per SM, 2 planes per CTA
    nullptr};
}  // namespace mpc
