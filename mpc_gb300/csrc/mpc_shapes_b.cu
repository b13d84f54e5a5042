// Kernel instantiations for grid shapes: 128,128,1024 256,256,512 (Nx,Ny,Nt).
#include "mpc_shapes.cuh"

namespace mpc {
extern const ShapeOps* const shape_list_b[];
const ShapeOps* const shape_list_b[] = {
    Shape<128,128,1024>::ops(),
    Shape<256,256,512>::ops(),
    nullptr};
}  // namespace mpc
