// Kernel instantiations for grid shapes: 256,256,2048 (Nx,Ny,Nt).
#include "mpc_shapes.cuh"

namespace mpc {
extern const ShapeOps* const shape_list_c[];
const ShapeOps* const shape_list_c[] = {
    Shape<256,256,2048>::ops(),
    nullptr};
}  // namespace mpc
