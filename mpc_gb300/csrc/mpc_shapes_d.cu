// Kernel instantiations for grid shapes: 512,512,1024 (Nx,Ny,Nt).
#include "mpc_shapes.cuh"

namespace mpc {
extern const ShapeOps* const shape_list_d[];
const ShapeOps* const shape_list_d[] = {
    Shape<512,512,1024>::ops(),
    nullptr};
}  // namespace mpc
