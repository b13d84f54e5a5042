// Kernel instantiations for grid shapes: 512,512,1024 (Nx,Ny,Nt), three variants.
#include "mpc_shapes.cuh"

namespace mpc {
extern const ShapeOps* const shape_list_d[];
const ShapeOps* const shape_list_d[] = {
    Shape<512,512,1024,1,256,16384,32,1,2>::ops(),   // plane in two passes: 256-thread CTAs on 16-wide
                                                     // column and row strips
    Shape<512,512,1024>::ops(),                      // plane clusters of 16 512-thread CTAs
    Shape<512,512,1024,1,256,16384,32,1,2,3>::ops(), // two passes, strip kernels at three CTAs per SM
    nullptr};
}  // namespace mpc
