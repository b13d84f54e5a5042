// Kernel instantiations for grid shapes: 128,128,1024 256,256,512 (Nx,Ny,Nt), four variants each.
#include "mpc_shapes.cuh"

namespace mpc {
extern const ShapeOps* const shape_list_b[];
const ShapeOps* const shape_list_b[] = {
    Shape<128,128,1024>::ops(),
    Shape<128,128,1024,1,256>::ops(),   // plane 256 threads x 2 per SM, clusters of 2
    Shape<128,128,1024,1,128,16384,32,1,2>::ops(),   // plane in two passes, 32-wide strips
    Shape<128,128,1024,1,128,16384,32,1,2,5>::ops(), // the same, strip kernels at five CTAs per SM
    Shape<128,128,1024,1,128,16384,32,1,3>::ops(),   // two passes, the y pass staged by TMA
    Shape<256,256,512>::ops(),
    Shape<256,256,512,1,256>::ops(),    // plane 256 threads x 2 per SM, clusters of 8
    Shape<256,256,512,1,128,16384,32,1,2>::ops(),    // plane in two passes, 16-wide strips
    Shape<256,256,512,1,128,16384,32,1,2,5>::ops(),  // the same, strip kernels at five CTAs per SM
    Shape<256,256,512,1,128,16384,32,1,3>::ops(),    // two passes, the y pass staged by TMA
    Shape<256,256,512,1,128,16384,32,1,4>::ops(),    // two passes, both staged by TMA
    nullptr};
}  // namespace mpc
