// Kernel instantiations for grid shapes: 256,256,2048 (Nx,Ny,Nt), eight layout / launch
// variants (identical results, except 1e-6 relative for the 16-sample chunks; variant 0 is the
// default, the autotuner times all).
#include "mpc_shapes.cuh"

namespace mpc {
extern const ShapeOps* const shape_list_c[];
const ShapeOps* const shape_list_c[] = {
    Shape<256,256,2048,1,128,8192,32,0,2>::ops(),  // 4-pencil tiles staged by cp.async (256-thread pencil
                                                   // CTAs); plane in two passes, 128-thread CTAs on
                                                   // 16-wide column and row strips
    Shape<256,256,2048,1,256,8192,32,0>::ops(),    // 4-pencil tiles; plane clusters of 8 256-thread CTAs
    Shape<256,256,2048,1,256>::ops(),              // 8-pencil tiles (512 threads), plane as above
    Shape<256,256,2048>::ops(),                    // SLO 2, plane 512 threads, clusters of 8 (2 planes)
    Shape<256,256,2048,1,512>::ops(),              // SLO 1, plane 512 threads, clusters of 4
    Shape<256,256,2048,1,256,16384,16>::ops(),     // SLO 1, 1024-thread pencil CTAs (16-sample chunks)
    Shape<256,256,2048,1,256,8192,32,0,2>::ops(),  // 4-pencil tiles, two-pass plane on 32-wide strips
    Shape<256,256,2048,1,128,8192,32,0,2,5>::ops(),  // as variant 0, strip kernels at five CTAs per SM
    Shape<256,256,2048,1,128,8192,32,0,3>::ops(),  // as variant 0, the y pass staged by TMA
    Shape<256,256,2048,1,128,8192,32,0,4>::ops(),  // as variant 0, both strip passes staged by TMA
    nullptr};
}  // namespace mpc
