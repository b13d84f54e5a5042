// mpc_shapes.cuh -- per-grid-shape launch configuration of the pencil and plane sweeps.
//
// A shape variant fixes the device layout and both sweeps' launch shapes:
//   pencil tile  P = TP / Nt pencils, P * Nt / CH threads per CTA, one per CH-sample chunk of the
//                nonlinear walk (TP = 16384, CH = 32: one 512-thread CTA per SM; TP = 8192: two
//                256-thread CTAs per SM; TP = 16384, CH = 16: one 1024-thread CTA per SM);
//   SLO          slots interleaved in the layout (default 2 when P = 8, so t-rows are 128 B);
//   LD           how the split-step pencil pass reads a tile (pencil_kernel);
//   PMB          PL = 2: resident strip CTAs per SM the strip kernels are compiled for (0: 512 / PT,
//                at 128 registers; more CTAs hide more load latency at fewer registers each);
//   PL           plane passes: 1, one cluster kernel per sweep (plane_kernel); 2, the y part on
//                column strips and the x part on row strips, two kernels over HBM without
//                clusters (plane_y_kernel, plane_x_kernel), one more pass over HBM but every SM
//                busy and no cluster barrier; 3, as 2 with the y part staged by TMA bulk tensor
//                copies (plane_y_tma_kernel: persistent 256-thread CTAs, 3 unit buffers each);
//                4, both parts staged by TMA (plane_x_tma_kernel for the x part, Nx = 256);
//   plane unit   PT threads per CTA and 512 / PT CTAs per SM, each CTA holding a
//                PLB = 128 KB * PT / 512 share of the unit; PL = 1: SLO == 2, the two interleaved
//                omega-planes split over CL CTAs; SLO == 1, planes larger than PLB split over
//                CL CTAs, smaller planes batched PB per CTA; PL = 2: strips of PLB bytes.
// Several variants of one grid may be compiled in; they differ only in speed.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <mutex>

#include "mpc_kernels.cuh"

namespace mpc {

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link to libcuda)
inline PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// The field (complex64, slot layout SLO = 1) as a 2-D FLOAT32 tensor of rows of 2 Nx floats,
// Ny * Nt rows, with boxes of box_x floats by box_rows rows.
inline cudaError_t field_tensor_map(CUtensorMap* m, const void* field, int Nx, long rows, int box_x, int box_rows,
                                    CUtensorMapSwizzle swz = CU_TENSOR_MAP_SWIZZLE_NONE) {
    PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
    if (!enc) return cudaErrorNotSupported;
    const cuuint64_t dims[2] = {(cuuint64_t)(2 * Nx), (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)(2 * Nx) * sizeof(float)};
    const cuuint32_t box[2] = {(cuuint32_t)box_x, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(field), dims, strides, box, estr,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, swz,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

struct ShapeOps {
    int Nx, Ny, Nt, P, SLO, CL, PB, PT, CH, LD, PL;
    int pencil_smem, plane_smem;
    cudaError_t (*setup)();
    cudaError_t (*pencil)(int mode, const PencilArgs&, int grid, cudaStream_t);
    cudaError_t (*plane)(const PlaneArgs&, int nclusters, cudaStream_t);
    int (*max_clusters)();
    int (*pencil_blocks_per_sm)();   // resident split-step pencil CTAs per SM
};

template <int NX, int NY, int NT, int SLO_ = 0, int PT = kThreads, int TP = kTilePoints, int CH = 32, int LD = 1,
          int PL = 1, int PMB = 0>
struct Shape {
    static constexpr int P = TP / NT;
    static constexpr int SLO = SLO_ > 0 ? SLO_ : ((P < 16) ? 16 / P : 1);
    static constexpr long PLANE_B = (long)NX * NY * 8;
    static constexpr long PLB = 131072L * PT / kThreads;
    static constexpr int CL = PL >= 2 ? 1
                              : (SLO == 2) ? (int)(PLANE_B * 2 / PLB) : (PLANE_B > PLB ? (int)(PLANE_B / PLB) : 1);
    static constexpr int PB = PL >= 2 ? 1
                              : (SLO == 2) ? 2 : (PLANE_B > PLB ? 1 : ((PLB / PLANE_B) < NT ? (int)(PLB / PLANE_B) : NT));
    // PL = 2: column strips of CXS columns and row strips of RYS rows, PLB bytes each
    static constexpr int CXS = (int)(PLB / (NY * 8L)), RYS = (int)(PLB / (NX * 8L));
    static_assert(PL == 1 || (PL >= 2 && PL <= 4 && SLO == 1 && CXS >= 2 && CXS <= NX && RYS >= 1 && RYS <= NY),
                  "two-pass planes: SLO 1, strips within the plane");
    // PL = 3: the TMA-staged y pass on 16-column strips (128 B box rows), 256 threads, 3 buffers
    static constexpr int TCX = 16, TTH = 256, TNB = 3;
    static_assert(PL < 3 || (NX % TCX == 0 && NY <= 256), "TMA boxes: 16 columns, at most 256 rows");
    static_assert(PL != 4 || (NX == 256 && NY % 16 == 0), "TMA x part: rows of 256, strips of 16 rows");
    static constexpr int XSMEM = 1024 + 3 * 32768 + 2 * 256 * 16 + ((twiddle_bytes(256) + 15) / 16) * 16 + 3 * 8 + 16;
    static_assert(SLO == 1 || SLO == 2, "slot interleave");
    static_assert(PT == 128 || PT == 256 || PT == 512, "plane threads");
    static_assert(P >= 4 && P <= NX * NY, "pencil tile must fit the grid");
    static_assert(CL >= 1 && CL <= 16 && NY % CL == 0 && NX % CL == 0, "cluster split");
    using PC = PencilCfg<NT, P, SLO, CH>;
    using LC = PlaneCfg<NX, NY, CL, PB, SLO>;
    static constexpr int TH = PC::TH;

    static cudaError_t setup() {
        cudaError_t e;
#define MPC_SET_SMEM(K, B)                                                                       \
    e = cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, B);                   \
    if (e != cudaSuccess) return e;
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_ENTRY_C128, CH, LD>), PC::smem(PM_ENTRY_C128));
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_ENTRY_C64, CH, LD>), PC::smem(PM_ENTRY_C64));
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_STEP, CH, LD>), PC::smem(PM_STEP));
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_EXIT_C128, CH, LD>), PC::smem(PM_EXIT_C128));
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_EXIT_C64, CH, LD>), PC::smem(PM_EXIT_C64));
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_TEMP, CH, LD>), PC::smem(PM_TEMP));
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_IONIZ, CH, LD>), PC::smem(PM_IONIZ));
        if constexpr (PL >= 2) {
            if constexpr (PL == 4) {
                MPC_SET_SMEM((plane_x_tma_kernel<NY, TTH, TNB>), XSMEM);
                int dev1 = 0, nsm1 = 0, bx1 = 0;
                if ((e = cudaGetDevice(&dev1)) != cudaSuccess) return e;
                if ((e = cudaDeviceGetAttribute(&nsm1, cudaDevAttrMultiProcessorCount, dev1)) != cudaSuccess) return e;
                if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bx1, plane_x_tma_kernel<NY, TTH, TNB>, TTH, XSMEM)) !=
                    cudaSuccess)
                    return e;
                if (bx1 <= 0) return cudaErrorInvalidConfiguration;
                tma_grid_x = bx1 * nsm1 < NT * (NY / 16) ? bx1 * nsm1 : NT * (NY / 16);
            }
            if constexpr (PL >= 3) {
                if (!tensor_map_encoder()) return cudaErrorNotSupported;
                MPC_SET_SMEM((plane_y_tma_kernel<NX, NY, TCX, TTH, TNB>), (StripYTmaCfg<NX, NY, TCX>::SMEM(TNB)));
                int dev0 = 0, nsm0 = 0, bt = 0;
                if ((e = cudaGetDevice(&dev0)) != cudaSuccess) return e;
                if ((e = cudaDeviceGetAttribute(&nsm0, cudaDevAttrMultiProcessorCount, dev0)) != cudaSuccess) return e;
                if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bt, plane_y_tma_kernel<NX, NY, TCX, TTH, TNB>, TTH,
                                                                       StripYTmaCfg<NX, NY, TCX>::SMEM(TNB))) != cudaSuccess)
                    return e;
                if (bt <= 0) return cudaErrorInvalidConfiguration;
                tma_grid_y = bt * nsm0 < NT * (NX / TCX) ? bt * nsm0 : NT * (NX / TCX);
            }
            MPC_SET_SMEM((plane_y_kernel<NX, NY, CXS, PT, PMB>), (StripYCfg<NX, NY, CXS>::SMEM));
            MPC_SET_SMEM((plane_x_kernel<NX, NY, RYS, PT, PMB>), (StripXCfg<NX, NY, RYS>::SMEM));
            int dev = 0, nsm = 0, by = 0, bx = 0;
            if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
            if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&by, plane_y_kernel<NX, NY, CXS, PT, PMB>, PT,
                                                                   StripYCfg<NX, NY, CXS>::SMEM)) != cudaSuccess)
                return e;
            if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bx, plane_x_kernel<NX, NY, RYS, PT, PMB>, PT,
                                                                   StripXCfg<NX, NY, RYS>::SMEM)) != cudaSuccess)
                return e;
            strip_grid_y = by * nsm < NT * (NX / CXS) ? by * nsm : NT * (NX / CXS);
            strip_grid_x = bx * nsm < NT * (NY / RYS) ? bx * nsm : NT * (NY / RYS);
            return (by > 0 && bx > 0) ? cudaSuccess : cudaErrorInvalidConfiguration;
        } else {
            MPC_SET_SMEM((plane_kernel<NX, NY, CL, PB, SLO, PT>), LC::SMEM);
            if (CL > 8) {
                e = cudaFuncSetAttribute(plane_kernel<NX, NY, CL, PB, SLO, PT>,
                                         cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
                if (e != cudaSuccess) return e;
            }
            return cudaSuccess;
        }
#undef MPC_SET_SMEM
    }

    static cudaError_t pencil(int mode, const PencilArgs& a, int grid, cudaStream_t st) {
        switch (mode) {
            case PM_ENTRY_C128: pencil_kernel<NT, P, SLO, PM_ENTRY_C128, CH, LD><<<grid, TH, PC::smem(PM_ENTRY_C128), st>>>(a); break;
            case PM_ENTRY_C64: pencil_kernel<NT, P, SLO, PM_ENTRY_C64, CH, LD><<<grid, TH, PC::smem(PM_ENTRY_C64), st>>>(a); break;
            case PM_STEP: pencil_kernel<NT, P, SLO, PM_STEP, CH, LD><<<grid, TH, PC::smem(PM_STEP), st>>>(a); break;
            case PM_EXIT_C128: pencil_kernel<NT, P, SLO, PM_EXIT_C128, CH, LD><<<grid, TH, PC::smem(PM_EXIT_C128), st>>>(a); break;
            case PM_EXIT_C64: pencil_kernel<NT, P, SLO, PM_EXIT_C64, CH, LD><<<grid, TH, PC::smem(PM_EXIT_C64), st>>>(a); break;
            case PM_TEMP: pencil_kernel<NT, P, SLO, PM_TEMP, CH, LD><<<grid, TH, PC::smem(PM_TEMP), st>>>(a); break;
            case PM_IONIZ: pencil_kernel<NT, P, SLO, PM_IONIZ, CH, LD><<<grid, TH, PC::smem(PM_IONIZ), st>>>(a); break;
            default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }

    // PL = 2, 3: resident-CTA grids of the strip kernels (set by setup)
    static inline int strip_grid_y = 0, strip_grid_x = 0, tma_grid_y = 0, tma_grid_x = 0;

    // the TMA-staged y pass from `in` to `out` (tensor maps encoded per launch: a few host
    // microseconds, no device work)
    static cudaError_t plane_y_tma(const PlaneArgs& a, int second, cudaStream_t st) {
        CUtensorMap tin, tout;
        cudaError_t e;
        if ((e = field_tensor_map(&tin, a.in, NX, (long)NY * NT, 2 * TCX, NY)) != cudaSuccess) return e;
        if ((e = field_tensor_map(&tout, a.out, NX, (long)NY * NT, 2 * TCX, NY)) != cudaSuccess) return e;
        plane_y_tma_kernel<NX, NY, TCX, TTH, TNB><<<tma_grid_y, TTH, StripYTmaCfg<NX, NY, TCX>::SMEM(TNB), st>>>(
            tin, tout, a, second, a.err);
        return cudaGetLastError();
    }

    // the TMA-staged x pass, in place on a.out (row strips of 16 rows, 16 swizzled boxes each)
    static cudaError_t plane_x_tma(const PlaneArgs& a, cudaStream_t st) {
        CUtensorMap tin, tout;
        cudaError_t e;
        if ((e = field_tensor_map(&tin, a.in, NX, (long)NY * NT, 32, 16, CU_TENSOR_MAP_SWIZZLE_128B)) != cudaSuccess)
            return e;
        if ((e = field_tensor_map(&tout, a.out, NX, (long)NY * NT, 32, 16, CU_TENSOR_MAP_SWIZZLE_128B)) != cudaSuccess)
            return e;
        if constexpr (PL == 4) plane_x_tma_kernel<NY, TTH, TNB><<<tma_grid_x, TTH, XSMEM, st>>>(tin, tout, a, a.err);
        return cudaGetLastError();
    }

    static cudaError_t plane(const PlaneArgs& a, int nclusters, cudaStream_t st) {
        if constexpr (PL == 4) {
            PlaneArgs b = a;
            b.in = a.out;   // the passes after the first run in place
            cudaError_t e;
            if ((e = plane_y_tma(a, 0, st)) != cudaSuccess) return e;
            if ((e = plane_x_tma(b, st)) != cudaSuccess) return e;
            if (a.lens) return plane_y_tma(b, 1, st);
            return cudaSuccess;
        } else if constexpr (PL == 3) {
            PlaneArgs b = a;
            b.in = a.out;   // the passes after the first run in place
            cudaError_t e;
            if ((e = plane_y_tma(a, 0, st)) != cudaSuccess) return e;
            plane_x_kernel<NX, NY, RYS, PT, PMB><<<strip_grid_x, PT, StripXCfg<NX, NY, RYS>::SMEM, st>>>(b);
            if ((e = cudaGetLastError()) != cudaSuccess) return e;
            if (a.lens) return plane_y_tma(b, 1, st);
            return cudaSuccess;
        } else if constexpr (PL == 2) {
            PlaneArgs b = a;
            b.in = a.out;   // the passes after the first run in place
            plane_y_kernel<NX, NY, CXS, PT, PMB><<<strip_grid_y, PT, StripYCfg<NX, NY, CXS>::SMEM, st>>>(a, 0);
            plane_x_kernel<NX, NY, RYS, PT, PMB><<<strip_grid_x, PT, StripXCfg<NX, NY, RYS>::SMEM, st>>>(b);
            if (a.lens) plane_y_kernel<NX, NY, CXS, PT, PMB><<<strip_grid_y, PT, StripYCfg<NX, NY, CXS>::SMEM, st>>>(b, 1);
            return cudaGetLastError();
        } else {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(nclusters * CL);
            cfg.blockDim = dim3(PT);
            cfg.dynamicSmemBytes = LC::SMEM;
            cfg.stream = st;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = CL;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            return cudaLaunchKernelEx(&cfg, plane_kernel<NX, NY, CL, PB, SLO, PT>, a);
        }
    }

    static int max_clusters() {
        if constexpr (PL >= 2) {
            return strip_grid_y;   // CTAs of the y pass (clusters of one)
        } else {
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3(CL);
            cfg.blockDim = dim3(PT);
            cfg.dynamicSmemBytes = LC::SMEM;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeClusterDimension;
            attr[0].val.clusterDim.x = CL;
            attr[0].val.clusterDim.y = 1;
            attr[0].val.clusterDim.z = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            int n = 0;
            if (cudaOccupancyMaxActiveClusters(&n, plane_kernel<NX, NY, CL, PB, SLO, PT>, &cfg) != cudaSuccess) return 0;
            return n;
        }
    }

    static int pencil_blocks_per_sm() {
        int n = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, pencil_kernel<NT, P, SLO, PM_STEP, CH, LD>, TH, PC::SMEM) !=
            cudaSuccess)
            return 0;
        return n;
    }

    static constexpr int plane_smem() {
        if constexpr (PL >= 2) return StripYCfg<NX, NY, CXS>::SMEM;
        else return LC::SMEM;
    }

    static const ShapeOps* ops() {
        static const ShapeOps o = {NX, NY, NT, P, SLO, CL, PB, PT, CH, LD, PL, PC::SMEM, plane_smem(), &setup, &pencil, &plane,
                                   &max_clusters, &pencil_blocks_per_sm};
        return &o;
    }
};

}  // namespace mpc
