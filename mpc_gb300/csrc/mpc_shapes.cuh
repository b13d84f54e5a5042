// mpc_shapes.cuh -- per-grid-shape launch configuration of the two sweeps.
//
// Tile and cluster shapes follow from shared-memory capacity (one 128 KB working set per
// CTA, one CTA per SM) and the >= 128 B row rule for strided HBM access:
//   pencil tile  P = 16384 / Nt pencils, SLO = 2 slots interleaved when P = 8, else 1;
//   plane unit   SLO == 2: the two interleaved omega-planes, split over CL = bytes/128 KB CTAs;
//                SLO == 1: planes over 128 KB are split over CL CTAs, smaller planes are
//                batched PB per CTA.
#pragma once
#include <cuda_runtime.h>

#include "mpc_kernels.cuh"

namespace mpc {

struct ShapeOps {
    int Nx, Ny, Nt, P, SLO, CL, PB;
    int pencil_smem, plane_smem;
    cudaError_t (*setup)();
    cudaError_t (*pencil)(int mode, const PencilArgs&, int grid, cudaStream_t);
    cudaError_t (*plane)(const PlaneArgs&, int nclusters, cudaStream_t);
    int (*max_clusters)();
};

template <int NX, int NY, int NT>
struct Shape {
    static constexpr int P = kTilePoints / NT;
    static constexpr int SLO = (P < 16) ? 16 / P : 1;
    static constexpr long PLANE_B = (long)NX * NY * 8;
    static constexpr int CL = (SLO == 2) ? (int)(PLANE_B * 2 / 131072) : (PLANE_B > 131072 ? (int)(PLANE_B / 131072) : 1);
    static constexpr int PB = (SLO == 2) ? 2 : (PLANE_B > 131072 ? 1 : ((131072 / PLANE_B) < NT ? (int)(131072 / PLANE_B) : NT));
    static_assert(P >= 8 && P <= NX * NY, "pencil tile must fit the grid");
    static_assert(CL >= 1 && CL <= 16 && NY % CL == 0 && NX % CL == 0, "cluster split");
    using PC = PencilCfg<NT, P, SLO>;
    using LC = PlaneCfg<NX, NY, CL, PB, SLO>;

    static cudaError_t setup() {
        cudaError_t e;
#define MPC_SET_SMEM(K, B)                                                                       \
    e = cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, B);                   \
    if (e != cudaSuccess) return e;
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_ENTRY_C128>), PC::SMEM);
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_ENTRY_C64>), PC::SMEM);
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_STEP>), PC::SMEM);
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_EXIT_C128>), PC::SMEM);
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_EXIT_C64>), PC::SMEM);
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_TEMP>), PC::SMEM);
        MPC_SET_SMEM((pencil_kernel<NT, P, SLO, PM_IONIZ>), PC::SMEM);
        MPC_SET_SMEM((plane_kernel<NX, NY, CL, PB, SLO>), LC::SMEM);
#undef MPC_SET_SMEM
        if (CL > 8) {
            e = cudaFuncSetAttribute(plane_kernel<NX, NY, CL, PB, SLO>,
                                     cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }

    static cudaError_t pencil(int mode, const PencilArgs& a, int grid, cudaStream_t st) {
        switch (mode) {
            case PM_ENTRY_C128: pencil_kernel<NT, P, SLO, PM_ENTRY_C128><<<grid, kThreads, PC::SMEM, st>>>(a); break;
            case PM_ENTRY_C64: pencil_kernel<NT, P, SLO, PM_ENTRY_C64><<<grid, kThreads, PC::SMEM, st>>>(a); break;
            case PM_STEP: pencil_kernel<NT, P, SLO, PM_STEP><<<grid, kThreads, PC::SMEM, st>>>(a); break;
            case PM_EXIT_C128: pencil_kernel<NT, P, SLO, PM_EXIT_C128><<<grid, kThreads, PC::SMEM, st>>>(a); break;
            case PM_EXIT_C64: pencil_kernel<NT, P, SLO, PM_EXIT_C64><<<grid, kThreads, PC::SMEM, st>>>(a); break;
            case PM_TEMP: pencil_kernel<NT, P, SLO, PM_TEMP><<<grid, kThreads, PC::SMEM, st>>>(a); break;
            case PM_IONIZ: pencil_kernel<NT, P, SLO, PM_IONIZ><<<grid, kThreads, PC::SMEM, st>>>(a); break;
            default: return cudaErrorInvalidValue;
        }
        return cudaGetLastError();
    }

    static cudaError_t plane(const PlaneArgs& a, int nclusters, cudaStream_t st) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(nclusters * CL);
        cfg.blockDim = dim3(kThreads);
        cfg.dynamicSmemBytes = LC::SMEM;
        cfg.stream = st;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = CL;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, plane_kernel<NX, NY, CL, PB, SLO>, a);
    }

    static int max_clusters() {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(CL);
        cfg.blockDim = dim3(kThreads);
        cfg.dynamicSmemBytes = LC::SMEM;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = CL;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, plane_kernel<NX, NY, CL, PB, SLO>, &cfg) != cudaSuccess) return 0;
        return n;
    }

    static const ShapeOps* ops() {
        static const ShapeOps o = {NX, NY, NT, P, SLO, CL, PB, PC::SMEM, LC::SMEM, &setup, &pencil, &plane, &max_clusters};
        return &o;
    }
};

}  // namespace mpc
