// mpc_noalloc.cu -- the nonlinear split-step operator for callers that cannot allocate.
//
// Some callers cannot call cudaMalloc: code that runs where allocation is not allowed or
// not safe (a host callback, a section of another library that has promised its caller
// not to allocate), processes whose device memory is handed out at start-up by a memory
// pool that owns every byte, and embedded hosts with a fixed device-memory budget.  They
// hold the field in device memory already and need the nonlinear step applied to it.
//
// mpc_nonlinear_noalloc does that without allocating anything: the work buffers of its
// kernel (one dA tile per resident CTA, the twiddle table, the omega table) live in the
// single file-scope array g_noalloc below, which every GPU that loads this library holds
// until the process exits.  Its kernel is the pencil sweep's nonlinear stage (Kerr,
// self-steepening through the spectral derivative, ADK ionization and plasma terms,
// propagation.c:164-327 and plasma.c:118-245 with the defects corrected) on a field given
// in real space, complex64, reference layout A[t*Nx*Ny + y*Nx + x], physical units.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "../../include/mpc_gpu.h"
#include "mpc_kernels.cuh"
#include "mpc_nlsetup.h"

namespace {

using mpc::kThreads;
using mpc::kTilePoints;
using mpc::NLConst;

constexpr int kMaxCtas = 64;      // resident CTAs the dA area serves (grid is capped to it)
constexpr int kMaxNt = 2048;      // longest t axis supported
constexpr size_t kDABytes = (size_t)kMaxCtas * kTilePoints * sizeof(float2);   // 8 MiB
constexpr size_t kTwOff = kDABytes;   // packed twiddle table (12 B per entry) in a 16 B-per-entry region
constexpr size_t kWposOff = kTwOff + (size_t)kMaxNt * 16;
constexpr size_t kNoallocBytes = kWposOff + (size_t)kMaxNt * sizeof(float);    // 8,429,568 B

// All scratch of mpc_nonlinear_noalloc: [dA tiles | twiddles | omega per position]
static __device__ __align__(256) unsigned char g_noalloc[kNoallocBytes];

// omega at each FFT position, computed on the host and passed by value (8 KB of kernel
// parameters), so that no call reads host memory asynchronously
struct WposTable {
    float v[kMaxNt];
};

// Packed W_Nt table (mpc_fft.cuh Twiddles: (c, s) then -(c^2 + s^2 - 1)) and the omega of
// each FFT position, into the static array.
__global__ void k_noalloc_tables(int Nt, WposTable wp, float2* tw, float* wpos) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Nt) return;
    double s, c;
    sincos(-2.0 * M_PI * (double)k / (double)Nt, &s, &c);
    const float cf = (float)c, sf = (float)s;
    tw[k] = make_float2(cf, sf);
    reinterpret_cast<float*>(tw + Nt)[k] = (float)-((double)cf * cf + (double)sf * sf - 1.0);
    wpos[k] = wp.v[k];
}

// omega at each position of the in-place forward sweep (radices 16, ..., 16, r_last;
// pos = sum span_s k_s, freq = k_1 + r_1 k_2 + ...), from the centred omega grid w
void omega_of_positions(int Nt, const double* w, WposTable* out) {
    for (int k = 0; k < Nt; k++) {
        int rem = k, freq = 0, mult = 1;
        for (int L = Nt; L > 1;) {
            const int R = (L >= 16) ? 16 : L;
            const int span = L / R;
            const int d = rem / span;
            rem -= d * span;
            freq += d * mult;
            mult *= R;
            L /= R;
        }
        out->v[k] = (float)w[(freq + Nt / 2) % Nt];
    }
}

// The nonlinear stage of the pencil sweep on a real-space complex64 field, in place:
// dA = IFFT_t(-i w FFT_t A)/Nt into this CTA's tile of the static dA area, then
// A *= exp(dz A_nl(A, dA)).
template <int NT, int P>
__global__ void __launch_bounds__(kThreads, 1)
    k_nonlinear_noalloc(float2* A, int NP, int ntiles, float in_scale, float out_scale, NLConst c, float2* dA_area,
                        const float2* tw_g, const float* wpos) {
    using Cfg = mpc::PencilCfg<NT, P, 1>;
    using V = typename Cfg::View;
    static_assert(Cfg::TH == kThreads, "one thread per 32-sample chunk");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* s = reinterpret_cast<float2*>(smem_raw);
    void* scan_mem = smem_raw + Cfg::SMEM_FIELD;
    unsigned char* tw_mem = smem_raw + Cfg::SMEM_FIELD + Cfg::SMEM_SCAN;
    const int tid = threadIdx.x;
    mpc::stage_twiddles<NT, kThreads>(tw_mem, tw_g, tid);
    const mpc::Twiddles tw = mpc::Twiddles::packed(tw_mem, NT);
    __syncthreads();
    float2* scr = dA_area + (size_t)blockIdx.x * NT * P;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int q0 = tile * P;
        if (c.sst_c != 0.0f) {
            for (int f = tid; f < NT * P; f += kThreads) {
                const int t = f / P, p = f - t * P;
                s[V::at(t, p)] = mpc::cscale(A[(size_t)t * NP + q0 + p], in_scale);
            }
            __syncthreads();
            mpc::dif_all<NT, NT, V, kThreads>(s, tw, tid);
            const float inv_nt = 1.0f / (float)NT;
            for (int f = tid; f < NT * P; f += kThreads) {
                const int pos = f / P, p = f - pos * P;
                const int i = V::at(pos, p);
                s[i] = mpc::cscale(mpc::mul_mi<false>(s[i]), wpos[pos] * inv_nt);
            }
            __syncthreads();
            mpc::dit_all<NT, NT, V, kThreads>(s, tw, tid);
            for (int f = tid; f < NT * P; f += kThreads) {
                const int t = f / P, p = f - t * P;
                scr[f] = s[V::at(t, p)];
            }
            __syncthreads();
        }
        for (int f = tid; f < NT * P; f += kThreads) {
            const int t = f / P, p = f - t * P;
            s[V::at(t, p)] = mpc::cscale(A[(size_t)t * NP + q0 + p], in_scale);
        }
        __syncthreads();
        float4 mx = make_float4(0.f, 0.f, 0.f, 0.f);
        mpc::nonlinear_tile<NT, P, false>(s, scr, c, scan_mem, tid, nullptr, nullptr, q0, NP, mx);
        __syncthreads();
        for (int f = tid; f < NT * P; f += kThreads) {
            const int t = f / P, p = f - t * P;
            A[(size_t)t * NP + q0 + p] = mpc::cscale(s[V::at(t, p)], out_scale);
        }
        __syncthreads();
    }
}

struct NtKernel {
    int nt;
    void (*fn)(float2*, int, int, float, float, NLConst, float2*, const float2*, const float*);
    int smem;
};
const NtKernel kKernels[] = {
    {64, k_nonlinear_noalloc<64, 256>, mpc::PencilCfg<64, 256, 1>::SMEM},
    {256, k_nonlinear_noalloc<256, 64>, mpc::PencilCfg<256, 64, 1>::SMEM},
    {512, k_nonlinear_noalloc<512, 32>, mpc::PencilCfg<512, 32, 1>::SMEM},
    {1024, k_nonlinear_noalloc<1024, 16>, mpc::PencilCfg<1024, 16, 1>::SMEM},
    {2048, k_nonlinear_noalloc<2048, 8>, mpc::PencilCfg<2048, 8, 1>::SMEM},
};

// errors are reported on stderr, as the reference's functions report theirs, and as the
// status code
int noalloc_fail(int code, const char* what, cudaError_t e = cudaSuccess) {
    if (e != cudaSuccess) fprintf(stderr, "mpc_nonlinear_noalloc: %s: %s\n", what, cudaGetErrorString(e));
    else fprintf(stderr, "mpc_nonlinear_noalloc: %s\n", what);
    return code;
}

}  // namespace

extern "C" int mpc_nonlinear_noalloc(const mpc_params* p, void* A_dev, double dz, void* stream) {
    if (!p || !A_dev || !p->w) return noalloc_fail(MPC_ERR_ARG, "null argument");
    const int Nx = p->dims[0], Ny = p->dims[1], Nt = p->dims[2];
    if (Nx <= 0 || Ny <= 0 || Nt <= 0) return noalloc_fail(MPC_ERR_ARG, "dims must be positive");
    if (Nt > kMaxNt)
        return noalloc_fail(MPC_ERR_SHAPE, "Nt exceeds the static scratch of mpc_nonlinear_noalloc (at most 2048)");
    int ki = -1;
    for (int i = 0; i < (int)(sizeof(kKernels) / sizeof(kKernels[0])); i++)
        if (kKernels[i].nt == Nt) ki = i;
    if (ki < 0) return noalloc_fail(MPC_ERR_SHAPE, "Nt must be 64, 256, 512, 1024 or 2048");
    const long NP = (long)Nx * Ny;
    const int P = kTilePoints / Nt;
    if (NP % P != 0 || NP > (1L << 30))
        return noalloc_fail(MPC_ERR_SHAPE, "Nx*Ny must be a multiple of 16384/Nt");
    if (!(p->w0 > 0)) return noalloc_fail(MPC_ERR_ARG, "w0 must be positive");
    const double fs = sqrt(mpc::kHBAR * p->w0 / mpc::kIUnit);
    const mpc::NLSetup setup = mpc::nl_setup(*p, fs);
    if (p->plasm == 1 && !setup.gas_ok) return noalloc_fail(MPC_ERR_ARG, "unknown gas");
    NLConst c = setup.nl;
    c.dz = (float)dz;
    WposTable wp;
    omega_of_positions(Nt, p->w, &wp);
    // The device address of g_noalloc, looked up on every call with the caller's device current
    // (in host code the symbol is a host-side stand-in and must never be passed to a kernel);
    // the lookup allocates nothing.  The first call on a device loads this library's device code.
    void* addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc);
    if (e != cudaSuccess || !addr) return noalloc_fail(MPC_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc)", e);
    e = cudaFuncSetAttribute(kKernels[ki].fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kKernels[ki].smem);
    if (e != cudaSuccess) return noalloc_fail(MPC_ERR_CUDA, "cudaFuncSetAttribute", e);
    unsigned char* base = static_cast<unsigned char*>(addr);
    float2* dA_area = reinterpret_cast<float2*>(base);
    float2* tw = reinterpret_cast<float2*>(base + kTwOff);
    float* wpos = reinterpret_cast<float*>(base + kWposOff);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    k_noalloc_tables<<<(Nt + 255) / 256, 256, 0, st>>>(Nt, wp, tw, wpos);
    e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(MPC_ERR_CUDA, "table kernel launch", e);
    const int ntiles = (int)(NP / P);
    const int grid = ntiles < kMaxCtas ? ntiles : kMaxCtas;
    kKernels[ki].fn<<<grid, kThreads, kKernels[ki].smem, st>>>(static_cast<float2*>(A_dev), (int)NP, ntiles,
                                                               (float)fs, (float)(1.0 / fs), c, dA_area, tw, wpos);
    e = cudaGetLastError();
    if (e != cudaSuccess) return noalloc_fail(MPC_ERR_CUDA, "nonlinear kernel launch", e);
    return MPC_OK;
}
