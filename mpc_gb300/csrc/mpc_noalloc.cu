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

#include <mutex>

#include "../../include/mpc_gpu.h"
#include "mpc_kernels.cuh"

namespace {

using mpc::kThreads;
using mpc::kTilePoints;
using mpc::NLConst;

constexpr int kMaxCtas = 64;      // resident CTAs the dA area serves (grid is capped to it)
constexpr int kMaxNt = 2048;      // longest t axis supported
constexpr size_t kDABytes = (size_t)kMaxCtas * kTilePoints * sizeof(float2);   // 8 MiB
constexpr size_t kTwOff = kDABytes;   // packed twiddle table (12 B per entry) in a 16 B-per-entry region
constexpr size_t kWposOff = kTwOff + (size_t)kMaxNt * 16;
constexpr size_t kWOff = kWposOff + (size_t)kMaxNt * sizeof(float);
constexpr size_t kNoallocBytes = kWOff + (size_t)kMaxNt * sizeof(double);      // 8,445,952 B
constexpr int kMaxDevices = 64;

// All scratch of mpc_nonlinear_noalloc: [dA tiles | twiddles | omega per position | omega grid]
static __device__ __align__(256) unsigned char g_noalloc[kNoallocBytes];

// constants.h:1-11
constexpr double ZW0 = 377.0, NC = 1.0, FCTR = 0.89, IH = 27.21, EF = 5.14220642e11;
constexpr double ME = 9.1094e-31, EL0 = 1.602e-19, NAVO = 6.02214e+23, T0 = 2.4188843265e-17;
constexpr double C0 = 299792458.0, HBAR = 1.054560652926899e-34;
constexpr double I_UNIT = 1e16;   // device units: |a|^2 = intensity / 1e16 W/m^2

// ionizpot and Natoms (plasma.c:4-115)
bool gas_constants(const char* gas, double* I1, double* I2, double* Natm, double* sig) {
    struct G { const char* n; double i1, i2, dens, M, sig; };
    static const G g[] = {
        {"Argon", 15.75962, 27.62967, 1.784 * 1e3, 39.941, 1.57e-20},
        {"Helium", 24.58741, 54.41778, 0.166e3, 4.002602, 6.11e-20},
        {"Neon", 21.5646, 40.96328, 0.9002e3, 20.1797, 1.65e-20},
        {"Air", 0.78084 * 14.53414 + 0.20946 * 13.61806 + 0.00934 * 15.75962,
         0.78084 * 29.6013 + 0.20946 * 35.11730 + 0.00934 * 27.62967, 1.205e3, 28.97, 10e-20},
        {"Nitrogen", 14.53414, 29.6013, 1.65e3, 14.0067, 10.2e-20},
        {"Xenon", 12.1298, 21.20979, 5.86e3, 5.761, 3.55e-20},
        {"Krypton", 13.99961, 24.35985, 3.749e3, 83.798, 1.15e-20},
    };
    for (const G& e : g)
        if (strncmp(gas, e.n, 9) == 0) {
            *I1 = e.i1;
            *I2 = e.i2;
            *Natm = e.dens * NAVO / e.M;
            *sig = e.sig;
            return true;
        }
    return false;
}

// FP32 constants of the nonlinear step from the run parameters (FP64 on the host), the same
// physics as the context-based path: ADK with n*_q = q/sqrt(2 Ip_q), drift velocity from w0.
bool nl_constants(const mpc_params& p, double fs, double dz, NLConst* out) {
    NLConst n;
    memset(&n, 0, sizeof n);
    const double fs2 = fs * fs;
    n.dz = (float)dz;
    n.gam = (float)(p.gamma2 / fs2);
    n.sst_c = p.sst_on == 1 ? (float)(p.gamma2 / (p.w0 * fs2)) : 0.0f;
    n.I_scale = (float)I_UNIT;
    const double E_c = sqrt(2.0 * ZW0 / NC) * FCTR / EF;
    n.E_c = (float)E_c;
    n.inv_E_c = (float)(1.0 / E_c);
    double I1 = 0, I2 = 0, Natm = 0, sig = 0;
    const bool gas_ok = gas_constants(p.gas, &I1, &I2, &Natm, &sig);
    if (p.plasm == 1 && !gas_ok) return false;
    if (gas_ok) {
        const double Iion[2] = {I1 / IH, I2 / IH};
        const double nq[2] = {1.0 / sqrt(2.0 * Iion[0]), 2.0 / sqrt(2.0 * Iion[1])};
        for (int s = 0; s < 2; s++) {
            const double Cnl = sqrt(pow(2.0, 2.0 * nq[s]) / (nq[s] * tgamma(nq[s] + 1.0) * tgamma(nq[s])));
            const double K1 = Cnl * Cnl * sqrt(6.0 / M_PI) * Iion[s];
            const double K3 = 2.0 * pow(2.0 * Iion[s], 1.5);
            n.l2K1[s] = (float)log2(K1);
            n.l2K3[s] = (float)log2(K3);
            n.K5[s] = (float)(2.0 * nq[s] - 1.5);
            n.K3l2e[s] = (float)(K3 / (3.0 * M_LN2));
        }
        const double Kon = p.deltat / T0;
        n.Kon = (float)Kon;
        n.Kuv = (float)(sig * p.rho_nt * EL0 * EF / (sqrt(2.0) * ME * p.w0));
        n.K4w0 = (float)((p.w0 / C0) / (p.n0 * p.rho_c) * p.w0 * p.w0);
        n.w0sq = (float)(p.w0 * p.w0);
        n.inv_w0 = (float)(1.0 / p.w0);
        n.invI1_Kon = (float)(Kon / I1);
        n.rho_half = (float)(p.rho_nt / 2.0);
    }
    n.plasma = (p.plasm == 1) ? 1 : 0;
    *out = n;
    return true;
}

// Packed W_Nt table (mpc_fft.cuh Twiddles: (c, s) then -(c^2 + s^2 - 1)) and omega at each
// FFT position of the in-place forward sweep (radices 16, ..., 16, r_last;
// pos = sum span_s k_s, freq = k_1 + r_1 k_2 + ...), from the centred omega grid w.
__global__ void k_noalloc_tables(int Nt, const double* w, float2* tw, float* wpos) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= Nt) return;
    double s, c;
    sincos(-2.0 * M_PI * (double)k / (double)Nt, &s, &c);
    const float cf = (float)c, sf = (float)s;
    tw[k] = make_float2(cf, sf);
    reinterpret_cast<float*>(tw + Nt)[k] = (float)-((double)cf * cf + (double)sf * sf - 1.0);
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
    wpos[k] = (float)w[(freq + Nt / 2) % Nt];
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

std::mutex g_setup_mutex;
void* g_dev_addr[kMaxDevices];            // device address of g_noalloc, per device
bool g_smem_ready[kMaxDevices][sizeof(kKernels) / sizeof(kKernels[0])];

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
    const double fs = sqrt(HBAR * p->w0 / I_UNIT);
    NLConst c;
    if (!nl_constants(*p, fs, dz, &c)) return noalloc_fail(MPC_ERR_ARG, "unknown gas");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_fail(MPC_ERR_CUDA, "cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices) return noalloc_fail(MPC_ERR_ARG, "device index beyond 63");
    {
        // once per device, with that device current: the device address of g_noalloc (in
        // host code the symbol is a host-side stand-in and must not be passed to a kernel)
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_dev_addr[dev]) {
            void* addr = nullptr;
            e = cudaGetSymbolAddress(&addr, g_noalloc);
            if (e != cudaSuccess || !addr) return noalloc_fail(MPC_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc)", e);
            g_dev_addr[dev] = addr;
        }
        if (!g_smem_ready[dev][ki]) {
            e = cudaFuncSetAttribute(kKernels[ki].fn, cudaFuncAttributeMaxDynamicSharedMemorySize, kKernels[ki].smem);
            if (e != cudaSuccess) return noalloc_fail(MPC_ERR_CUDA, "cudaFuncSetAttribute", e);
            g_smem_ready[dev][ki] = true;
        }
    }
    unsigned char* base = static_cast<unsigned char*>(g_dev_addr[dev]);
    float2* dA_area = reinterpret_cast<float2*>(base);
    float2* tw = reinterpret_cast<float2*>(base + kTwOff);
    float* wpos = reinterpret_cast<float*>(base + kWposOff);
    double* w = reinterpret_cast<double*>(base + kWOff);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    e = cudaMemcpyAsync(w, p->w, sizeof(double) * Nt, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return noalloc_fail(MPC_ERR_CUDA, "copy of the omega grid", e);
    k_noalloc_tables<<<(Nt + 255) / 256, 256, 0, st>>>(Nt, w, tw, wpos);
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
