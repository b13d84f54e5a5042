// mpc_capi.cu -- host side of libmpc_gpu.so: the C ABI of include/mpc_gpu.h.
//
// The context owns the device-resident field (complex64, slot layout, see mpc_kernels.cuh),
// the FFT twiddles and position->frequency tables of the three axes, the per-step phase
// tables (computed on the device in FP64 and rounded to complex64) and the scratch of the
// pencil sweep.  Every entry point returns an int status; CUDA errors are reported through
// mpc_last_error().  Host code only sequences kernels and evaluates scalar control logic
// (pass sign, step-size rule); all per-point arithmetic runs on the GPU.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/mpc_gpu.h"
#include "mpc_nlsetup.h"
#include "mpc_shapes.cuh"

using mpc::NLConst;
using mpc::PencilArgs;
using mpc::PlaneArgs;
using mpc::PlaneTables;
using mpc::ShapeOps;

namespace mpc {
extern const ShapeOps* const shape_list_a[];
extern const ShapeOps* const shape_list_b[];
extern const ShapeOps* const shape_list_c[];
extern const ShapeOps* const shape_list_d[];
}  // namespace mpc

// constants.h:1-11 (mpc_nlsetup.h)
static const double HBAR = mpc::kHBAR;
// device units: |a|^2 = intensity / I_UNIT
static const double I_UNIT = mpc::kIUnit;

static thread_local std::string g_err;
static int fail(int code, const char* what, cudaError_t e = cudaSuccess) {
    char buf[512];
    if (e != cudaSuccess) snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
    else snprintf(buf, sizeof buf, "%s", what);
    g_err = buf;
    return code;
}
#define CK(call, what)                                    \
    do {                                                  \
        cudaError_t _e = (call);                          \
        if (_e != cudaSuccess) return fail(MPC_ERR_CUDA, what, _e); \
    } while (0)

// ---------------------------------------------------------------------------------------
// small device kernels: tables, reductions, element-wise ADK
// ---------------------------------------------------------------------------------------
struct TabIn {
    const double* wr;     // centred k grid (Nx == Ny entries)
    const double* betas;  // centred, Nt
    const int* fx;        // position -> FFT frequency index
    const int* fy;
    const int* ft;
    int Nx, Ny, Nt;
    double zd, zp, k0, alpha, scale;
};

// FP64 factors of one linear step (propagation.c:375-391 and kernels.cu:47-54, corrected):
//   Rx[px] = exp(-i zd kap^2 / (2 k0)), kap = wr[m] - wr[N/2], m = centred index of freq(px);
//   D[pos] = scale * exp(zp (i beta[m] - alpha/2)).
// Phase arguments and their range reduction in FP64.
__global__ void k_phase64(TabIn in, double2* Rx, double2* Ry, double2* D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < in.Nx) {
        const int m = (in.fx[i] + in.Nx / 2) % in.Nx;
        const double kap = in.wr[m] - in.wr[in.Nx / 2];
        double s, c;
        sincos(-in.zd * kap * kap / (2.0 * in.k0), &s, &c);
        Rx[i] = make_double2(c, s);
    }
    if (i < in.Ny) {
        const int m = (in.fy[i] + in.Ny / 2) % in.Ny;
        const double kap = in.wr[m] - in.wr[in.Ny / 2];
        double s, c;
        sincos(-in.zd * kap * kap / (2.0 * in.k0), &s, &c);
        Ry[i] = make_double2(c, s);
    }
    if (i < in.Nt) {
        const int m = (in.ft[i] + in.Nt / 2) % in.Nt;
        const double amp = exp(-in.zp * in.alpha / 2.0) * in.scale;
        double s, c;
        sincos(in.zp * in.betas[m], &s, &c);
        D[i] = make_double2(amp * c, amp * s);
    }
}

__device__ __forceinline__ float4 split_df(double2 z) {
    const float hx = (float)z.x, hy = (float)z.y;
    return make_float4(hx, hy, (float)(z.x - (double)hx), (float)(z.y - (double)hy));
}

// Double-float tables of the plane sweep: Rx_df[px] and RyD_df[y * Nt + pos] = Ry[y] D[pos]
// (the product formed in FP64), and the same products slot-major, RyDT_df[pos * Ny + y], so that
// one slot's Ny factors are contiguous (the TMA-staged y pass copies them in one piece).
__global__ void k_split(const double2* Rx, const double2* Ry, const double2* D, int Nx, int Ny, int Nt,
                        float4* Rx_df, float4* RyD_df, float4* RyDT_df) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i < Nx) Rx_df[i] = split_df(Rx[i]);
    if (i < (long)Ny * Nt) {
        const long y = i / Nt, pos = i % Nt;
        const double2 a = Ry[y], b = D[pos];
        const float4 f = split_df(make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x));
        RyD_df[i] = f;
        RyDT_df[pos * Ny + y] = f;
    }
}

// exp(-i k0 r^2 / roc) for the mirror lens (lens bounce mode)
__global__ void k_lens(const double* r, int n, double k0, double roc, float2* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        double s, c;
        sincos(-k0 * r[i] * r[i] / roc, &s, &c);
        out[i] = make_float2((float)c, (float)s);
    }
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    v = (threadIdx.x < blockDim.x / 32) ? sh[threadIdx.x] : 0.0;
    if (w == 0)
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// sum |x|^2 of a complex64 array (FP32 per thread over a short run, FP64 across)
__global__ void k_norm2_c64(const float2* __restrict__ x, long n, double* out) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const float2 v = x[i];
        acc += (double)fmaf(v.x, v.x, v.y * v.y);
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) atomicAdd(out, acc);
}

// sum |a-b|^2 and sum |b|^2 of two complex128 arrays (setStep, propagation.c:624-633)
__global__ void k_diffnorm_c128(const double2* __restrict__ a, const double2* __restrict__ b, long n, double* out) {
    __shared__ double sh[32];
    double s1 = 0.0, s2 = 0.0;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double2 u = a[i], v = b[i];
        const double dx = v.x - u.x, dy = v.y - u.y;
        s1 += dx * dx + dy * dy;
        s2 += v.x * v.x + v.y * v.y;
    }
    s1 = block_sum(s1, sh);
    s2 = block_sum(s2, sh);
    if (threadIdx.x == 0) {
        atomicAdd(out, s1);
        atomicAdd(out + 1, s2);
    }
}

// The reductions below add each thread's values in FP32 over runs of kRun elements and the run
// sums in FP64 (within the thread, then across threads): GB300 issues FP64 at 1/64 of its FP32
// rate, and an FP64 add per element made these passes FP64-bound instead of HBM-bound.  A run sum
// of kRun non-negative FP32 terms is within kRun * 2^-24 (relative) of exact.
constexpr int kRun = 32;

// Richardson combination and error sums of one step-doubling attempt (MPC.c:350-381 and
// propagation.c:624-633, on the device field): out = (4 C2 - C1) / 3 (out may alias C1),
// sums[0] += |C2 - C1|^2, sums[1] += |C2|^2.
__global__ void k_richardson(const float2* C1, const float2* C2, float2* out, long n, double* sums) {
    __shared__ double sh[32];
    double s1 = 0.0, s2 = 0.0;
    const long stride = (long)gridDim.x * blockDim.x;
    long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    while (i < n) {
        float p1 = 0.0f, p2 = 0.0f;
        for (int j = 0; j < kRun && i < n; j++, i += stride) {
            const float2 a = C1[i], b = C2[i];
            const float dx = b.x - a.x, dy = b.y - a.y;
            p1 += fmaf(dx, dx, dy * dy);
            p2 += fmaf(b.x, b.x, b.y * b.y);
            out[i] = make_float2(fmaf(4.0f / 3.0f, b.x, -a.x / 3.0f), fmaf(4.0f / 3.0f, b.y, -a.y / 3.0f));
        }
        s1 += (double)p1;
        s2 += (double)p2;
    }
    s1 = block_sum(s1, sh);
    s2 = block_sum(s2, sh);
    if (threadIdx.x == 0) {
        atomicAdd(sums, s1);
        atomicAdd(sums + 1, s2);
    }
}

// E[q] = scale * sum over the Nt slots of |S[slot, q]|^2 (slot layout), one thread per pencil
__global__ void k_pencil_energy_slots(const float2* __restrict__ S, int NP, int Nt, int SLO, double scale, double* E) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= NP) return;
    double acc = 0.0;
    for (int s0 = 0; s0 < Nt; s0 += kRun) {
        float part = 0.0f;
        const int s1 = s0 + kRun < Nt ? s0 + kRun : Nt;
        for (int s = s0; s < s1; s++) {
            const float2 v = S[((size_t)(s / SLO) * NP + q) * SLO + (s % SLO)];
            part = fmaf(v.x, v.x, fmaf(v.y, v.y, part));
        }
        acc += (double)part;
    }
    E[q] = acc * scale;
}

// Moments of the field S (slot layout) for the step-size features:
// out = {sum |S|^2, sum w|S|^2, sum w^2|S|^2, sum x|S|^2, sum x^2|S|^2, sum y|S|^2, sum y^2|S|^2}
// (w = omega offset of the slot, x, y = transverse positions, rf = r in FP32) and
// mx = max |S|^2 (bit pattern).  A block takes whole omega-slots (w is the block's constant
// there) and walks their rows; blockDim.x = Nx clamped to [32, 256] (a multiple of 32).
__global__ void k_moments(const float2* __restrict__ S, int Nt, int NP, int Nx, int Ny, int SLO,
                          const float* __restrict__ wpos, const float* __restrict__ rf, double* out, unsigned int* mx) {
    __shared__ double sh[32];
    double m[7] = {0, 0, 0, 0, 0, 0, 0};
    float vmax = 0.0f;
    for (int slot = blockIdx.x; slot < Nt; slot += gridDim.x) {
        const size_t base = (size_t)(slot / SLO) * NP * SLO + (slot % SLO);
        double a[5] = {0, 0, 0, 0, 0};   // e, x e, x^2 e, y e, y^2 e of this slot
        for (int y0 = 0; y0 < Ny; y0 += kRun) {
            float p[5] = {0, 0, 0, 0, 0};
            const int y1 = y0 + kRun < Ny ? y0 + kRun : Ny;
            for (int y = y0; y < y1; y++) {
                const float yv = rf[y];
                for (int x = threadIdx.x; x < Nx; x += blockDim.x) {
                    const float2 v = S[base + (size_t)(y * Nx + x) * SLO];
                    const float e = fmaf(v.x, v.x, v.y * v.y);
                    const float xv = rf[x], xe = xv * e, ye = yv * e;
                    p[0] += e;
                    p[1] += xe;
                    p[2] = fmaf(xv, xe, p[2]);
                    p[3] += ye;
                    p[4] = fmaf(yv, ye, p[4]);
                    vmax = fmaxf(vmax, e);
                }
            }
#pragma unroll
            for (int k = 0; k < 5; k++) a[k] += (double)p[k];
        }
        const double w = wpos[slot];
        m[0] += a[0];
        m[1] += w * a[0];
        m[2] += w * w * a[0];
        m[3] += a[1];
        m[4] += a[2];
        m[5] += a[3];
        m[6] += a[4];
    }
    for (int k = 0; k < 7; k++) {
        const double t = block_sum(m[k], sh);
        if (threadIdx.x == 0) atomicAdd(out + k, t);
    }
    for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, __float_as_uint(vmax));
}

// spec[freq(pos)] = scale * sum_q |S[pos, q]|^2 for the slot layout; one block per slot
__global__ void k_spec(const float2* __restrict__ S, int NP, int SLO, const int* ft, double scale, double* spec) {
    __shared__ double sh[32];
    const int pos = blockIdx.x;
    double acc = 0.0;
    const size_t base = (size_t)(pos / SLO) * NP * SLO + (pos % SLO);
    int q = threadIdx.x;
    while (q < NP) {
        float part = 0.0f;
        for (int j = 0; j < kRun && q < NP; j++, q += blockDim.x) {
            const float2 v = S[base + (size_t)q * SLO];
            part = fmaf(v.x, v.x, fmaf(v.y, v.y, part));
        }
        acc += (double)part;
    }
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) spec[ft[pos]] = acc * scale;
}

// BP1[x] = sum_y E[y*Nx + x], BP2[y] = sum_x E[y*Nx + x] from per-pencil sums E
__global__ void k_beam_profiles(const double* E, int Nx, int Ny, double* BP1, double* BP2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < Nx) {
        double s = 0.0;
        for (int y = 0; y < Ny; y++) s += E[(size_t)y * Nx + i];
        BP1[i] = s;
    }
    if (i < Ny) {
        double s = 0.0;
        for (int x = 0; x < Nx; x++) s += E[(size_t)i * Nx + x];
        BP2[i] = s;
    }
}

struct ADKConst {
    double Kon1, Kon2, Kon3, Kon4, Kon5, Kon6;
};
// plasma.c:43-58 in FP64
__global__ void k_adk(long n, const double* __restrict__ E, double* r1, double* r2, ADKConst k) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double e = E[i];
        r1[i] = k.Kon1 * pow(k.Kon3 / e, k.Kon5) * exp(-k.Kon3 / (3.0 * e));
        r2[i] = k.Kon2 * pow(k.Kon4 / e, k.Kon6) * exp(-k.Kon4 / (3.0 * e));
    }
}

// ---------------------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------------------
struct TableSet {
    float4* Rx = nullptr;       // double-float Rx, Nx
    float4* RyD = nullptr;      // double-float Ry x D, Ny * Nt
    float4* RyDT = nullptr;     // the same, slot-major: Nt * Ny
    double2* f64 = nullptr;     // FP64 Rx (Nx), Ry (Ny), D (Nt); base of the allocation
};

struct mpc_ctx {
    const ShapeOps* ops = nullptr;
    int variant = 0;    // index of ops among the compiled variants of the grid
    int Nx = 0, Ny = 0, Nt = 0;
    long NP = 0, N = 0;
    mpc_params p{};
    std::vector<double> betas, wr, w, r;
    double fs = 1.0;    // device units per physical field unit
    NLConst nl{};
    float sst_c_full = 0.0f;  // self-steepening prefactor when switched on
    int ion_gas_ok = 0;
    double I1 = 0, I2 = 0;
    ADKConst adk{};
    cudaStream_t st = nullptr;
    int nsm = 0, pencil_grid = 0, plane_clusters = 0;
    int dev = 0;                // the device the context was created on
    float2* S = nullptr;        // state, slot layout
    float2* scratch = nullptr;
    double2* io = nullptr;      // complex128 staging, N
    double2* io2 = nullptr;     // second complex128 staging (setStep)
    float2 *twx = nullptr, *twy = nullptr, *twt = nullptr;  // packed twiddle tables
    float2 *C1 = nullptr, *C2 = nullptr;                    // step doubling (allocated on first use)
    double* hsd = nullptr;   // pinned: error sums and C2's beam profiles of the last attempt (2 + Nx + Ny)
    unsigned int* dstats = nullptr;  // running maxima of the split steps since the last reset (4),
                                     // then at dstats[4] the kernels' error word
    double* dmom = nullptr;          // field moments (7 doubles) and max |S|^2 (bits, after them)
    double sd_dz = 0.0;      // dz of the attempt in flight
    double sd_natural = 0.0; // the step before landing on a mirror plane shortened it
    int sd_clipped = 0;      // the attempt in flight was shortened to land on a mirror plane
    int capturing = 0;       // launches are being captured into a CUDA graph (no synchronous calls)
    float* wpos = nullptr;
    int *dfx = nullptr, *dfy = nullptr, *dft = nullptr;
    std::vector<int> hfx, hfy, hft;
    double *dwr = nullptr, *dbetas = nullptr, *dr = nullptr;
    float* rf = nullptr;        // r in FP32 (after dr in the same allocation)
    float2 *lensx = nullptr, *lensy = nullptr;
    double* penergy = nullptr;  // NP
    double* dred = nullptr;     // reduction outputs (2 Nt + Nx + Ny + 64 doubles)
    std::map<std::tuple<double, double, double>, TableSet> tables;
    TableSet ident;             // identity tables (zd = zp = 0, scale 1/(NxNy))
    mpc_state state{};
    int have_field = 0;
    long launches = 0;          // kernels launched by this context
    int profiling = 0;          // bracket sweeps with events
    struct Ev { int kind; cudaEvent_t a, b; };
    std::vector<Ev> events;     // kind 0 = pencil sweep, 1 = plane sweep
};

static void prof_begin(mpc_ctx* c, int kind, cudaEvent_t* a) {
    (void)kind;
    *a = nullptr;
    if (!c->profiling) return;
    cudaEventCreate(a);
    cudaEventRecord(*a, c->st);
}
static void prof_end(mpc_ctx* c, int kind, cudaEvent_t a) {
    if (!c->profiling || !a) return;
    cudaEvent_t b;
    cudaEventCreate(&b);
    cudaEventRecord(b, c->st);
    c->events.push_back(mpc_ctx::Ev{kind, a, b});
}
static void prof_clear(mpc_ctx* c) {
    for (auto& e : c->events) {
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    c->events.clear();
}

// Compiled variant `variant` (0 = the first) of a grid shape, or null.
static const ShapeOps* find_shape(int Nx, int Ny, int Nt, int variant = 0) {
    const ShapeOps* const* lists[] = {mpc::shape_list_a, mpc::shape_list_b, mpc::shape_list_c, mpc::shape_list_d};
    int k = 0;
    for (auto l : lists)
        for (int i = 0; l[i]; i++)
            if (l[i]->Nx == Nx && l[i]->Ny == Ny && l[i]->Nt == Nt && k++ == variant) return l[i];
    return nullptr;
}

// Position -> FFT frequency index of the in-place DIF sweep with radices 16,...,16,r_last
// (mpc_fft.cuh): pos = sum_s span_s k_s, freq = k_1 + r_1 k_2 + r_1 r_2 k_3 + ...
static std::vector<int> freq_of_pos(int N) {
    std::vector<int> radix, span;
    for (int L = N; L > 1;) {
        const int R = (L >= 16) ? 16 : L;
        radix.push_back(R);
        span.push_back(L / R);
        L /= R;
    }
    std::vector<int> f(N);
    for (int pos = 0; pos < N; pos++) {
        int rem = pos, freq = 0, mult = 1;
        for (size_t s = 0; s < radix.size(); s++) {
            const int k = rem / span[s];
            rem -= k * span[s];
            freq += k * mult;
            mult *= radix[s];
        }
        f[pos] = freq;
    }
    return f;
}

// Packed W_N table (mpc_fft.cuh Twiddles): N float2 W_N^k rounded to FP32 from FP64, then N
// float -(|W|^2 - 1) of the rounded values
static int upload_twiddles(int N, float2** d) {
    std::vector<float> h(3 * (size_t)N);
    for (int k = 0; k < N; k++) {
        const double a = -2.0 * M_PI * (double)k / (double)N;
        const float c = (float)cos(a), s = (float)sin(a);
        const double eps = (double)c * c + (double)s * s - 1.0;
        h[2 * k] = c;
        h[2 * k + 1] = s;
        h[2 * (size_t)N + k] = (float)-eps;
    }
    CK(cudaMalloc(d, mpc::twiddle_bytes(N)), "cudaMalloc twiddles");
    CK(cudaMemcpy(*d, h.data(), mpc::twiddle_bytes(N), cudaMemcpyHostToDevice), "copy twiddles");
    return MPC_OK;
}

static int pass_sign(double z, double Cav) { return ((int)(floor(z / Cav) + 1) % 2) * 2 - 1; }

// FP32 constants of the fused nonlinear step (plasma.c:118-245, propagation.c:244-327;
// A11 and A18 corrections applied), from the setup shared with mpc_noalloc.cu
static void build_nl(mpc_ctx* c) {
    const mpc::NLSetup s = mpc::nl_setup(c->p, c->fs);
    c->nl = s.nl;
    c->sst_c_full = s.sst_c_full;
    c->ion_gas_ok = s.gas_ok;
    c->I1 = s.I1;
    c->I2 = s.I2;
    c->adk = ADKConst{s.K1[0], s.K1[1], s.K3[0], s.K3[1], s.K5[0], s.K5[1]};
}

// one allocation: FP64 factors (Nx + Ny + Nt double2), double-float Rx (Nx) and RyD (Ny*Nt)
static int alloc_tables(mpc_ctx* c, TableSet* t) {
    const size_t n64 = (size_t)(c->Nx + c->Ny + c->Nt);
    const size_t bytes = n64 * sizeof(double2) + ((size_t)c->Nx + 2 * (size_t)c->Ny * c->Nt) * sizeof(float4);
    char* buf = nullptr;
    CK(cudaMalloc(&buf, bytes), "cudaMalloc tables");
    t->f64 = reinterpret_cast<double2*>(buf);
    t->Rx = reinterpret_cast<float4*>(buf + n64 * sizeof(double2));
    t->RyD = t->Rx + c->Nx;
    t->RyDT = t->RyD + (size_t)c->Ny * c->Nt;
    return MPC_OK;
}

static int split_tables(mpc_ctx* c, const TableSet& t) {
    const long n = (long)c->Ny * c->Nt;
    k_split<<<(int)((n + 255) / 256), 256, 0, c->st>>>(t.f64, t.f64 + c->Nx, t.f64 + c->Nx + c->Ny, c->Nx, c->Ny,
                                                       c->Nt, t.Rx, t.RyD, t.RyDT);
    CK(cudaGetLastError(), "k_split");
    c->launches++;
    return MPC_OK;
}

// Adaptive runs meet a new step length every few steps: once the cache holds more than 64
// table sets, free them all.  Called at the start of an operation, before its first
// get_tables, and never while launches are being captured: the sets an operation looks up stay
// valid until its launches are queued, and the stream synchronisation here retires every launch
// that used a freed set.
static void recycle_tables(mpc_ctx* c) {
    if (c->tables.size() <= 64 || c->capturing) return;
    cudaStreamSynchronize(c->st);
    for (auto& kv : c->tables) cudaFree(kv.second.f64);
    c->tables.clear();
}

static int get_tables(mpc_ctx* c, double zd, double zp, double scale, TableSet* out) {
    auto key = std::make_tuple(zd, zp, scale);
    auto it = c->tables.find(key);
    if (it != c->tables.end()) {
        *out = it->second;
        return MPC_OK;
    }
    TableSet t;
    int rc = alloc_tables(c, &t);
    if (rc) return rc;
    TabIn in{c->dwr, c->dbetas, c->dfx, c->dfy, c->dft, c->Nx, c->Ny, c->Nt, zd, zp, c->p.k0, c->p.alpha, scale};
    const int n = c->Nt > c->Nx ? c->Nt : c->Nx;
    k_phase64<<<(n + 255) / 256, 256, 0, c->st>>>(in, t.f64, t.f64 + c->Nx, t.f64 + c->Nx + c->Ny);
    CK(cudaGetLastError(), "k_phase64");
    if ((rc = split_tables(c, t))) return rc;
    c->launches++;
    c->tables[key] = t;
    *out = t;
    return MPC_OK;
}

static int launch_pencil(mpc_ctx* c, int mode, PencilArgs a) {
    a.scratch = c->scratch;
    a.tw = c->twt;
    a.wpos = c->wpos;
    a.NP = (int)c->NP;
    a.ntiles = (int)(c->NP / c->ops->P);
    cudaEvent_t ev;
    prof_begin(c, 0, &ev);
    CK(c->ops->pencil(mode, a, c->pencil_grid, c->st), "pencil kernel launch");
    prof_end(c, 0, ev);
    c->launches++;
    return MPC_OK;
}

static int launch_plane(mpc_ctx* c, const float2* in, float2* out, const TableSet& t1, const TableSet* t2) {
    PlaneArgs a{};
    a.in = in;
    a.out = out;
    a.twx = c->twx;
    a.twy = c->twy;
    a.t1 = PlaneTables{t1.Rx, t1.RyD, t1.RyDT};
    if (t2) {
        a.t2 = PlaneTables{t2->Rx, t2->RyD, t2->RyDT};
        a.lens = 1;
    } else {
        a.t2 = a.t1;
        a.lens = 0;
    }
    a.lensx = c->lensx;
    a.lensy = c->lensy;
    a.err = c->dstats + 4;
    a.Nt = c->Nt;
    a.NP = (int)c->NP;
    a.nunits = c->ops->SLO == 2 ? c->Nt / 2 : c->Nt / c->ops->PB;
    cudaEvent_t ev;
    prof_begin(c, 1, &ev);
    CK(c->ops->plane(a, c->plane_clusters, c->st), "plane kernel launch");
    prof_end(c, 1, ev);
    c->launches += c->ops->PL >= 2 ? 2 + a.lens : 1;
    return MPC_OK;
}

static int ensure_io(mpc_ctx* c, int which) {
    double2** b = which == 0 ? &c->io : &c->io2;
    if (!*b) {
        if (cudaMalloc(b, sizeof(double2) * c->N) != cudaSuccess) {
            *b = nullptr;
            return fail(MPC_ERR_NOMEM, "cudaMalloc complex128 staging");
        }
    }
    return MPC_OK;
}

// Field-sized host <-> device copies.  When the host buffer is page-locked and mapped into the
// address space of the context's device (cudaMallocHost, mpc_host_alloc or cudaHostRegister while
// that device was current), SMs move it with 16-byte loads and stores over the host link: on
// GB300 that runs at the link's rate every time, while a copy-engine transfer that follows a
// second or more without host-link traffic (the normal case after a propagation pass) was
// measured at a third of it or less.  Pageable or unaligned buffers go through cudaMemcpyAsync.
__global__ void k_host_copy(const float4* __restrict__ src, float4* __restrict__ dst, size_t n) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// the device address of page-locked host memory at p mapped for device dev (allocated or
// registered while dev was current), or null
static void* mapped_host(const void* p, int dev) {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (at.type == cudaMemoryTypeHost && at.device == dev) ? at.devicePointer : nullptr;
}

static int field_copy(mpc_ctx* c, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, const char* what) {
    const void* host = kind == cudaMemcpyHostToDevice ? src : dst;
    void* hdev = mapped_host(host, c->dev);
    const bool aligned = ((uintptr_t)dst % 16 == 0) && ((uintptr_t)src % 16 == 0) && bytes % 16 == 0;
    if (hdev && aligned && bytes > 0) {
        const float4* s = reinterpret_cast<const float4*>(kind == cudaMemcpyHostToDevice ? hdev : src);
        float4* d = reinterpret_cast<float4*>(kind == cudaMemcpyHostToDevice ? dst : hdev);
        k_host_copy<<<2 * c->nsm, 256, 0, c->st>>>(s, d, bytes / 16);
        CK(cudaGetLastError(), what);
        c->launches++;
        return MPC_OK;
    }
    CK(cudaMemcpyAsync(dst, src, bytes, kind, c->st), what);
    return MPC_OK;
}

extern "C" {

const char* mpc_version(void) { return "mpc_gb300 0.1 (sm_103a)"; }
const char* mpc_last_error(void) { return g_err.c_str(); }
int mpc_shape_supported(int Nx, int Ny, int Nt) { return find_shape(Nx, Ny, Nt) ? 1 : 0; }

int mpc_destroy(mpc_ctx* c) {
    if (!c) return MPC_OK;
    if (c->st) cudaStreamSynchronize(c->st);
    prof_clear(c);
    for (auto& kv : c->tables) cudaFree(kv.second.f64);
    if (c->ident.f64) cudaFree(c->ident.f64);
    if (c->hsd) cudaFreeHost(c->hsd);
    // only the base of each allocation: dfy/dft, dbetas/dr and lensy point inside dfx, dwr
    // and lensx, and cudaFree of an interior pointer fails and leaves an error pending in the
    // (process-wide) runtime for the caller's next CUDA call
    void* ptrs[] = {c->S,   c->scratch, c->io,  c->io2,     c->twx,    c->twy,  c->twt,
                    c->wpos, c->dfx,    c->dwr, c->lensx,   c->penergy, c->dred, c->C1, c->C2,
                    c->dstats, c->dmom};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
    return MPC_OK;
}

static int autotune_variant(const mpc_params* p, int* best);

int mpc_create(mpc_ctx** out, const mpc_params* p) {
    if (!out || !p) return fail(MPC_ERR_ARG, "null argument");
    *out = nullptr;
    const int Nx = p->dims[0], Ny = p->dims[1], Nt = p->dims[2];
    if (Nx != Ny) return fail(MPC_ERR_SHAPE, "the k grid wr of param.bin serves both x and y: Nx must equal Ny");
    if (!find_shape(Nx, Ny, Nt)) return fail(MPC_ERR_SHAPE, "grid shape not compiled into libmpc_gpu");
    if (p->variant < -1) return fail(MPC_ERR_ARG, "variant must be -1 (autotune) or a variant index");
    if (p->variant == -1) {
        mpc_params q = *p;
        int rc = autotune_variant(p, &q.variant);
        if (rc) return rc;
        return mpc_create(out, &q);
    }
    const ShapeOps* ops = find_shape(Nx, Ny, Nt, p->variant > 0 ? p->variant : 0);
    if (!ops) return fail(MPC_ERR_ARG, "no such kernel variant of this grid shape");
    if (!p->betas || !p->wr || !p->w || !p->r) return fail(MPC_ERR_ARG, "null parameter array");
    if (!(p->k0 > 0) || !(p->w0 > 0) || !(p->Cav > 0)) return fail(MPC_ERR_ARG, "k0, w0 and Cav must be positive");
    mpc_ctx* c = new mpc_ctx();
    c->ops = ops;
    c->variant = p->variant > 0 ? p->variant : 0;
    c->Nx = Nx;
    c->Ny = Ny;
    c->Nt = Nt;
    c->NP = (long)Nx * Ny;
    c->N = c->NP * Nt;
    c->p = *p;
    c->betas.assign(p->betas, p->betas + Nt);
    c->wr.assign(p->wr, p->wr + Ny);
    c->w.assign(p->w, p->w + Nt);
    c->r.assign(p->r, p->r + Ny);
    c->p.betas = c->betas.data();
    c->p.wr = c->wr.data();
    c->p.w = c->w.data();
    c->p.r = c->r.data();
    c->p.gas[8] = 0;
    c->fs = sqrt(HBAR * p->w0 / I_UNIT);
    build_nl(c);
    int rc;
#define TRY(x)                      \
    if ((rc = (x)) != MPC_OK) {     \
        mpc_destroy(c);             \
        return rc;                  \
    }
#define TRYC(x, what)                                  \
    {                                                  \
        cudaError_t _e = (x);                          \
        if (_e != cudaSuccess) {                       \
            mpc_destroy(c);                            \
            return fail(MPC_ERR_CUDA, what, _e);       \
        }                                              \
    }
    int dev = 0;
    TRYC(cudaGetDevice(&dev), "cudaGetDevice");
    c->dev = dev;
    TRYC(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, dev), "SM count");
    TRYC(ops->setup(), "kernel attribute setup");
    TRYC(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking), "cudaStreamCreate");
    const int ntiles = (int)(c->NP / ops->P);
    const int per_sm = ops->pencil_blocks_per_sm();
    if (per_sm <= 0) {
        mpc_destroy(c);
        return fail(MPC_ERR_CUDA, "pencil sweep configuration cannot be scheduled on this device");
    }
    c->pencil_grid = ntiles < c->nsm * per_sm ? ntiles : c->nsm * per_sm;
    const int nunits = ops->SLO == 2 ? Nt / 2 : Nt / ops->PB;
    int mc = ops->max_clusters();
    if (mc <= 0) {
        mpc_destroy(c);
        return fail(MPC_ERR_CUDA, "plane cluster configuration cannot be scheduled on this device");
    }
    c->plane_clusters = mc < nunits ? mc : nunits;
    if (cudaMalloc(&c->S, sizeof(float2) * c->N) != cudaSuccess) {
        mpc_destroy(c);
        return fail(MPC_ERR_NOMEM, "cudaMalloc field");
    }
    TRYC(cudaMalloc(&c->scratch, sizeof(float2) * (size_t)c->pencil_grid * ops->P * Nt), "cudaMalloc scratch");
    TRY(upload_twiddles(Nx, &c->twx));
    TRY(upload_twiddles(Ny, &c->twy));
    TRY(upload_twiddles(Nt, &c->twt));
    c->hfx = freq_of_pos(Nx);
    c->hfy = freq_of_pos(Ny);
    c->hft = freq_of_pos(Nt);
    TRYC(cudaMalloc(&c->dfx, sizeof(int) * (Nx + Ny + Nt)), "cudaMalloc freq tables");
    c->dfy = c->dfx + Nx;
    c->dft = c->dfy + Ny;
    TRYC(cudaMemcpy(c->dfx, c->hfx.data(), sizeof(int) * Nx, cudaMemcpyHostToDevice), "copy fx");
    TRYC(cudaMemcpy(c->dfy, c->hfy.data(), sizeof(int) * Ny, cudaMemcpyHostToDevice), "copy fy");
    TRYC(cudaMemcpy(c->dft, c->hft.data(), sizeof(int) * Nt, cudaMemcpyHostToDevice), "copy ft");
    {
        // omega of each t position: wbuff = fftshift(w) (propagation.c:170-177) indexed by freq(pos)
        std::vector<float> wp(Nt);
        for (int pos = 0; pos < Nt; pos++) wp[pos] = (float)c->w[(c->hft[pos] + Nt / 2) % Nt];
        TRYC(cudaMalloc(&c->wpos, sizeof(float) * Nt), "cudaMalloc wpos");
        TRYC(cudaMemcpy(c->wpos, wp.data(), sizeof(float) * Nt, cudaMemcpyHostToDevice), "copy wpos");
    }
    TRYC(cudaMalloc(&c->dwr, sizeof(double) * (Ny + Nt + Ny) + sizeof(float) * Ny), "cudaMalloc FP64 grids");
    c->dbetas = c->dwr + Ny;
    c->dr = c->dbetas + Nt;
    c->rf = reinterpret_cast<float*>(c->dr + Ny);
    TRYC(cudaMemcpy(c->dwr, c->wr.data(), sizeof(double) * Ny, cudaMemcpyHostToDevice), "copy wr");
    TRYC(cudaMemcpy(c->dbetas, c->betas.data(), sizeof(double) * Nt, cudaMemcpyHostToDevice), "copy betas");
    TRYC(cudaMemcpy(c->dr, c->r.data(), sizeof(double) * Ny, cudaMemcpyHostToDevice), "copy r");
    {
        std::vector<float> rf(c->r.begin(), c->r.end());
        TRYC(cudaMemcpy(c->rf, rf.data(), sizeof(float) * Ny, cudaMemcpyHostToDevice), "copy r (FP32)");
    }
    TRYC(cudaMalloc(&c->lensx, sizeof(float2) * (Nx + Ny)), "cudaMalloc lens");
    c->lensy = c->lensx + Nx;
    if (p->bounce_mode == MPC_BOUNCE_LENS && p->roc != 0.0) {
        k_lens<<<(Nx + 255) / 256, 256, 0, c->st>>>(c->dr, Nx, p->k0, p->roc, c->lensx);
        k_lens<<<(Ny + 255) / 256, 256, 0, c->st>>>(c->dr, Ny, p->k0, p->roc, c->lensy);
        TRYC(cudaGetLastError(), "k_lens");
    }
    TRYC(cudaMalloc(&c->penergy, sizeof(double) * c->NP), "cudaMalloc pencil energies");
    // reductions: temp [0, Nt), spec [Nt, 2 Nt), beam profiles and sums use the front
    TRYC(cudaMalloc(&c->dred, sizeof(double) * (2 * Nt + Nx + Ny + 64)), "cudaMalloc reductions");
    // four running maxima, then the kernels' error word (KernelError)
    TRYC(cudaMalloc(&c->dstats, 8 * sizeof(unsigned int)), "cudaMalloc step statistics");
    TRYC(cudaMemsetAsync(c->dstats, 0, 8 * sizeof(unsigned int), c->st), "memset step statistics");
    TRYC(cudaMalloc(&c->dmom, 8 * sizeof(double)), "cudaMalloc field moments");
    {
        TRY(alloc_tables(c, &c->ident));
        TabIn in{c->dwr, c->dbetas, c->dfx, c->dfy, c->dft, Nx, Ny, Nt, 0.0, 0.0, p->k0, p->alpha,
                 1.0 / (double)c->NP};
        const int n = Nt > Nx ? Nt : Nx;
        k_phase64<<<(n + 255) / 256, 256, 0, c->st>>>(in, c->ident.f64, c->ident.f64 + Nx, c->ident.f64 + Nx + Ny);
        TRYC(cudaGetLastError(), "k_phase64 identity");
        TRY(split_tables(c, c->ident));
    }
    TRYC(cudaStreamSynchronize(c->st), "context setup");
    c->state.dzz = p->dzz;
    c->state.puls_e = p->puls_e;
    c->state.signmem = 1;
#undef TRY
#undef TRYC
    *out = c;
    return MPC_OK;
}

// The autotuner: the fastest compiled variant of a grid on the current device.  Each variant
// (device layout, pencil tile, plane cluster shape and CTA size; all give identical results)
// runs 2 + 3 split steps -- one pencil sweep and one plane sweep each -- on a zero field in a
// context of its own, timed with CUDA events over the last 3.  The choice is cached per device
// and grid for the life of the process.  The nonlinear step's cost depends on the field, but
// the shapes compared here do not change that part.
static int pencil_step(mpc_ctx* c, double dz, float2* buf);

static int autotune_variant(const mpc_params* p, int* best) {
    static std::mutex mu;
    static std::map<std::tuple<int, int, int, int>, int> cache;
    int dev = 0;
    CK(cudaGetDevice(&dev), "cudaGetDevice");
    const auto key = std::make_tuple(dev, p->dims[0], p->dims[1], p->dims[2]);
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find(key);
    if (it != cache.end()) {
        *best = it->second;
        return MPC_OK;
    }
    int nvar = 0;
    while (find_shape(p->dims[0], p->dims[1], p->dims[2], nvar)) nvar++;
    float best_ms = 0.0f;
    *best = -1;
    for (int v = 0; v < nvar; v++) {
        mpc_params q = *p;
        q.variant = v;
        mpc_ctx* c = nullptr;
        if (mpc_create(&c, &q) != MPC_OK) {  // e.g. a cluster shape this device cannot place
            cudaGetLastError();                  // leave no error pending for the caller
            continue;
        }
        float ms = -1.0f;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        bool ok = cudaMemsetAsync(c->S, 0, sizeof(float2) * c->N, c->st) == cudaSuccess &&
                  cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess;
        TableSet t;
        ok = ok && get_tables(c, q.dzz, q.dzz, 1.0 / ((double)c->NP * c->Nt), &t) == MPC_OK;
        for (int i = 0; ok && i < 5; i++) {
            if (i == 2) ok = cudaEventRecord(e0, c->st) == cudaSuccess;
            ok = ok && pencil_step(c, q.dzz, nullptr) == MPC_OK && launch_plane(c, c->S, c->S, t, nullptr) == MPC_OK;
        }
        ok = ok && cudaEventRecord(e1, c->st) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess &&
             cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        mpc_destroy(c);
        if (ok && (*best < 0 || ms < best_ms)) {
            *best = v;
            best_ms = ms;
        }
    }
    if (*best < 0) return fail(MPC_ERR_CUDA, "autotuner: no kernel variant of this grid ran on this device");
    cache[key] = *best;
    return MPC_OK;
}

int mpc_variant_info(mpc_ctx* c, int* variant, int* info) {
    if (!c || !variant || !info) return fail(MPC_ERR_ARG, "null argument");
    *variant = c->variant;
    const int v[10] = {c->ops->P, c->ops->SLO, c->ops->CL, c->ops->PB, c->ops->PT, c->pencil_grid,
                       c->plane_clusters, c->ops->P * c->Nt / c->ops->CH, c->ops->LD, c->ops->PL};
    for (int i = 0; i < 10; i++) info[i] = v[i];
    return MPC_OK;
}

// The wait-limit probe: one thread waits on an mbarrier that no copy and no thread completes; the
// bounded wait gives up after kWaitLimitCycles and the kernel leaves KERR_WAIT_PROBE in *err.
__global__ void k_wait_limit_probe(unsigned int* err) {
    __shared__ uint64_t bar;
    mpc::mbar_init(&bar, 1);
    mpc::fence_mbar_init();
    if (!mpc::mbar_wait(&bar, 0)) atomicExch(err, mpc::KERR_WAIT_PROBE);
}

// After a stream synchronisation: a kernel that gave up a bounded wait left its code in the
// error word (the field is then incomplete).  The word is cleared once reported.
static int kernel_errors(mpc_ctx* c) {
    unsigned int w = 0;
    CK(cudaMemcpy(&w, c->dstats + 4, sizeof w, cudaMemcpyDeviceToHost), "D2H kernel error word");
    if (w == mpc::KERR_NONE) return MPC_OK;
    CK(cudaMemset(c->dstats + 4, 0, sizeof w), "clear kernel error word");
    return fail(MPC_ERR_TIMEOUT, w == mpc::KERR_TMA_TIMEOUT   ? "a bulk tensor load did not arrive within the wait limit"
                                 : w == mpc::KERR_WAIT_PROBE ? "the wait-limit probe's wait ran out"
                                                             : "kernel error word set");
}

int mpc_wait_limit_check(mpc_ctx* c) {
    if (!c) return fail(MPC_ERR_ARG, "null context");
    k_wait_limit_probe<<<1, 1, 0, c->st>>>(c->dstats + 4);
    CK(cudaGetLastError(), "k_wait_limit_probe");
    c->launches++;
    CK(cudaStreamSynchronize(c->st), "wait-limit probe");
    return kernel_errors(c);
}

int mpc_sync(mpc_ctx* c) {
    if (!c) return fail(MPC_ERR_ARG, "null context");
    CK(cudaStreamSynchronize(c->st), "stream synchronize");
    return kernel_errors(c);
}

int mpc_host_alloc(void** ptr, size_t bytes) {
    if (!ptr) return fail(MPC_ERR_ARG, "null argument");
    *ptr = nullptr;
    cudaError_t e = cudaMallocHost(ptr, bytes);
    if (e != cudaSuccess) return fail(MPC_ERR_NOMEM, "cudaMallocHost", e);
    return MPC_OK;
}

int mpc_host_free(void* ptr) {
    if (ptr) CK(cudaFreeHost(ptr), "cudaFreeHost");
    return MPC_OK;
}

int mpc_stream_handle(mpc_ctx* c, void** stream) {
    if (!c || !stream) return fail(MPC_ERR_ARG, "null argument");
    *stream = (void*)c->st;
    return MPC_OK;
}

long mpc_launch_count(mpc_ctx* c) { return c ? c->launches : -1; }

int mpc_profile(mpc_ctx* c, int on) {
    if (!c) return fail(MPC_ERR_ARG, "null context");
    CK(cudaStreamSynchronize(c->st), "profile sync");
    prof_clear(c);
    c->profiling = on ? 1 : 0;
    return MPC_OK;
}

int mpc_kernel_times(mpc_ctx* c, double* pencil_ms, long* n_pencil, double* plane_ms, long* n_plane) {
    if (!c || !pencil_ms || !n_pencil || !plane_ms || !n_plane) return fail(MPC_ERR_ARG, "null argument");
    CK(cudaStreamSynchronize(c->st), "profile sync");
    *pencil_ms = *plane_ms = 0.0;
    *n_pencil = *n_plane = 0;
    for (auto& e : c->events) {
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, e.a, e.b), "cudaEventElapsedTime");
        if (e.kind == 0) { *pencil_ms += ms; (*n_pencil)++; }
        else { *plane_ms += ms; (*n_plane)++; }
    }
    return MPC_OK;
}

int mpc_get_state(mpc_ctx* c, mpc_state* st) {
    if (!c || !st) return fail(MPC_ERR_ARG, "null argument");
    *st = c->state;
    return MPC_OK;
}
int mpc_set_state(mpc_ctx* c, const mpc_state* st) {
    if (!c || !st) return fail(MPC_ERR_ARG, "null argument");
    c->state = *st;
    return MPC_OK;
}

int mpc_field_upload(mpc_ctx* c, const double* A, int calibrate) {
    if (!c || !A) return fail(MPC_ERR_ARG, "null argument");
    int rc = ensure_io(c, 0);
    if (rc) return rc;
    if ((rc = field_copy(c, c->io, A, sizeof(double2) * c->N, cudaMemcpyHostToDevice, "H2D field"))) return rc;
    double k = 1.0;
    if (calibrate) {
        if (!(c->p.Esig > 0)) return fail(MPC_ERR_ARG, "Esig must be positive to calibrate");
        k = sqrt(c->p.puls_e / c->p.Esig);  // MPC.c:209 (A17: both parts)
    }
    PencilArgs a{};
    a.in = c->io;
    a.out = c->S;
    a.in_scale = c->fs * k / (double)c->Nt;
    rc = launch_pencil(c, mpc::PM_ENTRY_C128, a);
    if (rc) return rc;
    c->have_field = 1;
    return MPC_OK;
}

// download the device field (complex128, physical units); optional per-pencil energies
static int exit_to_io(mpc_ctx* c, int energies) {
    int rc = ensure_io(c, 0);
    if (rc) return rc;
    PencilArgs a{};
    a.in = c->S;
    a.out = c->io;
    a.out_scale = 1.0 / c->fs;
    a.pencil_energy = energies ? c->penergy : nullptr;
    return launch_pencil(c, mpc::PM_EXIT_C128, a);
}

int mpc_field_download(mpc_ctx* c, double* A) {
    if (!c || !A) return fail(MPC_ERR_ARG, "null argument");
    if (!c->have_field) return fail(MPC_ERR_STATE, "no field on the device");
    int rc = exit_to_io(c, 0);
    if (rc) return rc;
    if ((rc = field_copy(c, A, c->io, sizeof(double2) * c->N, cudaMemcpyDeviceToHost, "D2H field"))) return rc;
    CK(cudaStreamSynchronize(c->st), "download");
    return kernel_errors(c);
}

// one nonlinear step of the pencil sweep, in place on buf (default: the field S)
static int pencil_step(mpc_ctx* c, double dz, float2* buf = nullptr) {
    PencilArgs a{};
    a.in = buf ? buf : c->S;
    a.out = buf ? buf : c->S;
    a.stats = c->dstats;
    a.nl = c->nl;
    a.nl.dz = (float)dz;
    return launch_pencil(c, mpc::PM_STEP, a);
}

static int bounces_between(double z0, double z1, double Cav) {
    const double eps = 1e-9;
    return (int)(floor(z1 / Cav + eps) - floor(z0 / Cav + eps));
}

int mpc_run_fixed(mpc_ctx* c, int nsteps) {
    if (!c) return fail(MPC_ERR_ARG, "null context");
    if (!c->have_field) return fail(MPC_ERR_STATE, "no field on the device");
    if (nsteps <= 0) return MPC_OK;
    const double dz = c->state.dzz;
    const double Cav = c->p.Cav;
    const int lens = c->p.bounce_mode == MPC_BOUNCE_LENS;
    const double sNP = 1.0 / (double)c->NP, sN = 1.0 / ((double)c->NP * c->Nt);
    const long g0 = c->state.nstep;
    auto sign_of = [&](long g) -> int { return lens ? 1 : pass_sign((double)g * dz + 1e-9 * Cav, Cav); };
    auto bounce_after = [&](long g) -> int { return bounces_between((double)g * dz, (double)(g + 1) * dz, Cav); };
    int rc;
    TableSet t1, t2;
    recycle_tables(c);
    // first half step of step g0 on the normalised state
    int s_prev = sign_of(g0);
    if ((rc = get_tables(c, s_prev * dz / 2, dz / 2, sNP, &t1))) return rc;
    if ((rc = launch_plane(c, c->S, c->S, t1, nullptr))) return rc;
    for (int k = 0; k < nsteps; k++) {
        const long g = g0 + k;
        if ((rc = pencil_step(c, dz))) return rc;
        const int nb = bounce_after(g);
        const int last = (k == nsteps - 1);
        const int s_next = sign_of(g + 1);
        if (nb > 0) {
            for (int b = 0; b < nb; b++) c->state.puls_e *= c->p.Ab_M;  // A24 fix
        }
        if (lens && nb > 0) {
            if ((rc = get_tables(c, s_prev * dz / 2, dz / 2, sN, &t1))) return rc;
            if (last) t2 = c->ident;
            else if ((rc = get_tables(c, s_next * dz / 2, dz / 2, sNP, &t2))) return rc;
            if ((rc = launch_plane(c, c->S, c->S, t1, &t2))) return rc;
        } else if (last) {
            if ((rc = get_tables(c, s_prev * dz / 2, dz / 2, sN, &t1))) return rc;
            if ((rc = launch_plane(c, c->S, c->S, t1, nullptr))) return rc;
        } else {
            if ((rc = get_tables(c, (s_prev + s_next) * dz / 2, dz, sN, &t1))) return rc;
            if ((rc = launch_plane(c, c->S, c->S, t1, nullptr))) return rc;
        }
        s_prev = s_next;
    }
    c->state.nstep += nsteps;
    c->state.z = (double)c->state.nstep * dz;
    c->state.signmem = sign_of(c->state.nstep);
    return MPC_OK;
}

int mpc_ssfmprop(mpc_ctx* c, double* A, int sst_on, double dzz, int* signmem, double z, double* puls_e,
                 double* BP1, double* BP2, double* y1, double* y2, double* bps1, double* bps2, int change) {
    if (!c || !A || !signmem || !puls_e) return fail(MPC_ERR_ARG, "null argument");
    if (change == 1 && (!BP1 || !BP2 || !y1 || !y2 || !bps1 || !bps2)) return fail(MPC_ERR_ARG, "null diagnostic output");
    int rc = ensure_io(c, 0);
    if (rc) return rc;
    if ((rc = field_copy(c, c->io, A, sizeof(double2) * c->N, cudaMemcpyHostToDevice, "H2D field"))) return rc;
    PencilArgs a{};
    a.in = c->io;
    a.out = c->S;
    a.in_scale = c->fs / (double)c->Nt;
    if ((rc = launch_pencil(c, mpc::PM_ENTRY_C128, a))) return rc;
    // calcexpR's sign logic (propagation.c:377-382)
    int signum = pass_sign(z, c->p.Cav);
    if (-*signmem == signum) *signmem = -*signmem;
    if (c->p.bounce_mode == MPC_BOUNCE_LENS) signum = 1;
    const double sNP = 1.0 / (double)c->NP, sN = 1.0 / ((double)c->NP * c->Nt);
    TableSet t1, t2;
    recycle_tables(c);
    if ((rc = get_tables(c, signum * dzz / 2, dzz / 2, sNP, &t1))) return rc;
    if ((rc = get_tables(c, signum * dzz / 2, dzz / 2, sN, &t2))) return rc;
    if ((rc = launch_plane(c, c->S, c->S, t1, nullptr))) return rc;
    PencilArgs b{};
    b.in = c->S;
    b.out = c->S;
    b.nl = c->nl;
    b.nl.dz = (float)dzz;
    b.nl.sst_c = (sst_on == 1) ? c->sst_c_full : 0.0f;
    if ((rc = launch_pencil(c, mpc::PM_STEP, b))) return rc;
    if ((rc = launch_plane(c, c->S, c->S, t2, nullptr))) return rc;
    c->have_field = 1;
    if ((rc = exit_to_io(c, change == 1))) return rc;
    if ((rc = field_copy(c, A, c->io, sizeof(double2) * c->N, cudaMemcpyDeviceToHost, "D2H field"))) return rc;
    if (change == 1) {
        // propagation.c:334-341, as written (after calcexpR the condition cannot hold)
        const int s2 = pass_sign(z, c->p.Cav);
        if (*signmem == -s2) {
            *puls_e = *puls_e * c->p.Ab_M;
            *signmem *= -1;
        }
        k_beam_profiles<<<(c->Nx + 255) / 256, 256, 0, c->st>>>(c->penergy, c->Nx, c->Ny, c->dred, c->dred + c->Nx);
        CK(cudaGetLastError(), "k_beam_profiles");
        CK(cudaMemcpyAsync(BP1, c->dred, sizeof(double) * c->Nx, cudaMemcpyDeviceToHost, c->st), "D2H BP1");
        CK(cudaMemcpyAsync(BP2, c->dred + c->Nx, sizeof(double) * c->Ny, cudaMemcpyDeviceToHost, c->st), "D2H BP2");
    }
    CK(cudaStreamSynchronize(c->st), "ssfmprop");
    if (change == 1) {
        mpc_calc1oes(BP1, c->Nx, c->r.data(), bps1, y1);
        mpc_calc1oes(BP2, c->Ny, c->r.data(), bps2, y2);
    }
    return MPC_OK;
}

// 1/e^2 radius search (propagation.c:460-504), serial meaning of its parallel loops.
int mpc_calc1oes(const double* BP, int n, const double* r, double* vald, double* y) {
    double bpex = 0;
    int posi1 = 0, posi2 = 0;
    for (int k = 0; k < n; k++)
        if (BP[k] > bpex) bpex = BP[k];
    const double lvl = 1.0 / pow(exp(1.0), 2.0);
    double best = 0;
    for (int k = 0; k < n / 2; k++) {
        const double h = fabs(BP[k] / bpex - lvl);
        if (k == 0) best = h;
        else if (h < best) { best = h; posi1 = k; }
    }
    for (int k = n / 2; k < n; k++) {
        const double h = fabs(BP[k] / bpex - lvl);
        if (k == n / 2) best = h;
        else if (h < best) { best = h; posi2 = k; }
    }
    *vald = -r[posi1] + r[posi2];
    y[0] = r[posi1];
    y[1] = r[posi2];
    y[2] = BP[posi1];
    y[3] = BP[posi2];
    return MPC_OK;
}

int mpc_linearstep(mpc_ctx* c, double* A, const double* exp_D0, const double* expR) {
    if (!c || !A || !exp_D0 || !expR) return fail(MPC_ERR_ARG, "null argument");
    int rc = ensure_io(c, 0);
    if (rc) return rc;
    // caller tables (FP64) -> position order, conj(expR) along x and y, D scaled by 1/(Nx Ny);
    // reordering only on the host, the double-float split on the device
    const int Nx = c->Nx, Ny = c->Ny, Nt = c->Nt;
    std::vector<double2> h(Nx + Ny + Nt);
    for (int i = 0; i < Nx; i++) {
        const int f = c->hfx[i];
        h[i] = make_double2(expR[2 * f], -expR[2 * f + 1]);
    }
    for (int j = 0; j < Ny; j++) {
        const int f = c->hfy[j];
        h[Nx + j] = make_double2(expR[2 * f], -expR[2 * f + 1]);
    }
    const double sc = 1.0 / (double)c->NP;
    for (int k = 0; k < Nt; k++) {
        const int f = c->hft[k];
        h[Nx + Ny + k] = make_double2(exp_D0[2 * f] * sc, exp_D0[2 * f + 1] * sc);
    }
    TableSet t;
    if ((rc = alloc_tables(c, &t))) return rc;
    cudaError_t e = cudaMemcpyAsync(t.f64, h.data(), sizeof(double2) * h.size(), cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess && (rc = field_copy(c, c->io, A, sizeof(double2) * c->N, cudaMemcpyHostToDevice, "H2D field"))) {
        cudaStreamSynchronize(c->st);
        cudaFree(t.f64);
        return rc;
    }
    if (e == cudaSuccess && (rc = split_tables(c, t))) {
        cudaStreamSynchronize(c->st);
        cudaFree(t.f64);
        return rc;
    }
    if (e != cudaSuccess) {
        cudaStreamSynchronize(c->st);
        cudaFree(t.f64);
        return fail(MPC_ERR_CUDA, "H2D linearstep", e);
    }
    PencilArgs a{};
    a.in = c->io;
    a.out = c->S;
    a.in_scale = c->fs / (double)Nt;
    rc = launch_pencil(c, mpc::PM_ENTRY_C128, a);
    if (!rc) rc = launch_plane(c, c->S, c->S, t, nullptr);
    if (!rc) rc = exit_to_io(c, 0);
    if (!rc) rc = field_copy(c, A, c->io, sizeof(double2) * c->N, cudaMemcpyDeviceToHost, "D2H field");
    if (!rc) {
        e = cudaStreamSynchronize(c->st);
        if (e != cudaSuccess) rc = fail(MPC_ERR_CUDA, "linearstep", e);
    }
    cudaStreamSynchronize(c->st);
    cudaFree(t.f64);
    c->have_field = 1;
    return rc;
}

int mpc_calcexpR(mpc_ctx* c, double* expR, int* signmem, double z, double dzz) {
    if (!c || !expR || !signmem) return fail(MPC_ERR_ARG, "null argument");
    int signum = pass_sign(z, c->p.Cav);
    if (-*signmem == signum) *signmem = -*signmem;
    if (c->p.bounce_mode == MPC_BOUNCE_LENS) signum = 1;
    TableSet t;
    recycle_tables(c);
    int rc = get_tables(c, signum * dzz, 0.0, 1.0, &t);
    if (rc) return rc;
    std::vector<double2> h(c->Nx);
    CK(cudaMemcpyAsync(h.data(), t.f64, sizeof(double2) * c->Nx, cudaMemcpyDeviceToHost, c->st), "D2H table");
    CK(cudaStreamSynchronize(c->st), "calcexpR");
    // the device table is conj(expR) in position order; the reference returns expR in FFT order
    for (int px = 0; px < c->Nx; px++) {
        const int f = c->hfx[px];
        expR[2 * f] = h[px].x;
        expR[2 * f + 1] = -h[px].y;
    }
    return MPC_OK;
}

int mpc_ioniz(mpc_ctx* c, const double* A, double* tau_c, double* fe_sp) {
    if (!c || !A || !tau_c || !fe_sp) return fail(MPC_ERR_ARG, "null argument");
    if (!c->ion_gas_ok) return fail(MPC_ERR_ARG, "unknown gas");
    int rc = ensure_io(c, 0);
    if (rc) return rc;
    if ((rc = ensure_io(c, 1))) return rc;
    if ((rc = field_copy(c, c->io, A, sizeof(double2) * c->N, cudaMemcpyHostToDevice, "H2D field"))) return rc;
    PencilArgs a{};
    a.in = c->io;
    a.in_scale = c->fs;
    a.nl = c->nl;
    a.nl.plasma = 1;
    double* tau_d = reinterpret_cast<double*>(c->io2);
    double* fe_d = tau_d + c->N;
    a.tau_out = tau_d;
    a.fe_out = fe_d;
    if ((rc = launch_pencil(c, mpc::PM_IONIZ, a))) return rc;
    if ((rc = field_copy(c, tau_c, tau_d, sizeof(double) * c->N, cudaMemcpyDeviceToHost, "D2H tau_c"))) return rc;
    if ((rc = field_copy(c, fe_sp, fe_d, sizeof(double) * c->N, cudaMemcpyDeviceToHost, "D2H fe_sp"))) return rc;
    CK(cudaStreamSynchronize(c->st), "ioniz");
    return MPC_OK;
}

int mpc_ADK(mpc_ctx* c, long n, const double* E, double* r1, double* r2) {
    if (!c || !E || !r1 || !r2 || n < 0) return fail(MPC_ERR_ARG, "null argument");
    if (n == 0) return MPC_OK;
    double* d = nullptr;
    CK(cudaMalloc(&d, sizeof(double) * 3 * n), "cudaMalloc ADK");
    cudaError_t e = cudaMemcpyAsync(d, E, sizeof(double) * n, cudaMemcpyHostToDevice, c->st);
    if (e == cudaSuccess) {
        k_adk<<<(int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096), 256, 0, c->st>>>(n, d, d + n, d + 2 * n, c->adk);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(r1, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(r2, d + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->st);
    cudaFree(d);
    if (e != cudaSuccess) return fail(MPC_ERR_CUDA, "ADK", e);
    return MPC_OK;
}

// the dz rule of setStep (propagation.c:636-676) given err
static void step_rule(double err, double* dzz, double def_err, double dzmin, const double* y1, const double* y2, int* bad) {
    const double err_fact = pow(2.0, 1.0 / 3.0);
    *bad = 0;
    if (err > 2.0 * def_err) {
        const double u = *dzz / 2.0;
        if (u > dzmin) {
            *dzz = u;
            *bad = 1;
        }
    } else if (err > def_err && err < 2.0 * def_err) {
        const double u = *dzz / err_fact;
        if (u > dzmin) *dzz = u;
    } else if (err > 0.5 * def_err && err <= def_err) {
    } else {
        const double u = *dzz * err_fact;
        if (!(u > 100 * (y2[1] + y1[1]) / 2.0)) *dzz = u;
    }
}

int mpc_setStep(mpc_ctx* c, double* dzz, const double* C1, const double* C2, const double* y1, const double* y2,
                int* bad, double* err) {
    if (!c || !dzz || !C1 || !C2 || !y1 || !y2 || !bad || !err) return fail(MPC_ERR_ARG, "null argument");
    int rc = ensure_io(c, 0);
    if (rc) return rc;
    if ((rc = ensure_io(c, 1))) return rc;
    if ((rc = field_copy(c, c->io, C1, sizeof(double2) * c->N, cudaMemcpyHostToDevice, "H2D C1"))) return rc;
    if ((rc = field_copy(c, c->io2, C2, sizeof(double2) * c->N, cudaMemcpyHostToDevice, "H2D C2"))) return rc;
    CK(cudaMemsetAsync(c->dred, 0, 2 * sizeof(double), c->st), "memset");
    k_diffnorm_c128<<<c->nsm * 4, 256, 0, c->st>>>(c->io, c->io2, c->N, c->dred);
    CK(cudaGetLastError(), "k_diffnorm_c128");
    double s[2];
    CK(cudaMemcpyAsync(s, c->dred, sizeof s, cudaMemcpyDeviceToHost, c->st), "D2H sums");
    CK(cudaStreamSynchronize(c->st), "setStep");
    *err = sqrt(s[0]) / sqrt(s[1]);
    step_rule(*err, dzz, c->p.def_err, c->p.dzmin, y1, y2, bad);
    return MPC_OK;
}

int mpc_diag(mpc_ctx* c, double* temp, double* spec, double* BP1, double* BP2) {
    if (!c) return fail(MPC_ERR_ARG, "null context");
    if (!c->have_field) return fail(MPC_ERR_STATE, "no field on the device");
    const int Nt = c->Nt;
    double* dtemp = c->dred;
    double* dspec = c->dred + Nt;
    int rc;
    const double phys2 = 1.0 / (c->fs * c->fs);
    if (temp) {
        CK(cudaMemsetAsync(dtemp, 0, sizeof(double) * Nt, c->st), "memset temp");
        PencilArgs a{};
        a.in = c->S;
        a.temp = dtemp;
        a.out_scale = 1.0 / c->fs;
        if ((rc = launch_pencil(c, mpc::PM_TEMP, a))) return rc;
        CK(cudaMemcpyAsync(temp, dtemp, sizeof(double) * Nt, cudaMemcpyDeviceToHost, c->st), "D2H temp");
        CK(cudaStreamSynchronize(c->st), "temp");
    }
    if (spec) {
        // S = FFT_t(a)/Nt  ->  |FFT_t A|^2 = Nt^2 |S|^2 / fs^2
        k_spec<<<Nt, 256, 0, c->st>>>(c->S, (int)c->NP, c->ops->SLO, c->dft, (double)Nt * Nt * phys2, dspec);
        CK(cudaGetLastError(), "k_spec");
        CK(cudaMemcpyAsync(spec, dspec, sizeof(double) * Nt, cudaMemcpyDeviceToHost, c->st), "D2H spec");
        CK(cudaStreamSynchronize(c->st), "spec");
    }
    if (BP1 || BP2) {
        if ((rc = exit_to_io(c, 1))) return rc;
        double* d1 = c->dred;
        double* d2 = c->dred + c->Nx;
        k_beam_profiles<<<(c->Nx + 255) / 256, 256, 0, c->st>>>(c->penergy, c->Nx, c->Ny, d1, d2);
        CK(cudaGetLastError(), "k_beam_profiles");
        if (BP1) CK(cudaMemcpyAsync(BP1, d1, sizeof(double) * c->Nx, cudaMemcpyDeviceToHost, c->st), "D2H BP1");
        if (BP2) CK(cudaMemcpyAsync(BP2, d2, sizeof(double) * c->Ny, cudaMemcpyDeviceToHost, c->st), "D2H BP2");
        CK(cudaStreamSynchronize(c->st), "beam profiles");
    }
    return MPC_OK;
}

// Launch one step-doubling attempt on the context's stream, asynchronously: C1, C2, C2's beam
// profiles, the error sums and the Richardson field, with the sums and profiles copied to the
// pinned buffer hsd.  No synchronous call, so the launches can be captured into a graph.
static int step_double_launch(mpc_ctx* c) {
    if (!c->have_field) return fail(MPC_ERR_STATE, "no field on the device");
    for (float2** b : {&c->C1, &c->C2})
        if (!*b && cudaMalloc(b, sizeof(float2) * c->N) != cudaSuccess) {
            *b = nullptr;
            cudaGetLastError();
            return fail(MPC_ERR_NOMEM, "cudaMalloc step-doubling fields");
        }
    if (!c->hsd && cudaMallocHost(&c->hsd, sizeof(double) * (2 + c->Nx + c->Ny)) != cudaSuccess) {
        c->hsd = nullptr;
        cudaGetLastError();
        return fail(MPC_ERR_NOMEM, "cudaMallocHost step-doubling sums");
    }
    mpc_state& st = c->state;
    const double Cav = c->p.Cav;
    double dz = st.dzz;
    c->sd_clipped = 0;
    if (c->p.land_mirrors) {   // end the attempt on the next mirror plane rather than cross it
        const double room = (floor(st.z / Cav + 1e-9) + 1.0) * Cav - st.z;
        if (room > 1e-9 * Cav && 2.0 * dz > room) {
            c->sd_natural = dz;
            dz = room / 2.0;
            c->sd_clipped = 1;
        }
    }
    c->sd_dz = dz;
    // calcexpR's sign logic (propagation.c:377-382), evaluated at the attempt's z for all three steps
    int signum = pass_sign(st.z, Cav);
    if (-st.signmem == signum) st.signmem = -st.signmem;
    if (c->p.bounce_mode == MPC_BOUNCE_LENS) signum = 1;
    const double sNP = 1.0 / (double)c->NP, sN = 1.0 / ((double)c->NP * c->Nt);
    int rc;
    recycle_tables(c);
    // C1: one step of 2 dz
    TableSet a1, a2;
    if ((rc = get_tables(c, signum * dz, dz, sNP, &a1))) return rc;
    if ((rc = get_tables(c, signum * dz, dz, sN, &a2))) return rc;
    if ((rc = launch_plane(c, c->S, c->C1, a1, nullptr))) return rc;
    if ((rc = pencil_step(c, 2.0 * dz, c->C1))) return rc;
    if ((rc = launch_plane(c, c->C1, c->C1, a2, nullptr))) return rc;
    // C2: two steps of dz, the two middle half steps merged
    TableSet b1, bm, b2;
    if ((rc = get_tables(c, signum * dz / 2, dz / 2, sNP, &b1))) return rc;
    if ((rc = get_tables(c, signum * dz, dz, sN, &bm))) return rc;
    if ((rc = get_tables(c, signum * dz / 2, dz / 2, sN, &b2))) return rc;
    if ((rc = launch_plane(c, c->S, c->C2, b1, nullptr))) return rc;
    if ((rc = pencil_step(c, dz, c->C2))) return rc;
    if ((rc = launch_plane(c, c->C2, c->C2, bm, nullptr))) return rc;
    if ((rc = pencil_step(c, dz, c->C2))) return rc;
    if ((rc = launch_plane(c, c->C2, c->C2, b2, nullptr))) return rc;
    // beam profiles of C2 (the change == 1 step, propagation.c:343-361), physical units:
    // sum_t |A|^2 = Nt sum_omega |S|^2 / fs^2
    k_pencil_energy_slots<<<(int)((c->NP + 255) / 256), 256, 0, c->st>>>(c->C2, (int)c->NP, c->Nt, c->ops->SLO,
                                                                       (double)c->Nt / (c->fs * c->fs), c->penergy);
    CK(cudaGetLastError(), "k_pencil_energy_slots");
    double* dbp = c->dred + 2;
    k_beam_profiles<<<(c->Nx + 255) / 256, 256, 0, c->st>>>(c->penergy, c->Nx, c->Ny, dbp, dbp + c->Nx);
    CK(cudaGetLastError(), "k_beam_profiles");
    // error sums and the Richardson field (into C1)
    CK(cudaMemsetAsync(c->dred, 0, 2 * sizeof(double), c->st), "memset");
    k_richardson<<<c->nsm * 4, 256, 0, c->st>>>(c->C1, c->C2, c->C1, c->N, c->dred);
    CK(cudaGetLastError(), "k_richardson");
    c->launches += 3;
    CK(cudaMemcpyAsync(c->hsd, c->dred, sizeof(double) * (2 + c->Nx + c->Ny), cudaMemcpyDeviceToHost, c->st),
       "D2H sums");
    return MPC_OK;
}

// Decide a launched attempt once its stream has completed: the setStep rule, acceptance
// (pointer swap), z, mirror bounces crossed.
static int step_double_finish(mpc_ctx* c, double* BP1, double* BP2, int* bad, double* err) {
    mpc_state& st = c->state;
    const double* h = c->hsd;
    mpc_calc1oes(h + 2, c->Nx, c->r.data(), &st.bps1, st.y1);
    mpc_calc1oes(h + 2 + c->Nx, c->Ny, c->r.data(), &st.bps2, st.y2);
    if (BP1) memcpy(BP1, h + 2, sizeof(double) * c->Nx);
    if (BP2) memcpy(BP2, h + 2 + c->Nx, sizeof(double) * c->Ny);
    *err = sqrt(h[0]) / sqrt(h[1]);
    st.err = *err;
    if (c->sd_clipped) st.dzz = c->sd_dz;   // the rule judges the step taken
    step_rule(*err, &st.dzz, c->p.def_err, c->p.dzmin, st.y1, st.y2, bad);
    // a shortening that only served to land on a plane does not shrink the next step
    if (c->sd_clipped && !*bad && *err <= c->p.def_err && st.dzz < c->sd_natural) st.dzz = c->sd_natural;
    st.bad = *bad;
    st.attempts++;
    if (*bad) return MPC_OK;
    std::swap(c->S, c->C1);  // the accepted field (4 C2 - C1)/3
    const double z0 = st.z;
    st.z = z0 + 2.0 * c->sd_dz;  // A26: the step just taken
    const int nb = bounces_between(z0, st.z, c->p.Cav);
    int rc;
    for (int b = 0; b < nb; b++) {
        if (c->p.bounce_mode == MPC_BOUNCE_LENS && (rc = launch_plane(c, c->S, c->S, c->ident, &c->ident))) return rc;
        st.puls_e *= c->p.Ab_M;  // A24: the mirror loss the reference's bookkeeping never applies
    }
    if (st.z > c->p.dist) st.z = c->p.dist;
    st.nstep++;
    return MPC_OK;
}

int mpc_step_double(mpc_ctx* c, double* BP1, double* BP2, int* bad, double* err) {
    if (!c || !bad || !err) return fail(MPC_ERR_ARG, "null argument");
    int rc = step_double_launch(c);
    if (rc) return rc;
    CK(cudaStreamSynchronize(c->st), "step_double");
    return step_double_finish(c, BP1, BP2, bad, err);
}

// ---- batches of cells -------------------------------------------------------------------
// A batch runs the same call on many independent contexts (cells of a sweep, of any grid
// shapes) as one CUDA graph: the launches of every cell are captured on the cell's own stream,
// forked from and joined into the batch's stream, and the graph is launched once, so kernels of
// different cells overlap where one leaves SMs idle (tails, small grids) and the whole batch
// costs one launch from the host.
struct mpc_batch {
    std::vector<mpc_ctx*> cells;
    cudaStream_t st = nullptr;
    cudaEvent_t fork = nullptr;
    std::vector<cudaEvent_t> join;
    long graphs = 0, nodes = 0;
};

int mpc_batch_create(mpc_batch** out, int n, mpc_ctx* const* cells) {
    if (!out || n <= 0 || !cells) return fail(MPC_ERR_ARG, "null argument or empty batch");
    *out = nullptr;
    for (int i = 0; i < n; i++)
        if (!cells[i]) return fail(MPC_ERR_ARG, "null context in batch");
    mpc_batch* b = new mpc_batch();
    b->cells.assign(cells, cells + n);
    b->join.assign(n, nullptr);
    cudaError_t e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (int i = 0; i < n && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        mpc_batch_destroy(b);
        return fail(MPC_ERR_CUDA, "batch stream and events", e);
    }
    *out = b;
    return MPC_OK;
}

int mpc_batch_destroy(mpc_batch* b) {
    if (!b) return MPC_OK;
    if (b->st) cudaStreamSynchronize(b->st);
    for (cudaEvent_t e : b->join)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return MPC_OK;
}

// Capture per_cell(cell) for every active cell into one graph and run it to completion.
static int batch_graph(mpc_batch* b, const std::vector<char>& active, const std::function<int(mpc_ctx*)>& per_cell) {
    for (size_t i = 0; i < b->cells.size(); i++)
        if (active[i]) {
            CK(cudaStreamSynchronize(b->cells[i]->st), "batch: cell stream");
            recycle_tables(b->cells[i]);
        }
    CK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeRelaxed), "begin graph capture");
    int rc = MPC_OK;
    cudaError_t e = cudaEventRecord(b->fork, b->st);
    for (size_t i = 0; i < b->cells.size() && rc == MPC_OK && e == cudaSuccess; i++) {
        if (!active[i]) continue;
        mpc_ctx* c = b->cells[i];
        e = cudaStreamWaitEvent(c->st, b->fork, 0);
        if (e != cudaSuccess) break;
        c->capturing = 1;
        rc = per_cell(c);
        c->capturing = 0;
        if (rc == MPC_OK) e = cudaEventRecord(b->join[i], c->st);
        if (rc == MPC_OK && e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->join[i], 0);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t e_end = cudaStreamEndCapture(b->st, &g);
    if (rc != MPC_OK || e != cudaSuccess || e_end != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        if (rc != MPC_OK) return rc;
        return fail(MPC_ERR_CUDA, "batch graph capture", e != cudaSuccess ? e : e_end);
    }
    cudaGraphExec_t ge = nullptr;
    e = cudaGraphInstantiate(&ge, g, 0);
    size_t nn = 0;
    if (e == cudaSuccess) e = cudaGraphGetNodes(g, nullptr, &nn);
    if (e == cudaSuccess) e = cudaGraphLaunch(ge, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (ge) cudaGraphExecDestroy(ge);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return fail(MPC_ERR_CUDA, "batch graph", e);
    b->graphs++;
    b->nodes += (long)nn;
    return MPC_OK;
}

int mpc_batch_run_fixed(mpc_batch* b, int nsteps) {
    if (!b) return fail(MPC_ERR_ARG, "null batch");
    std::vector<char> active(b->cells.size(), 1);
    for (size_t i = 0; i < b->cells.size(); i++)
        if (!b->cells[i]->have_field) return fail(MPC_ERR_STATE, "a cell of the batch has no field");
    return batch_graph(b, active, [nsteps](mpc_ctx* c) { return mpc_run_fixed(c, nsteps); });
}

int mpc_batch_step_double(mpc_batch* b, int* bad, double* err) {
    if (!b || !bad || !err) return fail(MPC_ERR_ARG, "null argument");
    const size_t n = b->cells.size();
    std::vector<char> active(n, 0);
    int any = 0;
    for (size_t i = 0; i < n; i++) {
        mpc_ctx* c = b->cells[i];
        if (!c->have_field) return fail(MPC_ERR_STATE, "a cell of the batch has no field");
        active[i] = c->state.z < c->p.dist;
        any |= active[i];
        bad[i] = -1;
        err[i] = 0.0;
    }
    if (!any) return MPC_OK;
    int rc = batch_graph(b, active, [](mpc_ctx* c) { return step_double_launch(c); });
    if (rc) return rc;
    for (size_t i = 0; i < n; i++)
        if (active[i] && (rc = step_double_finish(b->cells[i], nullptr, nullptr, &bad[i], &err[i]))) return rc;
    return MPC_OK;
}

int mpc_batch_stats(mpc_batch* b, long* graphs, long* nodes) {
    if (!b || !graphs || !nodes) return fail(MPC_ERR_ARG, "null argument");
    *graphs = b->graphs;
    *nodes = b->nodes;
    return MPC_OK;
}

int mpc_step(mpc_ctx* c, double dzz) {
    if (!c) return fail(MPC_ERR_ARG, "null context");
    if (!c->have_field) return fail(MPC_ERR_STATE, "no field on the device");
    if (!(dzz > 0)) return fail(MPC_ERR_ARG, "dzz must be positive");
    mpc_state& st = c->state;
    int signum = pass_sign(st.z, c->p.Cav);  // calcexpR (propagation.c:377-382)
    if (-st.signmem == signum) st.signmem = -st.signmem;
    if (c->p.bounce_mode == MPC_BOUNCE_LENS) signum = 1;
    const double sNP = 1.0 / (double)c->NP, sN = 1.0 / ((double)c->NP * c->Nt);
    TableSet t1, t2;
    int rc;
    recycle_tables(c);
    if ((rc = get_tables(c, signum * dzz / 2, dzz / 2, sNP, &t1))) return rc;
    if ((rc = get_tables(c, signum * dzz / 2, dzz / 2, sN, &t2))) return rc;
    if ((rc = launch_plane(c, c->S, c->S, t1, nullptr))) return rc;
    if ((rc = pencil_step(c, dzz))) return rc;
    if ((rc = launch_plane(c, c->S, c->S, t2, nullptr))) return rc;
    const double z0 = st.z;
    st.z = z0 + dzz;
    const int nb = bounces_between(z0, st.z, c->p.Cav);
    for (int b = 0; b < nb; b++) {
        if (c->p.bounce_mode == MPC_BOUNCE_LENS && (rc = launch_plane(c, c->S, c->S, c->ident, &c->ident))) return rc;
        st.puls_e *= c->p.Ab_M;
    }
    if (st.z > c->p.dist) st.z = c->p.dist;
    st.nstep++;
    return MPC_OK;
}

int mpc_step_stats(mpc_ctx* c, float* out, int reset) {
    if (!c || !out) return fail(MPC_ERR_ARG, "null argument");
    unsigned int u[4];
    CK(cudaMemcpyAsync(u, c->dstats, sizeof u, cudaMemcpyDeviceToHost, c->st), "D2H step statistics");
    if (reset) CK(cudaMemsetAsync(c->dstats, 0, sizeof u, c->st), "reset step statistics");
    CK(cudaStreamSynchronize(c->st), "step statistics");
    for (int k = 0; k < 4; k++) memcpy(&out[k], &u[k], sizeof(float));
    // device units -> physical: |a|^2 -> intensity [W/m^2]
    out[0] = (float)((double)out[0] * I_UNIT);
    return MPC_OK;
}

int mpc_features(mpc_ctx* c, float* f) {
    if (!c || !f) return fail(MPC_ERR_ARG, "null argument");
    if (!c->have_field) return fail(MPC_ERR_STATE, "no field on the device");
    float stt[4];
    int rc = mpc_step_stats(c, stt, 0);
    if (rc) return rc;
    CK(cudaMemsetAsync(c->dmom, 0, 8 * sizeof(double), c->st), "memset moments");
    k_moments<<<c->Nt, c->Nx < 32 ? 32 : (c->Nx < 256 ? c->Nx : 256), 0, c->st>>>(c->S, c->Nt, (int)c->NP, c->Nx, c->Ny, c->ops->SLO, c->wpos,
                                                             c->rf, c->dmom, reinterpret_cast<unsigned int*>(c->dmom + 7));
    CK(cudaGetLastError(), "k_moments");
    c->launches++;
    double m[8];
    CK(cudaMemcpyAsync(m, c->dmom, sizeof m, cudaMemcpyDeviceToHost, c->st), "D2H moments");
    CK(cudaStreamSynchronize(c->st), "features");
    float smax;
    memcpy(&smax, &m[7], sizeof smax);
    const mpc_params& p = c->p;
    const mpc_state& st = c->state;
    const double E = m[0] > 0 ? m[0] : 1e-300;
    const double wm = m[1] / E, ws = sqrt(fmax(m[2] / E - wm * wm, 0.0));
    const double xm = m[3] / E, xs = sqrt(fmax(m[4] / E - xm * xm, 0.0));
    const double ym = m[5] / E, ys = sqrt(fmax(m[6] / E - ym * ym, 0.0));
    const double window = c->Nx * p.dr;
    const double energy = m[0] * (double)c->Nt / (c->fs * c->fs) * p.dr * p.dr * p.deltat * HBAR * p.w0;
    const double zc = st.z / p.Cav;
    const double v[16] = {
        log10(1e-30 + stt[0]),                          // peak intensity of the last steps [W/m^2]
        log10(1e-12 + stt[1]),                          // peak ionization fraction
        log10(1e-12 + stt[2]),                          // peak nonlinear phase rate [rad/m]
        log10(1e-12 + stt[3]),                          // peak amplitude rate [1/m]
        log10(1e-30 + energy),                          // pulse energy [J]
        ws / p.w0 * 1e2,                                // spectral rms width / w0 [%]
        wm / p.w0 * 1e2,                                // spectral centroid shift / w0 [%]
        xs / window,                                    // beam rms width x / window
        ys / window,                                    // beam rms width y / window
        log10(st.dzz / p.Cav),                          // current step / mirror separation
        zc - floor(zc),                                 // position within the pass
        log10(1e-30 + (double)smax / E),                // spectral-spatial peakiness
        log10(1e-30 + p.rho_nt) - 25.0,                 // neutral density
        log10(1e-12 + stt[2] * st.dzz),                 // nonlinear phase per step at the current dz
        (double)(p.plasm == 1),                         // plasma terms on
        (double)(p.sst_on == 1),                        // self-steepening on
    };
    for (int k = 0; k < 16; k++) f[k] = (float)v[k];
    return MPC_OK;
}

// Plain split steps of the learned controller with their adjacent linear half steps merged: the
// field is left with the last step's second half step pending (zd, zp), which the next step's
// first plane sweep takes together with its own first half (one sweep instead of two), and which
// flush_half applies on its own before anything that needs the whole step.
struct HalfStep {
    int pending = 0;
    double zd = 0.0, zp = 0.0;   // diffraction (signed) and dispersion lengths of the pending half
};

static int flush_half(mpc_ctx* c, HalfStep* h) {
    if (!h->pending) return MPC_OK;
    const double sN = 1.0 / ((double)c->NP * c->Nt);
    TableSet t;
    int rc;
    recycle_tables(c);
    if ((rc = get_tables(c, h->zd, h->zp, sN, &t))) return rc;
    if ((rc = launch_plane(c, c->S, c->S, t, nullptr))) return rc;
    h->pending = 0;
    return MPC_OK;
}

// one split step of dz at state.z (mpc_step's arithmetic), its second half step left pending;
// a step that ends on or crosses a mirror plane is completed and bounced (lens, loss)
static int merged_step(mpc_ctx* c, double dz, HalfStep* h) {
    mpc_state& st = c->state;
    int signum = pass_sign(st.z, c->p.Cav);  // calcexpR (propagation.c:377-382)
    if (-st.signmem == signum) st.signmem = -st.signmem;
    if (c->p.bounce_mode == MPC_BOUNCE_LENS) signum = 1;
    const double sNP = 1.0 / (double)c->NP, sN = 1.0 / ((double)c->NP * c->Nt);
    TableSet t;
    int rc;
    recycle_tables(c);
    if (h->pending) {
        if ((rc = get_tables(c, h->zd + signum * dz / 2, h->zp + dz / 2, sN, &t))) return rc;
    } else if ((rc = get_tables(c, signum * dz / 2, dz / 2, sNP, &t))) {
        return rc;
    }
    if ((rc = launch_plane(c, c->S, c->S, t, nullptr))) return rc;
    if ((rc = pencil_step(c, dz))) return rc;
    h->pending = 1;
    h->zd = signum * dz / 2;
    h->zp = dz / 2;
    const double z0 = st.z;
    st.z = z0 + dz;
    const int nb = bounces_between(z0, st.z, c->p.Cav);
    if (nb > 0 && (rc = flush_half(c, h))) return rc;
    for (int b = 0; b < nb; b++) {
        if (c->p.bounce_mode == MPC_BOUNCE_LENS && (rc = launch_plane(c, c->S, c->S, c->ident, &c->ident))) return rc;
        st.puls_e *= c->p.Ab_M;
    }
    if (st.z > c->p.dist) st.z = c->p.dist;
    st.nstep++;
    return MPC_OK;
}

int mpc_run_learned_hold(mpc_ctx* c, mpc_mlp* mlp, double safety, int check_every, int fallback_len, int hold,
                         mpc_learned_stats* out) {
    if (!c || !mlp || !out || !(safety > 0) || check_every < 1 || fallback_len < 0 || hold < 1)
        return fail(MPC_ERR_ARG, "bad argument");
    if (!c->have_field) return fail(MPC_ERR_STATE, "no field on the device");
    memset(out, 0, sizeof *out);
    mpc_state& st = c->state;
    const double Cav = c->p.Cav, dist = c->p.dist, dzmin = c->p.dzmin;
    int rc, bad;
    double err;
    float f[MPC_NFEATURES], stt[4];
    int fb = 1;  // open with one step-doubling attempt (it also provides the first statistics)
    int since_check = 0, held = 0;
    double dz_last = st.dzz, dz_net = 0.0;
    HalfStep half;
    recycle_tables(c);
    while (st.z < dist * (1.0 - 1e-12)) {
        if (fb > 0) {
            if ((rc = flush_half(c, &half))) return rc;
            const double h = st.dzz;
            if ((rc = mpc_step_double(c, nullptr, nullptr, &bad, &err))) return rc;
            out->fallback_attempts++;
            out->executed_steps += 3;
            if (!bad) {
                fb--;
                dz_last = 2.0 * h;
            }
            held = 0;
            continue;
        }
        if (held == 0) {   // a new prediction: features of the whole step
            if ((rc = flush_half(c, &half))) return rc;
            if ((rc = mpc_features(c, f))) return rc;
            if ((rc = mpc_step_stats(c, stt, 1))) return rc;
            float y = 0.0f;
            if ((rc = mpc_mlp_predict1(mlp, f, &y))) return fail(rc, "network prediction failed");
            dz_net = safety * Cav * exp((double)y);
            if (!(dz_net > 0) || !isfinite(dz_net)) dz_net = dz_last;
            dz_net = fmin(dz_net, 2.0 * dz_last);
            dz_net = Cav * exp2(floor(16.0 * log2(dz_net / Cav)) / 16.0);   // cached phase tables stay few
            dz_net = fmax(dz_net, dzmin);
            held = hold;
        }
        double dz = dz_net;
        // land on the next mirror plane rather than step across it, so each bounce is applied
        // where the mirror is
        const double next_plane = (floor(st.z / Cav + 1e-9) + 1.0) * Cav;
        if (next_plane - st.z > 1e-9 * Cav) dz = fmin(dz, next_plane - st.z);
        dz = fmin(dz, dist - st.z);
        if (++since_check >= check_every) {
            since_check = 0;
            out->checks++;
            if ((rc = flush_half(c, &half))) return rc;
            st.dzz = dz / 2.0;
            if ((rc = mpc_step_double(c, nullptr, nullptr, &bad, &err))) return rc;
            out->executed_steps += 3;
            held = 0;
            if (bad || err > c->p.def_err) {
                out->check_failures++;
                fb = fallback_len;
            } else {
                dz_last = dz;
            }
            continue;
        }
        if ((rc = merged_step(c, dz, &half))) return rc;
        held--;
        out->steps++;
        out->executed_steps++;
        out->dz_min = out->steps == 1 ? dz : fmin(out->dz_min, dz);
        out->dz_max = fmax(out->dz_max, dz);
        dz_last = dz;
        st.dzz = dz;
    }
    return flush_half(c, &half);
}

int mpc_run_learned(mpc_ctx* c, mpc_mlp* mlp, double safety, int check_every, int fallback_len,
                    mpc_learned_stats* out) {
    return mpc_run_learned_hold(c, mlp, safety, check_every, fallback_len, 1, out);
}

int mpc_mirror_bounce(mpc_ctx* c, int mode) {
    if (!c) return fail(MPC_ERR_ARG, "null context");
    if (!c->have_field) return fail(MPC_ERR_STATE, "no field on the device");
    if (mode == MPC_BOUNCE_LENS) {
        if (c->p.roc == 0.0) return fail(MPC_ERR_ARG, "lens bounce needs the mirror radius of curvature roc");
        if (c->p.bounce_mode != MPC_BOUNCE_LENS) {
            k_lens<<<(c->Nx + 255) / 256, 256, 0, c->st>>>(c->dr, c->Nx, c->p.k0, c->p.roc, c->lensx);
            k_lens<<<(c->Ny + 255) / 256, 256, 0, c->st>>>(c->dr, c->Ny, c->p.k0, c->p.roc, c->lensy);
            CK(cudaGetLastError(), "k_lens");
        }
        int rc = launch_plane(c, c->S, c->S, c->ident, &c->ident);
        if (rc) return rc;
    } else if (mode == MPC_BOUNCE_SIGNFLIP) {
        c->state.signmem = -c->state.signmem;
    } else {
        return fail(MPC_ERR_ARG, "unknown bounce mode");
    }
    c->state.puls_e *= c->p.Ab_M;
    return MPC_OK;
}

int mpc_energy(mpc_ctx* c, double* energy) {
    if (!c || !energy) return fail(MPC_ERR_ARG, "null argument");
    if (!c->have_field) return fail(MPC_ERR_STATE, "no field on the device");
    CK(cudaMemsetAsync(c->dred, 0, sizeof(double), c->st), "memset");
    k_norm2_c64<<<c->nsm * 4, 256, 0, c->st>>>(c->S, c->N, c->dred);
    CK(cudaGetLastError(), "k_norm2_c64");
    double s = 0;
    CK(cudaMemcpyAsync(&s, c->dred, sizeof s, cudaMemcpyDeviceToHost, c->st), "D2H energy");
    CK(cudaStreamSynchronize(c->st), "energy");
    // sum_t |a|^2 = Nt sum_omega |S|^2 ;  |A|^2 = |a|^2 / fs^2
    *energy = s * (double)c->Nt / (c->fs * c->fs) * c->p.dr * c->p.dr * c->p.deltat * HBAR * c->p.w0;
    return MPC_OK;
}

}  // extern "C"
