// mpc_oracle64.cu -- FP64 GPU restatement of the split-step propagator (TEST INFRASTRUCTURE).
//
// The CPU oracle (mpc_oracle.c) step for step, on a complex128 device field: the checker of the
// complex64 product path on whole runs of the large cells.  Nothing in the product links it.
// Built with --fmad=false: every pointwise FP64 operation rounds as the CPU oracle's (which is
// compiled with -ffp-contract=off); the FP64 math functions (pow, exp, sin, cos) are CUDA's and
// agree with the host's to an ulp or two.
#include <cuda_runtime.h>
#include <cufft.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "mpc_oracle64.h"

// constants.h:1-11
#define ZW0 377.0
#define NC 1.0
#define FCTR 0.89
#define IH 27.21
#define EF 5.14220642e11
#define ME 9.1094e-31
#define EL0 1.602e-19
#define T0 2.4188843265e-17
#define C0 299792458.0
#define HBAR 1.054560652926899e-34
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static thread_local std::string g_err;
static int fail(const char* what, const char* detail = "") {
    g_err = std::string(what) + (detail[0] ? ": " : "") + detail;
    return -1;
}
#define CK(x, what)                                                       \
    do {                                                                  \
        cudaError_t e_ = (x);                                             \
        if (e_ != cudaSuccess) return fail(what, cudaGetErrorString(e_)); \
    } while (0)
#define CF(x, what)                                         \
    do {                                                    \
        if ((x) != CUFFT_SUCCESS) return fail(what, "cufft"); \
    } while (0)

struct or64_ctx {
    or_params p;
    or_switches sw;
    std::vector<double> betas, wr, w, r;
    char gas[16];
    int Nx, Ny, Nt;
    long NP, N;
    cudaStream_t st = nullptr;
    cufftHandle plan3 = 0, plant = 0;
    double2 *A = nullptr, *C1 = nullptr, *C2 = nullptr, *buf = nullptr;
    double2* tab = nullptr;      // expD0 (Nt), expRx (Nx), expRy (Ny)
    double* wbuff = nullptr;     // fftshift(w), Nt
    double* red = nullptr;       // reductions: 2 sums + per-pencil energies (NP)
    double* W = nullptr;         // ionization terms, 5 N (plasma on; allocated on first use)
    std::vector<double> henergy;
    // ionization constants (plasma.c:118-213)
    double Kon, I1, Kon1, Kon2, Kon3, Kon4, Kon5, Kon6, K1, K2, K3, K4, K5;
};

// ---------------------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 conj2(double2 a) { return make_double2(a.x, -a.y); }

// propagation.c:65-108 after the transforms: the three diagonal factors and the 1/N scale,
// applied in the CPU oracle's order (D, conj Ry, conj Rx, scale)
__global__ void k_linear_factors(double2* A, long N, int Nx, int Ny, const double2* D, const double2* Rx,
                                 const double2* Ry, double s) {
    const long NP = (long)Nx * Ny;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < N; q += (long)gridDim.x * blockDim.x) {
        const long k = q / NP;
        const long rem = q - k * NP;
        const int j = (int)(rem / Nx), i = (int)(rem - (long)j * Nx);
        double2 a = cmul(A[q], D[k]);
        a = cmul(a, conj2(Ry[j]));
        a = cmul(a, conj2(Rx[i]));
        A[q] = make_double2(a.x * s, a.y * s);
    }
}

// propagation.c:196 / mpc_oracle.c or_sst: dA = -1.0 * I * dA * wbuff[k]
__global__ void k_deriv(double2* d, long N, long NP, const double* wbuff) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < N; q += (long)gridDim.x * blockDim.x) {
        const double2 v = d[q];
        const double wk = wbuff[q / NP];
        d[q] = make_double2(v.y * wk, -v.x * wk);
    }
}

struct NLArgs {
    double gamma2, w0, dzz, rho_nt, Kon, I1;
    double Kon1, Kon2, Kon3, Kon4, Kon5, Kon6, K1, K2, K3, K4, K5;
    double g_sst;   // gamma2 / w0
    int sst_on, plasm, Nt;
    long NP;
};

// The nonlinear step (propagation.c:164-327, plasma.c:118-245, corrected, the prefix run forward
// in t) in three passes with the CPU oracle's operations in its order: the per-point ionization
// terms (every point in parallel), the prefix along t (one pencil per thread), then the combine
// and the apply (every point in parallel).  d holds the unnormalised IFFT_t of -i w FFT_t A
// (sst_on) and is not read otherwise.
// W[0] = W1 (then fe_sp), W[1] = W2, W[2] = Wava, W[3] = sigma, W[4] = tau_c; N values each.
__global__ void k_ion_terms(const double2* A, NLArgs a, long N, double* W) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < N; q += (long)gridDim.x * blockDim.x) {
        const double2 Aq = A[q];
        const double absA = hypot(Aq.x, Aq.y);
        double Ip = pow(absA, 2) * HBAR * a.w0;                      // plasma.c:133-139
        if (Ip == 0) Ip = 1e-30;
        const double E0 = sqrt(2.0 * ZW0 * Ip / NC) * FCTR;          // :145-149
        const double dat = fabs(E0) / EF;
        double r1 = a.Kon1 * pow(a.Kon3 / dat, a.Kon5) * exp(-a.Kon3 / (3.0 * dat));
        double r2 = a.Kon2 * pow(a.Kon4 / dat, a.Kon6) * exp(-a.Kon4 / (3.0 * dat));
        if (isnan(r1)) r1 = 0.0;                                      // :184-192
        if (isnan(r2)) r2 = 0.0;
        const double ve = sqrt(a.K1 * pow(E0, 2.0) / (a.K2 * pow(0.0 + a.w0, 2.0)));   // A18
        const double tc = 1.0 / (a.K3 * ve);                          // :203-213
        const double sg = isinf(tc) ? 0.0 : a.K4 * tc / (1.0 + a.K5 * pow(tc, 2.0));  // A27
        W[q] = r1;
        W[N + q] = r2;
        W[2 * N + q] = sg * Ip / a.I1;
        W[3 * N + q] = sg;
        W[4 * N + q] = tc;
    }
}

// the prefix along t of one pencil per thread (plasma.c:223-231 forward, :238-241): W[0] := fe_sp
__global__ void k_ion_prefix(NLArgs a, long N, double* W) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= a.NP) return;
    double R = 0.0, ions1 = 0.0, ions2 = 0.0;   // ions1[k], ions2[k] before slice k
    for (int k = 0; k < a.Nt; k++) {
        const long q = (long)k * a.NP + i;
        const double W1 = W[q], W2 = W[N + q], Wava = W[2 * N + q], sg = W[3 * N + q];
        W[q] = (ions1 * 1.0 + ions2 * 2.0) * sg;
        R = R + W1 * a.Kon;
        R = R + (1.0 - R) * Wava * a.Kon;
        const double n1 = 1.0 - exp(-R) - ions2;
        const double n2 = ions2 + W2 * a.Kon * ions1;
        ions1 = n1;
        ions2 = n2;
    }
}

// the combine (propagation.c:283-309, A13) and the apply (:317-327, A14); W is read only with
// plasma on
__global__ void k_nl_apply(double2* A, const double2* d, NLArgs a, long N, const double* W) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < N; q += (long)gridDim.x * blockDim.x) {
        const double2 Aq = A[q];
        double sre = 0.0, sim = 0.0;
        if (a.sst_on == 1) {
            const double2 dv = d[q];
            const double dx = dv.x / (double)a.Nt, dy = dv.y / (double)a.Nt;
            // 2 d conj(A) + A conj(d)
            const double p = 2.0 * dx, qq = 2.0 * dy;
            const double t1r = p * Aq.x - qq * (-Aq.y), t1i = p * (-Aq.y) + qq * Aq.x;
            const double t2r = Aq.x * dx - Aq.y * (-dy), t2i = Aq.x * (-dy) + Aq.y * dx;
            sre = a.g_sst * (t1r + t2r);
            sim = a.g_sst * (t1i + t2i);
        }
        const double absA = hypot(Aq.x, Aq.y);
        double anr, ani;
        if (a.plasm == 1) {
            const double z1 = a.gamma2 * pow(absA, 2.0);
            const double pl = a.rho_nt * W[q] / 2.0;
            const double z2y = a.w0 * W[4 * N + q] * pl;
            anr = (0.0 - sre - pl);
            ani = (z1 - sim - z2y);
        } else {
            const double tempab = pow(absA, 2.0);
            anr = -sre;
            ani = a.gamma2 * tempab - sim;
        }
        const double er = exp(a.dzz * anr);
        const double ei = a.dzz * ani;
        const double c = cos(ei), s = sin(ei);
        const double nx = Aq.x * er * c - Aq.y * er * s;
        const double ny = Aq.y * er * c + Aq.x * er * s;
        A[q] = make_double2(nx, ny);
    }
}

// sum_t |A|^2 per pencil (propagation.c:343-354 before the sums over x or y)
__global__ void k_pencil_energy(const double2* A, long NP, int Nt, double* E) {
    const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
    if (i >= NP) return;
    double s = 0.0;
    for (int k = 0; k < Nt; k++) {
        const double2 v = A[(long)k * NP + i];
        const double m = hypot(v.x, v.y);
        s += pow(m, 2.0);
    }
    E[i] = s;
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    __syncthreads();
    return t;
}

// setStep's sums (propagation.c:624-633): sums[0] += |C2 - C1|^2, sums[1] += |C2|^2
__global__ void k_err_sums(const double2* C1, const double2* C2, long N, double* sums) {
    __shared__ double sh[32];
    double s1 = 0.0, s2 = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < N; q += (long)gridDim.x * blockDim.x) {
        const double2 a = C1[q], b = C2[q];
        const double m1 = hypot(b.x - a.x, b.y - a.y), m2 = hypot(b.x, b.y);
        s1 += pow(m1, 2);
        s2 += pow(m2, 2);
    }
    s1 = block_sum(s1, sh);
    s2 = block_sum(s2, sh);
    if (threadIdx.x == 0) {
        atomicAdd(&sums[0], s1);
        atomicAdd(&sums[1], s2);
    }
}

__global__ void k_sum_abs2(const double2* A, long N, double* sum) {
    __shared__ double sh[32];
    double s = 0.0;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < N; q += (long)gridDim.x * blockDim.x) {
        const double2 a = A[q];
        s += a.x * a.x + a.y * a.y;
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) atomicAdd(sum, s);
}

// MPC.c:377-381: A = (4/3) C2 - (1/3) C1
__global__ void k_richardson(double2* A, const double2* C1, const double2* C2, long N) {
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < N; q += (long)gridDim.x * blockDim.x) {
        const double2 a = C1[q], b = C2[q];
        A[q] = make_double2((4.0 / 3.0) * b.x - (1.0 / 3.0) * a.x, (4.0 / 3.0) * b.y - (1.0 / 3.0) * a.y);
    }
}

// or_mirror_lens: A *= cexp(-I k0 r2 / roc), r2 = r[i]^2 + r[j]^2
__global__ void k_lens(double2* A, long N, int Nx, int Ny, const double* r, double k0, double roc) {
    const long NP = (long)Nx * Ny;
    for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < N; q += (long)gridDim.x * blockDim.x) {
        const long rem = q % NP;
        const int j = (int)(rem / Nx), i = (int)(rem - (long)j * Nx);
        const double r2 = r[i] * r[i] + r[j] * r[j];
        const double ph = ((-k0) * r2) / roc;
        const double2 f = make_double2(cos(ph), sin(ph));
        A[q] = cmul(A[q], f);
    }
}

// ---------------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------------
static int grid_for(long n) {
    long b = (n + 255) / 256;
    return (int)(b < 152L * 16 ? b : 152L * 16);
}

static int pass_sign(double z, double Cav) { return ((int)(floor(z / Cav) + 1) % 2) * 2 - 1; }  // propagation.c:378

static int bounces_between(double z0, double z1, double Cav) {
    const double eps = 1e-9;
    return (int)(floor(z1 / Cav + eps) - floor(z0 / Cav + eps));
}

// The factors of one linear half step (propagation.c:128-158): expD0 (Nt), then the x and y
// diffraction tables (Nx, Ny), with calcexpR's sign bookkeeping on *signmem.
typedef std::vector<or_complex> Tables;
static void half_step_tables(or64_ctx* c, double dzz, int* signmem, double z, Tables* t) {
    const or_params* p = &c->p;
    t->resize((size_t)c->Nt + c->Nx + c->Ny);
    or_expD0(t->data(), c->Nt, dzz, p->alpha, p->betas);
    or_calcexpR(t->data() + c->Nt, c->Nx, c->Ny, signmem, z, p->Cav, p->k0, dzz / 2, p->wr, &c->sw);
    or_calcexpR(t->data() + c->Nt + c->Nx, c->Ny, c->Ny, signmem, z, p->Cav, p->k0, dzz / 2, p->wr, &c->sw);
}

// or_linearstep (propagation.c:65-108) with the factors `t`, or with the products t * u: two
// consecutive linear half steps with no nonlinear step between them are one transform pair with
// the product of their diagonal factors (the same operator; only FP64 rounding differs).
static int linearstep(or64_ctx* c, double2* A, const Tables& t, const Tables* u = nullptr) {
    Tables m;
    const Tables* f = &t;
    if (u) {
        m.resize(t.size());
        for (size_t i = 0; i < t.size(); i++) m[i] = t[i] * (*u)[i];
        f = &m;
    }
    CK(cudaMemcpyAsync(c->tab, f->data(), sizeof(double2) * f->size(), cudaMemcpyHostToDevice, c->st), "H2D tables");
    CF(cufftExecZ2Z(c->plan3, (cufftDoubleComplex*)A, (cufftDoubleComplex*)A, CUFFT_FORWARD), "fft3 fwd");
    const double2* D = c->tab;
    k_linear_factors<<<grid_for(c->N), 256, 0, c->st>>>(A, c->N, c->Nx, c->Ny, D, D + c->Nt, D + c->Nt + c->Nx,
                                                        1.0 / (double)c->N);
    CK(cudaGetLastError(), "k_linear_factors");
    CF(cufftExecZ2Z(c->plan3, (cufftDoubleComplex*)A, (cufftDoubleComplex*)A, CUFFT_INVERSE), "fft3 inv");
    // the host tables may change before the copy has been consumed: wait for it
    CK(cudaStreamSynchronize(c->st), "tables in use");
    return 0;
}

static int beam_profiles(or64_ctx* c, const double2* A, double* BP1, double* BP2) {
    double* E = c->red + 2;
    k_pencil_energy<<<(int)((c->NP + 255) / 256), 256, 0, c->st>>>(A, c->NP, c->Nt, E);
    CK(cudaGetLastError(), "k_pencil_energy");
    CK(cudaMemcpyAsync(c->henergy.data(), E, sizeof(double) * c->NP, cudaMemcpyDeviceToHost, c->st), "D2H E");
    CK(cudaStreamSynchronize(c->st), "beam profiles");
    memset(BP1, 0, sizeof(double) * c->Nx);
    memset(BP2, 0, sizeof(double) * c->Ny);
    for (int j = 0; j < c->Ny; j++)
        for (int i = 0; i < c->Nx; i++) {
            const double e = c->henergy[(size_t)j * c->Nx + i];
            BP1[i] += e;
            BP2[j] += e;
        }
    return 0;
}

// The nonlinear step of propagation.c:164-327 on device field A: the SST derivative
// (t transforms, -i w) and the three nonlinear passes.
static int nonlinear(or64_ctx* c, double2* A, double dzz) {
    const or_params* p = &c->p;
    if (p->sst_on == 1) {
        CK(cudaMemcpyAsync(c->buf, A, sizeof(double2) * c->N, cudaMemcpyDeviceToDevice, c->st), "copy dA");
        CF(cufftExecZ2Z(c->plant, (cufftDoubleComplex*)c->buf, (cufftDoubleComplex*)c->buf, CUFFT_FORWARD), "fft t fwd");
        k_deriv<<<grid_for(c->N), 256, 0, c->st>>>(c->buf, c->N, c->NP, c->wbuff);
        CK(cudaGetLastError(), "k_deriv");
        CF(cufftExecZ2Z(c->plant, (cufftDoubleComplex*)c->buf, (cufftDoubleComplex*)c->buf, CUFFT_INVERSE), "fft t inv");
    }
    NLArgs a;
    a.gamma2 = p->gamma2;
    a.w0 = p->w0;
    a.dzz = dzz;
    a.rho_nt = p->rho_nt;
    a.Kon = c->Kon;
    a.I1 = c->I1;
    a.Kon1 = c->Kon1; a.Kon2 = c->Kon2; a.Kon3 = c->Kon3; a.Kon4 = c->Kon4; a.Kon5 = c->Kon5; a.Kon6 = c->Kon6;
    a.K1 = c->K1; a.K2 = c->K2; a.K3 = c->K3; a.K4 = c->K4; a.K5 = c->K5;
    a.g_sst = p->gamma2 / p->w0;
    a.sst_on = p->sst_on;
    a.plasm = p->plasm;
    a.Nt = c->Nt;
    a.NP = c->NP;
    if (p->plasm == 1) {
        if (!c->W) CK(cudaMalloc(&c->W, sizeof(double) * 5 * c->N), "cudaMalloc ionization terms");
        k_ion_terms<<<grid_for(c->N), 256, 0, c->st>>>(A, a, c->N, c->W);
        CK(cudaGetLastError(), "k_ion_terms");
        k_ion_prefix<<<(int)((c->NP + 127) / 128), 128, 0, c->st>>>(a, c->N, c->W);
        CK(cudaGetLastError(), "k_ion_prefix");
    }
    k_nl_apply<<<grid_for(c->N), 256, 0, c->st>>>(A, c->buf, a, c->N, c->W);
    CK(cudaGetLastError(), "k_nl_apply");
    return 0;
}

// propagation.c:334-361 after the step (change == 1): the as-written bounce bookkeeping, the beam
// profiles and their 1/e^2 sizes
static int step_diagnostics(or64_ctx* c, const double2* A, int* signmem, double z, double* puls_e, double* BP1,
                            double* BP2, double* y1, double* y2, double* bps1, double* bps2) {
    const or_params* p = &c->p;
    const int signum = pass_sign(z, p->Cav);
    if (*signmem == -signum) {
        *puls_e = *puls_e * p->Ab_M;
        *signmem *= -1;
    }
    if (beam_profiles(c, A, BP1, BP2)) return -1;
    or_calc1oes(BP1, c->Nx, p->r, bps1, y1);
    or_calc1oes(BP2, c->Ny, p->r, bps2, y2);
    return 0;
}

// or_ssfmprop (propagation.c:111-372) on device field A
static int ssfmprop(or64_ctx* c, double2* A, double dzz, int* signmem, double z, double* puls_e, double* BP1,
                    double* BP2, double* y1, double* y2, double* bps1, double* bps2, int change) {
    Tables t;
    half_step_tables(c, dzz, signmem, z, &t);
    if (linearstep(c, A, t)) return -1;
    if (nonlinear(c, A, dzz)) return -1;
    if (linearstep(c, A, t)) return -1;
    if (change == 1 && step_diagnostics(c, A, signmem, z, puls_e, BP1, BP2, y1, y2, bps1, bps2)) return -1;
    return 0;
}

static int lens(or64_ctx* c, double2* A) {
    k_lens<<<grid_for(c->N), 256, 0, c->st>>>(A, c->N, c->Nx, c->Ny, c->red + 2 + c->NP, c->p.k0, c->p.roc);
    CK(cudaGetLastError(), "k_lens");
    return 0;
}

extern "C" {

const char* or64_last_error(void) { return g_err.c_str(); }

int or64_destroy(or64_ctx* c) {
    if (!c) return 0;
    if (c->st) cudaStreamSynchronize(c->st);
    if (c->plan3) cufftDestroy(c->plan3);
    if (c->plant) cufftDestroy(c->plant);
    for (void* ptr : {(void*)c->A, (void*)c->C1, (void*)c->C2, (void*)c->buf, (void*)c->tab, (void*)c->wbuff,
                      (void*)c->red, (void*)c->W})
        if (ptr) cudaFree(ptr);
    if (c->st) cudaStreamDestroy(c->st);
    delete c;
    return 0;
}

int or64_create(or64_ctx** out, const or_params* p, const or_switches* sw) {
    if (!out || !p || !sw) return fail("null argument");
    or_switches def;
    or_default_switches(&def);
    def.bounce_lens = sw->bounce_lens;
    if (memcmp(&def, sw, sizeof(def)) != 0) return fail("the GPU oracle restates the corrected physics only");
    or64_ctx* c = new or64_ctx();
    c->p = *p;
    c->sw = *sw;
    c->Nx = p->Nx;
    c->Ny = p->Ny;
    c->Nt = p->Nt;
    c->NP = (long)p->Nx * p->Ny;
    c->N = c->NP * p->Nt;
    c->betas.assign(p->betas, p->betas + p->Nt);
    c->wr.assign(p->wr, p->wr + p->Ny);
    c->w.assign(p->w, p->w + p->Nt);
    c->r.assign(p->r, p->r + p->Ny);
    c->p.betas = c->betas.data();
    c->p.wr = c->wr.data();
    c->p.w = c->w.data();
    c->p.r = c->r.data();
    memcpy(c->gas, p->gas, sizeof(c->gas));
    c->henergy.resize(c->NP);
    // ionization constants, plasma.c:118-213 as or_ioniz states them
    {
        double I2 = 0, Iion[2], nq[2], f_lm[2], mq[2], C_nl[2], lq[2] = {0.0, 0.0};
        or_ionizpot(p->gas, &c->I1, &I2);
        Iion[0] = c->I1 / IH;
        Iion[1] = I2 / IH;
        nq[0] = 1.0 / sqrt(2.0 * Iion[0]);                    // A11
        nq[1] = 2.0 / sqrt(2.0 * Iion[1]);
        f_lm[0] = f_lm[1] = 1.0;
        mq[0] = mq[1] = 0.0;
        C_nl[0] = sqrt(pow(2.0, 2.0 * nq[0]) * pow(nq[0] * tgamma(nq[0] + lq[0] + 1.0) * tgamma(nq[0] - lq[0]), -1.0));
        C_nl[1] = sqrt(pow(2.0, 2.0 * nq[1]) * pow(nq[1] * tgamma(nq[1] + lq[1] + 1.0) * tgamma(nq[1] - lq[1]), -1.0));
        double Natm = 0, sigm_coll = 0;
        or_Natoms(p->gas, &Natm, &sigm_coll);
        const double k0 = p->w0 / C0;
        c->Kon = p->deltat / T0;
        c->K1 = 2.0 * pow(EL0, 2.0);
        c->K2 = 4.0 * pow(ME, 2.0);
        c->K3 = sigm_coll * p->rho_nt;
        c->K4 = k0 / (p->n0 * p->rho_c) * p->w0;
        c->K5 = pow(p->w0, 2);
        c->Kon1 = pow(fabs(C_nl[0]), 2.0) * sqrt(6.0 / M_PI) * f_lm[0] * Iion[0];
        c->Kon2 = pow(fabs(C_nl[1]), 2.0) * sqrt(6.0 / M_PI) * f_lm[1] * Iion[1];
        c->Kon3 = 2.0 * pow(2.0 * Iion[0], 3.0 / 2.0);
        c->Kon4 = 2.0 * pow(2.0 * Iion[1], 3.0 / 2.0);
        c->Kon5 = 2.0 * nq[0] - mq[0] - 3.0 / 2.0;
        c->Kon6 = 2.0 * nq[1] - mq[1] - 3.0 / 2.0;
    }
#define CKD(x, what)                          \
    do {                                      \
        cudaError_t e_ = (x);                 \
        if (e_ != cudaSuccess) {              \
            or64_destroy(c);                  \
            return fail(what, cudaGetErrorString(e_)); \
        }                                     \
    } while (0)
    CKD(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking), "stream");
    CKD(cudaMalloc(&c->A, sizeof(double2) * c->N), "cudaMalloc field");
    CKD(cudaMalloc(&c->buf, sizeof(double2) * c->N), "cudaMalloc buffer");
    CKD(cudaMalloc(&c->tab, sizeof(double2) * (c->Nt + c->Nx + c->Ny)), "cudaMalloc tables");
    CKD(cudaMalloc(&c->wbuff, sizeof(double) * c->Nt), "cudaMalloc wbuff");
    CKD(cudaMalloc(&c->red, sizeof(double) * (2 + c->NP + c->Ny)), "cudaMalloc reductions");
    // wbuff = fftshift(w) (propagation.c:170-177); r for the mirror lens after the energies
    std::vector<double> wb(c->w);
    for (int k = 0; k < c->Nt / 2; k++) {
        wb[k] = c->w[c->Nt / 2 + k];
        wb[c->Nt / 2 + k] = c->w[k];
    }
    CKD(cudaMemcpy(c->wbuff, wb.data(), sizeof(double) * c->Nt, cudaMemcpyHostToDevice), "H2D wbuff");
    CKD(cudaMemcpy(c->red + 2 + c->NP, c->r.data(), sizeof(double) * c->Ny, cudaMemcpyHostToDevice), "H2D r");
    if (cufftPlan3d(&c->plan3, c->Nt, c->Ny, c->Nx, CUFFT_Z2Z) != CUFFT_SUCCESS) {
        or64_destroy(c);
        return fail("cufftPlan3d");
    }
    int n[1] = {c->Nt};
    if (cufftPlanMany(&c->plant, 1, n, n, (int)c->NP, 1, n, (int)c->NP, 1, CUFFT_Z2Z, (int)c->NP) != CUFFT_SUCCESS) {
        or64_destroy(c);
        return fail("cufftPlanMany t");
    }
    if (cufftSetStream(c->plan3, c->st) != CUFFT_SUCCESS || cufftSetStream(c->plant, c->st) != CUFFT_SUCCESS) {
        or64_destroy(c);
        return fail("cufftSetStream");
    }
#undef CKD
    *out = c;
    return 0;
}

int or64_upload(or64_ctx* c, const double* A) {
    if (!c || !A) return fail("null argument");
    CK(cudaMemcpyAsync(c->A, A, sizeof(double2) * c->N, cudaMemcpyHostToDevice, c->st), "H2D field");
    CK(cudaStreamSynchronize(c->st), "upload");
    return 0;
}

int or64_download(or64_ctx* c, double* A) {
    if (!c || !A) return fail("null argument");
    CK(cudaMemcpyAsync(A, c->A, sizeof(double2) * c->N, cudaMemcpyDeviceToHost, c->st), "D2H field");
    CK(cudaStreamSynchronize(c->st), "download");
    return 0;
}

int or64_ssfmprop(or64_ctx* c, double dzz, int* signmem, double z, double* puls_e, double* BP1, double* BP2,
                  double* y1, double* y2, double* bps1, double* bps2, int change) {
    if (!c || !signmem || !puls_e) return fail("null argument");
    if (change == 1 && (!BP1 || !BP2 || !y1 || !y2 || !bps1 || !bps2)) return fail("null diagnostic output");
    if (ssfmprop(c, c->A, dzz, signmem, z, puls_e, BP1, BP2, y1, y2, bps1, bps2, change)) return -1;
    CK(cudaStreamSynchronize(c->st), "ssfmprop");
    return 0;
}

// or_run_fixed, with the adjacent linear half steps of consecutive steps merged into one
// transform pair (not across a mirror lens, which sits between them)
int or64_run_fixed(or64_ctx* c, or_state* st, int nsteps) {
    if (!c || !st) return fail("null argument");
    if (nsteps <= 0) return 0;
    const or_params* p = &c->p;
    Tables cur, next;
    double zs = (double)st->nstep * st->dzz;
    half_step_tables(c, st->dzz, &st->signmem, zs + 1e-9 * p->Cav, &cur);
    if (linearstep(c, c->A, cur)) return -1;
    for (int s = 0; s < nsteps; s++) {
        if (nonlinear(c, c->A, st->dzz)) return -1;
        st->nstep++;
        st->z = (double)st->nstep * st->dzz;
        const int nb = bounces_between(zs, st->z, p->Cav);
        const int last = (s == nsteps - 1);
        if (nb > 0 || last) {
            if (linearstep(c, c->A, cur)) return -1;
            for (int b = 0; b < nb; b++) {
                if (c->sw.bounce_lens && lens(c, c->A)) return -1;
                st->puls_e *= p->Ab_M;
            }
            zs = st->z;
            if (!last) {
                half_step_tables(c, st->dzz, &st->signmem, zs + 1e-9 * p->Cav, &cur);
                if (linearstep(c, c->A, cur)) return -1;
            }
        } else {
            zs = st->z;
            half_step_tables(c, st->dzz, &st->signmem, zs + 1e-9 * p->Cav, &next);
            if (linearstep(c, c->A, cur, &next)) return -1;
            cur.swap(next);
        }
    }
    CK(cudaStreamSynchronize(c->st), "run_fixed");
    return 0;
}

// or_double_step
int or64_double_step(or64_ctx* c, or_state* st, double dz_used, int force, int* own_bad, double* own_err) {
    if (!c || !st) return fail("null argument");
    const or_params* p = &c->p;
    for (double2** b : {&c->C1, &c->C2})
        if (!*b) CK(cudaMalloc(b, sizeof(double2) * c->N), "cudaMalloc step-doubling fields");
    const double dz = dz_used > 0 ? dz_used : st->dzz;
    CK(cudaMemcpyAsync(c->C1, c->A, sizeof(double2) * c->N, cudaMemcpyDeviceToDevice, c->st), "C1 = A");
    CK(cudaMemcpyAsync(c->C2, c->A, sizeof(double2) * c->N, cudaMemcpyDeviceToDevice, c->st), "C2 = A");
    std::vector<double> BP1(c->Nx), BP2(c->Ny);
    if (ssfmprop(c, c->C1, 2 * dz, &st->signmem, st->z, &st->puls_e, BP1.data(), BP2.data(), st->y1, st->y2,
                 &st->bps1, &st->bps2, 0))
        return -1;
    {   // C2: two steps of dz, the middle half steps merged
        Tables t1, t2;
        half_step_tables(c, dz, &st->signmem, st->z, &t1);
        if (linearstep(c, c->C2, t1) || nonlinear(c, c->C2, dz)) return -1;
        half_step_tables(c, dz, &st->signmem, st->z, &t2);
        if (linearstep(c, c->C2, t1, &t2) || nonlinear(c, c->C2, dz) || linearstep(c, c->C2, t2)) return -1;
        if (step_diagnostics(c, c->C2, &st->signmem, st->z, &st->puls_e, BP1.data(), BP2.data(), st->y1, st->y2,
                             &st->bps1, &st->bps2))
            return -1;
    }
    st->attempts++;
    CK(cudaMemsetAsync(c->red, 0, 2 * sizeof(double), c->st), "memset sums");
    k_err_sums<<<grid_for(c->N), 256, 0, c->st>>>(c->C1, c->C2, c->N, c->red);
    CK(cudaGetLastError(), "k_err_sums");
    double sums[2];
    CK(cudaMemcpyAsync(sums, c->red, sizeof(sums), cudaMemcpyDeviceToHost, c->st), "D2H sums");
    CK(cudaStreamSynchronize(c->st), "sums");
    st->err = sqrt(sums[0]) / sqrt(sums[1]);
    st->dzz = dz;
    int bad = 0;
    or_step_rule(st->err, &st->dzz, p->def_err, p->dzmin, st->y1, st->y2, &bad);
    if (own_bad) *own_bad = bad;
    if (own_err) *own_err = st->err;
    if (force >= 0) bad = !force;
    st->bad = bad;
    if (bad == 0) {
        k_richardson<<<grid_for(c->N), 256, 0, c->st>>>(c->A, c->C1, c->C2, c->N);
        CK(cudaGetLastError(), "k_richardson");
        const double z0 = st->z;
        st->z = st->z + 2.0 * dz;                            // A26: the step just taken
        const int nb = bounces_between(z0, st->z, p->Cav);
        for (int b = 0; b < nb; b++) {
            if (c->sw.bounce_lens && lens(c, c->A)) return -1;
            st->puls_e *= p->Ab_M;
        }
        if (st->z > p->dist) st->z = p->dist;
        st->nstep++;
    }
    CK(cudaStreamSynchronize(c->st), "double_step");
    return 0;
}

int or64_energy(or64_ctx* c, double* e) {
    if (!c || !e) return fail("null argument");
    CK(cudaMemsetAsync(c->red, 0, sizeof(double), c->st), "memset");
    k_sum_abs2<<<grid_for(c->N), 256, 0, c->st>>>(c->A, c->N, c->red);
    CK(cudaGetLastError(), "k_sum_abs2");
    CK(cudaMemcpyAsync(e, c->red, sizeof(double), cudaMemcpyDeviceToHost, c->st), "D2H energy");
    CK(cudaStreamSynchronize(c->st), "energy");
    return 0;
}

}  // extern "C"
