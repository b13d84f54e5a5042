// mpc_kernels.cuh -- the split-step propagator's sweeps over HBM and their helpers.
//
// Device layout of the field between sweeps ("slot layout"): the field is kept in the
// (x, y, omega) domain, omega in FFT position order.  Slots are interleaved in groups of
// SLO: element (slot s, pencil q = y*Nx + x) lives at ((s/SLO)*Nx*Ny + q)*SLO + s%SLO.
// SLO = 2 makes the t-rows of an 8-pencil tile 128 B; the default variants use SLO = 1 (rows of
// P * 8 B), which keeps every omega-plane contiguous for the plane passes.
//
// Sweep 1, pencil pass (one CTA per tile of P neighbouring (x,y) pencils, all of t):
//   IFFT_t of -i*omega*S -> dA,  IFFT_t of S -> A,  nonlinear step N(dz) (Kerr, self-
//   steepening, ADK ionization with two affine prefix scans along t, plasma absorption and
//   defocusing, A *= exp(dz*A_nl)),  FFT_t -> S.
// Sweep 2, plane pass, the linear step factorised as (IFFT_x Rx FFT_x)(IFFT_y Ry D FFT_y):
//   either one kernel per unit of omega-planes on a thread-block cluster (FFT_y, Ry(ky) D(omega)
//   / (Nx Ny Nt), IFFT_y on columns; the columns become rows in one exchange between the
//   cluster's CTAs through distributed shared memory; FFT_x, Rx(kx), IFFT_x on rows), or two
//   kernels without clusters, the y part on column strips and the x part on row strips.
#pragma once
#include <cooperative_groups.h>
#include <type_traits>
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpc_fft.cuh"
#include "mpc_tma.cuh"

namespace cg = cooperative_groups;

namespace mpc {

constexpr int kThreads = 512;          // threads of a one-CTA-per-SM launch (128 registers each)
constexpr int kTilePoints = 16384;     // default pencil tile: P * Nt complex points (128 KB)
// butterflies of a pencil thread unrolled together per FFT stage (the plane sweep keeps 1: its
// kernels are at the register limit)
#ifndef MPC_PENCIL_UNROLL
#define MPC_PENCIL_UNROLL 4
#endif
constexpr int kPencilUnroll = MPC_PENCIL_UNROLL;
// dA samples loaded ahead of use in the nonlinear walk, and the first walk's unroll (tuning builds
// set them with MPC_NVCC_EXTRA, e.g. "-DMPC_DA_PREFETCH=8")
#ifndef MPC_DA_PREFETCH
#define MPC_DA_PREFETCH 4
#endif
#ifndef MPC_S1_UNROLL
#define MPC_S1_UNROLL 8
#endif
constexpr int kDAPrefetch = MPC_DA_PREFETCH;
constexpr int kS1Unroll = MPC_S1_UNROLL;
static_assert(kDAPrefetch >= 1 && kDAPrefetch <= 32, "dA prefetch depth within a 32-sample chunk");

// FP32 constants of the nonlinear step, computed on the host in FP64.
struct NLConst {
    float dz;        // step length [m]
    float gam;       // gamma2 / fs^2: Kerr phase per unit |a|^2 [1/m]
    float sst_c;     // gamma2 / (w0 fs^2), 0 when self-steepening is off
    float I_scale;   // intensity [W/m^2] per unit |a|^2
    float E_c;       // field in atomic units = sqrt(I) * E_c
    float inv_E_c;   // 1 / E_c
    float l2K1[2], l2K3[2], K5[2], K3l2e[2];  // ADK: log2 K1, log2 K3, K5, K3 log2(e) / 3
    float Kon;       // deltat / T0
    float Kuv;       // sigma_coll rho_nt v_e per unit F (v_e = e E0 / (sqrt 2 me w0))
    float K4w0;      // k0 w0^2 / (n0 rho_c)
    float w0sq;      // w0^2
    float inv_w0;    // 1 / w0
    float invI1_Kon; // Kon / I1 (I1 in eV, as the reference divides by it)
    float rho_half;  // rho_nt / 2
    int plasma;      // 1 = ionization and plasma terms on
};

// Pencil tile view: line = pencil p, element (pos, p).  For P < 16 a pad of P slots every
// 2^SH positions and every 32 positions keeps the FFT stages and the per-thread t walks free
// of shared-memory bank conflicts (SH = 4 for P = 8, 3 for P = 4).  The pad depends on pos
// only through pos >> SH and pos >> 5, so a walk of CH samples from a multiple of CH has the
// same offsets everywhere, at(t0 + i, p) - at(t0, p) == walk(i), for CH = 32 and, when SH = 4,
// for CH = 16.
template <int NT, int P>
struct PencilView {
    static constexpr int NLINES = P;
    static constexpr int SH = (P < 8) ? 3 : 4;
    static constexpr __host__ __device__ __forceinline__ int at(int pos, int p) {
        if constexpr (P < 16) return pos * P + p + P * ((pos >> SH) + (pos >> 5));
        else return pos * P + p;
    }
    static constexpr __host__ __device__ __forceinline__ int walk(int i) { return at(i, 0) - at(0, 0); }
    static constexpr int SIZE = (P < 16) ? (NT * P + P * ((NT >> SH) + NT / 32)) : NT * P;
    static_assert(P >= 4, "pencil tile of at least 4 pencils");
};

enum PencilMode : int {
    PM_ENTRY_C128 = 0,  // real-space complex128 (reference layout, physical units) -> S
    PM_ENTRY_C64 = 1,   // real-space complex64 (reference layout, device units) -> S
    PM_STEP = 2,        // S -> N(dz) -> S
    PM_EXIT_C128 = 3,   // S -> real-space complex128 (physical units) + per-pencil energy
    PM_EXIT_C64 = 4,    // S -> real-space complex64 (device units) + per-pencil energy
    PM_TEMP = 5,        // S -> temporal profile sums only (no store)
    PM_IONIZ = 6,       // real-space complex128 -> tau_c, freeelectrons_sp (FP64, reference layout)
};

struct PencilArgs {
    const void* in;          // input field (layout by mode)
    void* out;               // output field (may alias in)
    float2* scratch;         // per-CTA dA scratch, gridDim.x * Nt * P complex64
    const float2* tw;        // W_Nt table, packed (mpc_fft.cuh Twiddles)
    const float* wpos;       // omega of each t position (FFT position order), Nt
    double* pencil_energy;   // EXIT: sum_t |out|^2 per pencil, Nx*Ny
    double* temp;            // TEMP: sum_xy |out|^2 per t, Nt (accumulated)
    double* tau_out;         // IONIZ: tau_c, reference layout
    double* fe_out;          // IONIZ: freeelectrons_sp, reference layout
    unsigned int* stats;     // STEP: running maxima of the step (nonlinear_tile), or null
    double in_scale;         // ENTRY: input multiplier (to device units, includes 1/Nt)
    double out_scale;        // EXIT/TEMP: output multiplier (from device units)
    int NP;                  // Nx * Ny
    int ntiles;              // NP / P
    NLConst nl;
};

// ---------------------------------------------------------------------------------------
// Affine-map scans of the ionization prefix (plasma.c:223-231, run forward in t).
//   R_k = (1 - b_k)(R_{k-1} + a_k) + b_k          map (B, C): R -> (1-B) R + C
//   (u, v)_{k+1} = (u_k + c2_k v_k, g_k - u_k)     map (M, o): x -> M x + o
// with a_k = W1 Kon, b_k = Wava Kon, c2_k = W2 Kon, g_k = 1 - exp(-R_k); u = ions2,
// v = ions1, both zero before the first slice; fe_sp[k] = (v_k + 2 u_k) sigma_k.
// Chunk maps are composed in FP32 inside a thread's CH points and across chunks in FP64.  Across
// chunks the R map is held as (D, C) = (1 - B, C), R -> D R + C, so that composing two maps is one
// FP64 product and one FP64 FMA (GB300 issues FP64 at 1/64 of its FP32 rate).  D keeps 1 - B to
// FP64's absolute precision (1e-16), which is what the product D R needs; B's own relative
// precision does not enter.
// ---------------------------------------------------------------------------------------
struct MapR { double D, C; };
struct MapUV { double m00, m01, m10, m11, o0, o1; };

__device__ __forceinline__ MapR compose(const MapR& first, const MapR& then) {
    MapR r;
    r.D = then.D * first.D;
    r.C = fma(then.D, first.C, then.C);
    return r;
}
__device__ __forceinline__ MapUV compose(const MapUV& f, const MapUV& t) {
    MapUV r;
    r.m00 = t.m00 * f.m00 + t.m01 * f.m10;
    r.m01 = t.m00 * f.m01 + t.m01 * f.m11;
    r.m10 = t.m10 * f.m00 + t.m11 * f.m10;
    r.m11 = t.m10 * f.m01 + t.m11 * f.m11;
    r.o0 = t.m00 * f.o0 + t.m01 * f.o1 + t.o0;
    r.o1 = t.m10 * f.o0 + t.m11 * f.o1 + t.o1;
    return r;
}
template <class M>
__device__ __forceinline__ M map_ident();
template <>
__device__ __forceinline__ MapR map_ident<MapR>() { return MapR{1.0, 0.0}; }
template <>
__device__ __forceinline__ MapUV map_ident<MapUV>() { return MapUV{1.0, 0.0, 0.0, 1.0, 0.0, 0.0}; }

template <class M>
__device__ __forceinline__ M shfl_up_map(const M& m, int off) {
    M r;
    double* dst = reinterpret_cast<double*>(&r);
    const double* src = reinterpret_cast<const double*>(&m);
#pragma unroll
    for (int i = 0; i < (int)(sizeof(M) / sizeof(double)); i++) dst[i] = __shfl_up_sync(0xffffffffu, src[i], off);
    return r;
}

// Exclusive scan over the TPP chunk maps of each of P pencils, in place in `maps`
// (index p * TPP + c).  One warp per pencil; each lane composes TPP/32 (or 1) chunks.
template <class M, int P, int TPP>
__device__ __forceinline__ void scan_chunks(M* maps, int tid) {
    const int warp = tid >> 5, lane = tid & 31;
    constexpr int NW = P * TPP / 32;       // the CTA has one thread per chunk
    constexpr int CPL = (TPP + 31) / 32;
    for (int p = warp; p < P; p += NW) {
        M* row = maps + p * TPP;
        M acc = map_ident<M>();
        const int c0 = lane * CPL;
#pragma unroll
        for (int j = 0; j < CPL; j++)
            if (c0 + j < TPP) acc = compose(acc, row[c0 + j]);
        // inclusive warp scan of lane aggregates
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const M prev = shfl_up_map(acc, off);
            if (lane >= off) acc = compose(prev, acc);
        }
        M excl = shfl_up_map(acc, 1);
        if (lane == 0) excl = map_ident<M>();
        __syncwarp();
#pragma unroll
        for (int j = 0; j < CPL; j++) {
            if (c0 + j < TPP) {
                const M own = row[c0 + j];
                row[c0 + j] = excl;
                excl = compose(excl, own);
            }
        }
        __syncwarp();
    }
}

// Small-argument elementary functions, from their Taylor series (|x| below the stated bound;
// the CUDA library function is called outside it).  Per split step the nonlinear phase is
// < 0.25 rad and the amplitude exponent < 1/64, so the series branch is the one taken.
// 1 - exp(-x), x >= 0: alternating series to x^6/720 (relative truncation < x^6/5040 < 8e-10)
__device__ __forceinline__ float one_minus_exp_neg(float x) {
    if (x < 0.125f)
        return x * (1.0f - x * (0.5f - x * (1.0f / 6.0f - x * (1.0f / 24.0f - x * (1.0f / 120.0f - x * (1.0f / 720.0f))))));
    return 1.0f - expf(-x);
}
// exp(x): series to x^4/24 for |x| < 1/64 (truncation < |x|^5/120 < 1e-11)
__device__ __forceinline__ float exp_small(float x) {
    if (fabsf(x) < 0.015625f) return 1.0f + x * (1.0f + x * (0.5f + x * (1.0f / 6.0f + x * (1.0f / 24.0f))));
    return expf(x);
}
// sin and cos: series to x^7/7! and x^8/8! for |x| < 1/4 (truncation < 3e-11)
__device__ __forceinline__ void sincos_small(float x, float* sn, float* cs) {
    if (fabsf(x) < 0.25f) {
        const float x2 = x * x;
        *sn = x * (1.0f - x2 * (1.0f / 6.0f - x2 * (1.0f / 120.0f - x2 * (1.0f / 5040.0f))));
        *cs = 1.0f - x2 * (0.5f - x2 * (1.0f / 24.0f - x2 * (1.0f / 720.0f - x2 * (1.0f / 40320.0f))));
    } else {
        sincosf(x, sn, cs);
    }
}

// Per-point ionization coefficients of one sample (plasma.c:133-213 in FP32, A18 fix
// applied).  The ADK rates are evaluated in the log2 domain:
//   log2 W = log2 K1 + K5 (log2 K3 - log2 F) - K3 / (3 F ln 2).
// Second-stage probabilities c2 below 2^-60 per slice are flushed to zero: their whole-pencil
// effect on ions2 is < Nt 2^-60 < 2e-15, far below FP32 resolution, and a tile without any
// second-stage ionization then skips the (ions2, ions1) scan, which is exact there.
constexpr float kC2Flush = 8.673617e-19f;   // 2^-60
struct IonPoint {
    float a, b, c2;  // scan coefficients W1 Kon, Wava Kon, W2 Kon
    float qw;        // sigma w0 tau_c = K4 w0 / (u^2 + w0^2) (defocusing weight)
    float sigma;     // K4 tau_c / (1 + w0^2 tau_c^2)
    float u;         // 1 / tau_c = sigma_coll rho_nt v_e
};
// SECOND = false: the second stage is known to flush to zero for every sample of the tile (the
// first walk's test), so its rate is not evaluated and c2 = 0, the value it would flush to.
template <bool SECOND = true>
__device__ __forceinline__ IonPoint ion_point(float2 a, const NLConst& c) {
    IonPoint r;
    float I = fmaf(a.x, a.x, a.y * a.y) * c.I_scale;
    if (I == 0.0f) I = 1e-30f;                   // plasma.c:136-138
    const float rs = rsqrtf(I);
    const float F = I * rs * c.E_c;              // |E| in atomic units
    const float invF = rs * c.inv_E_c;
    const float l2F = __log2f(F);
    float w[2] = {0.0f, 0.0f};
#pragma unroll
    for (int st = 0; st < (SECOND ? 2 : 1); st++) {
        const float e2 = c.l2K1[st] + c.K5[st] * (c.l2K3[st] - l2F) - c.K3l2e[st] * invF;
        w[st] = (e2 > -126.0f) ? exp2f(e2) : 0.0f;
    }
    const float u = c.Kuv * F;
    const float qw = __fdividef(c.K4w0, fmaf(u, u, c.w0sq));
    r.sigma = qw * u * c.inv_w0;
    r.qw = qw;
    r.u = u;
    r.a = w[0] * c.Kon;
    r.b = r.sigma * I * c.invI1_Kon;
    if constexpr (SECOND) {
        const float c2 = w[1] * c.Kon;
        r.c2 = (c2 >= kC2Flush) ? c2 : 0.0f;
    } else {
        r.c2 = 0.0f;
    }
    return r;
}

// The first walk of the ionization scan needs only a and b of each sample, and whether any
// sample of the tile may have a second-stage probability c2 at or above the flush threshold.
// That is decided on the exponent, e2 > log2(threshold / Kon) - 1, without the second exp2: a
// conservative test (a tile flagged whose c2 all flush runs the exact (ions2, ions1) scan with
// zero coefficients).
struct IonAB {
    float a, b;
    bool second;
};
__device__ __forceinline__ float ion_second_threshold(const NLConst& c) { return __log2f(kC2Flush / c.Kon) - 1.0f; }
__device__ __forceinline__ IonAB ion_point_ab(float2 a, const NLConst& c, float e2thr) {
    IonAB r;
    float I = fmaf(a.x, a.x, a.y * a.y) * c.I_scale;
    if (I == 0.0f) I = 1e-30f;                   // plasma.c:136-138
    const float rs = rsqrtf(I);
    const float F = I * rs * c.E_c;
    const float invF = rs * c.inv_E_c;
    const float l2F = __log2f(F);
    const float e1 = c.l2K1[0] + c.K5[0] * (c.l2K3[0] - l2F) - c.K3l2e[0] * invF;
    const float e2 = c.l2K1[1] + c.K5[1] * (c.l2K3[1] - l2F) - c.K3l2e[1] * invF;
    const float u = c.Kuv * F;
    const float qw = __fdividef(c.K4w0, fmaf(u, u, c.w0sq));
    r.a = ((e1 > -126.0f) ? exp2f(e1) : 0.0f) * c.Kon;
    r.b = qw * u * c.inv_w0 * I * c.invI1_Kon;
    r.second = e2 > e2thr;
    return r;
}

// Nonlinear step on a tile holding A(t) of P pencils in shared memory (natural t order).
// IONIZ_ONLY = false: A *= exp(dz * A_nl) in place (propagation.c:244-327 with the A13/A14
// fixes).  IONIZ_ONLY = true: write tau_c and freeelectrons_sp (plasma.c:118-245 outputs)
// in the reference layout instead, A untouched.  Thread (p = tid % P, ch = tid / P) walks
// the CH samples t = CH ch .. CH ch + CH - 1 of pencil p.  The step's running maxima go to `mx`:
// {|a|^2 (device units), ionization fraction, |Im A_nl| (phase rate, rad/m), |Re A_nl| (1/m)}.
template <int NT, int P, bool IONIZ_ONLY, int CH = 32>
__device__ __forceinline__ void nonlinear_tile(float2* s, const float2* __restrict__ scr, const NLConst& c,
                                               void* scan_mem, int tid, double* tau_out, double* fe_out,
                                               int q0, int NP, float4& mx) {
    using V = PencilView<NT, P>;
    static_assert(CH == 32 || (CH == 16 && V::SH == 4), "walk offsets need a chunk-aligned pad");
    constexpr int TPP = NT / CH;
    const int p = tid % P;
    const int ch = tid / P;
    const int t0 = ch * CH;
    float2* w = s + V::at(t0, p);   // this thread's CH samples: w[V::walk(i)]
    const float2* dA = scr + t0 * P + p;   // dA of the same samples: dA[i * P]
    if (c.plasma) {
        MapR* mr = reinterpret_cast<MapR*>(scan_mem);
        MapUV* muv = reinterpret_cast<MapUV*>(scan_mem);
        // S1: chunk map of the R recurrence (FP32 within the chunk)
        int any2 = 0;
        {
            float B = 0.0f, C = 0.0f;
            const float e2thr = ion_second_threshold(c);
#pragma unroll kS1Unroll
            for (int i = 0; i < CH; i++) {
                const IonAB ip = ion_point_ab(w[V::walk(i)], c, e2thr);
                const float Ck = fmaf(1.0f - ip.b, ip.a, ip.b);
                C = fmaf(1.0f - ip.b, C, Ck);
                B = fmaf(-B, ip.b, B + ip.b);
                any2 |= ip.second;
            }
            mr[p * TPP + ch] = MapR{1.0 - (double)B, (double)C};
        }
        any2 = __syncthreads_or(any2);
        scan_chunks<MapR, P, TPP>(mr, tid);   // carries across chunks in FP64
        __syncthreads();
        const float Rin = (float)mr[p * TPP + ch].C;
        float u = 0.0f, v = (Rin > 0.0f) ? one_minus_exp_neg(Rin) : 0.0f;
        if (any2) {
            __syncthreads();
            // S2: chunk map of the (ions2, ions1) recurrence
            float R = Rin;
            float m00 = 1.f, m01 = 0.f, m10 = 0.f, m11 = 1.f, o0 = 0.f, o1 = 0.f;
#pragma unroll 4
            for (int i = 0; i < CH; i++) {
                const IonPoint ip = ion_point<true>(s[V::at(t0 + i, p)], c);
                R = fmaf(1.0f - ip.b, R + ip.a, ip.b);
                const float g = one_minus_exp_neg(R);
                const float n00 = fmaf(ip.c2, m10, m00), n01 = fmaf(ip.c2, m11, m01);
                const float no0 = fmaf(ip.c2, o1, o0), no1 = g - o0;
                m10 = -m00;
                m11 = -m01;
                m00 = n00;
                m01 = n01;
                o1 = no1;
                o0 = no0;
            }
            muv[p * TPP + ch] = MapUV{m00, m01, m10, m11, o0, o1};
            __syncthreads();
            scan_chunks<MapUV, P, TPP>(muv, tid);
            __syncthreads();
            u = (float)muv[p * TPP + ch].o0;
            v = (float)muv[p * TPP + ch].o1;
        }
        // S3: apply the nonlinear step (or emit the ionization outputs).  The dA samples come
        // from L2: a ring of kDAPrefetch registers loads each kDAPrefetch samples ahead.  Tiles
        // without second-stage ionization (any2 == 0) take the walk without the second rate.
        auto walk = [&](auto second) {
            constexpr bool SECOND = decltype(second)::value;
            float R = Rin;
            float2 ring[kDAPrefetch];
            if (!IONIZ_ONLY && c.sst_c != 0.0f) {
#pragma unroll
                for (int k = 0; k < kDAPrefetch; k++) ring[k] = dA[k * P];
            }
#pragma unroll kDAPrefetch
            for (int i = 0; i < CH; i++) {
                const int t = t0 + i;
                float2 dAi = make_float2(0.0f, 0.0f);
                if (!IONIZ_ONLY && c.sst_c != 0.0f) {
                    dAi = ring[i % kDAPrefetch];
                    if (i + kDAPrefetch < CH) ring[i % kDAPrefetch] = dA[(i + kDAPrefetch) * P];
                }
                const float2 a = w[V::walk(i)];
                const IonPoint ip = ion_point<SECOND>(a, c);
                R = fmaf(1.0f - ip.b, R + ip.a, ip.b);
                const float g = one_minus_exp_neg(R);
                const float ions = fmaf(2.0f, u, v);     // state before slice t (plasma.c:238-241)
                const float nu = fmaf(ip.c2, v, u);
                v = g - u;
                u = nu;
                if constexpr (IONIZ_ONLY) {
                    const size_t gi = (size_t)t * NP + q0 + p;
                    tau_out[gi] = 1.0 / (double)ip.u;
                    fe_out[gi] = (double)ions * (double)ip.sigma;
                    continue;
                }
                const float pl = c.rho_half * ions;
                const float a2 = fmaf(a.x, a.x, a.y * a.y);
                float re = -pl * ip.sigma;
                float im = fmaf(c.gam, a2, -pl * ip.qw);
                if (c.sst_c != 0.0f) {
                    const float2 sd = cmulc(dAi, a);  // dA * conj(A)
                    re = fmaf(-3.0f * c.sst_c, sd.x, re);
                    im = fmaf(-c.sst_c, sd.y, im);
                }
                const float amp = exp_small(c.dz * re);
                float sn, cs;
                sincos_small(c.dz * im, &sn, &cs);
                w[V::walk(i)] = cmul(a, make_float2(amp * cs, amp * sn));
                mx = make_float4(fmaxf(mx.x, a2), fmaxf(mx.y, ions), fmaxf(mx.z, fabsf(im)), fmaxf(mx.w, fabsf(re)));
            }
        };
        if (any2) walk(std::true_type{});
        else walk(std::false_type{});
    } else {
        float2 ring[kDAPrefetch];
        if (c.sst_c != 0.0f) {
#pragma unroll
            for (int k = 0; k < kDAPrefetch; k++) ring[k] = dA[k * P];
        }
#pragma unroll kDAPrefetch
        for (int i = 0; i < CH; i++) {
            const float2 a = w[V::walk(i)];
            const float a2 = fmaf(a.x, a.x, a.y * a.y);
            float re = 0.0f;
            float im = c.gam * a2;
            if (c.sst_c != 0.0f) {
                const float2 dAi = ring[i % kDAPrefetch];
                if (i + kDAPrefetch < CH) ring[i % kDAPrefetch] = dA[(i + kDAPrefetch) * P];
                const float2 sd = cmulc(dAi, a);
                re = -3.0f * c.sst_c * sd.x;
                im = fmaf(-c.sst_c, sd.y, im);
            }
            const float amp = exp_small(c.dz * re);
            float sn, cs;
            sincos_small(c.dz * im, &sn, &cs);
            w[V::walk(i)] = cmul(a, make_float2(amp * cs, amp * sn));
            mx = make_float4(fmaxf(mx.x, a2), mx.y, fmaxf(mx.z, fabsf(im)), fmaxf(mx.w, fabsf(re)));
        }
    }
}

// Block-wide maximum of each component of v into stats[0..3] (non-negative floats, whose
// bit patterns order like the values); one atomic per component and CTA.
template <int TH>
__device__ __forceinline__ void stats_max(float4 v, unsigned int* stats, float* red, int tid) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        v.x = fmaxf(v.x, __shfl_xor_sync(0xffffffffu, v.x, o));
        v.y = fmaxf(v.y, __shfl_xor_sync(0xffffffffu, v.y, o));
        v.z = fmaxf(v.z, __shfl_xor_sync(0xffffffffu, v.z, o));
        v.w = fmaxf(v.w, __shfl_xor_sync(0xffffffffu, v.w, o));
    }
    if ((tid & 31) == 0) reinterpret_cast<float4*>(red)[tid >> 5] = v;
    __syncthreads();
    if (tid < 4) {
        float m = 0.0f;
        for (int w = 0; w < TH / 32; w++) m = fmaxf(m, red[4 * w + tid]);
        atomicMax(&stats[tid], __float_as_uint(m));
    }
}

// ---------------------------------------------------------------------------------------
// Pencil pass
// ---------------------------------------------------------------------------------------
// Shared memory of a pencil CTA: [field tile][scan maps][W_Nt twiddles][FP64 t sums (TEMP)].
// One thread per CH-sample chunk of the nonlinear walk: TH = P * Nt / CH threads (CH = 16 puts
// 1024 threads, 64 registers each, in a CTA: twice the warps to hide latency).
template <int NT, int P, int SLO, int CH = 32>
struct PencilCfg {
    using View = PencilView<NT, P>;
    static constexpr int TPP = NT / CH;                 // chunks per pencil
    static constexpr int TH = P * TPP;                  // threads per CTA
    static constexpr int SMEM_FIELD = View::SIZE * 8;  // bytes
    static constexpr int SMEM_SCAN = P * TPP * (int)sizeof(MapUV);
    static constexpr int SMEM_TW = twiddle_bytes(NT);
    static constexpr int SMEM_TEMP = NT * 8;            // FP64 temporal sums (TEMP mode only)
    static constexpr int SMEM = SMEM_FIELD + SMEM_SCAN + SMEM_TW;
    // the TEMP mode keeps its sums in the scan area (unused there) when they fit
    static constexpr bool TEMP_IN_SCAN = SMEM_SCAN >= SMEM_TEMP;
    static constexpr int SMEM_TEMP_MODE = TEMP_IN_SCAN ? SMEM : SMEM + SMEM_TEMP;
    static constexpr int smem(int mode) { return mode == 5 ? SMEM_TEMP_MODE : SMEM; }
    static_assert(TH % 32 == 0 && TH <= 1024, "pencil CTA size");
    static_assert((P * SLO) % 2 == 0, "rows must be whole float4s");
};

// Element order of the two complex values of a float4 row chunk.  For SLO = 2 the pair is
// (pos 2r, pos 2r + 1) of one pencil; odd rows store them in the opposite order so that
// the four rows a warp touches fall on both halves of the shared-memory banks.
// load a slot-layout tile into shared memory
template <int NT, int P, int SLO, int TH>
__device__ __forceinline__ void load_tile(float2* s, const float2* __restrict__ g, int q0, int NP, int tid) {
    using V = PencilView<NT, P>;
    constexpr int F4_PER_ROW = P * SLO / 2;
    constexpr int ROWS = NT / SLO;
    const float4* g4 = reinterpret_cast<const float4*>(g);
    for (int f = tid; f < ROWS * F4_PER_ROW; f += TH) {
        const int row = f / F4_PER_ROW, c = f - row * F4_PER_ROW;
        const size_t gi = (((size_t)row * NP + q0) * SLO) / 2 + c;
        const float4 v = __ldg(&g4[gi]);
        int pos0, p0, pos1, p1;
        if constexpr (SLO == 2) { pos0 = 2 * row; pos1 = pos0 + 1; p0 = p1 = c; }
        else { pos0 = pos1 = row; p0 = 2 * c; p1 = p0 + 1; }
        const float2 e0 = make_float2(v.x, v.y), e1 = make_float2(v.z, v.w);
        if (SLO == 2 && (row & 1)) {
            s[V::at(pos1, p1)] = e1;
            s[V::at(pos0, p0)] = e0;
        } else {
            s[V::at(pos0, p0)] = e0;
            s[V::at(pos1, p1)] = e1;
        }
    }
}

// Slot-layout index of spectrum position pos of pencil q (a multiple-of-P tile start plus line)
template <int SLO>
__device__ __forceinline__ size_t slot_index(int pos, int q, int NP) {
    return ((size_t)(pos / SLO) * NP + q) * SLO + (pos % SLO);
}

// Asynchronous tile load for the SLO = 1 layout: every 16 B chunk of a t-row (pencils 2c and
// 2c + 1 at one position) is copied from global to shared memory by cp.async, all of them in
// flight at once.  Both addresses are 16 B aligned: NP and q0 are even, and P and the view's
// pad are even.  Ends with the wait and a CTA barrier.
template <int NT, int P, int TH>
__device__ __forceinline__ void load_tile_async(float2* s, const float2* __restrict__ g, int q0, int NP, int tid) {
    using V = PencilView<NT, P>;
    static_assert(P % 2 == 0, "16 B chunks of two pencils");
    constexpr int F4_PER_ROW = P / 2;
    const float4* g4 = reinterpret_cast<const float4*>(g);
    for (int f = tid; f < NT * F4_PER_ROW; f += TH) {
        const int row = f / F4_PER_ROW, c = f - row * F4_PER_ROW;
        const float4* src = g4 + (((size_t)row * NP + q0) / 2 + c);
        const unsigned dst = (unsigned)__cvta_generic_to_shared(s + V::at(row, 2 * c));
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
}

// The tile's spectrum into shared memory (pencil view), then a CTA barrier.
template <int NT, int P, int SLO, int TH>
__device__ __forceinline__ void stage_tile(float2* s, const float2* __restrict__ g, int q0, int NP, int tid) {
    if constexpr (SLO == 1) {
        load_tile_async<NT, P, TH>(s, g, q0, NP, tid);
    } else {
        load_tile<NT, P, SLO, TH>(s, g, q0, NP, tid);
        __syncthreads();
    }
}

// First stage of the derivative's inverse t transform over a staged tile: S(pos) from shared
// memory times -i omega(pos).
template <class V>
struct SmemDerivSource {
    const float2* s;
    const float* __restrict__ wpos;
    static constexpr bool active = true;
    template <int R>
    __device__ __forceinline__ void operator()(float2 (&v)[R], int pos0, int line) const {
        const float2* p0 = s + V::at(pos0, line);
#pragma unroll
        for (int q = 0; q < R; q++) v[q] = cscale(mul_mi<false>(p0[V::at(q, 0) - V::at(0, 0)]), __ldg(&wpos[pos0 + q]));
    }
};

// First stage of an inverse t transform reading the tile's spectrum straight from global memory
// (through L2: the tile is read twice per step and written once, by this CTA only); DERIV
// multiplies by -i omega(pos), the spectrum of the time derivative.  A warp's loads for one q
// are P-pencil row segments of 8 positions.
template <int P, int SLO, bool DERIV>
struct TileSource {
    const float2* __restrict__ g;
    const float* __restrict__ wpos;
    int q0, NP;
    static constexpr bool active = true;
    template <int R>
    __device__ __forceinline__ void operator()(float2 (&v)[R], int pos0, int line) const {
#pragma unroll
        for (int q = 0; q < R; q++) v[q] = __ldcg(&g[slot_index<SLO>(pos0 + q, q0 + line, NP)]);
        if constexpr (DERIV) {
#pragma unroll
            for (int q = 0; q < R; q++) v[q] = cscale(mul_mi<false>(v[q]), __ldg(&wpos[pos0 + q]));
        }
    }
};

// Last stage of the forward t transform writing the tile's spectrum to global memory.
template <int P, int SLO>
struct TileSink {
    float2* __restrict__ g;
    int q0, NP;
    static constexpr bool active = true;
    template <int R>
    __device__ __forceinline__ void operator()(const float2 (&v)[R], int pos0, int S, int line) const {
#pragma unroll
        for (int q = 0; q < R; q++) g[slot_index<SLO>(pos0 + S * q, q0 + line, NP)] = v[q];
    }
};

// Fused into the last stage of the derivative's inverse transform: dA(t) of pencil `line` goes
// to the CTA's scratch tile [t][p] (L2) instead of shared memory; a warp's stores for one q
// cover consecutive t of all P pencils.
template <int P>
struct ScratchSink {
    float2* __restrict__ scr;
    static constexpr bool active = true;
    template <int R>
    __device__ __forceinline__ void operator()(const float2 (&v)[R], int t0, int S, int line) const {
#pragma unroll
        for (int q = 0; q < R; q++) scr[(t0 + S * q) * P + line] = v[q];
    }
};

template <int NT, int P, int SLO, int TH>
__device__ __forceinline__ void store_tile(const float2* s, float2* __restrict__ g, int q0, int NP, int tid) {
    using V = PencilView<NT, P>;
    constexpr int F4_PER_ROW = P * SLO / 2;
    constexpr int ROWS = NT / SLO;
    float4* g4 = reinterpret_cast<float4*>(g);
    for (int f = tid; f < ROWS * F4_PER_ROW; f += TH) {
        const int row = f / F4_PER_ROW, c = f - row * F4_PER_ROW;
        const size_t gi = (((size_t)row * NP + q0) * SLO) / 2 + c;
        int pos0, p0, pos1, p1;
        if constexpr (SLO == 2) { pos0 = 2 * row; pos1 = pos0 + 1; p0 = p1 = c; }
        else { pos0 = pos1 = row; p0 = 2 * c; p1 = p0 + 1; }
        float2 e0, e1;
        if (SLO == 2 && (row & 1)) {
            e1 = s[V::at(pos1, p1)];
            e0 = s[V::at(pos0, p0)];
        } else {
            e0 = s[V::at(pos0, p0)];
            e1 = s[V::at(pos1, p1)];
        }
        g4[gi] = make_float4(e0.x, e0.y, e1.x, e1.y);
    }
}

// LD: how the split step reads the tile (0: staged in shared memory by cp.async, best with
// 32 B t-rows; 1: loaded by the first transform stages, best with 64 B and wider rows).
template <int NT, int P, int SLO, int MODE, int CH = 32, int LD = 1>
__global__ void __launch_bounds__(PencilCfg<NT, P, SLO, CH>::TH, (PencilCfg<NT, P, SLO, CH>::TH >= kThreads ? 1 : 2))
    pencil_kernel(PencilArgs args) {
    using Cfg = PencilCfg<NT, P, SLO, CH>;
    using V = typename Cfg::View;
    constexpr int TH = Cfg::TH;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* s = reinterpret_cast<float2*>(smem_raw);
    void* scan_mem = smem_raw + Cfg::SMEM_FIELD;
    unsigned char* tw_mem = smem_raw + Cfg::SMEM_FIELD + Cfg::SMEM_SCAN;
    double* tsum = reinterpret_cast<double*>(Cfg::TEMP_IN_SCAN ? smem_raw + Cfg::SMEM_FIELD : smem_raw + Cfg::SMEM);
    const int tid = threadIdx.x;
    const int NP = args.NP;
    stage_twiddles<NT, TH>(tw_mem, args.tw, tid);
    const Twiddles tw = Twiddles::packed(tw_mem, NT);
    __syncthreads();

    if constexpr (MODE == PM_TEMP) {
        for (int t = tid; t < NT; t += TH) tsum[t] = 0.0;
        __syncthreads();
    }
    float4 mx = make_float4(0.f, 0.f, 0.f, 0.f);   // STEP: this thread's maxima over its tiles

    for (int tile = blockIdx.x; tile < args.ntiles; tile += gridDim.x) {
        const int q0 = tile * P;
        if constexpr (MODE == PM_IONIZ) {
            for (int f = tid; f < NT * P; f += TH) {
                const int t = f / P, p = f - (f / P) * P;
                const size_t gi = (size_t)t * NP + q0 + p;
                const double2 v = __ldg(&reinterpret_cast<const double2*>(args.in)[gi]);
                s[V::at(t, p)] = make_float2((float)(v.x * args.in_scale), (float)(v.y * args.in_scale));
            }
            __syncthreads();
            float4 unused = make_float4(0.f, 0.f, 0.f, 0.f);
            nonlinear_tile<NT, P, true, CH>(s, nullptr, args.nl, scan_mem, tid, args.tau_out, args.fe_out, q0, NP, unused);
            __syncthreads();
        } else if constexpr (MODE == PM_ENTRY_C128 || MODE == PM_ENTRY_C64) {
            // real-space input, reference layout A[t*NP + q]
            for (int f = tid; f < NT * P; f += TH) {
                const int t = f / P, p = f - (f / P) * P;
                const size_t gi = (size_t)t * NP + q0 + p;
                float2 e;
                if constexpr (MODE == PM_ENTRY_C128) {
                    const double2 v = __ldg(&reinterpret_cast<const double2*>(args.in)[gi]);
                    e = make_float2((float)(v.x * args.in_scale), (float)(v.y * args.in_scale));
                } else {
                    e = cscale(__ldg(&reinterpret_cast<const float2*>(args.in)[gi]), (float)args.in_scale);
                }
                s[V::at(t, p)] = e;
            }
            __syncthreads();
            dif_all<NT, NT, V, TH, kPencilUnroll>(s, tw, tid);
            store_tile<NT, P, SLO, TH>(s, reinterpret_cast<float2*>(args.out), q0, NP, tid);
            __syncthreads();
        } else if constexpr (MODE == PM_EXIT_C128 || MODE == PM_EXIT_C64 || MODE == PM_TEMP) {
            load_tile<NT, P, SLO, TH>(s, reinterpret_cast<const float2*>(args.in), q0, NP, tid);
            __syncthreads();
            dit_all<NT, NT, V, TH, kPencilUnroll>(s, tw, tid);
            if constexpr (MODE == PM_TEMP) {
                const double inv = args.out_scale * args.out_scale;
                for (int t = tid; t < NT; t += TH) {
                    float acc = 0.0f;
#pragma unroll 8
                    for (int p = 0; p < P; p++) {
                        const float2 e = s[V::at(t, p)];
                        acc = fmaf(e.x, e.x, fmaf(e.y, e.y, acc));
                    }
                    tsum[t] += (double)acc * inv;
                }
            } else {
                for (int f = tid; f < NT * P; f += TH) {
                    const int t = f / P, p = f - (f / P) * P;
                    const size_t gi = (size_t)t * NP + q0 + p;
                    const float2 e = s[V::at(t, p)];
                    if constexpr (MODE == PM_EXIT_C128) {
                        const double sc = args.out_scale;
                        reinterpret_cast<double2*>(args.out)[gi] = make_double2((double)e.x * sc, (double)e.y * sc);
                    } else {
                        reinterpret_cast<float2*>(args.out)[gi] = cscale(e, (float)args.out_scale);
                    }
                }
                // per-pencil energy sum_t |A|^2 (physical units)
                if (args.pencil_energy) {
                    const int p = tid % P, part = tid / P;           // TH/P partial sums per pencil
                    constexpr int PARTS = TH / P;
                    float acc = 0.0f;
                    for (int t = part; t < NT; t += PARTS) {
                        const float2 e = s[V::at(t, p)];
                        acc = fmaf(e.x, e.x, fmaf(e.y, e.y, acc));
                    }
                    double* red = reinterpret_cast<double*>(scan_mem);
                    __syncthreads();
                    red[part * P + p] = (double)acc;
                    __syncthreads();
                    if (tid < P) {
                        double tot = 0.0;
                        for (int k = 0; k < PARTS; k++) tot += red[k * P + tid];
                        args.pencil_energy[q0 + tid] = tot * args.out_scale * args.out_scale;
                    }
                }
            }
            __syncthreads();
        } else {  // PM_STEP
            const NLConst& c = args.nl;
            const float2* gin = reinterpret_cast<const float2*>(args.in);
            float2* scr = args.scratch + (size_t)blockIdx.x * NT * P;
            // dA = IFFT_t(-i omega S): the time derivative of the self-steepening term, kept in
            // this CTA's scratch tile [t][p] (L2-resident) until the nonlinear walk
            // (LD = 1: the transforms' first stages load the spectrum from global memory; LD = 0:
            // it is staged in shared memory by bulk asynchronous copies first)
            if (c.sst_c != 0.0f) {
                if constexpr (LD == 1) {
                    dit_all<NT, NT, V, TH, kPencilUnroll, false>(
                        s, tw, tid, TileSource<P, SLO, true>{gin, args.wpos, q0, NP}, ScratchSink<P>{scr});
                } else {
                    stage_tile<NT, P, SLO, TH>(s, gin, q0, NP, tid);
                    dit_all<NT, NT, V, TH, kPencilUnroll, false>(s, tw, tid, SmemDerivSource<V>{s, args.wpos},
                                                                  ScratchSink<P>{scr});
                }
            }
            // A = IFFT_t(S)
            if constexpr (LD == 1) {
                dit_all<NT, NT, V, TH, kPencilUnroll>(s, tw, tid, TileSource<P, SLO, false>{gin, args.wpos, q0, NP});
            } else {
                stage_tile<NT, P, SLO, TH>(s, gin, q0, NP, tid);
                dit_all<NT, NT, V, TH, kPencilUnroll>(s, tw, tid);
            }

            nonlinear_tile<NT, P, false, CH>(s, scr, c, scan_mem, tid, nullptr, nullptr, q0, NP, mx);
            __syncthreads();
            dif_all<NT, NT, V, TH, kPencilUnroll>(s, tw, tid, TileSink<P, SLO>{reinterpret_cast<float2*>(args.out), q0, NP});
        }
    }
    if constexpr (MODE == PM_TEMP) {
        __syncthreads();
        for (int t = tid; t < NT; t += TH) atomicAdd(&args.temp[t], tsum[t]);
    }
    if constexpr (MODE == PM_STEP) {
        if (args.stats) stats_max<TH>(mx, args.stats, reinterpret_cast<float*>(scan_mem), tid);
    }
}

// ---------------------------------------------------------------------------------------
// Plane pass
// ---------------------------------------------------------------------------------------
// Linear-step factors as double-float complex numbers (x, y = high parts, z, w = low parts,
// split from FP64).  Rounded once to complex64 the same factor would be applied every step
// with the same rounding error, which adds up coherently over thousands of steps; the
// low parts remove that systematic error.
struct PlaneTables {
    const float4* Rx;   // Nx, x position order: exp(-i zd kx^2 / (2 k0))
    const float4* RyD;  // Ny * Nt, [y position][slot position]: Ry(ky) D(omega) scale
    const float4* RyDT; // the same factors slot-major, Nt * Ny: [slot position][y position]
};

struct PlaneArgs {
    const float2* in;
    float2* out;
    const float2* twx;       // W_Nx table, packed (mpc_fft.cuh Twiddles)
    const float2* twy;       // W_Ny table, packed
    PlaneTables t1;      // first (or only) linear operator
    PlaneTables t2;      // second half after the mirror lens (lens != 0)
    const float2* lensx; // exp(-i k0 x^2 / roc), real x order
    const float2* lensy;
    int lens;            // 1: L(t1) -> lens -> L(t2)
    int Nt;
    int NP;
    int nunits;          // number of cluster work units
    unsigned int* err;   // error word of the TMA-staged kernels (KernelError), device memory
};

template <int NX, int NY, int CL, int PB, int SLO>
struct PlaneCfg {
    static constexpr int RY = NY / CL;   // rows per CTA (row view)
    static constexpr int CX = NX / CL;   // columns per CTA (column view)
    static constexpr int RS = CX + 1;    // padded row stride
    static constexpr int RSZ = PB * RY * RS;  // region (one partner block), complex64
    static constexpr int SIZE = CL * RSZ;
    static constexpr int SMEM = SIZE * 8 + twiddle_bytes(NX) + twiddle_bytes(NY);
    static_assert(SLO == 1 || PB == SLO, "interleaved slots are processed together");
    static_assert((RSZ % 2) == 0, "regions are moved as float4");
};

template <int NX, int NY, int CL, int PB, int SLO>
struct RowView {
    using C = PlaneCfg<NX, NY, CL, PB, SLO>;
    static constexpr int NLINES = PB * C::RY;
    static constexpr __host__ __device__ __forceinline__ int at(int x, int l) {
        return (x / C::CX) * C::RSZ + l * C::RS + (x % C::CX);
    }
};
template <int NX, int NY, int CL, int PB, int SLO>
struct ColView {
    using C = PlaneCfg<NX, NY, CL, PB, SLO>;
    static constexpr int NLINES = PB * C::CX;
    static constexpr __host__ __device__ __forceinline__ int at(int y, int l) {
        const int pl = l / C::CX, xl = l - pl * C::CX;
        return (y / C::RY) * C::RSZ + (pl * C::RY + (y % C::RY)) * C::RS + xl;
    }
};

// Swap region g of this CTA with region `rank` of CTA g, for every g != rank.
template <int CL, int RSZ, int NTHR>
__device__ __forceinline__ void cluster_exchange(float2* s, cg::cluster_group& cluster, int rank, int tid) {
    if constexpr (CL > 1) {
        constexpr int F4 = RSZ / 2;               // float4 per region
        constexpr int KR = (CL >= 4) ? 2 : 1;     // partners per round
        constexpr int PER = (KR * F4 + NTHR - 1) / NTHR;
        cluster.sync();
        for (int k0 = 1; k0 < CL; k0 += KR) {
            float4 buf[PER];
#pragma unroll
            for (int i = 0; i < PER; i++) {
                const int f = tid + i * NTHR;
                if (f < KR * F4) {
                    const int kk = k0 + f / F4;
                    if (kk < CL) {
                        const int g = rank ^ kk;
                        const float4* rem = reinterpret_cast<const float4*>(cluster.map_shared_rank(s, g));
                        buf[i] = rem[rank * F4 + (f % F4)];
                    }
                }
            }
            cluster.sync();
#pragma unroll
            for (int i = 0; i < PER; i++) {
                const int f = tid + i * NTHR;
                if (f < KR * F4) {
                    const int kk = k0 + f / F4;
                    if (kk < CL) {
                        const int g = rank ^ kk;
                        reinterpret_cast<float4*>(s)[g * F4 + (f % F4)] = buf[i];
                    }
                }
            }
        }
        __syncthreads();
    }
}

// Ry(py) D(slot) (double-float) at column-view positions y (FFT position order) of line
// l = pl * CX + xl, plane pl of the unit.
template <int CX, int SLO, int PB>
struct YFactors {
    const float4* __restrict__ RyD;
    int Nt, unit;
    template <int R>
    __device__ __forceinline__ void operator()(float2 (&v)[R], int y0, int line) const {
        const int pl = line / CX;
        const int slot = (SLO == 1) ? unit * PB + pl : unit * SLO + pl;
        const float4* f = RyD + (size_t)y0 * Nt + slot;
#pragma unroll
        for (int q = 0; q < R; q++) v[q] = cmul_df(v[q], __ldg(&f[(size_t)q * Nt]));
    }
};
// Rx(px) (double-float) at row-view positions x, from shared or global memory
struct XFactorsAny {
    const float4* Rx;
    template <int R>
    __device__ __forceinline__ void operator()(float2 (&v)[R], int x0, int) const {
#pragma unroll
        for (int q = 0; q < R; q++) v[q] = cmul_df(v[q], Rx[x0 + q]);
    }
};
// Rx(px) (double-float) at row-view positions x (FFT position order).
struct XFactors {
    const float4* __restrict__ Rx;
    template <int R>
    __device__ __forceinline__ void operator()(float2 (&v)[R], int x0, int) const {
#pragma unroll
        for (int q = 0; q < R; q++) v[q] = cmul_df(v[q], __ldg(&Rx[x0 + q]));
    }
};

// Move this CTA's share of a unit between global and shared memory: ROWS, the rows
// y in [rank RY, rank RY + RY) (row view, NX * 8 B contiguous per row and plane); otherwise
// the columns x in [rank CX, rank CX + CX) of every row (column view, CX * 8 B per row and
// plane).  STORE: shared -> global.  SLO == 2: one float4 holds both slots of one x.
template <int NX, int NY, int CL, int PB, int SLO, int NTHR, bool ROWS, bool STORE>
__device__ __forceinline__ void plane_move(float2* s, const float2* __restrict__ gin, float2* __restrict__ gout,
                                           int rank, int unit, int NP, int tid) {
    using C = PlaneCfg<NX, NY, CL, PB, SLO>;
    using RV = RowView<NX, NY, CL, PB, SLO>;
    using CV = ColView<NX, NY, CL, PB, SLO>;
    constexpr int W = ROWS ? NX : C::CX;    // x extent moved per row
    constexpr int NR = ROWS ? C::RY : NY;   // rows moved per plane block
    static_assert((W * SLO) % 2 == 0, "rows move as float4");
    constexpr int F4_ROW = W * SLO / 2;
    const int x0 = ROWS ? 0 : rank * C::CX;
    const int y0 = ROWS ? rank * C::RY : 0;
#pragma unroll 8
    for (int f = tid; f < PB / SLO * NR * F4_ROW; f += NTHR) {
        const int c = f % F4_ROW;
        const int r = f / F4_ROW;
        const int yr = r % NR, plb = r / NR;  // plb: plane block (SLO == 1: plane)
        const int y = y0 + yr;
        size_t gi;
        int i0, i1;
        if constexpr (SLO == 1) {
            gi = ((size_t)(unit * PB + plb) * NP + (size_t)y * NX + x0) / 2 + c;
            if constexpr (ROWS) {
                i0 = RV::at(2 * c, plb * C::RY + yr);
                i1 = RV::at(2 * c + 1, plb * C::RY + yr);
            } else {
                i0 = CV::at(y, plb * C::CX + 2 * c);
                i1 = CV::at(y, plb * C::CX + 2 * c + 1);
            }
        } else {
            gi = (size_t)unit * NP + (size_t)y * NX + x0 + c;
            if constexpr (ROWS) {
                i0 = RV::at(c, yr);
                i1 = RV::at(c, C::RY + yr);
            } else {
                i0 = CV::at(y, c);
                i1 = CV::at(y, C::CX + c);
            }
        }
        if constexpr (STORE) {
            const float2 e0 = s[i0], e1 = s[i1];
            reinterpret_cast<float4*>(gout)[gi] = make_float4(e0.x, e0.y, e1.x, e1.y);
        } else {
            const float4 v = __ldg(reinterpret_cast<const float4*>(gin) + gi);
            s[i0] = make_float2(v.x, v.y);
            s[i1] = make_float2(v.z, v.w);
        }
    }
}

// NTHR threads per CTA; 512 / NTHR CTAs per SM (the register file holds 512 threads at
// 128 registers).  The linear step factorises, IFFT_xy Rx Ry D FFT_xy =
// (IFFT_x Rx FFT_x)(IFFT_y Ry D FFT_y), so a unit is loaded by columns, takes its y part in
// the column view, moves to the row view in one cluster exchange, takes its x part and is
// stored by rows.  With the mirror lens: y(t1), exchange, x(t1), lens, x(t2), exchange,
// y(t2), stored by columns.
template <int NX, int NY, int CL, int PB, int SLO, int NTHR>
__global__ void __launch_bounds__(NTHR, (NTHR >= 512 ? 1 : 512 / NTHR)) plane_kernel(PlaneArgs a) {
    using C = PlaneCfg<NX, NY, CL, PB, SLO>;
    using RV = RowView<NX, NY, CL, PB, SLO>;
    using CV = ColView<NX, NY, CL, PB, SLO>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* s = reinterpret_cast<float2*>(smem_raw);
    unsigned char* twx_mem = smem_raw + C::SIZE * 8;
    unsigned char* twy_mem = twx_mem + twiddle_bytes(NX);
    cg::cluster_group cluster = cg::this_cluster();
    const int rank = (int)cluster.block_rank();
    const int tid = threadIdx.x;
    const int cid = blockIdx.x / CL, ncl = gridDim.x / CL;
    const int NP = a.NP;
    stage_twiddles<NX, NTHR>(twx_mem, a.twx, tid);
    stage_twiddles<NY, NTHR>(twy_mem, a.twy, tid);
    const Twiddles twx = Twiddles::packed(twx_mem, NX), twy = Twiddles::packed(twy_mem, NY);
    __syncthreads();

    for (int unit = cid; unit < a.nunits; unit += ncl) {
        plane_move<NX, NY, CL, PB, SLO, NTHR, false, false>(s, a.in, nullptr, rank, unit, NP, tid);
        __syncthreads();
        dif_op_dit<NY, NY, CV, NTHR, 1>(s, twy, tid, YFactors<C::CX, SLO, PB>{a.t1.RyD, a.Nt, unit});
        cluster_exchange<CL, C::RSZ, NTHR>(s, cluster, rank, tid);
        dif_op_dit<NX, NX, RV, NTHR, 1>(s, twx, tid, XFactors{a.t1.Rx});
        if (a.lens) {
            // mirror lens in real (x, y): exp(-i k0 (x^2 + y^2)/roc) = lensx[x] * lensy[y]
            for (int e = tid; e < PB * C::RY * NX; e += NTHR) {
                const int x = e % NX;
                const int l = e / NX;
                const int yl = l % C::RY;
                const int y = rank * C::RY + yl;
                const int idx = RV::at(x, l);
                s[idx] = cmul(s[idx], cmul(__ldg(&a.lensx[x]), __ldg(&a.lensy[y])));
            }
            __syncthreads();
            dif_op_dit<NX, NX, RV, NTHR, 1>(s, twx, tid, XFactors{a.t2.Rx});
            cluster_exchange<CL, C::RSZ, NTHR>(s, cluster, rank, tid);
            dif_op_dit<NY, NY, CV, NTHR, 1>(s, twy, tid, YFactors<C::CX, SLO, PB>{a.t2.RyD, a.Nt, unit});
            plane_move<NX, NY, CL, PB, SLO, NTHR, false, true>(s, nullptr, a.out, rank, unit, NP, tid);
        } else {
            plane_move<NX, NY, CL, PB, SLO, NTHR, true, true>(s, nullptr, a.out, rank, unit, NP, tid);
        }
        __syncthreads();
    }
    cluster.sync();
}

// ---------------------------------------------------------------------------------------
// Plane pass in two passes over HBM (no clusters), for planes that a cluster of 2-CTA-per-SM
// blocks cannot hold: the linear step's y part on column strips, then its x part on row strips
// (IFFT_xy Rx Ry D FFT_xy = (IFFT_x Rx FFT_x)(IFFT_y Ry D FFT_y)).  Slot layout SLO = 1.  Each
// CTA reads and writes only its own strip, so both passes run in place.
// ---------------------------------------------------------------------------------------
// strip of CXS columns of one omega-plane: line = column, position = y
template <int NY, int CXS>
struct StripYView {
    static constexpr int NLINES = CXS;
    static constexpr __host__ __device__ __forceinline__ int at(int y, int l) { return y * CXS + l; }
};
// strip of RYS rows: line = row, position = x, rows padded by one element (bank spread)
template <int NX, int RYS>
struct StripXView {
    static constexpr int NLINES = RYS;
    static constexpr __host__ __device__ __forceinline__ int at(int x, int l) { return l * (NX + 1) + x; }
};

template <int NX, int NY, int CXS>
struct StripYCfg {
    static constexpr int SIZE = NY * CXS;
    // [strip][the slot's NY factors Ry(y) D(slot), 16 B each][W_NY twiddles]
    static constexpr int SMEM = SIZE * 8 + NY * 16 + twiddle_bytes(NY);
    // at least 16 columns: the rows of a warp's butterfly loads then fill all 32 banks
    static_assert(CXS >= 16 && CXS % 2 == 0 && NX % CXS == 0, "whole float4 column strips");
};
template <int NX, int NY, int RYS>
struct StripXCfg {
    static constexpr int SIZE = RYS * (NX + 1);
    // rows of up to 256 points: the x factors of both tables staged in shared memory once per CTA
    static constexpr bool XSTAGE = NX <= 256;
    static constexpr int SMEM = ((SIZE * 8 + 15) / 16) * 16 + (XSTAGE ? 2 * NX * 16 : 0) + twiddle_bytes(NX);
    static_assert(NY % RYS == 0 && NX % 2 == 0, "whole row strips");
};


// Ry(y) D(slot) of the unit's slot from shared memory (staged once per unit)
struct YSmemFactors {
    const float4* f;   // NY factors of the unit's slot, shared memory
    template <int R>
    __device__ __forceinline__ void operator()(float2 (&v)[R], int y0, int) const {
#pragma unroll
        for (int q = 0; q < R; q++) v[q] = cmul_df(v[q], f[y0 + q]);
    }
};

// Resident CTAs per SM a strip kernel is compiled for: MINB, or 512 / NTHR (128 registers).
__host__ __device__ constexpr int strip_min_blocks(int NTHR, int MINB) {
    return MINB > 0 ? MINB : (NTHR >= 512 ? 1 : 512 / NTHR);
}

// y part: units are (slot, strip of CXS columns); `second` selects the table set t2.
template <int NX, int NY, int CXS, int NTHR, int MINB = 0>
__global__ void __launch_bounds__(NTHR, strip_min_blocks(NTHR, MINB)) plane_y_kernel(PlaneArgs a, int second) {
    using C = StripYCfg<NX, NY, CXS>;
    using V = StripYView<NY, CXS>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* s = reinterpret_cast<float2*>(smem_raw);
    float4* fac = reinterpret_cast<float4*>(smem_raw + C::SIZE * 8);
    unsigned char* tw_mem = smem_raw + C::SIZE * 8 + NY * 16;
    const int tid = threadIdx.x;
    stage_twiddles<NY, NTHR>(tw_mem, a.twy, tid);
    const Twiddles tw = Twiddles::packed(tw_mem, NY);
    __syncthreads();
    const float4* RyDT = second ? a.t2.RyDT : a.t1.RyDT;
    constexpr int STRIPS = NX / CXS;
    constexpr int F4_ROW = CXS / 2;
    const int units = a.Nt * STRIPS;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
        const int slot = unit / STRIPS, x0 = (unit - slot * STRIPS) * CXS;
        const float4* g4 = reinterpret_cast<const float4*>(a.in) + ((size_t)slot * a.NP + x0) / 2;
        // the slot's factors, shared by the strip's CXS columns
        for (int y = tid; y < NY; y += NTHR) fac[y] = __ldg(&RyDT[(size_t)slot * NY + y]);
#pragma unroll 8
        for (int f = tid; f < NY * F4_ROW; f += NTHR) {
            const int y = f / F4_ROW, c = f - y * F4_ROW;
            reinterpret_cast<float4*>(s)[(y * CXS) / 2 + c] = __ldg(&g4[(size_t)y * (NX / 2) + c]);
        }
        __syncthreads();
        dif_op_dit<NY, NY, V, NTHR, 1>(s, tw, tid, YSmemFactors{fac});
        float4* o4 = reinterpret_cast<float4*>(a.out) + ((size_t)slot * a.NP + x0) / 2;
#pragma unroll 8
        for (int f = tid; f < NY * F4_ROW; f += NTHR) {
            const int y = f / F4_ROW, c = f - y * F4_ROW;
            o4[(size_t)y * (NX / 2) + c] = reinterpret_cast<const float4*>(s)[(y * CXS) / 2 + c];
        }
        __syncthreads();
    }
}

// y part with TMA staging: a persistent CTA walks its units (slot, strip of CXS columns) with
// NBUF unit buffers in shared memory; warp 0 keeps NBUF - 1 units in flight as 2-D bulk tensor
// loads (box: CXS complex columns x NY rows of one omega-plane, landing in the StripYView layout)
// plus a bulk copy of the slot's NY factors Ry(y) D(slot) (the slot-major table, 16 B each) on
// the same mbarrier, and each finished unit leaves by a bulk tensor store, so no thread spends
// instructions or registers on moving the strips and every factor is read from shared memory
// (all CXS columns of a row share it).  tin / tout map the field as float rows of 2 Nx values,
// Ny * Nt rows.  A load that does not arrive within the wait limit sets *err and ends the kernel.
template <int NX, int NY, int CXS>
struct StripYTmaCfg {
    static constexpr int UNIT_BYTES = NY * CXS * 8;
    static constexpr int FAC_BYTES = NY * 16;   // one slot's Ry(y) D(slot) factors, double-float
    static_assert(UNIT_BYTES % 128 == 0 && CXS * 8 % 16 == 0, "unit buffers of whole 128 B lines");
    static constexpr __host__ __device__ int FAC_OFF(int nbuf) { return nbuf * UNIT_BYTES; }
    static constexpr __host__ __device__ int TW_OFF(int nbuf) { return FAC_OFF(nbuf) + nbuf * FAC_BYTES; }
    static constexpr __host__ __device__ int BAR_OFF(int nbuf) { return TW_OFF(nbuf) + ((twiddle_bytes(NY) + 15) / 16) * 16; }
    static constexpr __host__ __device__ int SMEM(int nbuf) { return 128 + BAR_OFF(nbuf) + nbuf * 8 + 16; }
};

template <int NX, int NY, int CXS, int NTHR, int NBUF>
__global__ void __launch_bounds__(NTHR, 512 / NTHR)
    plane_y_tma_kernel(const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tout, PlaneArgs a,
                       int second, unsigned int* err) {
    using C = StripYTmaCfg<NX, NY, CXS>;
    using V = StripYView<NY, CXS>;
    extern __shared__ __align__(128) unsigned char smem_dyn[];
    // unit buffers on a 128-byte boundary of the shared window (the launch adds 128 B of slack)
    unsigned char* smem_raw = smem_dyn + ((128u - (smem_addr(smem_dyn) & 127u)) & 127u);
    unsigned char* tw_mem = smem_raw + C::TW_OFF(NBUF);
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + C::BAR_OFF(NBUF));
    int& s_arrived = *reinterpret_cast<int*>(bars + NBUF);
    const int tid = threadIdx.x;
    constexpr int STRIPS = NX / CXS;
    const int units = a.Nt * STRIPS;
    const int nmine = blockIdx.x < units ? (units - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    if (tid == 0) {
        for (int b = 0; b < NBUF; b++) mbar_init(&bars[b], 1);
        fence_mbar_init();
    }
    stage_twiddles<NY, NTHR>(tw_mem, a.twy, tid);
    const Twiddles tw = Twiddles::packed(tw_mem, NY);
    const float4* RyDT = second ? a.t2.RyDT : a.t1.RyDT;
    __syncthreads();
    auto buf = [&](int k) { return reinterpret_cast<float2*>(smem_raw + (k % NBUF) * C::UNIT_BYTES); };
    auto fac = [&](int k) {
        return reinterpret_cast<float4*>(smem_raw + C::FAC_OFF(NBUF) + (k % NBUF) * C::FAC_BYTES);
    };
    const int warp = tid >> 5, lane = tid & 31;
    // the copies of a unit are issued by warp 0: lane 0 arms the mbarrier with the unit's bytes and
    // loads the strip, lane 1 the slot's factors
    auto issue = [&](int k) {
        const int unit = (int)blockIdx.x + k * (int)gridDim.x;
        const int slot = unit / STRIPS, x0 = (unit - slot * STRIPS) * CXS;
        if (lane == 0) mbar_arrive_expect_tx(&bars[k % NBUF], C::UNIT_BYTES + C::FAC_BYTES);
        __syncwarp();
        if (lane == 0) tma_load_2d(buf(k), &tin, 2 * x0, slot * NY, &bars[k % NBUF]);
        if (lane == 1) bulk_load(fac(k), RyDT + (size_t)slot * NY, C::FAC_BYTES, &bars[k % NBUF]);
    };
    if (warp == 0)
        for (int k = 0; k < NBUF - 1 && k < nmine; k++) issue(k);
    for (int k = 0; k < nmine; k++) {
        const int unit = (int)blockIdx.x + k * (int)gridDim.x;
        const int slot = unit / STRIPS, x0 = (unit - slot * STRIPS) * CXS;
        // one thread decides whether the unit arrived in time, so that the whole CTA takes the
        // same branch; then every thread observes the completed phase itself
        if (tid == 0) s_arrived = mbar_wait(&bars[k % NBUF], (uint32_t)((k / NBUF) & 1)) ? 1 : 0;
        __syncthreads();
        if (!s_arrived) {
            if (tid == 0) {
                atomicExch(err, KERR_TMA_TIMEOUT);
                // the loads still in flight target the later buffers: wait (bounded) for them
                for (int j = k + 1; j < k + NBUF - 1 && j < nmine; j++) mbar_wait(&bars[j % NBUF], (uint32_t)((j / NBUF) & 1));
                bulk_wait<0>();
            }
            return;
        }
        mbar_wait(&bars[k % NBUF], (uint32_t)((k / NBUF) & 1));   // completed: returns at once
        float2* s = buf(k);
        dif_op_dit<NY, NY, V, NTHR, 1, YSmemFactors, false>(s, tw, tid, YSmemFactors{fac(k)});
        fence_proxy_async_smem();   // this thread's results, before the bulk store reads them
        __syncthreads();
        if (warp == 0) {
            if (lane == 0) {
                tma_store_2d(&tout, 2 * x0, slot * NY, s);
                bulk_commit();
            }
            if (k + NBUF - 1 < nmine) {
                if (lane == 0) bulk_wait_read<1>();   // the previous unit's store has left its buffer
                issue(k + NBUF - 1);
            }
        }
    }
    if (tid == 0) bulk_wait<0>();
}

// x part with TMA staging, for rows of 256 = 16 x 16 points.  A unit is 16 rows of one omega-plane
// (32 KB, contiguous in HBM), loaded as 16 boxes of 16 rows x 16 complex (128 B box rows) with the
// 128-byte swizzle: box b (x = 16 b .. 16 b + 15) lands at byte 2048 b, row l at 128 l within it,
// and the 16-byte chunk c of the row at chunk c ^ (l & 7).  With that layout the transform's
// stages are free of bank conflicts when the span-16 stages put the 16 butterflies j of one row on
// a half-warp and the span-1 pass moves 16-byte pairs with 8 rows per quarter-warp.  The
// arithmetic is that of dif_op_dit with radix 16 (the same operations in the same order).
__device__ __forceinline__ int xsw_offset(int x, int l) {   // byte offset of element (row l, x)
    return ((x >> 4) << 11) + (l << 7) + ((((x & 15) >> 1) ^ (l & 7)) << 4) + ((x & 1) << 3);
}

template <int NTHR>
__device__ __forceinline__ void x16_span16(unsigned char* buf, Twiddles tw, int tid, bool inverse) {
    // 16 rows x 16 butterflies j, j fastest
    for (int item = tid; item < 256; item += NTHR) {
        const int j = item & 15, l = item >> 4;
        float2 v[16];
#pragma unroll
        for (int q = 0; q < 16; q++) v[q] = *reinterpret_cast<const float2*>(buf + xsw_offset(j + 16 * q, l));
        const float2* t = tw.w + j;   // stage L = 256 of the staged W_256 table starts at 0
        if (!inverse) {
            dft<16, false>(v);
#pragma unroll
            for (int k = 1; k < 16; k++) v[k] = cmul(v[k], t[(k - 1) * 16]);
        } else {
            const float* te = tw.e + j;
#pragma unroll
            for (int k = 1; k < 16; k++) {
                const float2 u = cmulc(v[k], t[(k - 1) * 16]);
                const float e = te[(k - 1) * 16];
                v[k] = make_float2(fmaf(u.x, e, u.x), fmaf(u.y, e, u.y));
            }
            dft<16, true>(v);
        }
#pragma unroll
        for (int q = 0; q < 16; q++) *reinterpret_cast<float2*>(buf + xsw_offset(j + 16 * q, l)) = v[q];
    }
}

template <int NTHR>
__device__ __forceinline__ void x16_middle(unsigned char* buf, const float4* Rx, int tid) {
    // the span-1 forward stage, the Rx factors and the span-1 inverse stage, on 16 consecutive
    // x of one row; rows fastest (8 rows per quarter-warp), pairs of complex per 16-byte access
    for (int item = tid; item < 256; item += NTHR) {
        const int l = item & 15, b = item >> 4;
        unsigned char* row = buf + (b << 11) + (l << 7);
        float2 v[16];
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const float4 f = *reinterpret_cast<const float4*>(row + ((c ^ (l & 7)) << 4));
            v[2 * c] = make_float2(f.x, f.y);
            v[2 * c + 1] = make_float2(f.z, f.w);
        }
        dft<16, false>(v);
#pragma unroll
        for (int q = 0; q < 16; q++) v[q] = cmul_df(v[q], Rx[16 * b + q]);   // shared memory
        dft<16, true>(v);
#pragma unroll
        for (int c = 0; c < 8; c++)
            *reinterpret_cast<float4*>(row + ((c ^ (l & 7)) << 4)) = make_float4(v[2 * c].x, v[2 * c].y, v[2 * c + 1].x,
                                                                                   v[2 * c + 1].y);
    }
}

// IFFT_x Rx FFT_x on the 16 rows of a swizzled unit; ends with a CTA barrier unless TAIL = false
template <int NTHR, bool TAIL = true>
__device__ __forceinline__ void x16_linear(unsigned char* buf, Twiddles tw, const float4* Rx, int tid) {
    x16_span16<NTHR>(buf, tw, tid, false);
    __syncthreads();
    x16_middle<NTHR>(buf, Rx, tid);
    __syncthreads();
    x16_span16<NTHR>(buf, tw, tid, true);
    if constexpr (TAIL) __syncthreads();
}

template <int NY, int NTHR, int NBUF>
__global__ void __launch_bounds__(NTHR, 512 / NTHR)
    plane_x_tma_kernel(const __grid_constant__ CUtensorMap tin, const __grid_constant__ CUtensorMap tout, PlaneArgs a,
                       unsigned int* err) {
    constexpr int NX = 256, RYS = 16, UNIT_BYTES = RYS * NX * 8;
    extern __shared__ __align__(1024) unsigned char smem_dyn[];
    // unit buffers on a 1024-byte boundary of the shared window, where the 128-byte swizzle's
    // pattern starts (the launch adds 1 KB of slack)
    unsigned char* smem_raw = smem_dyn + ((1024u - (smem_addr(smem_dyn) & 1023u)) & 1023u);
    float4* rx1 = reinterpret_cast<float4*>(smem_raw + NBUF * UNIT_BYTES);   // Rx of t1, then of t2
    float4* rx2 = rx1 + NX;
    unsigned char* tw_mem = reinterpret_cast<unsigned char*>(rx2 + NX);
    uint64_t* bars = reinterpret_cast<uint64_t*>(tw_mem + ((twiddle_bytes(NX) + 15) / 16) * 16);
    int& s_arrived = *reinterpret_cast<int*>(bars + NBUF);
    const int tid = threadIdx.x;
    constexpr int STRIPS = NY / RYS;
    for (int i = tid; i < NX; i += NTHR) {   // the x factors of both tables, once per CTA
        rx1[i] = __ldg(&a.t1.Rx[i]);
        rx2[i] = __ldg(&a.t2.Rx[i]);
    }
    const int units = a.Nt * STRIPS;
    const int nmine = blockIdx.x < units ? (units - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    if (tid == 0) {
        for (int b = 0; b < NBUF; b++) mbar_init(&bars[b], 1);
        fence_mbar_init();
    }
    stage_twiddles<NX, NTHR>(tw_mem, a.twx, tid);
    const Twiddles tw = Twiddles::packed(tw_mem, NX);
    __syncthreads();
    auto buf = [&](int k) { return smem_raw + (k % NBUF) * UNIT_BYTES; };
    auto coords = [&](int k, int* row0) {
        const int unit = (int)blockIdx.x + k * (int)gridDim.x;
        const int slot = unit / STRIPS, y0 = (unit - slot * STRIPS) * RYS;
        *row0 = slot * NY + y0;
        return y0;
    };
    const int warp = tid >> 5, lane = tid & 31;
    // the copies of a unit are issued by warp 0, one box per lane (lanes 0..15): lane 0 arms the
    // mbarrier with the unit's bytes first
    auto issue = [&](int k) {
        int row0;
        coords(k, &row0);
        if (lane == 0) mbar_arrive_expect_tx(&bars[k % NBUF], UNIT_BYTES);
        __syncwarp();
        if (lane < NX / 16) tma_load_2d(buf(k) + lane * 2048, &tin, 32 * lane, row0, &bars[k % NBUF]);
    };
    if (warp == 0)
        for (int k = 0; k < NBUF - 1 && k < nmine; k++) issue(k);
    for (int k = 0; k < nmine; k++) {
        int row0;
        const int y0 = coords(k, &row0);
        if (tid == 0) s_arrived = mbar_wait(&bars[k % NBUF], (uint32_t)((k / NBUF) & 1)) ? 1 : 0;
        __syncthreads();
        if (!s_arrived) {
            if (warp == 0) {
                if (lane == 0) {
                    atomicExch(err, KERR_TMA_TIMEOUT);
                    for (int j = k + 1; j < k + NBUF - 1 && j < nmine; j++)
                        mbar_wait(&bars[j % NBUF], (uint32_t)((j / NBUF) & 1));
                }
                if (lane < NX / 16) bulk_wait<0>();   // each lane's own stores
                __syncwarp();
            }
            return;
        }
        mbar_wait(&bars[k % NBUF], (uint32_t)((k / NBUF) & 1));   // completed: returns at once
        unsigned char* u = buf(k);
        if (a.lens) {
            x16_linear<NTHR>(u, tw, rx1, tid);
            for (int e = tid; e < RYS * NX; e += NTHR) {
                const int x = e % NX, r = e / NX;
                float2* pe = reinterpret_cast<float2*>(u + xsw_offset(x, r));
                *pe = cmul(*pe, cmul(__ldg(&a.lensx[x]), __ldg(&a.lensy[y0 + r])));
            }
            __syncthreads();
            x16_linear<NTHR, false>(u, tw, rx2, tid);
        } else {
            x16_linear<NTHR, false>(u, tw, rx1, tid);
        }
        fence_proxy_async_smem();   // this thread's results, before the bulk stores read them
        __syncthreads();
        if (warp == 0) {
            if (lane < NX / 16) {
                tma_store_2d(&tout, 32 * lane, row0, u + lane * 2048);
                bulk_commit();
            }
            if (k + NBUF - 1 < nmine) {
                // lane b refills box b of the buffer its own store of the previous unit read
                if (lane < NX / 16) bulk_wait_read<1>();
                issue(k + NBUF - 1);
            }
        }
    }
    if (warp == 0 && lane < NX / 16) bulk_wait<0>();
}

// x part: units are (slot, strip of RYS rows); with the mirror lens, x(t1), the lens, x(t2).
template <int NX, int NY, int RYS, int NTHR, int MINB = 0>
__global__ void __launch_bounds__(NTHR, strip_min_blocks(NTHR, MINB)) plane_x_kernel(PlaneArgs a) {
    using C = StripXCfg<NX, NY, RYS>;
    using V = StripXView<NX, RYS>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2* s = reinterpret_cast<float2*>(smem_raw);
    float4* rx_s = reinterpret_cast<float4*>(smem_raw + ((C::SIZE * 8 + 15) / 16) * 16);
    unsigned char* tw_mem = reinterpret_cast<unsigned char*>(rx_s) + (C::XSTAGE ? 2 * NX * 16 : 0);
    const int tid = threadIdx.x;
    stage_twiddles<NX, NTHR>(tw_mem, a.twx, tid);
    const Twiddles tw = Twiddles::packed(tw_mem, NX);
    const float4* rx1 = a.t1.Rx;
    const float4* rx2 = a.t2.Rx;
    if constexpr (C::XSTAGE) {
        for (int i = tid; i < NX; i += NTHR) {
            rx_s[i] = __ldg(&a.t1.Rx[i]);
            rx_s[NX + i] = __ldg(&a.t2.Rx[i]);
        }
        rx1 = rx_s;
        rx2 = rx_s + NX;
    }
    __syncthreads();
    constexpr int STRIPS = NY / RYS;
    constexpr int F4_ROW = NX / 2;
    const int units = a.Nt * STRIPS;
    for (int unit = blockIdx.x; unit < units; unit += gridDim.x) {
        const int slot = unit / STRIPS, y0 = (unit - slot * STRIPS) * RYS;
        const float4* g4 = reinterpret_cast<const float4*>(a.in) + ((size_t)slot * a.NP + (size_t)y0 * NX) / 2;
#pragma unroll 8
        for (int f = tid; f < RYS * F4_ROW; f += NTHR) {
            const int r = f / F4_ROW, c = f - r * F4_ROW;
            const float4 v = __ldg(&g4[f]);
            s[V::at(2 * c, r)] = make_float2(v.x, v.y);
            s[V::at(2 * c + 1, r)] = make_float2(v.z, v.w);
        }
        __syncthreads();
        dif_op_dit<NX, NX, V, NTHR, 1>(s, tw, tid, XFactorsAny{rx1});
        if (a.lens) {
            for (int e = tid; e < RYS * NX; e += NTHR) {
                const int x = e % NX, r = e / NX;
                const int idx = V::at(x, r);
                s[idx] = cmul(s[idx], cmul(__ldg(&a.lensx[x]), __ldg(&a.lensy[y0 + r])));
            }
            __syncthreads();
            dif_op_dit<NX, NX, V, NTHR, 1>(s, tw, tid, XFactorsAny{rx2});
        }
        float4* o4 = reinterpret_cast<float4*>(a.out) + ((size_t)slot * a.NP + (size_t)y0 * NX) / 2;
#pragma unroll 8
        for (int f = tid; f < RYS * F4_ROW; f += NTHR) {
            const int r = f / F4_ROW, c = f - r * F4_ROW;
            const float2 e0 = s[V::at(2 * c, r)], e1 = s[V::at(2 * c + 1, r)];
            o4[f] = make_float4(e0.x, e0.y, e1.x, e1.y);
        }
        __syncthreads();
    }
}

}  // namespace mpc
