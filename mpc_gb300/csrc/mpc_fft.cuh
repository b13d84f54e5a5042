// mpc_fft.cuh -- complex64 arithmetic and in-shared-memory FFT stages for sm_103a.
//
// The propagator's transforms (t pencils, x rows, y columns) are all batched power-of-two
// FFTs done in shared memory: a forward transform is an in-place decimation-in-frequency
// (DIF) sweep that leaves the spectrum in digit-reversed "position" order, an inverse is the
// exact transpose sweep (decimation in time, DIT) that takes position order back to natural
// order.  Nothing between a forward and an inverse transform needs natural frequency order,
// so no reordering pass ever runs; diagonal operators (dispersion, diffraction, -i*omega) are
// indexed through a position -> frequency table built on the host (mpc_freq_of_pos).
//
// Radix plan of a length-L stage: 16 while L >= 16, else L (so 2048 = 16*16*8,
// 1024 = 16*16*4, 512 = 16*16*2, 256 = 16*16, 128 = 16*8, 64 = 16*4).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mpc {

// Complex add and subtract as packed FP32x2 instructions (one instruction for both parts; each
// part rounded exactly as the scalar operation): a - b is computed as fma(b, -1, a), whose
// single rounding of the exact a - b equals the subtraction's.
#ifndef MPC_PACKED_F32X2
#define MPC_PACKED_F32X2 1
#endif
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
#if MPC_PACKED_F32X2
    return __fadd2_rn(a, b);
#else
    return make_float2(a.x + b.x, a.y + b.y);
#endif
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
#if MPC_PACKED_F32X2
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
#else
    return make_float2(a.x - b.x, a.y - b.y);
#endif
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// a * conj(b)
__device__ __forceinline__ float2 cmulc(float2 a, float2 b) {
    return make_float2(fmaf(a.x, b.x, a.y * b.y), fmaf(a.y, b.x, -a.x * b.y));
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
// multiply by -i (forward kernel sign) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}
// The butterflies' constant factors (sqrt(1/2), cos(pi/8), sin(pi/8)) are applied as a high
// FP32 part plus a low correction (exact value minus high part, from FP64).  Rounded to FP32
// alone they are off unit modulus by 3e-8..6e-8, and since every forward/inverse round trip
// applies the same constants, that error would accumulate linearly over the steps of a run
// (about -2e-7 energy per split step); with the low parts it is ~1e-15.
constexpr double kSqrtHalf = 0.70710678118654752440;
constexpr double kCos8 = 0.92387953251128675613;   // cos(pi/8)
constexpr double kSin8 = 0.38268343236508977173;   // sin(pi/8)
constexpr float kH = (float)kSqrtHalf, kHl = (float)(kSqrtHalf - (double)(float)kSqrtHalf);
constexpr float kC8 = (float)kCos8, kC8l = (float)(kCos8 - (double)(float)kCos8);
constexpr float kS8 = (float)kSin8, kS8l = (float)(kSin8 - (double)(float)kSin8);

// t * sqrt(1/2) with the low-part correction
__device__ __forceinline__ float mul_h(float t) { return fmaf(t, kH, t * kHl); }

// a * (z.hi + z.lo): double-float complex factor z = (x, y) + (z, w)
__device__ __forceinline__ float2 cmul_df(float2 a, float4 z) {
    const float cr = fmaf(a.x, z.z, -a.y * z.w);
    const float ci = fmaf(a.x, z.w, a.y * z.z);
    return make_float2(fmaf(a.x, z.x, fmaf(-a.y, z.y, cr)), fmaf(a.x, z.y, fmaf(a.y, z.x, ci)));
}

// multiply by exp(-+i*pi/4) = (1 -+ i)/sqrt(2)
template <bool INV>
__device__ __forceinline__ float2 mul_w8(float2 a) {
    return INV ? make_float2(mul_h(a.x - a.y), mul_h(a.x + a.y))
               : make_float2(mul_h(a.x + a.y), mul_h(a.y - a.x));
}
// multiply by exp(-+3i*pi/4) = (-1 -+ i)/sqrt(2)
template <bool INV>
__device__ __forceinline__ float2 mul_w83(float2 a) {
    return INV ? make_float2(mul_h(-a.x - a.y), mul_h(a.x - a.y))
               : make_float2(mul_h(a.y - a.x), mul_h(-a.x - a.y));
}

// ---- small DFTs in registers, natural order in and out, unnormalised ------------------
template <bool INV>
__device__ __forceinline__ void dft2(float2& a, float2& b) {
    const float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <bool INV>
__device__ __forceinline__ void dft4(float2& x0, float2& x1, float2& x2, float2& x3) {
    const float2 s02 = cadd(x0, x2), d02 = csub(x0, x2);
    const float2 s13 = cadd(x1, x3), d13 = mul_mi<INV>(csub(x1, x3));
    x0 = cadd(s02, s13);
    x2 = csub(s02, s13);
    x1 = cadd(d02, d13);
    x3 = csub(d02, d13);
}

template <int R, bool INV>
__device__ __forceinline__ void dft(float2 (&v)[R]);

template <>
__device__ __forceinline__ void dft<2, false>(float2 (&v)[2]) { dft2<false>(v[0], v[1]); }
template <>
__device__ __forceinline__ void dft<2, true>(float2 (&v)[2]) { dft2<true>(v[0], v[1]); }
template <>
__device__ __forceinline__ void dft<4, false>(float2 (&v)[4]) { dft4<false>(v[0], v[1], v[2], v[3]); }
template <>
__device__ __forceinline__ void dft<4, true>(float2 (&v)[4]) { dft4<true>(v[0], v[1], v[2], v[3]); }

// 8 = 4 x 2: n = 2 n1 + n2, k = k1 + 4 k2
template <bool INV>
__device__ __forceinline__ void dft8(float2 (&v)[8]) {
    dft4<INV>(v[0], v[2], v[4], v[6]);   // Y[0][k1] at v[0],v[2],v[4],v[6]
    dft4<INV>(v[1], v[3], v[5], v[7]);   // Y[1][k1] at v[1],v[3],v[5],v[7]
    v[3] = mul_w8<INV>(v[3]);
    v[5] = mul_mi<INV>(v[5]);
    v[7] = mul_w83<INV>(v[7]);
    float2 o[8];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
        o[k1] = cadd(v[2 * k1], v[2 * k1 + 1]);
        o[k1 + 4] = csub(v[2 * k1], v[2 * k1 + 1]);
    }
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = o[i];
}
template <>
__device__ __forceinline__ void dft<8, false>(float2 (&v)[8]) { dft8<false>(v); }
template <>
__device__ __forceinline__ void dft<8, true>(float2 (&v)[8]) { dft8<true>(v); }

// 16 = 4 x 4: n = 4 n1 + n2, k = k1 + 4 k2, inner twiddle W16^(n2 k1)
template <bool INV>
__device__ __forceinline__ void dft16(float2 (&v)[16]) {
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) dft4<INV>(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]);
    // now v[n2 + 4 k1] = Y[n2][k1]
    const float sg = INV ? 1.0f : -1.0f;
    const float4 w1 = make_float4(kC8, sg * kS8, kC8l, sg * kS8l);      // W16^1
    const float4 w3 = make_float4(kS8, sg * kC8, kS8l, sg * kC8l);      // W16^3
    const float4 w9 = make_float4(-kC8, -sg * kS8, -kC8l, -sg * kS8l);  // W16^9
    v[5] = cmul_df(v[5], w1);         // n2=1,k1=1
    v[9] = mul_w8<INV>(v[9]);         // n2=1,k1=2 : W16^2
    v[13] = cmul_df(v[13], w3);       // n2=1,k1=3
    v[6] = mul_w8<INV>(v[6]);         // n2=2,k1=1 : W16^2
    v[10] = mul_mi<INV>(v[10]);       // n2=2,k1=2 : W16^4
    v[14] = mul_w83<INV>(v[14]);      // n2=2,k1=3 : W16^6
    v[7] = cmul_df(v[7], w3);         // n2=3,k1=1
    v[11] = mul_w83<INV>(v[11]);      // n2=3,k1=2 : W16^6
    v[15] = cmul_df(v[15], w9);       // n2=3,k1=3
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) dft4<INV>(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
    // now v[4 k1 + k2] = X[k1 + 4 k2]; transpose to natural order
    float2 o[16];
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++)
#pragma unroll
        for (int k2 = 0; k2 < 4; k2++) o[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = o[i];
}
template <>
__device__ __forceinline__ void dft<16, false>(float2 (&v)[16]) { dft16<false>(v); }
template <>
__device__ __forceinline__ void dft<16, true>(float2 (&v)[16]) { dft16<true>(v); }

template <int L>
struct Radix {
    static constexpr int R = (L >= 16) ? 16 : L;
};

// ---- batched in-place stages over a shared-memory view --------------------------------
// View: NLINES independent lines of length N; element `pos` of line `l` lives at
// V::at(pos, l).  Work items are (line, butterfly) pairs, lines fastest across threads.
// tw: twiddle table of W_N, packed as N float2 w[k] = (c, s) = exp(-2 pi i k / N) rounded to
// FP32 from FP64, followed by N float e[k] = -eps with eps = c^2 + s^2 - 1 (computed in FP64
// from the rounded values).  The forward (DIF) stage multiplies by (c, s); the inverse (DIT)
// stage by conj(c, s) * (1 - eps), so every forward/inverse round trip has gain 1 - eps^2 per
// path instead of 1 + eps: rounded twiddles alone lose ~6e-8 of the energy per split step.
// In global memory the table is in natural order k; the kernels copy it to shared memory in
// "staged" order (stage_twiddles): for each stage of sub-length L (span S = L/R) the R - 1
// factors W_N^(j k N/L), k = 1..R-1, of every j < S, stored at [(k - 1) S + j].  The threads of
// a warp that read one k then read consecutive words (the natural-order index j k N/L puts the
// 4..8 j of a warp in one bank at the middle stage of a 2048-point transform), and each
// butterfly's R - 1 addresses are one base plus compile-time offsets.
//
// Every view used here is "stage separable": for a butterfly of span S starting at
// base = b*L + j (j < S), V::at(base + S*q, l) == V::at(base, l) + V::at(S*q, 0) - V::at(0, 0),
// so the R addresses of a butterfly are one computed base plus compile-time offsets
// (tests/test_host.py checks the property for every view and stage of the library).

struct Twiddles {
    const float2* w;  // N entries (c, s)
    const float* e;   // N entries -eps
    // a packed table of N entries starting at p (shared or global memory)
    __host__ __device__ static Twiddles packed(const void* p, int N) {
        Twiddles t;
        t.w = static_cast<const float2*>(p);
        t.e = reinterpret_cast<const float*>(t.w + N);
        return t;
    }
};
// bytes of a packed table of N entries
__host__ __device__ constexpr int twiddle_bytes(int N) { return N * 12; }

// First entry of the stage of sub-length L in the staged table of W_N: the stages before it
// (sub-lengths N, N/R, ...) hold L' - L'/R' entries each; all stages together hold fewer than N.
__host__ __device__ constexpr int tw_stage_offset(int N, int L) {
    return N == L ? 0 : (N - N / (N >= 16 ? 16 : N)) + tw_stage_offset(N / (N >= 16 ? 16 : N), L);
}

// Copy the natural-order table `src` (global) into shared memory `dst` in staged order.
// Entries past the last stage are zero (never read).
template <int N, int NTH>
__device__ __forceinline__ void stage_twiddles(void* dst, const float2* __restrict__ src, int tid) {
    float2* w = static_cast<float2*>(dst);
    float* e = reinterpret_cast<float*>(w + N);
    const float* se = reinterpret_cast<const float*>(src + N);
    for (int i = tid; i < N; i += NTH) {
        int L = N, off = 0, flat = -1;
        while (L > 1) {
            const int R = (L >= 16) ? 16 : L, S = L / R, cnt = L - S;
            if (i < off + cnt) {
                const int k = (i - off) / S + 1, j = (i - off) % S;
                flat = j * k * (N / L);
                break;
            }
            off += cnt;
            L /= R;
        }
        if (flat >= 0) {
            w[i] = __ldg(&src[flat]);
            e[i] = __ldg(&se[flat]);
        } else {
            w[i] = make_float2(0.0f, 0.0f);
            e[i] = 0.0f;
        }
    }
}

// Loads and stores fused into a transform's first or last stage, in place of shared memory.
// A SRC (active) gives the first stage of an inverse transform its inputs: src(v, pos0, line)
// fills v with positions pos0 .. pos0 + R - 1 of one line.  A SINK (active) takes the results
// of the last stage: sink(v, i0, S, line) gets indices i0 + S q, q < R (natural order after an
// inverse transform, position order after a forward one, where S = 1).
struct NoOp {
    static constexpr bool active = false;
};

// Warp-local tail.  The last two stages of a transform (sub-length L2 = 16 * Ll, then the span-1
// stage of radix Ll) work inside sub-transforms of L2 points.  When a warp's 32 work items of the
// stage L2 are exactly one such sub-transform (NL * Ll == 32 lines x butterflies) and the warps
// share the sub-transforms evenly, the span-1 stage can give each warp the same sub-transforms it
// had in stage L2: the barrier between the two stages is then a warp barrier (__syncwarp), and the
// warps run the tail independently.  Used where those conditions hold (the 2048-point transforms of
// 4-pencil tiles on 256 threads); per butterfly the arithmetic is unchanged.
__host__ __device__ constexpr int tail_last(int N) { return N <= 16 ? N : tail_last(N / 16); }
template <int N, int NL, int NTH>
struct WarpTail {
    static constexpr int LL = tail_last(N);      // radix (and length) of the span-1 stage
    static constexpr int L2 = 16 * LL;           // sub-transform length of the tail
    static constexpr int NW = NTH / 32;
    static constexpr int PPS = 16 / LL;          // warp passes per sub-transform in the span-1 stage
    static constexpr bool ok = N > L2 && NTH % 32 == 0 && NL * LL == 32 && 16 % LL == 0 &&
                               ((N / 16) * NL) % NTH == 0 && (N / L2) % NW == 0 &&
                               ((N / LL) * NL) % NTH == 0 && ((N / LL) * NL) / NTH == ((N / L2) / NW) * PPS;
    // item (line, butterfly g) of pass u of the span-1 stage for thread tid
    __device__ __forceinline__ static void item(int tid, int u, int& line, int& g) {
        const int w = tid >> 5, lane = tid & 31;
        const int sub = w + NW * (u / PPS);
        const int i = (u % PPS) * 32 + lane;
        line = i % NL;
        g = sub * 16 + i / NL;
    }
};

// DIF stage of sub-length L (span S = L/R): y_k = W_L^(j k) * sum_q x_q W_R^(q k).
// NTH threads share the stage's TOT butterflies; UNR of a thread's butterflies are unrolled
// together so that their shared-memory loads overlap.
template <int N, int L, class V, int NTH, int UNR, class SINK = NoOp>
__device__ __forceinline__ void dif_stage(float2* s, Twiddles tw, int tid, const SINK& sink = SINK{}) {
    constexpr int R = Radix<L>::R;
    constexpr int S = L / R;
    constexpr int NB = N / R;
    constexpr int TOT = NB * V::NLINES;
    using WT = WarpTail<N, V::NLINES, NTH>;
    constexpr bool WTAIL = WT::ok && S == 1;
#pragma unroll UNR
    for (int idx = tid; idx < TOT; idx += NTH) {
        int line, g;
        if constexpr (WTAIL) {
            WT::item(tid, (idx - tid) / NTH, line, g);
        } else {
            line = idx % V::NLINES;
            g = idx / V::NLINES;
        }
        const int b = g / S, j = g - (g / S) * S;
        float2* p0 = s + V::at(b * L + j, line);
        float2 v[R];
#pragma unroll
        for (int q = 0; q < R; q++) v[q] = p0[V::at(S * q, 0) - V::at(0, 0)];
        dft<R, false>(v);
        if (S > 1) {
            const float2* t = tw.w + tw_stage_offset(N, L) + j;
#pragma unroll
            for (int k = 1; k < R; k++) v[k] = cmul(v[k], t[(k - 1) * S]);
        }
        if constexpr (S == 1 && SINK::active) {
            sink(v, b * L, 1, line);
        } else {
#pragma unroll
            for (int q = 0; q < R; q++) p0[V::at(S * q, 0) - V::at(0, 0)] = v[q];
        }
    }
}

// DIT stage (exact transpose of the DIF stage with conjugate twiddles).  CORR = false skips the
// (1 - eps) magnitude correction, for transforms whose result is not fed back into the field
// (the time derivative of the self-steepening term).  The stage with span 1 (the first of the
// inverse transform) loads through SRC; the stage of sub-length N (the last) stores through SINK.
template <int N, int L, class V, int NTH, int UNR, bool CORR = true, class SRC = NoOp, class SINK = NoOp>
__device__ __forceinline__ void dit_stage(float2* s, Twiddles tw, int tid, const SRC& src = SRC{},
                                          const SINK& sink = SINK{}) {
    constexpr int R = Radix<L>::R;
    constexpr int S = L / R;
    constexpr int NB = N / R;
    constexpr int TOT = NB * V::NLINES;
    using WT = WarpTail<N, V::NLINES, NTH>;
    constexpr bool WTAIL = WT::ok && S == 1;
#pragma unroll UNR
    for (int idx = tid; idx < TOT; idx += NTH) {
        int line, g;
        if constexpr (WTAIL) {
            WT::item(tid, (idx - tid) / NTH, line, g);
        } else {
            line = idx % V::NLINES;
            g = idx / V::NLINES;
        }
        const int b = g / S, j = g - (g / S) * S;
        float2* p0 = s + V::at(b * L + j, line);
        float2 v[R];
        if constexpr (S == 1 && SRC::active) {
            src(v, b * L, line);
        } else {
#pragma unroll
            for (int q = 0; q < R; q++) v[q] = p0[V::at(S * q, 0) - V::at(0, 0)];
        }
        if (S > 1) {
            const float2* t = tw.w + tw_stage_offset(N, L) + j;
            const float* te = tw.e + tw_stage_offset(N, L) + j;
#pragma unroll
            for (int k = 1; k < R; k++) {
                const float2 u = cmulc(v[k], t[(k - 1) * S]);
                if constexpr (CORR) {
                    const float e = te[(k - 1) * S];
                    v[k] = make_float2(fmaf(u.x, e, u.x), fmaf(u.y, e, u.y));
                } else {
                    v[k] = u;
                }
            }
        }
        dft<R, true>(v);
        if constexpr (L == N && SINK::active) {
            sink(v, b * L + j, S, line);
        } else {
#pragma unroll
            for (int q = 0; q < R; q++) p0[V::at(S * q, 0) - V::at(0, 0)] = v[q];
        }
    }
}

// Whole forward transform (natural -> position order).  Ends with a __syncthreads.
template <int N, int L, class V, int NTH, int UNR = 1, class SINK = NoOp>
__device__ __forceinline__ void dif_all(float2* s, Twiddles tw, int tid, const SINK& sink = SINK{}) {
    dif_stage<N, L, V, NTH, UNR, SINK>(s, tw, tid, sink);
    using WT = WarpTail<N, V::NLINES, NTH>;
    if constexpr (WT::ok && L == WT::L2) __syncwarp();   // the span-1 stage stays inside the warp
    else __syncthreads();
    constexpr int R = Radix<L>::R;
    if constexpr (L / R > 1) dif_all<N, L / R, V, NTH, UNR, SINK>(s, tw, tid, sink);
}

// Whole inverse transform (position -> natural order), unnormalised.  Ends with a sync.
template <int N, int L, class V, int NTH, int UNR = 1, bool CORR = true, class SRC = NoOp, class SINK = NoOp>
__device__ __forceinline__ void dit_all(float2* s, Twiddles tw, int tid, const SRC& src = SRC{},
                                        const SINK& sink = SINK{}) {
    constexpr int R = Radix<L>::R;
    if constexpr (L / R > 1) dit_all<N, L / R, V, NTH, UNR, CORR, SRC, SINK>(s, tw, tid, src, sink);
    dit_stage<N, L, V, NTH, UNR, CORR, SRC, SINK>(s, tw, tid, src, sink);
    using WT = WarpTail<N, V::NLINES, NTH>;
    if constexpr (WT::ok && L == WT::LL) __syncwarp();   // stage L2 reads only this warp's results
    else __syncthreads();
}

// Forward transform, a diagonal operator in position order, inverse transform: the span-1 stage
// of the forward transform, the operator and the span-1 stage of the inverse work on the same R
// positions of a line, so they run in registers in one pass (op(v, pos0, line) multiplies the
// values of positions pos0 .. pos0 + R - 1).  Same arithmetic as dif_all, a pass applying op,
// then dit_all.  Ends with a __syncthreads unless TAIL = false (the caller then fences and
// synchronises itself).
template <int N, int L, class V, int NTH, int UNR, class OP, bool TAIL = true>
__device__ __forceinline__ void dif_op_dit(float2* s, Twiddles tw, int tid, const OP& op) {
    constexpr int R = Radix<L>::R;
    if constexpr (L / R > 1) {
        dif_stage<N, L, V, NTH, UNR>(s, tw, tid);
        __syncthreads();
        dif_op_dit<N, L / R, V, NTH, UNR, OP>(s, tw, tid, op);
        dit_stage<N, L, V, NTH, UNR>(s, tw, tid);
        if constexpr (TAIL) __syncthreads();
    } else {
        constexpr int TOT = (N / R) * V::NLINES;
#pragma unroll UNR
        for (int idx = tid; idx < TOT; idx += NTH) {
            const int line = idx % V::NLINES;
            const int b = idx / V::NLINES;
            float2* p0 = s + V::at(b * L, line);
            float2 v[R];
#pragma unroll
            for (int q = 0; q < R; q++) v[q] = p0[V::at(q, 0) - V::at(0, 0)];
            dft<R, false>(v);
            op(v, b * L, line);
            dft<R, true>(v);
#pragma unroll
            for (int q = 0; q < R; q++) p0[V::at(q, 0) - V::at(0, 0)] = v[q];
        }
        if constexpr (TAIL) __syncthreads();
    }
}

}  // namespace mpc
