/*
 * mpc_oracle.c -- FP64 CPU restatement of the kmecseki/MPC split-step propagator.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, and the timed CPU baseline).  Nothing in the
 * product path links or calls this file.  Each function cites the reference lines it
 * restates; where the reference is defective a defect number A<n> in the comments names
 * the switch in or_switches that selects corrected (1) or as-written (0) arithmetic.  The FFT is this file's own iterative radix-2 (the reference used FFTW
 * guru plans, propagation.c:554-603, which are not available here); it is checked
 * against numpy.fft by tests/test_oracle.py.
 */
#include "mpc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* constants.h:1-11 */
#define ZW0 377.0
#define NC 1.0
#define FCTR 0.89
#define IH 27.21
#define EF 5.14220642e11
#define ME 9.1094e-31
#define EL0 1.602e-19
#define NAVO 6.02214e+23
#define T0 2.4188843265e-17
#define C0 299792458.0
#define HBAR 1.054560652926899e-34

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

void or_default_switches(or_switches *sw) {
    sw->diffr_phase = 1;
    sw->diffr_fftorder = 1;
    sw->diffr_center = 1;
    sw->plasma_imag = 1;
    sw->nl_apply = 1;
    sw->ion_forward = 1;
    sw->ion_nq = 1;
    sw->ve_omega0 = 1;
    sw->energy_both = 1;
    sw->mirror_loss = 1;
    sw->z_advance_used = 1;
    sw->sigma_limit = 1;
    sw->bounce_lens = 0;
}

void or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* ------------------------------------------------------------------------------------
 * FFT: iterative radix-2 decimation in time on BLK lines at once, the lines interleaved
 * in a work buffer (element i of line b at buf[i*BLK + b]) so the inner loop runs over
 * neighbouring lines.  Twiddles exp(-2 pi i j/n) come from sin/cos in FP64.
 * ---------------------------------------------------------------------------------- */
#define BLK 8

static void make_twiddles(int n, or_complex *tw, int *rev) {
    for (int j = 0; j < n / 2; j++) {
        double a = -2.0 * M_PI * (double)j / (double)n;
        tw[j] = cos(a) + I * sin(a);
    }
    int lg = 0;
    while ((1 << lg) < n) lg++;
    for (int i = 0; i < n; i++) {
        int r = 0;
        for (int b = 0; b < lg; b++)
            if (i & (1 << b)) r |= 1 << (lg - 1 - b);
        rev[i] = r;
    }
}

/* transform nb (<= BLK) lines whose element i sits at base[b] + i*stride */
static void fft_block(or_complex *const *base, int nb, long stride, int n, int sign,
                      const or_complex *tw, const int *rev, or_complex *buf) {
    for (int i = 0; i < n; i++) {
        const long src = (long)rev[i] * stride;
        for (int b = 0; b < nb; b++) buf[(long)i * BLK + b] = base[b][src];
        for (int b = nb; b < BLK; b++) buf[(long)i * BLK + b] = 0;
    }
    for (int len = 2; len <= n; len <<= 1) {
        const int half = len >> 1, step = n / len;
        for (int s = 0; s < n; s += len) {
            for (int j = 0; j < half; j++) {
                or_complex wj = tw[j * step];
                if (sign > 0) wj = conj(wj);
                or_complex *u = buf + (long)(s + j) * BLK;
                or_complex *v = buf + (long)(s + j + half) * BLK;
                for (int b = 0; b < BLK; b++) {
                    const or_complex t = v[b] * wj;
                    v[b] = u[b] - t;
                    u[b] = u[b] + t;
                }
            }
        }
    }
    for (int i = 0; i < n; i++) {
        const long dst = (long)i * stride;
        for (int b = 0; b < nb; b++) base[b][dst] = buf[(long)i * BLK + b];
    }
}

/* Batched strided FFTs with the strides of the FFTW guru plans, propagation.c:563-603. */
void or_fft_axis(or_complex *A, int Nx, int Ny, int Nt, int axis, int sign) {
    int n;
    long stride, nlines;
    if (axis == 0) { n = Nx; stride = 1; nlines = (long)Ny * Nt; }
    else if (axis == 1) { n = Ny; stride = Nx; nlines = (long)Nx * Nt; }
    else { n = Nt; stride = (long)Nx * Ny; nlines = (long)Nx * Ny; }
    if (n <= 1) return;
    or_complex *tw = (or_complex *)malloc(sizeof(or_complex) * (n / 2 + 1));
    int *rev = (int *)malloc(sizeof(int) * n);
    make_twiddles(n, tw, rev);
    const long nblk = (nlines + BLK - 1) / BLK;
#pragma omp parallel
    {
        or_complex *buf = (or_complex *)malloc(sizeof(or_complex) * (long)n * BLK);
        or_complex *base[BLK];
#pragma omp for schedule(static)
        for (long bl = 0; bl < nblk; bl++) {
            int nb = 0;
            for (long l = bl * BLK; l < nlines && nb < BLK; l++, nb++) {
                long off;
                if (axis == 0) off = l * Nx;                       /* line (j,k): row start */
                else if (axis == 1) {                              /* line (i,k) */
                    long i = l % Nx, k = l / Nx;
                    off = k * (long)Nx * Ny + i;
                } else off = l;                                    /* line (i,j) */
                base[nb] = A + off;
            }
            fft_block(base, nb, stride, n, sign, tw, rev, buf);
        }
        free(buf);
    }
    free(tw);
    free(rev);
}

/* kernels.cu:47-54 (calcexpD0CUDA) / propagation.c:150-153, then fftshift axis 0
 * (propagation.c:393-402): swap the two halves. */
void or_expD0(or_complex *out, int Nt, double dzz, double alpha, const double *betas) {
    or_complex *tmp = (or_complex *)malloc(sizeof(or_complex) * Nt);
    for (int k = 0; k < Nt; k++) tmp[k] = cexp(dzz / 2.0 * (I * betas[k] - alpha / 2.0));
    for (int k = 0; k < Nt / 2; k++) {
        out[k] = tmp[Nt / 2 + k];
        out[Nt / 2 + k] = tmp[k];
    }
    free(tmp);
}

static int pass_sign(double z, double Cav) {
    /* propagation.c:378 */
    return ((int)(floor(z / Cav) + 1) % 2) * 2 - 1;
}

/* propagation.c:375-391.  As written the exponent is real (the i of the commented line
 * 389 is dropped, A12), the table stays in centred order while the linear step indexes
 * it in FFT order (A12), and the centre is the mean of the two middle entries (A23). */
void or_calcexpR(or_complex *expR, int n, int nwr, int *signmem, double z, double Cav,
                 double k0, double dzh, const double *wr, const or_switches *sw) {
    int signum = pass_sign(z, Cav);
    if (-*signmem == signum) *signmem = -*signmem;
    if (sw->bounce_lens) signum = 1;
    const double wc = sw->diffr_center ? wr[nwr / 2] : (wr[nwr / 2 - 1] + wr[nwr / 2]) / 2.0;
    for (int p = 0; p < n; p++) {
        /* position p of the table as the linear step indexes it */
        const int m = sw->diffr_fftorder ? (p + n / 2) % n : p;
        const double kap2 = pow(wr[m] - wc, 2);
        const double arg = signum * (-1.0 / (2.0 * k0) * dzh * (-1.0)) * kap2;
        if (sw->diffr_phase) expR[p] = cexp(I * arg);
        else expR[p] = exp(arg);
    }
}

/* propagation.c:65-108 (FFTW branch; A9: the index is j*Nx + i). */
void or_linearstep(or_complex *A, int Nx, int Ny, int Nt, const or_complex *expD0,
                   const or_complex *expRx, const or_complex *expRy) {
    const long NP = (long)Nx * Ny, N = NP * Nt;
    or_fft_axis(A, Nx, Ny, Nt, 2, -1);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < Nt; k++)
        for (long i = 0; i < NP; i++) A[k * NP + i] *= expD0[k];
    or_fft_axis(A, Nx, Ny, Nt, 2, +1);
    or_fft_axis(A, Nx, Ny, Nt, 1, -1);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < Nt; k++)
        for (long j = 0; j < Ny; j++)
            for (long i = 0; i < Nx; i++) A[k * NP + j * Nx + i] *= conj(expRy[j]);
    or_fft_axis(A, Nx, Ny, Nt, 1, +1);
    or_fft_axis(A, Nx, Ny, Nt, 0, -1);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < Nt; k++)
        for (long j = 0; j < Ny; j++)
            for (long i = 0; i < Nx; i++) A[k * NP + j * Nx + i] *= conj(expRx[i]);
    or_fft_axis(A, Nx, Ny, Nt, 0, +1);
    const double s = 1.0 / (double)N;
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N; q++) A[q] *= s;
}

/* propagation.c:164-177 (wbuff = fftshift(w)) and 215-233 (FFTW branch of the SST). */
void or_sst(const or_complex *A, int Nx, int Ny, int Nt, const double *w, double gamma2,
            double w0, or_complex *sst) {
    const long NP = (long)Nx * Ny, N = NP * Nt;
    double *wbuff = (double *)malloc(sizeof(double) * Nt);
    memcpy(wbuff, w, sizeof(double) * Nt);
    for (int k = 0; k < Nt / 2; k++) {
        wbuff[k] = w[Nt / 2 + k];
        wbuff[Nt / 2 + k] = w[k];
    }
    or_complex *dA = (or_complex *)malloc(sizeof(or_complex) * N);
    memcpy(dA, A, sizeof(or_complex) * N);
    or_fft_axis(dA, Nx, Ny, Nt, 2, -1);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < Nt; k++)
        for (long i = 0; i < NP; i++) dA[k * NP + i] = -1.0 * I * dA[k * NP + i] * wbuff[k];
    or_fft_axis(dA, Nx, Ny, Nt, 2, +1);
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N; q++) {
        const or_complex d = dA[q] / (double)Nt;
        sst[q] = gamma2 / w0 * (2.0 * d * conj(A[q]) + A[q] * conj(d));
    }
    free(dA);
    free(wbuff);
}

/* plasma.c:4-40 */
void or_ionizpot(const char *gas, double *I1, double *I2) {
    if (strcmp(gas, "Argon") == 0) { *I1 = 15.75962; *I2 = 27.62967; }
    if (strcmp(gas, "Helium") == 0) { *I1 = 24.58741; *I2 = 54.41778; }
    if (strcmp(gas, "Neon") == 0) { *I1 = 21.5646; *I2 = 40.96328; }
    if (strcmp(gas, "Air") == 0) {
        *I1 = 0.78084 * 14.53414 + 0.20946 * 13.61806 + 0.00934 * 15.75962;
        *I2 = 0.78084 * 29.6013 + 0.20946 * 35.11730 + 0.00934 * 27.62967;
    }
    if (strcmp(gas, "Nitrogen") == 0) { *I1 = 14.53414; *I2 = 29.6013; }
    if (strcmp(gas, "Xenon") == 0) { *I1 = 12.1298; *I2 = 21.20979; }
    if (strcmp(gas, "Krypton") == 0) { *I1 = 13.99961; *I2 = 24.35985; }
}

/* plasma.c:61-115.  Number density at 1 bar = density[g/m^3] * N_A / M[g/mol].  The
 * xenon molar mass 5.761 (plasma.c:103) is kept as written. */
void or_Natoms(const char *gas, double *Natm, double *sigm_coll) {
    if (strcmp(gas, "Argon") == 0) { *Natm = 1.784 * 1e3 * NAVO / 39.941; *sigm_coll = 1.57e-20; }
    if (strcmp(gas, "Helium") == 0) { *Natm = 0.166e3 * NAVO / 4.002602; *sigm_coll = 6.11e-20; }
    if (strcmp(gas, "Neon") == 0) { *Natm = 0.9002e3 * NAVO / 20.1797; *sigm_coll = 1.65e-20; }
    if (strcmp(gas, "Air") == 0) { *Natm = 1.205e3 * NAVO / 28.97; *sigm_coll = 10e-20; }
    if (strcmp(gas, "Nitrogen") == 0) { *Natm = 1.65e3 * NAVO / 14.0067; *sigm_coll = 10.2e-20; }
    if (strcmp(gas, "Xenon") == 0) { *Natm = 5.86e3 * NAVO / 5.761; *sigm_coll = 3.55e-20; }
    if (strcmp(gas, "Krypton") == 0) { *Natm = 3.749e3 * NAVO / 83.798; *sigm_coll = 1.15e-20; }
}

/* plasma.c:43-58 (A11: fabs on C_nl instead of an int abs) */
void or_ADK(double *rates1, double *rates2, long n, const double *C_nl, const double *f_lm,
            const double *nq, const double *mq, const double *Ei, const double *E) {
    const double Kon1 = pow(fabs(C_nl[0]), 2.0) * sqrt(6.0 / M_PI) * f_lm[0] * Ei[0];
    const double Kon2 = pow(fabs(C_nl[1]), 2.0) * sqrt(6.0 / M_PI) * f_lm[1] * Ei[1];
    const double Kon3 = 2.0 * pow(2.0 * Ei[0], 3.0 / 2.0);
    const double Kon4 = 2.0 * pow(2.0 * Ei[1], 3.0 / 2.0);
    const double Kon5 = 2.0 * nq[0] - mq[0] - 3.0 / 2.0;
    const double Kon6 = 2.0 * nq[1] - mq[1] - 3.0 / 2.0;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; i++) {
        rates1[i] = Kon1 * pow(Kon3 / E[i], Kon5) * exp(-Kon3 / (3.0 * E[i]));
        rates2[i] = Kon2 * pow(Kon4 / E[i], Kon6) * exp(-Kon4 / (3.0 * E[i]));
    }
}

/* Quantum numbers and prefactors, plasma.c:264-287 (A11). */
static void adk_consts(const char *gas, const or_switches *sw, double *I1, double *I2,
                       double Iion[2], double nq[2], double f_lm[2], double mq[2],
                       double C_nl[2]) {
    or_ionizpot(gas, I1, I2);
    Iion[0] = *I1 / IH;
    Iion[1] = *I2 / IH;
    double lq[2] = {0.0, 0.0};
    if (sw->ion_nq) {
        nq[0] = 1.0 / sqrt(2.0 * Iion[0]);
        nq[1] = 2.0 / sqrt(2.0 * Iion[1]);
    } else {
        /* as written nq[0] uses Iion[1]; nq[1] reads Iion[2], past the end of a 2-element
         * array, so that value is undefined and the corrected one is used instead */
        nq[0] = pow(2 * Iion[1], -0.5);
        nq[1] = 2.0 / sqrt(2.0 * Iion[1]);
    }
    f_lm[0] = f_lm[1] = 1.0;
    mq[0] = mq[1] = 0.0;
    C_nl[0] = sqrt(pow(2.0, 2.0 * nq[0]) *
                   pow(nq[0] * tgamma(nq[0] + lq[0] + 1.0) * tgamma(nq[0] - lq[0]), -1.0));
    const double e1 = sw->ion_nq ? 2.0 * nq[1] : nq[1];
    C_nl[1] = sqrt(pow(2.0, e1) *
                   pow(nq[1] * tgamma(nq[1] + lq[1] + 1.0) * tgamma(nq[1] - lq[1]), -1.0));
}

/* plasma.c:118-245, one (x,y) pencil at a time.  The per-point arithmetic is that of the
 * reference's whole-field loops; only the storage is per pencil. */
void or_ioniz(const or_complex *A, int Nx, int Ny, int Nt, double w0, double deltat,
              const char *gas, double rho_c, const double *w, double rho_nt, double n0,
              double *tau_c, double *fe_sp, const or_switches *sw) {
    const long NP = (long)Nx * Ny;
    const double Kon = deltat / T0;
    const double k0 = w0 / C0;
    double I1 = 0, I2 = 0, Iion[2], nq[2], f_lm[2], mq[2], C_nl[2];
    adk_consts(gas, sw, &I1, &I2, Iion, nq, f_lm, mq, C_nl);
    double Natm = 0, sigm_coll = 0;
    or_Natoms(gas, &Natm, &sigm_coll);
    const double K1 = 2.0 * pow(EL0, 2.0);
    const double K2 = 4.0 * pow(ME, 2.0);
    const double K3 = sigm_coll * rho_nt;
    const double K4 = k0 / (n0 * rho_c) * w0;
    const double K5 = pow(w0, 2);
    const double Kon1 = pow(fabs(C_nl[0]), 2.0) * sqrt(6.0 / M_PI) * f_lm[0] * Iion[0];
    const double Kon2 = pow(fabs(C_nl[1]), 2.0) * sqrt(6.0 / M_PI) * f_lm[1] * Iion[1];
    const double Kon3 = 2.0 * pow(2.0 * Iion[0], 3.0 / 2.0);
    const double Kon4 = 2.0 * pow(2.0 * Iion[1], 3.0 / 2.0);
    const double Kon5 = 2.0 * nq[0] - mq[0] - 3.0 / 2.0;
    const double Kon6 = 2.0 * nq[1] - mq[1] - 3.0 / 2.0;

#pragma omp parallel
    {
        double *W1 = (double *)malloc(sizeof(double) * Nt);
        double *W2 = (double *)malloc(sizeof(double) * Nt);
        double *Wava = (double *)malloc(sizeof(double) * Nt);
        double *sig = (double *)malloc(sizeof(double) * Nt);
        double *ions1 = (double *)malloc(sizeof(double) * (Nt + 1));
        double *ions2 = (double *)malloc(sizeof(double) * (Nt + 1));
#pragma omp for schedule(static)
        for (long i = 0; i < NP; i++) {
            for (int k = 0; k < Nt; k++) {
                const long q = (long)k * NP + i;
                double Ip = pow(cabs(A[q]), 2) * HBAR * w0;           /* :133-139 */
                if (Ip == 0) Ip = 1e-30;
                const double E0 = sqrt(2.0 * ZW0 * Ip / NC) * FCTR;   /* :145-149 */
                const double dat = fabs(E0) / EF;
                double r1 = Kon1 * pow(Kon3 / dat, Kon5) * exp(-Kon3 / (3.0 * dat));
                double r2 = Kon2 * pow(Kon4 / dat, Kon6) * exp(-Kon4 / (3.0 * dat));
                if (isnan(r1)) r1 = 0.0;                               /* :184-192 */
                if (isnan(r2)) r2 = 0.0;
                const double wk = sw->ve_omega0 ? 0.0 : w[k];          /* A18 */
                const double ve = sqrt(K1 * pow(E0, 2.0) / (K2 * pow(wk + w0, 2.0)));
                const double tc = 1.0 / (K3 * ve);                     /* :203-213 */
                /* A27: when ve underflows to 0, tau_c = inf and the formula gives inf/inf;
                 * its limit is 0 */
                const double sg = (sw->sigma_limit && isinf(tc)) ? 0.0 : K4 * tc / (1.0 + K5 * pow(tc, 2.0));
                tau_c[q] = tc;
                sig[k] = sg;
                Wava[k] = sg * Ip / I1;
                W1[k] = r1;
                W2[k] = r2;
            }
            for (int k = 0; k <= Nt; k++) ions1[k] = ions2[k] = 0.0;
            double R = 0.0;
            /* :223-231.  As written k runs down from Nt-1 and reads ions[k] before it is
             * written (A15); corrected it runs up. */
            for (int s = 0; s < Nt; s++) {
                const int k = sw->ion_forward ? s : Nt - 1 - s;
                R = R + W1[k] * Kon;
                R = R + (1.0 - R) * Wava[k] * Kon;
                ions1[k + 1] = 1.0 - exp(-R) - ions2[k];
                ions2[k + 1] = ions2[k] + W2[k] * Kon * ions1[k];
            }
            for (int k = 0; k < Nt; k++)                                /* :238-241 */
                fe_sp[(long)k * NP + i] = (ions1[k] * 1.0 + ions2[k] * 2.0) * sig[k];
        }
        free(W1); free(W2); free(Wava); free(sig); free(ions1); free(ions2);
    }
}

/* propagation.c:460-504, with the serial meaning of its (racy) parallel loops. */
void or_calc1oes(const double *BP, int n, const double *r, double *vald1oes, double *y) {
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
    *vald1oes = -r[posi1] + r[posi2];
    y[0] = r[posi1];
    y[1] = r[posi2];
    y[2] = BP[posi1];
    y[3] = BP[posi2];
}

void or_beam_profiles(const or_complex *A, int Nx, int Ny, int Nt, double *BP1, double *BP2) {
    const long NP = (long)Nx * Ny;
    memset(BP1, 0, sizeof(double) * Nx);
    memset(BP2, 0, sizeof(double) * Ny);
    for (long k = 0; k < Nt; k++)
        for (long j = 0; j < Ny; j++)
            for (long i = 0; i < Nx; i++) {
                const double a = pow(cabs(A[k * NP + j * Nx + i]), 2.0);
                BP1[i] += a;
                BP2[j] += a;
            }
}

/* propagation.c:111-372 */
void or_ssfmprop(or_complex *A, const or_params *p, double dzz, int *signmem, double z,
                 double *puls_e, double *BP1, double *BP2, double *y1, double *y2,
                 double *bps1, double *bps2, int change, const or_switches *sw) {
    const int Nx = p->Nx, Ny = p->Ny, Nt = p->Nt;
    const long NP = (long)Nx * Ny, N = NP * Nt;
    or_complex *expD0 = (or_complex *)malloc(sizeof(or_complex) * Nt);
    or_complex *expRx = (or_complex *)malloc(sizeof(or_complex) * Nx);
    or_complex *expRy = (or_complex *)malloc(sizeof(or_complex) * Ny);
    or_expD0(expD0, Nt, dzz, p->alpha, p->betas);
    or_calcexpR(expRx, Nx, Ny, signmem, z, p->Cav, p->k0, dzz / 2, p->wr, sw);
    or_calcexpR(expRy, Ny, Ny, signmem, z, p->Cav, p->k0, dzz / 2, p->wr, sw);
    or_linearstep(A, Nx, Ny, Nt, expD0, expRx, expRy);

    or_complex *buffer = (or_complex *)calloc(N, sizeof(or_complex));
    if (p->sst_on == 1) or_sst(A, Nx, Ny, Nt, p->w, p->gamma2, p->w0, buffer);

    or_complex *A_nl = (or_complex *)malloc(sizeof(or_complex) * N);
    if (p->plasm == 1) {
        double *tau_c = (double *)malloc(sizeof(double) * N);
        double *fe = (double *)malloc(sizeof(double) * N);
        or_ioniz(A, Nx, Ny, Nt, p->w0, p->deltat, p->gas, p->rho_c, p->w, p->rho_nt, p->n0,
                 tau_c, fe, sw);
#pragma omp parallel for schedule(static)
        for (long q = 0; q < N; q++) {                       /* :283-293 (A13) */
            const double z1 = p->gamma2 * pow(cabs(A[q]), 2.0);
            const double pl = p->rho_nt * fe[q] / 2.0;
            const double z2y = sw->plasma_imag ? p->w0 * tau_c[q] * pl
                                               : (1.0 + p->w0 * tau_c[q]) * pl;
            A_nl[q] = (0.0 - creal(buffer[q]) - pl) + I * (z1 - cimag(buffer[q]) - z2y);
        }
        free(tau_c);
        free(fe);
    } else {
#pragma omp parallel for schedule(static)
        for (long q = 0; q < N; q++) {                       /* :303-309 */
            const double tempab = pow(cabs(A[q]), 2.0);
            A_nl[q] = -creal(buffer[q]) + I * (p->gamma2 * tempab - cimag(buffer[q]));
        }
    }
#pragma omp parallel for schedule(static)
    for (long q = 0; q < N; q++) {                           /* :317-327 (A14) */
        const double er = exp(dzz * creal(A_nl[q]));
        const double ei = dzz * cimag(A_nl[q]);
        const double c = cos(ei), s = sin(ei);
        double x = creal(A[q]), y = cimag(A[q]);
        if (sw->nl_apply) {
            const double nx = x * er * c - y * er * s;
            const double ny = y * er * c + x * er * s;
            x = nx;
            y = ny;
        } else {
            x = x * er * c - y * er * s;
            y = y * er * s + x * er * c;
        }
        A[q] = x + I * y;
    }
    free(A_nl);
    free(buffer);

    or_linearstep(A, Nx, Ny, Nt, expD0, expRx, expRy);

    if (change == 1) {                                       /* :334-341 */
        const int signum = pass_sign(z, p->Cav);
        if (*signmem == -signum) {
            *puls_e = *puls_e * p->Ab_M;
            *signmem *= -1;
        }
        or_beam_profiles(A, Nx, Ny, Nt, BP1, BP2);           /* :343-361 */
        or_calc1oes(BP1, Nx, p->r, bps1, y1);
        or_calc1oes(BP2, Ny, p->r, bps2, y2);
    }
    free(expD0);
    free(expRx);
    free(expRy);
}

/* propagation.c:636-676: the dz update for a local error err. */
void or_step_rule(double err, double *dzz, double def_err, double dzmin, const double *y1,
                  const double *y2, int *bad) {
    double ujdz;
    *bad = 0;
    const double err_fact = pow(2.0, (1.0 / 3.0));
    if (err > 2.0 * def_err) {
        ujdz = *dzz / 2.0;
        if (ujdz > dzmin) {
            *dzz = ujdz;
            *bad = 1;
            return;
        }
    } else if (err > def_err && err < 2.0 * def_err) {
        ujdz = *dzz / err_fact;
        if (ujdz > dzmin) *dzz = ujdz;
    } else if (err > 0.5 * def_err && err <= def_err) {
        /* keep */
    } else {
        ujdz = *dzz * err_fact;
        if (!(ujdz > 100 * (y2[1] + y1[1]) / 2.0)) *dzz = ujdz;
    }
}

/* propagation.c:616-677 (printing dropped): the error sums (:624-633), then the rule. */
void or_setStep(long n, double *dzz, const or_complex *C1, const or_complex *C2,
                double def_err, double dzmin, const double *y1, const double *y2, int *bad,
                double *err) {
    double sum1 = 0, sum2 = 0;
    for (long i = 0; i < n; i++) {
        const or_complex CC = C2[i] - C1[i];
        sum1 += pow(cabs(CC), 2);
        sum2 += pow(cabs(C2[i]), 2);
    }
    *err = sqrt(sum1) / sqrt(sum2);
    or_step_rule(*err, dzz, def_err, dzmin, y1, y2, bad);
}

/* MPC.c:389-449 (GPU branch: intensity sums; the spectrum stays in FFT order). */
void or_diag(const or_complex *A, int Nx, int Ny, int Nt, double *temp, double *spec) {
    const long NP = (long)Nx * Ny, N = NP * Nt;
    for (long k = 0; k < Nt; k++) {
        double s = 0;
        for (long i = 0; i < NP; i++) {
            const or_complex a = A[k * NP + i];
            s += creal(a) * creal(a) + cimag(a) * cimag(a);
        }
        temp[k] = s;
    }
    or_complex *C = (or_complex *)malloc(sizeof(or_complex) * N);
    memcpy(C, A, sizeof(or_complex) * N);
    or_fft_axis(C, Nx, Ny, Nt, 2, -1);
    for (long k = 0; k < Nt; k++) {
        double s = 0;
        for (long i = 0; i < NP; i++) {
            const or_complex a = C[k * NP + i];
            s += creal(a) * creal(a) + cimag(a) * cimag(a);
        }
        spec[k] = s;
    }
    free(C);
}

/* MPC.c:206-216 (A17: both parts scaled) */
void or_calibrate(or_complex *A, long n, double puls_e, double Esig, const or_switches *sw) {
    const double Ksn = sqrt(puls_e / Esig);
    for (long i = 0; i < n; i++) {
        if (sw->energy_both) A[i] *= Ksn;
        else A[i] = Ksn * creal(A[i]) + I * cimag(A[i]);
    }
}

void or_mirror_lens(or_complex *A, int Nx, int Ny, int Nt, const double *r, double k0,
                    double roc) {
    const long NP = (long)Nx * Ny;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < Nt; k++)
        for (long j = 0; j < Ny; j++)
            for (long i = 0; i < Nx; i++) {
                const double r2 = r[i] * r[i] + r[j] * r[j];
                A[k * NP + j * Nx + i] *= cexp(-I * k0 * r2 / roc);
            }
}

/* Number of mirror planes (multiples of Cav) crossed going from z0 to z1. */
static int bounces_between(double z0, double z1, double Cav) {
    const double eps = 1e-9;
    return (int)(floor(z1 / Cav + eps) - floor(z0 / Cav + eps));
}

void or_run_fixed(or_complex *A, const or_params *p, or_state *st, int nsteps,
                  const or_switches *sw) {
    for (int s = 0; s < nsteps; s++) {
        /* the pass index is taken from the step count so that z = s*dz lands on the
         * mirror planes exactly */
        const double zs = (double)st->nstep * st->dzz;
        /* a relative 1e-9 nudge keeps floor(z/Cav) exact when z = s*dz rounds below a plane */
        or_ssfmprop(A, p, st->dzz, &st->signmem, zs + 1e-9 * p->Cav, &st->puls_e, NULL, NULL,
                    NULL, NULL, NULL, NULL, 0, sw);
        st->nstep++;
        st->z = (double)st->nstep * st->dzz;
        const int nb = bounces_between(zs, st->z, p->Cav);
        if (nb > 0) {
            if (sw->bounce_lens)
                for (int b = 0; b < nb; b++) or_mirror_lens(A, p->Nx, p->Ny, p->Nt, p->r, p->k0, p->roc);
            if (sw->mirror_loss)
                for (int b = 0; b < nb; b++) st->puls_e *= p->Ab_M;
        }
    }
}

void or_double_step(or_complex *A, or_complex *C1, or_complex *C2,
                    const or_params *p, or_state *st, const or_switches *sw) {
    const long N = (long)p->Nx * p->Ny * p->Nt;
    double *BP1 = (double *)malloc(sizeof(double) * p->Nx);
    double *BP2 = (double *)malloc(sizeof(double) * p->Ny);
    memcpy(C1, A, sizeof(or_complex) * N);
    memcpy(C2, A, sizeof(or_complex) * N);
    const double dz_used = st->dzz;
    or_ssfmprop(C1, p, 2 * dz_used, &st->signmem, st->z, &st->puls_e, BP1, BP2, st->y1, st->y2,
                &st->bps1, &st->bps2, 0, sw);
    or_ssfmprop(C2, p, dz_used, &st->signmem, st->z, &st->puls_e, BP1, BP2, st->y1, st->y2,
                &st->bps1, &st->bps2, 0, sw);
    or_ssfmprop(C2, p, dz_used, &st->signmem, st->z, &st->puls_e, BP1, BP2, st->y1, st->y2,
                &st->bps1, &st->bps2, 1, sw);
    st->attempts++;
    or_setStep(N, &st->dzz, C1, C2, p->def_err, p->dzmin, st->y1, st->y2, &st->bad, &st->err);
    if (st->bad == 0) {
        for (long i = 0; i < N; i++) A[i] = (4.0 / 3.0) * C2[i] - (1.0 / 3.0) * C1[i];
        const double z0 = st->z;
        /* A26: the reference advances z by twice the step size chosen for the NEXT step
         * (MPC.c:352,383); corrected it advances by the step just taken. */
        st->z = st->z + 2.0 * (sw->z_advance_used ? dz_used : st->dzz);
        const int nb = bounces_between(z0, st->z, p->Cav);
        if (nb > 0) {
            if (sw->bounce_lens)
                for (int b = 0; b < nb; b++) or_mirror_lens(A, p->Nx, p->Ny, p->Nt, p->r, p->k0, p->roc);
            if (sw->mirror_loss)
                for (int b = 0; b < nb; b++) st->puls_e *= p->Ab_M;
        }
        if (st->z > p->dist) st->z = p->dist;
        st->nstep++;
    }
    free(BP1);
    free(BP2);
}
