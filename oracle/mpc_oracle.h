/*
 * mpc_oracle.h -- FP64 CPU restatement of the kmecseki/MPC split-step propagator.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle: tests, the smoke check and the
 * bench's cpu_baseline / reference arm may call it, as the checker.  The product
 * (mpc_gb300/, include/mpc_gpu.h) never links, imports or runs it.
 *
 * Parity status: the reference ships no tests, fixtures or golden vectors, and its
 * full propagator cannot be built (invalid Makefile, FFTW and MPI absent).  The pieces
 * of plasma.c / propagation.c that compile on their own (ADK, ionizpot, Natoms,
 * ioniz as written, calcexpR as written, calc1oes, setStep) are compiled from the
 * reference sources into oracle/_ref by oracle/build_ref.sh and pin this file's
 * restatement of them (tests/golden/ holds the vectors).  The FFT/linear step is
 * pinned against numpy.fft, the whole step against analytic known answers.
 *
 * Field layout everywhere: A[k*Nx*Ny + j*Nx + i], i = x (fastest), j = y, k = t
 * (kernels.cu:74,79; propagation.c:514-536).  Complex values are C99 double complex
 * (layout of cufftDoubleComplex / numpy complex128).
 */
#ifndef MPC_ORACLE_H
#define MPC_ORACLE_H
/* C99 double complex in C; the layout-identical std::complex<double> when the header is
 * included from C++ (the FP64 GPU oracle, mpc_oracle64.cu) */
#ifdef __cplusplus
#include <complex>
typedef std::complex<double> or_complex;
extern "C" {
#else
#include <complex.h>
typedef double complex or_complex;
#endif

/* Run parameters in the order of param.bin (MPC.c:77,180-203) plus the mirror
 * radius of curvature, which the reference does not have (lens bounce mode). */
typedef struct {
    int Nx, Ny, Nt;
    double dist, dzz;
    const double *betas;  /* Nt, centred omega order */
    double alpha, Cav, k0;
    const double *wr;     /* Ny, centred k grid (also used for x, as the reference does) */
    int sst_on;
    const double *w;      /* Nt, centred omega grid */
    double gamma2, w0;
    int plasm;
    double deltat, rho_c, rho_nt, n0, puls_e, Ab_M;
    const double *r;      /* Ny, transverse positions */
    double dr, def_err, dzmin, Esig;
    char gas[16];
    double roc;           /* mirror radius of curvature (lens bounce mode only) */
} or_params;

/* One switch per reference defect that changes numbers.  1 = corrected (default),
 * 0 = as written.  A<n> numbers the defect; the comment states it. */
typedef struct {
    int diffr_phase;    /* A12: i restored in the diffraction exponent (propagation.c:386-389) */
    int diffr_fftorder; /* A12: diffraction table reordered to FFT order */
    int diffr_center;   /* A23: centre wc = wr[N/2] (zero of the FFT grid) instead of mean of middle two */
    int plasma_imag;    /* A13: (1 + i w0 tau_c) instead of (1 + w0 tau_c) in the imaginary part */
    int nl_apply;       /* A14: correct complex product A*exp(dz*A_nl) */
    int ion_forward;    /* A15: ionization prefix runs forward in t */
    int ion_nq;         /* A11: n*_q = q/sqrt(2 Ip_q), C_nl with 2^(2n*) */
    int ve_omega0;      /* A18: drift velocity uses w0 only */
    int energy_both;    /* A17: energy calibration scales both parts */
    int mirror_loss;    /* A24: mirror loss bookkeeping fires on the pass change */
    int z_advance_used; /* A26: z advances by the step just taken, not the next one */
    int sigma_limit;    /* A27: sigma = 0 when tau_c overflows (as written inf/inf = NaN) */
    int bounce_lens;    /* bounce mode: 0 = diffraction sign flip (reference), 1 = mirror lens phase */
} or_switches;

void or_default_switches(or_switches *sw);
void or_set_threads(int n);

/* Unnormalised strided 1-D FFTs along one axis of the 3-D field.
 * axis 0 = x, 1 = y, 2 = t; sign -1 = forward (exp(-i..)), +1 = inverse. */
void or_fft_axis(or_complex *A, int Nx, int Ny, int Nt, int axis, int sign);

/* exp(dzz/2*(i*betas - alpha/2)) then fftshift (kernels.cu:47-54, propagation.c:150-156,393-402). */
void or_expD0(or_complex *out, int Nt, double dzz, double alpha, const double *betas);

/* Diffraction table and sign update (propagation.c:375-391).  n = table length,
 * nwr = length of wr (Ny).  dzh is the half step (the caller passes dzz/2). */
void or_calcexpR(or_complex *expR, int n, int nwr, int *signmem, double z, double Cav,
                 double k0, double dzh, const double *wr, const or_switches *sw);

/* Linear step (propagation.c:65-108, FFTW ordering with the A9 index fix). */
void or_linearstep(or_complex *A, int Nx, int Ny, int Nt, const or_complex *expD0,
                   const or_complex *expRx, const or_complex *expRy);

/* Self-steepening term sst = gamma2/w0*(2 dA A* + A dA*), dA = IFFT_t[-i w FFT_t A]/Nt
 * (propagation.c:164-233). */
void or_sst(const or_complex *A, int Nx, int Ny, int Nt, const double *w, double gamma2,
            double w0, or_complex *sst);

void or_ionizpot(const char *gas, double *I1, double *I2);            /* plasma.c:4-40 */
void or_Natoms(const char *gas, double *Natm, double *sigm_coll);     /* plasma.c:61-115 */
void or_ADK(double *rates1, double *rates2, long n, const double *C_nl, const double *f_lm,
            const double *nq, const double *mq, const double *Ei, const double *E); /* plasma.c:43-58 */
/* Ionization (plasma.c:118-245): outputs tau_c and freeelectrons_sp, N values each. */
void or_ioniz(const or_complex *A, int Nx, int Ny, int Nt, double w0, double deltat,
              const char *gas, double rho_c, const double *w, double rho_nt, double n0,
              double *tau_c, double *fe_sp, const or_switches *sw);

/* 1/e^2 beam size (propagation.c:460-504). */
void or_calc1oes(const double *BP, int n, const double *r, double *vald1oes, double *y);

/* Beam profiles BP1[x] = sum_{y,t}|A|^2, BP2[y] = sum_{x,t}|A|^2 (propagation.c:343-354). */
void or_beam_profiles(const or_complex *A, int Nx, int Ny, int Nt, double *BP1, double *BP2);

/* One symmetric split step (propagation.c:111-372). */
void or_ssfmprop(or_complex *A, const or_params *p, double dzz, int *signmem, double z,
                 double *puls_e, double *BP1, double *BP2, double *y1, double *y2,
                 double *bps1, double *bps2, int change, const or_switches *sw);

/* The dz rule of setStep (propagation.c:636-676) for a given local error err: writes dzz
 * and bad.  y1, y2 are the beam-size records of calc1oes (y[1] caps the growth of dz). */
void or_step_rule(double err, double *dzz, double def_err, double dzmin, const double *y1,
                  const double *y2, int *bad);

/* Step-size control (propagation.c:616-677).  Returns nothing; writes dzz, bad, err. */
void or_setStep(long n, double *dzz, const or_complex *C1, const or_complex *C2,
                double def_err, double dzmin, const double *y1, const double *y2, int *bad,
                double *err);

/* temp[k] = sum_xy |A|^2, spec[k] = sum_xy |FFT_t A|^2 in FFT order (MPC.c:389-449). */
void or_diag(const or_complex *A, int Nx, int Ny, int Nt, double *temp, double *spec);

/* Energy calibration (MPC.c:206-216): A *= sqrt(puls_e/Esig). */
void or_calibrate(or_complex *A, long n, double puls_e, double Esig, const or_switches *sw);

/* Mirror lens phase exp(-i k0 (x^2+y^2)/roc) with x = r[i], y = r[j] (lens bounce mode). */
void or_mirror_lens(or_complex *A, int Nx, int Ny, int Nt, const double *r, double k0,
                    double roc);

/* Driver state carried between steps (MPC.c:234-238). */
typedef struct {
    double z, dzz, err, puls_e, bps1, bps2;
    int signmem, bad, nstep, attempts;
    double y1[4], y2[4];
} or_state;

/* Fixed-step run: nsteps calls of ssfmprop(dzz), z advancing by dzz each; in lens
 * mode the mirror phase is applied after each step that ends on a pass boundary. */
void or_run_fixed(or_complex *A, const or_params *p, or_state *st, int nsteps,
                  const or_switches *sw);

/* One step-doubling attempt (MPC.c:269-383 with the A4 fix: C1 = C2 = A first).
 * C1, C2 are N-sized work buffers.  On accept A = (4 C2 - C1)/3, z += 2 dzz. */
void or_double_step(or_complex *A, or_complex *C1, or_complex *C2,
                    const or_params *p, or_state *st, const or_switches *sw);

#ifdef __cplusplus
}
#endif
#endif
