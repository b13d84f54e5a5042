/*
 * mpc_gpu.h -- C ABI of the GB300 split-step propagator (libmpc_gpu.so).
 *
 * Drop-in boundary for the hot path of kmecseki/MPC: the entry points below replace the
 * C functions declared in the reference's propagation.h and plasma.h, with the same
 * argument meaning.  Differences, all deliberate:
 *   - the six FFT plan handles of createPlans become one opaque context (mpc_ctx);
 *   - every call returns an int status (MPC_OK = 0) and never exits the process;
 *   - the physics is the reference's with its numerical defects corrected;
 *   - a device-resident field API (mpc_field_*, mpc_run_*) avoids the per-step host copies
 *     the reference makes.
 * Field layout everywhere: A[k*Nx*Ny + j*Nx + i] (i = x fastest, k = t slowest), complex128
 * as interleaved doubles (the layout of cufftDoubleComplex), physical units as in MPC.c.
 * One CUDA stream per context; a context is used from one host thread at a time.
 */
#ifndef MPC_GPU_H
#define MPC_GPU_H
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MPC_OK = 0,
    MPC_ERR_ARG = 1,        /* null pointer or invalid value */
    MPC_ERR_SHAPE = 2,      /* grid shape not compiled into this library */
    MPC_ERR_CUDA = 3,       /* a CUDA runtime call failed (mpc_last_error has the text) */
    MPC_ERR_NOMEM = 4,      /* device allocation failed */
    MPC_ERR_NONFINITE = 5,  /* the field became NaN/Inf */
    MPC_ERR_STATE = 6,      /* call out of order (e.g. no field uploaded) */
    MPC_ERR_IO = 7,         /* file could not be read/written */
    MPC_ERR_UNSUPPORTED = 8, /* option not implemented on the device path */
    MPC_ERR_TIMEOUT = 9     /* a bounded device-side wait ran out; the kernel stopped early */
};

enum { MPC_BOUNCE_SIGNFLIP = 0, MPC_BOUNCE_LENS = 1 };

/* Run parameters: the param.bin record in the order MPC.c:77,180-203 reads it, plus
 * the mirror model (the reference only has the diffraction sign flip). */
typedef struct {
    int dims[3];            /* Nx, Ny, Nt */
    double dist, dzz;
    const double *betas;    /* Nt, propagation constant beta(omega) - beta0 - beta1*omega, centred omega order */
    double alpha, Cav, k0;
    const double *wr;       /* Ny, centred transverse wavenumber grid (used for x and y) */
    int sst_on;
    const double *w;        /* Nt, centred angular-frequency offset grid */
    double gamma2, w0;
    int plasm;
    double deltat, rho_c, rho_nt, n0, puls_e, Ab_M;
    const double *r;        /* Ny, transverse positions */
    double dr, def_err, dzmin, Esig;
    char gas[9];
    int bounce_mode;        /* MPC_BOUNCE_SIGNFLIP (reference) or MPC_BOUNCE_LENS */
    double roc;             /* mirror radius of curvature [m], lens mode */
    int variant;            /* compiled kernel variant of this grid (layout and launch shapes; all
                               give the same results): 0 = default, k = the k-th, -1 = the
                               fastest, timed when the context is created */
    int land_mirrors;       /* step doubling: 0 = as the reference, a bounce is applied after the
                               attempt that crosses a mirror plane; 1 = an attempt that would cross
                               the next plane is shortened to end on it */
} mpc_params;

typedef struct mpc_ctx mpc_ctx;

/* Library version string and the text of the last error on this thread. */
const char *mpc_version(void);
const char *mpc_last_error(void);
/* 1 if kernels for this grid are compiled in. */
int mpc_shape_supported(int Nx, int Ny, int Nt);

/* Replaces createPlans (propagation.c:508-613): builds twiddle, frequency and phase tables
 * and the device buffers for this grid.  The parameter arrays are copied. */
int mpc_create(mpc_ctx **ctx, const mpc_params *p);
int mpc_destroy(mpc_ctx *ctx);

/* One symmetric split step L(dzz/2) N(dzz) L(dzz/2) on a host complex128 field, in place
 * (propagation.c:111-372, ssfmprop).  signmem, puls_e, BP1 (Nx), BP2 (Ny), y1[4], y2[4],
 * bps1, bps2 are updated as the reference updates them; the beam diagnostics (BP1, BP2,
 * y1, y2, bps1, bps2) only when change == 1. */
int mpc_ssfmprop(mpc_ctx *ctx, double *A, int sst_on, double dzz, int *signmem, double z,
                 double *puls_e, double *BP1, double *BP2, double *y1, double *y2,
                 double *bps1, double *bps2, int change);

/* Linear step on a host complex128 field with caller tables (propagation.c:3-108):
 * exp_D0[Nt] in FFT order (after fftshift), expR[Nx] in the order the corrected
 * calcexpR returns it (FFT order), applied as conj(expR) along y and x. */
int mpc_linearstep(mpc_ctx *ctx, double *A, const double *exp_D0, const double *expR);

/* Diffraction table (propagation.c:375-391, corrected: imaginary exponent, FFT order,
 * centre wr[N/2]) into expR[Nx] (complex128); updates *signmem like the reference. */
int mpc_calcexpR(mpc_ctx *ctx, double *expR, int *signmem, double z, double dzz);

/* Ionization (plasma.c:118-245, corrected): tau_c[N] and freeelectrons_sp[N] (FP64) for a
 * host complex128 field, computed on the device. */
int mpc_ioniz(mpc_ctx *ctx, const double *A, double *tau_c, double *freeelectrons_sp);

/* ADK rates (plasma.c:43-58) of both ionization stages for n field values E (atomic units),
 * corrected constants of plasma.c:264-287 for the context's gas, computed on the device. */
int mpc_ADK(mpc_ctx *ctx, long n, const double *E, double *rates1, double *rates2);

/* 1/e^2 beam size from a beam profile BP[n] and positions r[n] (propagation.c:460-504):
 * *vald1oes = r[p2] - r[p1], y = {r[p1], r[p2], BP[p1], BP[p2]}.  Host scalar search. */
int mpc_calc1oes(const double *BP, int n, const double *r, double *vald1oes, double *y);

/* Step-size control (propagation.c:616-677): err = |C2-C1|/|C2| reduced on the device,
 * then the reference's dz rule.  C1, C2 host complex128 fields. */
int mpc_setStep(mpc_ctx *ctx, double *dzz, const double *C1, const double *C2,
                const double *y1, const double *y2, int *bad, double *err);

/* ---- device-resident field (the fast path) ---------------------------------------- */
/* Upload / download a host complex128 field (physical units); upload optionally applies
 * the energy calibration of MPC.c:206-216 (both parts scaled). */
int mpc_field_upload(mpc_ctx *ctx, const double *A, int calibrate);
int mpc_field_download(mpc_ctx *ctx, double *A);

/* Run state of the device-resident loop (MPC.c:234-238). */
typedef struct {
    double z, dzz, err, puls_e, bps1, bps2;
    int signmem, bad, nstep, attempts;
    double y1[4], y2[4];
} mpc_state;
int mpc_get_state(mpc_ctx *ctx, mpc_state *st);
int mpc_set_state(mpc_ctx *ctx, const mpc_state *st);

/* nsteps fixed split steps of length state.dzz on the device-resident field, merging the
 * half linear steps of consecutive steps; mirror bounces (lens phase or diffraction sign
 * flip) at every multiple of Cav.  Updates state.z, nstep, puls_e. */
int mpc_run_fixed(mpc_ctx *ctx, int nsteps);

/* One attempt of the reference's adaptive step (the body of the MPC.c:269-383 loop, with
 * the defects corrected) on the device-resident field: C1 = one split step of 2*dzz and
 * C2 = two split steps of dzz from the same field, the diffraction sign taken from state.z
 * for all three (calcexpR, propagation.c:375-391); err = |C2 - C1| / |C2| reduced on the
 * device in FP64, and setStep's rule (propagation.c:616-677) picks the next state.dzz.
 * Accepted (*bad = 0): the field becomes (4 C2 - C1) / 3, state.z advances by 2*dzz (the step
 * just taken), each mirror plane crossed applies a bounce (the lens phase in lens mode, the
 * mirror loss Ab_M on puls_e), nstep += 1.  Rejected (*bad = 1): the field is unchanged and
 * state.dzz halved.  BP1 (Nx) and BP2 (Ny) receive C2's beam profiles (NULL to skip); state
 * y1, y2, bps1, bps2 are updated from them; attempts += 1. */
int mpc_step_double(mpc_ctx *ctx, double *BP1, double *BP2, int *bad, double *err);

/* One split step L(dzz/2) N(dzz) L(dzz/2) of any length on the device-resident field at
 * state.z (the device form of ssfmprop, propagation.c:111-372, with the diffraction sign of
 * calcexpR): state.z += dzz, mirror planes crossed apply a bounce as in mpc_step_double. */
int mpc_step(mpc_ctx *ctx, double dzz);

/* ---- learned step-size control (no counterpart in the reference) -------------------- */
/* Running maxima over the split steps since the last reset: {peak intensity [W/m^2], peak
 * ionization fraction, peak nonlinear phase rate |Im A_nl| [rad/m], peak amplitude rate
 * |Re A_nl| [1/m]}, gathered inside the pencil sweep; reset != 0 restarts them. */
int mpc_step_stats(mpc_ctx *ctx, float out[4], int reset);
#define MPC_NFEATURES 16
/* The step-size controller's 16 features of the device field and state (one reduction pass
 * over the field plus the step statistics): log10 peak intensity, log10 peak ionization, log10
 * phase rate, log10 amplitude rate, log10 energy, spectral rms width and centroid shift (% of
 * w0), beam rms widths x, y (/ window), log10(dzz/Cav), position within the pass, log10 field
 * peakiness, log10 density - 25, log10 phase per step at dzz, plasma flag, self-steepening flag. */
int mpc_features(mpc_ctx *ctx, float f[MPC_NFEATURES]);

/* The network of the learned controller: 16 features -> 64 -> 64 -> 1 (SiLU), predicting
 * log(dz / Cav) of the next step.  Weights are MPC_MLP_NWEIGHTS floats packed as W1[64][16],
 * b1[64], W2[64][64], b2[64], W3[64], b3; inputs are normalised as (x - mean) / std and the
 * output de-normalised as y_mean + y_std * out.  Training and inference run in this
 * library's own kernels on the GPU (minibatch Adam on the mean squared error in normalised
 * units).  Host arrays throughout: X is n x 16 row-major, y has n entries. */
#define MPC_MLP_NWEIGHTS 5313
typedef struct mpc_mlp mpc_mlp;
int mpc_mlp_num_weights(void);
int mpc_mlp_create(mpc_mlp **mlp, unsigned long long seed);   /* uniform(+-1/sqrt(fan_in)) init */
int mpc_mlp_destroy(mpc_mlp *mlp);
int mpc_mlp_set_normalization(mpc_mlp *mlp, const float mean[MPC_NFEATURES], const float stdv[MPC_NFEATURES],
                              float y_mean, float y_std);
/* out = {mean[16], std[16], y_mean, y_std} */
int mpc_mlp_get_normalization(mpc_mlp *mlp, float out[2 * MPC_NFEATURES + 2]);
int mpc_mlp_get_weights(mpc_mlp *mlp, float *w);
int mpc_mlp_set_weights(mpc_mlp *mlp, const float *w);      /* also restarts Adam */
/* Mean squared error (normalised units) over all n samples and its gradient w.r.t. the weights. */
int mpc_mlp_loss_grad(mpc_mlp *mlp, const float *X, const float *y, int n, float *grad, float *loss);
/* epochs of minibatch Adam (lr, beta 0.9 / 0.999), a Fisher-Yates shuffle per epoch from seed;
 * final_loss = the last epoch's mean loss. */
int mpc_mlp_train(mpc_mlp *mlp, const float *X, const float *y, int n, int epochs, int batch, float lr,
                  unsigned long long seed, float *final_loss);
int mpc_mlp_predict(mpc_mlp *mlp, const float *X, int n, float *y);
/* One sample, without allocating (the controller's per-step call). */
int mpc_mlp_predict1(mpc_mlp *mlp, const float x[MPC_NFEATURES], float *y);

/* The learned controller (run to state.z = dist): plain split steps (mpc_step's arithmetic) of
 * dz = safety * Cav * exp(network(features)), capped at twice the previous step, quantised
 * down to 16 steps per octave of Cav and shortened to land on the next mirror plane; the run
 * opens with one step-doubling attempt, and every check_every steps the step is taken as a
 * step-doubling attempt instead, whose error checks the network: above def_err, the next
 * fallback_len accepted steps are plain step doubling (mpc_step_double) before the network is
 * used again.  Consecutive plain steps share one plane sweep (the second linear half step of one
 * and the first of the next, as mpc_run_fixed does). */
typedef struct {
    int steps;              /* plain steps at the network's dz */
    int checks;             /* periodic step-doubling checks */
    int check_failures;     /* checks whose error exceeded def_err (each starts a fallback) */
    int fallback_attempts;  /* step-doubling attempts outside the checks */
    long executed_steps;    /* split steps executed (3 per step-doubling attempt) */
    double dz_min, dz_max;  /* range of the network's steps [m] */
} mpc_learned_stats;
int mpc_run_learned(mpc_ctx *ctx, mpc_mlp *mlp, double safety, int check_every, int fallback_len,
                    mpc_learned_stats *out);
/* As mpc_run_learned, with one prediction (feature pass, network call) held for `hold`
 * consecutive plain steps (no counterpart in the reference; mpc_run_learned is hold = 1). */
int mpc_run_learned_hold(mpc_ctx *ctx, mpc_mlp *mlp, double safety, int check_every, int fallback_len, int hold,
                         mpc_learned_stats *out);

/* One mirror bounce of the device-resident field, now: MPC_BOUNCE_LENS multiplies it by the
 * mirror's focusing phase exp(-i k0 (x^2 + y^2) / roc); MPC_BOUNCE_SIGNFLIP flips
 * state.signmem, the reference's bookkeeping of a bounce (propagation.c:334-341; the
 * diffraction sign of later steps follows from z).  Either way state.puls_e *= Ab_M. */
int mpc_mirror_bounce(mpc_ctx *ctx, int mode);

/* Diagnostics of the device-resident field (MPC.c:389-449, propagation.c:343-361):
 * temp[Nt] = sum_xy |A|^2, spec[Nt] = sum_xy |FFT_t A|^2 (FFT order), BP1[Nx], BP2[Ny];
 * any pointer may be NULL. */
int mpc_diag(mpc_ctx *ctx, double *temp, double *spec, double *BP1, double *BP2);

/* Total energy sum |A|^2 dx dy dt hbar w0 of the device-resident field (FP64 reduction). */
int mpc_energy(mpc_ctx *ctx, double *energy);

/* Synchronise the context's stream; returns MPC_ERR_CUDA on an asynchronous fault. */
int mpc_sync(mpc_ctx *ctx);

/* ---- batches of independent cells (no counterpart in the reference) ----------------- */
/* A batch runs one call on many contexts -- the cells of a parameter sweep, of any compiled
 * grid shapes -- as one CUDA graph per call: each cell's launches are captured on the cell's
 * stream (forked from and joined into the batch's stream) and the graph is launched once, so
 * the cells' kernels overlap and the host issues one launch per call.  The contexts stay owned
 * by the caller and must outlive the batch; each call waits for the cells' pending work first. */
typedef struct mpc_batch mpc_batch;
int mpc_batch_create(mpc_batch **batch, int n, mpc_ctx *const *cells);
int mpc_batch_destroy(mpc_batch *batch);
/* mpc_run_fixed(cell, nsteps) for every cell, as one graph. */
int mpc_batch_run_fixed(mpc_batch *batch, int nsteps);
/* One mpc_step_double attempt of every cell with state.z < dist, as one graph, then each
 * cell's decision: bad[i] / err[i] as mpc_step_double returns them, bad[i] = -1 for cells
 * that have finished.  bad and err hold n entries. */
int mpc_batch_step_double(mpc_batch *batch, int *bad, double *err);
/* Graphs launched and their total node count, since creation. */
int mpc_batch_stats(mpc_batch *batch, long *graphs, long *nodes);

/* ---- measurement and host buffers (no counterpart in the reference) ---------------- */
/* Page-locked host buffer for fast host<->device copies of the field.  Field-sized transfers
 * to or from page-locked, 16-byte aligned host memory mapped for the context's device (this
 * allocator, cudaMallocHost or cudaHostRegister called while that device is current) are done
 * by the library's SM copy kernel, at the host link's rate in every call; other host memory
 * goes through cudaMemcpyAsync. */
int mpc_host_alloc(void **ptr, size_t bytes);
int mpc_host_free(void *ptr);
/* The cudaStream_t every kernel of this context is launched on. */
int mpc_stream_handle(mpc_ctx *ctx, void **stream);
/* Number of kernels this context has launched so far. */
long mpc_launch_count(mpc_ctx *ctx);
/* The compiled kernel variant this context runs (the autotuner's pick when created with
 * variant = -1) and its launch shapes: info = {P pencils per tile, SLO slots interleaved,
 * CL CTAs per plane cluster, PB planes per cluster unit, PT plane threads per CTA,
 * pencil CTAs launched, plane clusters launched, pencil threads per CTA, LD pencil tile load
 * mode (0 staged by cp.async, 1 read by the first transform stage), PL plane passes (1 one
 * cluster kernel, 2 column-strip and row-strip kernels)}. */
int mpc_variant_info(mpc_ctx *ctx, int *variant, int info[10]);
/* With on != 0, every pencil and plane sweep is bracketed by CUDA events on the context's
 * stream; mpc_kernel_times sums their durations since the last enable (synchronises). */
int mpc_profile(mpc_ctx *ctx, int on);
int mpc_kernel_times(mpc_ctx *ctx, double *pencil_ms, long *n_pencil, double *plane_ms, long *n_plane);

/* Self-check of the bounded device-side waits (no counterpart in the reference): launches a
 * one-thread kernel that waits on an mbarrier nothing completes.  The wait gives up after about
 * a second and leaves its code in the context's kernel error word, which this call reads and
 * clears: it returns MPC_ERR_TIMEOUT when the limit works, and the context stays usable.  Every
 * wait of the library's TMA-staged kernels is bounded the same way; mpc_sync and
 * mpc_field_download report such a timeout as MPC_ERR_TIMEOUT. */
int mpc_wait_limit_check(mpc_ctx *ctx);

/* ---- allocation-free nonlinear step (no counterpart in the reference) -------------- */
/* The nonlinear half of a split step, A *= exp(dz * A_nl(A)) with Kerr, self-steepening,
 * ionization and plasma terms, applied in place to a field the caller already holds in
 * device memory: complex64, real space, layout A[t*Nx*Ny + y*Nx + x], physical units,
 * physics parameters from p (only dims, w, gamma2, w0, sst_on, plasm, deltat, rho_c,
 * rho_nt, n0 and gas are read).
 *
 * For callers that cannot allocate device memory -- code running where cudaMalloc is not
 * allowed or not safe (inside a host callback, or under another library's promise not to
 * allocate), processes whose device memory is owned entirely by a pool handed out at
 * start-up, hosts with a fixed device-memory budget -- this call allocates nothing: no
 * cudaMalloc, no cudaFree, no context.  Its work buffers are one static device array of
 * 8,429,568 bytes inside libmpc_gpu.so, which every GPU that loads the library holds
 * until the process exits.  Limits: Nt one of 64, 256, 512, 1024, 2048 (at most 2048),
 * Nx*Ny a multiple of 16384/Nt; larger or other sizes are rejected with MPC_ERR_SHAPE.
 *
 * Every call looks up the device address of that array on the current device (an
 * allocation-free runtime query) and passes the omega grid to the device by value, so the
 * call keeps no pointer to p or its arrays after it returns.  The first call on a device
 * loads the library's device code: make it before any stream capture begins.  Every call
 * shares the array and leaves its contents behind; nothing in it needs to start at zero
 * (each call rewrites what it reads).  Calls that overlap on the GPU -- on different
 * streams, or from several host threads -- race on the array.  The work is queued on
 * `stream` (a cudaStream_t, NULL for the legacy stream) and the call returns without
 * waiting; errors are printed to stderr and returned as MPC_ERR_*. */
int mpc_nonlinear_noalloc(const mpc_params *p, void *A_dev, double dz, void *stream);

#ifdef __cplusplus
}
#endif
#endif
