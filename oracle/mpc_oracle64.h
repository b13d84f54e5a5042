/*
 * mpc_oracle64.h -- FP64 GPU restatement of the split-step propagator.
 *
 * TEST INFRASTRUCTURE ONLY, like the CPU oracle (mpc_oracle.c) it follows step for step: the
 * checker of the complex64 product path at grid sizes and run lengths the CPU oracle cannot
 * reach (a whole 3,200-step run of a 256x256x2048 cell).  The field is complex128 on the device
 * in the reference layout A[k*Nx*Ny + j*Nx + i]; the transforms are cuFFT Z2Z (the reference's
 * own GPU FFT library, propagation.c:11-57); every pointwise operation is FP64 and compiled
 * without FMA contraction, so that it rounds as the CPU oracle does.  The phase tables, the
 * beam-size search and the step-size rule are the CPU oracle's own host functions.
 *
 * Only the corrected physics is restated (or_default_switches), with either mirror model
 * (bounce_lens); or64_create rejects other switch settings.
 */
#ifndef MPC_ORACLE64_H
#define MPC_ORACLE64_H
#include "mpc_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or64_ctx or64_ctx;

const char *or64_last_error(void);

/* A context on the current device: the field, the derivative buffer, the two step-doubling
 * fields C1, C2 (allocated on the first attempt) and the ionization terms (5 x 8 N bytes, on
 * the first step with plasma), the cuFFT plans and the tables.  Returns 0 or -1. */
int or64_create(or64_ctx **out, const or_params *p, const or_switches *sw);
int or64_destroy(or64_ctx *c);

/* N complex128 values, host memory, reference layout. */
int or64_upload(or64_ctx *c, const double *A);
int or64_download(or64_ctx *c, double *A);

/* or_ssfmprop (propagation.c:111-372) on the resident field. */
int or64_ssfmprop(or64_ctx *c, double dzz, int *signmem, double z, double *puls_e, double *BP1,
                  double *BP2, double *y1, double *y2, double *bps1, double *bps2, int change);

/* or_run_fixed: nsteps fixed steps of st->dzz. */
int or64_run_fixed(or64_ctx *c, or_state *st, int nsteps);

/* or_double_step (MPC.c:269-383): one step-doubling attempt.  dz_used > 0 replaces st->dzz as
 * the attempt's step (to follow another integrator's schedule, e.g. one that shortens steps to
 * land on the mirror planes).  force < 0: the attempt is accepted or rejected by this oracle's
 * own rule; force = 0 / 1: rejected / accepted as the followed integrator decided, the rule still
 * run (own_bad, own_err: its decision and local error, for comparing the two). */
int or64_double_step(or64_ctx *c, or_state *st, double dz_used, int force, int *own_bad,
                     double *own_err);

/* sum |A|^2 of the resident field (FP64) */
int or64_energy(or64_ctx *c, double *e);

#ifdef __cplusplus
}
#endif
#endif
