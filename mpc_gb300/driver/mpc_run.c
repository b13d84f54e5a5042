/*
 * mpc_run -- the run driver of the multipass-cell propagator, in place of the reference's
 * MPC.c (MPC.c:23-596), on libmpc_gpu.so through include/mpc_gpu.h.
 *
 *   mpc_run [-r] [-n NRUN] [-d DATADIR] [-m signflip|lens] [-R ROC] [-f CHUNK] [-v VARIANT] [-L]
 *
 * Files and formats are the reference's (MPC.c:77-110, 159-203, 489-509, 521-537, 558):
 *   DATADIR%04d/param.bin            run parameters, read field by field (MPC.c:180-203)
 *   DATADIR/datar.bin, datai.bin     initial field, N raw doubles each, x fastest, t slowest
 *   DATADIR%04d/bp1.bin, bp2.bin     per accepted step: Nx / Ny doubles (beam profiles)
 *   DATADIR%04d/temp.bin, spec.bin   per accepted step: Nt doubles (sum_xy |A|^2, sum_xy |FFT_t A|^2)
 *   DATADIR%04d/other.bin            per accepted step: "%f\t%f\n" of err and the next dzz
 *   DATADIR%04d/resdata.bin          checkpoint every 10 steps: the field, N complex128
 *   DATADIR%04d/resparam.bin         checkpoint: double dzz, double z, int signmem, double puls_e, int nstep+1
 *   DATADIR%04d/out.bin              the final field, N interleaved complex128
 * At each checkpoint the five diagnostic files are copied to *.bak; -r (resume) restores those
 * copies, reopens them for appending and continues from resdata.bin / resparam.bin.
 *
 * Stepping: by default the reference's adaptive step doubling (one mpc_step_double call per
 * loop iteration of MPC.c:269-383).  -f CHUNK runs fixed steps of param.bin's dzz instead
 * (mpc_run_fixed, CHUNK steps between diagnostic records; other.bin then records err = 0).
 * -m lens -R ROC models each mirror as a focusing phase of radius of curvature ROC [m]
 * (param.bin carries no ROC); the default is the reference's diffraction sign flip.  -L ends
 * step-doubling attempts on the mirror planes instead of stepping across them.
 *
 * Differences from MPC.c, all deliberate: the field is calibrated with both parts scaled
 * (MPC.c:213 scales the real part only) and only on a fresh run (the checkpointed field is
 * calibrated already); resume parameters are always read (MPC.c:240 reads them only in MPI
 * mode); out.bin is written only at the end (MPC.c:92 truncates it when resuming); z advances by
 * the step just taken; diagnostic files are copied once per checkpoint by the driver itself
 * (MPC.c:38-41 shells out to cp, twice).
 */
#include <errno.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/mpc_gpu.h"

#define CHECKPOINT_EVERY 10

static void die(const char *what) {
    fprintf(stderr, "mpc_run: %s\n", what);
    exit(1);
}

static void check(int rc, const char *what) {
    if (rc != MPC_OK) {
        fprintf(stderr, "mpc_run: %s: status %d: %s\n", what, rc, mpc_last_error());
        exit(1);
    }
}

static FILE *open_in(const char *dir, const char *name, const char *mode) {
    char path[4096];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, mode);
    if (!f) {
        fprintf(stderr, "mpc_run: cannot open %s: %s\n", path, strerror(errno));
        exit(1);
    }
    return f;
}

/* copy src to dst; 0 on success */
static int copy_file(const char *src, const char *dst) {
    FILE *a = fopen(src, "rb");
    if (!a) return -1;
    FILE *b = fopen(dst, "wb");
    if (!b) {
        fclose(a);
        return -1;
    }
    char buf[1 << 16];
    size_t n;
    int rc = 0;
    while ((n = fread(buf, 1, sizeof buf, a)) > 0)
        if (fwrite(buf, 1, n, b) != n) {
            rc = -1;
            break;
        }
    fclose(a);
    if (fclose(b) != 0) rc = -1;
    return rc;
}

static void read_exact(void *dst, size_t size, size_t n, FILE *f, const char *what) {
    if (fread(dst, size, n, f) != n) {
        fprintf(stderr, "mpc_run: %s: file too short\n", what);
        exit(1);
    }
}

static void write_exact(const void *src, size_t size, size_t n, FILE *f, const char *what) {
    if (fwrite(src, size, n, f) != n) {
        fprintf(stderr, "mpc_run: writing %s failed\n", what);
        exit(1);
    }
}

/* param.bin, in the order MPC.c:77,180-203 reads it */
static void read_params(const char *dir, mpc_params *p, double **arrays) {
    FILE *f = open_in(dir, "param.bin", "rb");
    memset(p, 0, sizeof *p);
    read_exact(p->dims, sizeof(int), 3, f, "param.bin dims");
    const int Ny = p->dims[1], Nt = p->dims[2];
    if (p->dims[0] <= 0 || Ny <= 0 || Nt <= 0) die("param.bin: invalid dims");
    double *betas = malloc(sizeof(double) * Nt), *wr = malloc(sizeof(double) * Ny);
    double *w = malloc(sizeof(double) * Nt), *r = malloc(sizeof(double) * Ny);
    if (!betas || !wr || !w || !r) die("out of host memory");
    read_exact(&p->dist, sizeof(double), 1, f, "param.bin dist");
    read_exact(&p->dzz, sizeof(double), 1, f, "param.bin dzz");
    read_exact(betas, sizeof(double), Nt, f, "param.bin betas");
    read_exact(&p->alpha, sizeof(double), 1, f, "param.bin alpha");
    read_exact(&p->Cav, sizeof(double), 1, f, "param.bin Cav");
    read_exact(&p->k0, sizeof(double), 1, f, "param.bin k0");
    read_exact(wr, sizeof(double), Ny, f, "param.bin wr");
    read_exact(&p->sst_on, sizeof(int), 1, f, "param.bin sst_on");
    read_exact(w, sizeof(double), Nt, f, "param.bin w");
    read_exact(&p->gamma2, sizeof(double), 1, f, "param.bin gamma2");
    read_exact(&p->w0, sizeof(double), 1, f, "param.bin w0");
    read_exact(&p->plasm, sizeof(int), 1, f, "param.bin plasm");
    double six[6];
    read_exact(six, sizeof(double), 6, f, "param.bin deltat..Ab_M");
    p->deltat = six[0];
    p->rho_c = six[1];
    p->rho_nt = six[2];
    p->n0 = six[3];
    p->puls_e = six[4];
    p->Ab_M = six[5];
    read_exact(r, sizeof(double), Ny, f, "param.bin r");
    double four[4];
    read_exact(four, sizeof(double), 4, f, "param.bin dr..Esig");
    p->dr = four[0];
    p->def_err = four[1];
    p->dzmin = four[2];
    p->Esig = four[3];
    read_exact(p->gas, 1, 9, f, "param.bin gas");
    p->gas[8] = 0;
    fclose(f);
    p->betas = betas;
    p->wr = wr;
    p->w = w;
    p->r = r;
    arrays[0] = betas;
    arrays[1] = wr;
    arrays[2] = w;
    arrays[3] = r;
}

static const char *kDiagFiles[5] = {"bp1.bin", "bp2.bin", "temp.bin", "spec.bin", "other.bin"};

int main(int argc, char **argv) {
    int resume = 0, nrun = 0, chunk = 0, variant = -1, bounce = MPC_BOUNCE_SIGNFLIP, land = 0;
    double roc = 0.0;
    const char *datadir = ".";
    for (int i = 1; i < argc; i++) {
        const char *a = argv[i];
        const char *v = (i + 1 < argc) ? argv[i + 1] : NULL;
        if (!strcmp(a, "-r")) resume = 1;
        else if (!strcmp(a, "-n") && v) nrun = atoi(argv[++i]);
        else if (!strcmp(a, "-d") && v) datadir = argv[++i];
        else if (!strcmp(a, "-f") && v) chunk = atoi(argv[++i]);
        else if (!strcmp(a, "-v") && v) variant = atoi(argv[++i]);
        else if (!strcmp(a, "-L")) land = 1;
        else if (!strcmp(a, "-R") && v) roc = atof(argv[++i]);
        else if (!strcmp(a, "-m") && v) {
            const char *m = argv[++i];
            if (!strcmp(m, "lens")) bounce = MPC_BOUNCE_LENS;
            else if (!strcmp(m, "signflip")) bounce = MPC_BOUNCE_SIGNFLIP;
            else die("-m takes signflip or lens");
        } else {
            fprintf(stderr, "usage: %s [-r] [-n NRUN] [-d DATADIR] [-m signflip|lens] [-R ROC] [-f CHUNK] [-v VARIANT] [-L]\n",
                    argv[0]);
            return 2;
        }
    }
    if (bounce == MPC_BOUNCE_LENS && !(roc > 0)) die("-m lens needs -R ROC > 0");
    char cpath[4096];
    snprintf(cpath, sizeof cpath, "%s%04d", datadir, nrun);   /* MPC.c:73 */
    printf("Using directory %s\n", cpath);

    mpc_params p;
    double *arrays[4];
    read_params(cpath, &p, arrays);
    p.bounce_mode = bounce;
    p.roc = roc;
    p.variant = variant;
    p.land_mirrors = land;
    const int Nx = p.dims[0], Ny = p.dims[1], Nt = p.dims[2];
    const size_t N = (size_t)Nx * Ny * Nt;
    printf("Matrix dimensions are: %d x %d x %d.\n", Nx, Ny, Nt);

    double *A = NULL;
    check(mpc_host_alloc((void **)&A, sizeof(double) * 2 * N), "pinned field buffer");
    double *BP1 = calloc(Nx, sizeof(double)), *BP2 = calloc(Ny, sizeof(double));
    double *temp = calloc(Nt, sizeof(double)), *spec = calloc(Nt, sizeof(double));
    if (!BP1 || !BP2 || !temp || !spec) die("out of host memory");

    FILE *fd[5];
    mpc_state st;
    memset(&st, 0, sizeof st);
    int nstep = 0;
    double z = 0.0, dzz = p.dzz, puls_e = p.puls_e;
    int signmem = 1;
    if (resume) {
        printf("Resuming previous run!\n");
        for (int k = 0; k < 5; k++) {   /* restore the copies of the last checkpoint */
            char path[4200], bak[4300];
            snprintf(path, sizeof path, "%s/%s", cpath, kDiagFiles[k]);
            snprintf(bak, sizeof bak, "%s.bak", path);
            if (copy_file(bak, path) != 0) {
                fprintf(stderr, "mpc_run: cannot restore %s\n", bak);
                return 1;
            }
            fd[k] = open_in(cpath, kDiagFiles[k], k < 4 ? "ab" : "a");
        }
        FILE *f = open_in(cpath, "resdata.bin", "rb");
        read_exact(A, sizeof(double), 2 * N, f, "resdata.bin");
        fclose(f);
        f = open_in(cpath, "resparam.bin", "rb");   /* A16: always read */
        read_exact(&dzz, sizeof(double), 1, f, "resparam.bin dzz");
        read_exact(&z, sizeof(double), 1, f, "resparam.bin z");
        read_exact(&signmem, sizeof(int), 1, f, "resparam.bin signmem");
        read_exact(&puls_e, sizeof(double), 1, f, "resparam.bin puls_e");
        read_exact(&nstep, sizeof(int), 1, f, "resparam.bin nstep");
        fclose(f);
    } else {
        FILE *fr = open_in(datadir, "datar.bin", "rb"), *fi = open_in(datadir, "datai.bin", "rb");
        double *buf = malloc(sizeof(double) * N);
        if (!buf) die("out of host memory");
        read_exact(buf, sizeof(double), N, fr, "datar.bin");
        for (size_t i = 0; i < N; i++) A[2 * i] = buf[i];
        read_exact(buf, sizeof(double), N, fi, "datai.bin");
        for (size_t i = 0; i < N; i++) A[2 * i + 1] = buf[i];
        free(buf);
        fclose(fr);
        fclose(fi);
        for (int k = 0; k < 5; k++) fd[k] = open_in(cpath, kDiagFiles[k], k < 4 ? "wb" : "w");
    }

    mpc_ctx *ctx = NULL;
    check(mpc_create(&ctx, &p), "mpc_create");
    check(mpc_field_upload(ctx, A, resume ? 0 : 1), "mpc_field_upload");   /* MPC.c:206-216 */
    check(mpc_get_state(ctx, &st), "mpc_get_state");
    st.z = z;
    st.dzz = dzz;
    st.signmem = signmem;
    st.puls_e = puls_e;
    st.nstep = (chunk > 0) ? (int)llround(z / dzz) : nstep;
    check(mpc_set_state(ctx, &st), "mpc_set_state");
    int variant_used = 0, info[10];
    check(mpc_variant_info(ctx, &variant_used, info), "mpc_variant_info");
    if (info[9] >= 2)
        printf("Kernel variant %d (pencil tile %d, plane in two strip passes of %d-thread CTAs)\n", variant_used,
               info[0], info[4]);
    else
        printf("Kernel variant %d (pencil tile %d, plane cluster %d x %d threads)\n", variant_used, info[0], info[2],
               info[4]);

    const long total_fixed = (chunk > 0) ? (long)llround(p.dist / dzz) : 0;
    while (chunk > 0 ? st.nstep < total_fixed : st.z < p.dist) {
        double err = 0.0;
        if (chunk > 0) {
            const long left = total_fixed - st.nstep;
            check(mpc_run_fixed(ctx, (int)(left < chunk ? left : chunk)), "mpc_run_fixed");
            check(mpc_diag(ctx, temp, spec, BP1, BP2), "mpc_diag");
        } else {
            int bad = 0;
            check(mpc_step_double(ctx, BP1, BP2, &bad, &err), "mpc_step_double");
            if (bad) continue;   /* MPC.c:345-348 */
            check(mpc_diag(ctx, temp, spec, NULL, NULL), "mpc_diag");
        }
        check(mpc_get_state(ctx, &st), "mpc_get_state");
        write_exact(BP1, sizeof(double), Nx, fd[0], "bp1.bin");
        write_exact(BP2, sizeof(double), Ny, fd[1], "bp2.bin");
        write_exact(temp, sizeof(double), Nt, fd[2], "temp.bin");
        write_exact(spec, sizeof(double), Nt, fd[3], "spec.bin");
        fprintf(fd[4], "%f\t%f\n", err, st.dzz);
        for (int k = 0; k < 5; k++) fflush(fd[k]);
        printf("We are here: %5.2f\n", st.z * 100.0 / p.dist);
        if (nstep % CHECKPOINT_EVERY == 0) {   /* MPC.c:521-537 */
            printf("We are at step %d, writing checkpoint data into files.\n", nstep);
            check(mpc_field_download(ctx, A), "mpc_field_download");
            FILE *f = open_in(cpath, "resdata.bin", "wb");
            write_exact(A, sizeof(double), 2 * N, f, "resdata.bin");
            fclose(f);
            const int stepn = nstep + 1;
            f = open_in(cpath, "resparam.bin", "wb");
            write_exact(&st.dzz, sizeof(double), 1, f, "resparam.bin");
            write_exact(&st.z, sizeof(double), 1, f, "resparam.bin");
            write_exact(&st.signmem, sizeof(int), 1, f, "resparam.bin");
            write_exact(&st.puls_e, sizeof(double), 1, f, "resparam.bin");
            write_exact(&stepn, sizeof(int), 1, f, "resparam.bin");
            fclose(f);
            for (int k = 0; k < 5; k++) {
                char path[4200], bak[4300];
                snprintf(path, sizeof path, "%s/%s", cpath, kDiagFiles[k]);
                snprintf(bak, sizeof bak, "%s.bak", path);
                if (copy_file(path, bak) != 0) fprintf(stderr, "mpc_run: warning: cannot back up %s\n", path);
            }
        }
        nstep++;
    }
    check(mpc_field_download(ctx, A), "mpc_field_download");
    FILE *fo = open_in(cpath, "out.bin", "wb");
    write_exact(A, sizeof(double), 2 * N, fo, "out.bin");
    fclose(fo);
    for (int k = 0; k < 5; k++) fclose(fd[k]);
    printf("Done: z = %g m, %d accepted steps, %d attempts.\n", st.z, nstep, st.attempts);
    mpc_destroy(ctx);
    mpc_host_free(A);
    free(BP1);
    free(BP2);
    free(temp);
    free(spec);
    for (int k = 0; k < 4; k++) free(arrays[k]);
    return 0;
}
