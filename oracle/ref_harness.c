/*
 * ref_harness.c - driver for the compiled reference force layer (TEST INFRASTRUCTURE).
 *
 * Replays the start of the reference's main() (src/mspms2.c:34-51): opening(),
 * readins(), fnValidateInput(), init_vars(), frclong(), frcshort(), in the directory
 * holding in.mspms / cfg.mspms / xyz.mspms, then writes every force and energy the
 * two calls produce, plus the derived globals, to a binary file:
 *   int32 natom; double fxl[n], fyl[n], fzl[n], fxs[n], fys[n], fzs[n];
 *   double energies[18] (mg_energies order); double derived[24] (see below).
 * With a repeat count R > 0 it then times R further frclong() calls and R frcshort()
 * calls and prints "frclong_s=<seconds per call> frcshort_s=<...>".
 *
 * With "md <nsteps> <md.bin>" after the repeat count it then runs nsteps steps of the
 * reference's own integrator for the input's ensemble (what_ensemble NVT: vver_nh_3,
 * src/nvtnh.c:11; NVE: vver, src/md.c:22; NPT: npt_respa, src/nptnh.c:134), starting
 * from the velocities init_vars() drew, and writes
 *   int32 natom, nstep_inner, what_ensemble, nsteps; double scalars[12] = {delt, treq,
 *   qq, qqs, gg, ggs, nfree, ps, ss, pss, sss, 0}; double x,y,z,vx,vy,vz[n] (start);
 *   per step (0 = start, then 1..nsteps) double log[12] = {ukin, uinter, uintra, ushift,
 *   ps, ss, pss, sss, tinst, unhts, unhtss, 0}; double x,y,z,vx,vy,vz[n] (end).
 * For NPT the scalars are {delt, treq, Qts, Qbs, preq, isLJlrcOn, nfree, vts, vbs, rts,
 * boxlx, pljlrc} and the per-step record {ukin, uinter, uintra, ushift, vts, vbs, rts,
 * utsbs, tinst, pinst, boxlx, boxv}.
 * With "hmc <nmoves> <nstep_md> <hmc.bin> <vel.bin>" after the repeat count it runs nmoves
 * canonical HMC moves through the reference's own md_move() over vver() (src/dispmd.c:12-103,
 * src/md.c:22-85), each from velocities read from vel.bin (per move vx, vy, vz [n]) in
 * place of velinit()'s draw, with the kinetic energy formed as velinit() ends
 * (src/initvars.c:198-228), then frclong() and frcshort() as hmc() calls them
 * (src/hmc.c:31-36). md_move() runs unchanged; the vver() it calls is wrapped to copy the
 * positions after its last step, so the proposal is kept even when the move is rejected.
 * Writes int32 natom, nmoves, nstep_md; per move double {ukin, uinter, uintra, ushift}
 * before, {dH, isAccept, uinter, ushift} after, {ukin, uinter, uintra, ushift} of the
 * proposal, then the proposal and the final x, y, z [n].
 * A further argument trj_every > 0 makes the run write the reference's trajectory file
 * (trj.mspms in the input directory, trajectory() of src/dumpxyz.c) the way its main loop
 * does (src/mspms2.c:57-60, :123-126), and its checkpoint (saveit(), sav.mspms) after the
 * last step with istep = nsteps.
 */
#include <stdio.h>
#include <stdlib.h>
#include <time.h>
#include <string.h>
#include <unistd.h>
#include "mspms2.h"

int opening();
int fnValidateInput();
int vver();
int vver_nh_3();
int npt_respa();
bool md_move(int (*pfn_md_scheme)(), int nStepMD);

/* vver() that keeps the positions after the last step of an HMC trajectory */
static int rec_steps, rec_k;
static double *rec_x, *rec_y, *rec_z, rec_e[4];
static int vver_rec(void) {
    int r = vver();
    if (++rec_k == rec_steps) {
        memcpy(rec_x, xx, sizeof(double) * natom);
        memcpy(rec_y, yy, sizeof(double) * natom);
        memcpy(rec_z, zz, sizeof(double) * natom);
        rec_e[0] = ukin;
        rec_e[1] = uinter;
        rec_e[2] = uintra;
        rec_e[3] = ushift;
    }
    return r;
}
int trajectory();
int saveit();

static void abs_path(const char *name, char *out, size_t len) {
    if (name[0] != '/' && getcwd(out, len - 1)) {
        snprintf(out + strlen(out), len - strlen(out), "/%s", name);
    } else {
        snprintf(out, len, "%s", name);
    }
}

static void write_state(FILE *fp, int n) {
    fwrite(xx, sizeof(double), n, fp);
    fwrite(yy, sizeof(double), n, fp);
    fwrite(zz, sizeof(double), n, fp);
    fwrite(vx, sizeof(double), n, fp);
    fwrite(vy, sizeof(double), n, fp);
    fwrite(vz, sizeof(double), n, fp);
}

static void write_log(FILE *fp) {
    if (what_ensemble == NPT) {
        double l[12] = {ukin, uinter, uintra, ushift, vts, vbs, rts, utsbs, tinst, pinst, boxlx, boxv};
        fwrite(l, sizeof(double), 12, fp);
        return;
    }
    double l[12] = {ukin, uinter, uintra, ushift, ps, ss, pss, sss, tinst, unhts, unhtss, 0.0};
    fwrite(l, sizeof(double), 12, fp);
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s <dir> <out.bin> [repeat [md <nsteps> <md.bin> | hmc <nmoves> <nstep_md> <hmc.bin> "
                        "<vel.bin>]]\n", argv[0]);
        return 2;
    }
    char outabs[4096];
    abs_path(argv[2], outabs, sizeof(outabs));
    int repeat = argc > 3 ? atoi(argv[3]) : 0;
    int md_steps = 0, hmc_moves = 0, hmc_steps = 0;
    char mdabs[4096] = {0}, velabs[4096] = {0};
    int trj_every = 0;
    if (argc > 8 && !strcmp(argv[4], "hmc")) {
        hmc_moves = atoi(argv[5]);
        hmc_steps = atoi(argv[6]);
        abs_path(argv[7], mdabs, sizeof(mdabs));
        abs_path(argv[8], velabs, sizeof(velabs));
    } else if (argc > 6 && !strcmp(argv[4], "md")) {
        md_steps = atoi(argv[5]);
        abs_path(argv[6], mdabs, sizeof(mdabs));
        if (argc > 7) trj_every = atoi(argv[7]);
    }
    if (chdir(argv[1]) != 0) { perror("chdir"); return 2; }
    opening();
    readins();
    fnValidateInput();
    init_vars();
    frclong();
    frcshort();
    FILE *fp = fopen(outabs, "wb");
    if (!fp) { perror("out"); return 2; }
    int n = natom;
    fwrite(&n, sizeof(int), 1, fp);
    fwrite(fxl, sizeof(double), n, fp);
    fwrite(fyl, sizeof(double), n, fp);
    fwrite(fzl, sizeof(double), n, fp);
    fwrite(fxs, sizeof(double), n, fp);
    fwrite(fys, sizeof(double), n, fp);
    fwrite(fzs, sizeof(double), n, fp);
    double e[18] = {uvdw, ushift, ureal, uexcl, ufourier, uself, uvacuum, uelec,
                    usflj, uotherff, uinter, virial_inter,
                    ubond, uangle, udih, uimp, uintra, virial_intra};
    fwrite(e, sizeof(double), 18, fp);
    double d[24] = {rcutoffsq, rcutonsq, rcutoffelecsq, roff2_minus_ron2_cube, shift1, shift4,
                    wolfvcon1, wolfvcon2, wolfvcon3, wolffcon1, wolffcon2,
                    Bfactor_ewald, Vfactor_ewald, TWOPI_LX, TWOPI_LY, TWOPI_LZ, twopi_over_3v,
                    kappa, coulomb_prefactor, boxlx, boxly, boxlz, sigma_base, epsilon_base};
    fwrite(d, sizeof(double), 24, fp);
    fclose(fp);
    if (repeat > 0) {
        double t0 = now_s();
        for (int r = 0; r < repeat; r++) frclong();
        double t1 = now_s();
        for (int r = 0; r < repeat; r++) frcshort();
        double t2 = now_s();
        printf("frclong_s=%.9g frcshort_s=%.9g\n", (t1 - t0) / repeat, (t2 - t1) / repeat);
    }
    if (hmc_moves > 0) {
        FILE *fv = fopen(velabs, "rb"), *fh = fopen(mdabs, "wb");
        if (!fv || !fh) { perror("hmc files"); return 2; }
        int hdr[3] = {n, hmc_moves, hmc_steps};
        fwrite(hdr, sizeof(int), 3, fh);
        rec_x = (double *)malloc(sizeof(double) * n);
        rec_y = (double *)malloc(sizeof(double) * n);
        rec_z = (double *)malloc(sizeof(double) * n);
        for (int m = 0; m < hmc_moves; m++) {
            if (fread(vx, sizeof(double), n, fv) != (size_t)n || fread(vy, sizeof(double), n, fv) != (size_t)n ||
                fread(vz, sizeof(double), n, fv) != (size_t)n) {
                fprintf(stderr, "hmc: short velocity file\n");
                return 2;
            }
            int specie_id, sample_atom_id;
            ukin = 0.0;
            for (int ii = 0; ii < n; ii++) {
                get_specie_and_relative_atom_id(ii, &specie_id, &sample_atom_id);
                ukin += sample_mole[specie_id].aw[sample_atom_id] * (vx[ii] * vx[ii] + vy[ii] * vy[ii] + vz[ii] * vz[ii]);
            }
            ukin = 0.5 * ukin;
            tinst = 2.0 * ukin / nfree;
            frclong();
            frcshort();
            double pre[4] = {ukin, uinter, uintra, ushift};
            rec_steps = hmc_steps;
            rec_k = 0;
            bool acc = md_move(&vver_rec, hmc_steps);
            double post[4] = {dH, acc ? 1.0 : 0.0, uinter, ushift};
            fwrite(pre, sizeof(double), 4, fh);
            fwrite(post, sizeof(double), 4, fh);
            fwrite(rec_e, sizeof(double), 4, fh);
            fwrite(rec_x, sizeof(double), n, fh);
            fwrite(rec_y, sizeof(double), n, fh);
            fwrite(rec_z, sizeof(double), n, fh);
            fwrite(xx, sizeof(double), n, fh);
            fwrite(yy, sizeof(double), n, fh);
            fwrite(zz, sizeof(double), n, fh);
        }
        fclose(fv);
        fclose(fh);
    }
    if (md_steps > 0) {
        int (*scheme)() = what_ensemble == NVT ? vver_nh_3
                          : (what_ensemble == NVE ? vver : (what_ensemble == NPT ? npt_respa : NULL));
        if (!scheme) { fprintf(stderr, "md mode supports NVT, NVE and NPT only\n"); return 2; }
        if (repeat > 0) { frclong(); frcshort(); }
        FILE *fm = fopen(mdabs, "wb");
        if (!fm) { perror("md out"); return 2; }
        int hdr[4] = {n, nstep_inner, what_ensemble, md_steps};
        fwrite(hdr, sizeof(int), 4, fm);
        double sc[12] = {delt, treq, qq, qqs, gg, ggs, (double)nfree, ps, ss, pss, sss, 0.0};
        if (what_ensemble == NPT) {
            double snpt[12] = {delt, treq, Qts, Qbs, preq, (double)isLJlrcOn, (double)nfree, vts, vbs, rts, boxlx,
                               pljlrc};
            memcpy(sc, snpt, sizeof(sc));
        }
        fwrite(sc, sizeof(double), 12, fm);
        write_state(fm, n);
        write_log(fm);
        if (trj_every > 0) trajectory();
        for (int k = 0; k < md_steps; k++) {
            scheme();
            write_log(fm);
            istep = k + 1;
            if (trj_every > 0 && istep % trj_every == 0) trajectory();
        }
        write_state(fm, n);
        fclose(fm);
        if (trj_every > 0) {
            fflush(fptrj);
            istep = md_steps;
            saveit();
        }
    }
    return 0;
}
