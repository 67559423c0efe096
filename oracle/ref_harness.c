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
 */
#include <stdio.h>
#include <stdlib.h>
#include <time.h>
#include <string.h>
#include <unistd.h>
#include "mspms2.h"

int opening();
int fnValidateInput();

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s <dir> <out.bin> [repeat]\n", argv[0]);
        return 2;
    }
    const char *outname = argv[2];
    char outabs[4096];
    if (outname[0] != '/') {
        if (!getcwd(outabs, sizeof(outabs) - 1)) return 2;
        snprintf(outabs + strlen(outabs), sizeof(outabs) - strlen(outabs), "/%s", outname);
    } else {
        snprintf(outabs, sizeof(outabs), "%s", outname);
    }
    int repeat = argc > 3 ? atoi(argv[3]) : 0;
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
    return 0;
}
