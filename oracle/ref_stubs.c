/*
 * ref_stubs.c - link-time stand-ins for the parts of the reference that cannot be
 * compiled here (TEST INFRASTRUCTURE, linked only into oracle/_ref/mspms_ref_force).
 *
 *  - the mylibtasos Fortran sources (no Fortran compiler): the four Fortran entry points called by
 *    src/sffrc.c:149-222 and :1322-1337 are provided on top of the C restatement
 *    orc_tasos_force(). Grid sizing follows mylibtasos/initialize.f90:41-110 with
 *    grid_spacing = 0.2 A (mylibtasos/global.f90:214) and no symmetry
 *    (global.f90:235); the text grid format follows mylibtasos/grid.f90:54-129.
 *  - GSL (src/misc.c:127) and the DFT metal-cluster force field (src/dftmcff.c): not on
 *    the nonbonded path; calling them aborts.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "mspms_oracle.h"

double gsl_sf_gamma_inc(double a, double x) {
    (void)a; (void)x;
    fprintf(stderr, "ref_stubs: gsl_sf_gamma_inc is not available\n");
    abort();
}
int fnMetalClusterFF_Cu(void) { fprintf(stderr, "ref_stubs: no DFT FF\n"); abort(); }
int fnMetalClusterFF_Ag(void) { fprintf(stderr, "ref_stubs: no DFT FF\n"); abort(); }

#define TAS_MAX 12
static int tas_n;
static int tas_ngx, tas_ngy, tas_ngz;
static double tas_hx, tas_hy, tas_hz, tas_cuc;
static char tas_file[TAS_MAX][256];
static double *tas_values[TAS_MAX];
static orc_tasos tas_grid[TAS_MAX];

void initpotentialgrid_(int *tnuatoms, double *auc, double *buc, double *cuc, int *na, int *nb,
                        int *nc, double *radius) {
    (void)na; (void)nb; (void)nc; (void)radius;
    const double spacing = 0.2;
    tas_n = *tnuatoms;
    tas_ngx = (int)lround(*auc / spacing);
    tas_hx = *auc / tas_ngx;
    tas_ngy = (int)lround(*buc / spacing);
    tas_hy = *buc / tas_ngy;
    tas_ngz = (int)lround(*cuc / spacing);
    tas_hz = *cuc / tas_ngz;
    tas_cuc = *cuc;
}

void pass_grid_file_name_(char *name, int *idx) {
    if (*idx >= 1 && *idx <= TAS_MAX) {
        strncpy(tas_file[*idx - 1], name, 255);
        tas_file[*idx - 1][255] = 0;
    }
}

void read_grids_(int *nspecies) {
    int nx = tas_ngx + 2, ny = tas_ngy + 2, nz = tas_ngz + 2;
    for (int s = 0; s < *nspecies && s < TAS_MAX; s++) {
        FILE *fp = fopen(tas_file[s], "r");
        if (!fp) { fprintf(stderr, "ref_stubs: cannot open grid %s\n", tas_file[s]); exit(1); }
        double *v = (double *)malloc(sizeof(double) * 8 * (size_t)nx * ny * nz);
        for (long long i = 0; i < 8LL * nx * ny * nz; i++)
            if (fscanf(fp, "%lf", &v[i]) != 1) { fprintf(stderr, "ref_stubs: short grid\n"); exit(1); }
        fclose(fp);
        tas_values[s] = v;
        orc_tasos *g = &tas_grid[s];
        g->nx = nx; g->ny = ny; g->nz = nz;
        g->hx = tas_hx; g->hy = tas_hy; g->hz = tas_hz; g->cuc = tas_cuc;
        g->values = v;
        g->min_pe = orc_tasos_min_pe(g);
    }
}

void cforce_atom_(int *atomid, double *x, double *y, double *z, double *pe, double *force) {
    int t = *atomid;
    if (t < 1 || t > tas_n) { *atomid = -9999; return; }
    double p, f[3];
    if (orc_tasos_force(&tas_grid[t - 1], MG_COMPAT_ALL, *x, *y, *z, &p, f) != 0) {
        *atomid = -9999;
        return;
    }
    *pe = p;
    force[0] = f[0]; force[1] = f[1]; force[2] = f[2];
}
