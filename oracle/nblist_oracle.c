/*
 * nblist_oracle.c - CPU builder of the cluster-pair list (TEST INFRASTRUCTURE).
 *
 * Restates the GPU build of mspms2_gb300/csrc/mg_nblist.cu step by step with the same
 * FP64 operations in the same order (compiled with -ffp-contract=off), so the two must
 * agree bit for bit: the clusters (site membership and order) and the list of
 * (i-cluster, j-cluster, periodic image) entries in order. The column grid (ncx, ncy)
 * and the small-box choice are inputs, taken from the GPU build under test.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mspms_oracle.h"

#define CL 8

typedef struct key { double z; int i; } key;

static int key_cmp(const void *a, const void *b) {
    const key *p = (const key *)a, *q = (const key *)b;
    if (p->z < q->z) return -1;
    if (p->z > q->z) return 1;
    return (p->i > q->i) - (p->i < q->i);
}

/* products with reciprocals rounded once, as the GPU build takes them */
static int column_of(double w, double icw, int nc) {
    int c = (int)floor(w * icw);
    return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}
#define WIN_MARGIN 1e-9 /* columns added on each side of a search window */

static double gap2(double loi, double hii, double loj, double hij, double s) {
    double a = (loj + s) - hii;
    double b = loi - (hij + s);
    double g = fmax(0.0, fmax(a, b));
    return g * g;
}

int orc_nblist_build2(const double *x, const double *y, const double *z, int n, double lx, double ly,
                      double lz, double rlist, int ncx, int ncy, int small, double zcap, int *out_ncl,
                      int *cluster_atoms, int cluster_cap, long long *out_npairs, int *pairs, int *shifts,
                      long long pair_cap) {
    double L[3] = {lx, ly, lz};
    const double *P[3] = {x, y, z};
    double *w = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    int ncol = ncx * ncy;
    int *col = (int *)malloc(sizeof(int) * (size_t)n);
    int *cnt = (int *)calloc((size_t)ncol + 1, sizeof(int));
    double cwx = lx / ncx, cwy = ly / ncy;
    double iL[3] = {1.0 / lx, 1.0 / ly, 1.0 / lz}, icwx = 1.0 / cwx, icwy = 1.0 / cwy;
    for (int a = 0; a < n; a++) {
        for (int d = 0; d < 3; d++) {
            double m = floor(P[d][a] * iL[d]);
            w[(size_t)d * n + a] = P[d][a] - m * L[d];
        }
        col[a] = column_of(w[(size_t)n + a], icwy, ncy) * ncx + column_of(w[a], icwx, ncx);
        cnt[col[a]]++;
    }
    int *start = (int *)calloc((size_t)ncol + 1, sizeof(int));
    for (int c = 0; c < ncol; c++) start[c + 1] = start[c] + cnt[c];
    key *keys = (key *)malloc(sizeof(key) * (size_t)(n > 0 ? n : 1));
    int *fill = (int *)calloc((size_t)ncol, sizeof(int));
    for (int a = 0; a < n; a++) {
        int c = col[a];
        keys[start[c] + fill[c]++] = (key){w[2 * (size_t)n + a], a};
    }
    /* clusters: consecutive z-sorted sites of a column, cut after 8 sites or when a site
       lies more than zcap above the cluster's first site */
    int *clstart = (int *)calloc((size_t)ncol + 1, sizeof(int));
    int ncl = 0;
    for (int c = 0; c < ncol; c++) {
        qsort(keys + start[c], (size_t)cnt[c], sizeof(key), key_cmp);
        clstart[c] = ncl;
        int first = 0;
        for (int i = 0; i < cnt[c]; i++)
            if (i == 0 || i - first == CL || keys[start[c] + i].z - keys[start[c] + first].z > zcap) {
                ncl++;
                first = i;
            }
    }
    clstart[ncol] = ncl;
    *out_ncl = ncl;
    double *bb = (double *)malloc(sizeof(double) * 6 * (size_t)(ncl > 0 ? ncl : 1));
    int *catoms = (int *)malloc(sizeof(int) * CL * (size_t)(ncl > 0 ? ncl : 1));
    for (int c = 0; c < ncol; c++) {
        int q = clstart[c], first = 0;
        for (int i = 0; i <= cnt[c]; i++) {
            int cut = (i == cnt[c]) || (i > 0 && (i - first == CL ||
                                                  keys[start[c] + i].z - keys[start[c] + first].z > zcap));
            if (!cut) continue;
            if (i > 0) {
                double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
                for (int s = 0; s < CL; s++) {
                    int a = first + s < i ? keys[start[c] + first + s].i : -1;
                    catoms[(size_t)q * CL + s] = a;
                    if (a < 0) continue;
                    for (int d = 0; d < 3; d++) {
                        double v = w[(size_t)d * n + a];
                        lo[d] = fmin(lo[d], v);
                        hi[d] = fmax(hi[d], v);
                    }
                }
                for (int d = 0; d < 3; d++) {
                    bb[(size_t)q * 6 + d] = lo[d];
                    bb[(size_t)q * 6 + 3 + d] = hi[d];
                }
                q++;
            }
            first = i;
        }
    }
    if (cluster_atoms && ncl * CL <= cluster_cap) memcpy(cluster_atoms, catoms, sizeof(int) * CL * (size_t)ncl);
    long long np = 0;
    double r2 = rlist * rlist;
    for (int I = 0; I < ncl; I++) {
        if (small) {
            for (int J = 0; J < ncl; J++, np++)
                if (np < pair_cap) {
                    pairs[2 * np] = I; pairs[2 * np + 1] = J;
                    shifts[3 * np] = shifts[3 * np + 1] = shifts[3 * np + 2] = 0;
                }
            continue;
        }
        const double *bi = bb + (size_t)I * 6;
        int cx0 = (int)floor((bi[0] - rlist) * icwx - WIN_MARGIN), cx1 = (int)floor((bi[3] + rlist) * icwx + WIN_MARGIN);
        int cy0 = (int)floor((bi[1] - rlist) * icwy - WIN_MARGIN), cy1 = (int)floor((bi[4] + rlist) * icwy + WIN_MARGIN);
        for (int uy = cy0; uy <= cy1; uy++) {
            int wy = uy % ncy;
            if (wy < 0) wy += ncy;
            int iy = (uy - wy) / ncy;
            double sy = (double)iy * ly;
            for (int ux = cx0; ux <= cx1; ux++) {
                int wx = ux % ncx;
                if (wx < 0) wx += ncx;
                int ix = (ux - wx) / ncx;
                double sx = (double)ix * lx;
                int c = wy * ncx + wx;
                for (int J = clstart[c]; J < clstart[c + 1]; J++) {
                    const double *bj = bb + (size_t)J * 6;
                    double dxy = gap2(bi[0], bi[3], bj[0], bj[3], sx) + gap2(bi[1], bi[4], bj[1], bj[4], sy);
                    if (!(dxy < r2)) continue;
                    for (int iz = -1; iz <= 1; iz++) {
                        double sz = (double)iz * lz;
                        double d2 = dxy + gap2(bi[2], bi[5], bj[2], bj[5], sz);
                        if (!(d2 < r2)) continue;
                        if (np < pair_cap) {
                            pairs[2 * np] = I; pairs[2 * np + 1] = J;
                            shifts[3 * np] = ix; shifts[3 * np + 1] = iy; shifts[3 * np + 2] = iz;
                        }
                        np++;
                    }
                }
            }
        }
    }
    *out_npairs = np;
    free(w); free(col); free(cnt); free(start); free(clstart); free(keys); free(fill);
    free(bb); free(catoms);
    return 0;
}

int orc_nblist_build(const double *x, const double *y, const double *z, int natom, double lx,
                     double ly, double lz, double rlist, int *out_ncl, int *cluster_atoms,
                     int cluster_cap, long long *out_npairs, int *pairs, int *shifts,
                     long long pair_cap) {
    double vol = lx * ly * lz;
    double cw = fmin(cbrt(8.0 * vol / natom), 0.75 * rlist);
    int ncx = (int)floor(lx / cw), ncy = (int)floor(ly / cw);
    if (ncx < 1) ncx = 1;
    if (ncy < 1) ncy = 1;
    int small = lx < 2.0 * rlist + 2.0 * (lx / ncx) || ly < 2.0 * rlist + 2.0 * (ly / ncy) ||
                lz < 2.0 * rlist + 2.0 * cw;
    return orc_nblist_build2(x, y, z, natom, lx, ly, lz, rlist, ncx, ncy, small, cw, out_ncl, cluster_atoms,
                             cluster_cap, out_npairs, pairs, shifts, pair_cap);
}
