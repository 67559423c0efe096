/*
 * mspms_oracle.h - CPU restatement of the mspms2 force layer (TEST INFRASTRUCTURE).
 *
 * This is the checker for the GPU engine, never part of the product path: only
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm load it.
 * It restates, in plain scalar FP64 C with the reference's loop and operation order,
 *   frclong()  src/frclong.c:20-1233 (with the self-pair fix of src/frclong.c:86),
 *   frcshort() src/frcshort.c:20-91 and the bonded kernels,
 *   the pair kernels of src/ljfrc.c and src/elecfrc.c,
 *   the solid-fluid models of src/sffrc.c,
 *   the Tasos tricubic Hermite library (mylibtasos/forces.f90:6-173,
 *   cubicinterpolation.f90:9-116, cubicauxiliary.f90, pbc.f90:69-85),
 * and a CPU cluster-pair list builder that must agree bit-for-bit with the GPU one.
 * Parity of the restatement itself is pinned against the compiled reference
 * (oracle/_ref, built by oracle/build_ref.sh) through tests/golden.
 */
#ifndef MSPMS_ORACLE_H_
#define MSPMS_ORACLE_H_

#include "../include/mspms2_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_tasos {
    int nx, ny, nz;          /* nodes per axis (ngx+2 ...) */
    double hx, hy, hz, cuc;
    const double *values;    /* [nz][ny][nx][8] */
    double min_pe;           /* min of F over the nodes (mylibtasos/grid.f90:97) */
} orc_tasos;

typedef struct orc_myinterp {
    int ncx, ncy, ncz;
    double itvl_x, itvl_y, itvl_z, xmin, ymin, zmax;
    const double *coeff;     /* [4][32][ncube] */
} orc_myinterp;

typedef struct orc_system {
    int nspecies;
    const mg_species *sp;
    mg_params p;
    double lx, ly, lz;
    /* solid-fluid */
    int ntasos;                   /* tables 1..ntasos in tasos[0..ntasos-1] */
    const orc_tasos *tasos;
    int ntube;
    const double *tube_x, *tube_y, *tube_r;
    double solid_sigma, solid_epsilon, const_3pisq_theta;
    int nsolid;
    const double *solid_x, *solid_y, *solid_z;
    int nmyinterp;
    const orc_myinterp *myinterp;
} orc_system;

/* Work window for bounded CPU-baseline samples: only i-molecules in
 * [imol_begin, imol_end) of the inter-molecular loop and only every k_stride-th
 * reciprocal vector are evaluated. A zeroed struct (or NULL) means the full call. */
typedef struct orc_window {
    int imol_begin, imol_end;
    int k_stride;
    int skip_intra;
    int k_offset; /* with k_stride > 1: the k-vectors numbered k_offset mod k_stride */
} orc_window;

int orc_natom(const orc_system *s);
/* frclong(): forces into f{x,y,z}l (overwritten), energies into e. Returns a flag word:
 * bit 0 = a site left a Tasos/my-interp table. */
int orc_frclong(const orc_system *s, const double *x, const double *y, const double *z,
                double *fxl, double *fyl, double *fzl, mg_energies *e, const orc_window *w);
/* orc_frclong on nthreads host threads (pair rows and k-vectors shared out, per-thread
 * partial sums added in thread order); the result differs from the serial call only by the
 * order of the sums. slice/nslices = 0/1 is the full call; slice k of n > 1 evaluates the
 * k-th of n equal shares of the pair rows and the k-vectors numbered k mod n (the O(N) terms
 * in slice 0 only), so the slices' forces sum to the full call. Returns the flag word of orc_frclong, or -1 for a bad slice. */
int orc_frclong_mt(const orc_system *s, const double *x, const double *y, const double *z,
                   double *fxl, double *fyl, double *fzl, mg_energies *e, int nthreads, int slice,
                   int nslices);
int orc_frcshort(const orc_system *s, const double *x, const double *y, const double *z,
                 double *fxs, double *fys, double *fzs, mg_energies *e);
/* Count of inter-molecular site pairs (different molecules, neither GHOST_FULL) with
 * MIC distance^2 < r2 (FP64), counted once. */
long long orc_count_pairs(const orc_system *s, const double *x, const double *y,
                          const double *z, double r2);

/* Scalar pair kernels with the reference's signatures and formulas. */
void orc_ljfrc(const mg_params *p, double rijsq, double sigmaij, double epsilonij,
               double *uij, double *fij, double *uijshift);
void orc_ewald_real(const mg_params *p, double rijsq, double chargeij, double *uij, double *fij);
void orc_ewald_excl(const mg_params *p, double rijsq, double chargeij, double *uij, double *fij);
void orc_wolf_real(const mg_params *p, double rijsq, double chargeij, double *uij, double *fij);

/* Tasos CForce_atom for 1-based AtomID; x,y,z in A. Returns 0 or -9999 (out of grid).
 * pe in K, force in K/A. */
int orc_tasos_force(const orc_tasos *g, unsigned compat, double x, double y, double z,
                    double *pe, double force[3]);
double orc_tasos_min_pe(const orc_tasos *g);

/* Integrators (md_oracle.c): nsteps of vver() (src/md.c:22-85) or vver_nh_3()
 * (src/nvtnh.c:11-271) as chosen by p->scheme, after one force evaluation at the start,
 * with the same arguments and per-step record as mg_md_run. Returns 0. */
int orc_md_run(const orc_system *s, const mg_md_params *p, int nsteps, double *x, double *y, double *z,
               double *vx, double *vy, double *vz, mg_md_state *state, double *log);

/* One replica of mg_hmc_batch: nmoves canonical moves of the reference's hmc()
 * (velinit with the Philox streams of include/mg_philox.h, frclong, md_move over vver,
 * the Metropolis test of src/dispmd.c:48-66). Same outputs as mg_hmc_batch for that
 * replica. Returns 0. */
int orc_hmc_replica(const orc_system *s, const mg_hmc_params *p, int replica, int move0, int nmoves, double *x,
                    double *y, double *z, int *accepted, double *dh_log, double *energy);

/* The velocities mg_hmc_batch draws for move `move` of replica `replica` (velinit with the
 * Philox streams, the momentum removed, rescaled with hp->rescale), for n sites. */
int orc_hmc_velocities(const mg_hmc_params *hp, int replica, int move, int n, double *vx, double *vy, double *vz);
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
int orc_npt_run(const orc_system *s, const mg_npt_params *p, int nsteps, double *x, double *y, double *z,
                double *vx, double *vy, double *vz, double *box, mg_npt_state *st, double *log);
int orc_siman_run(const orc_system *s, const mg_siman_params *p, double *x, double *y, double *z, double *vx,
                  double *vy, double *vz, mg_md_state *st, int *nstages, double *stage_log);

/* CPU cluster-pair builder (same predicate, same op order as the GPU build); the
 * second form takes the column grid and small-box choice of the build under test. */
int orc_nblist_build(const double *x, const double *y, const double *z, int natom,
                     double lx, double ly, double lz, double rlist,
                     int *out_ncl, int *cluster_atoms, int cluster_cap,
                     long long *out_npairs, int *pairs, int *shifts, long long pair_cap);
int orc_nblist_build2(const double *x, const double *y, const double *z, int natom, double lx,
                      double ly, double lz, double rlist, int ncx, int ncy, int small, double zcap, int *out_ncl,
                      int *cluster_atoms, int cluster_cap, long long *out_npairs, int *pairs,
                      int *shifts, long long pair_cap);

#ifdef __cplusplus
}
#endif
#endif
