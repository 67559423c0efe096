/*
 * mspms_oracle.c - CPU restatement of the mspms2 force layer (TEST INFRASTRUCTURE:
 * the checker the GPU engine is compared with; it never runs on the product path).
 *
 * Arithmetic follows the reference expression by expression (FP64, same loop order,
 * same accumulation order), so that on the same inputs it reproduces the compiled
 * reference to the last few ulps. Build with -ffp-contract=off.
 *
 * Deviations from the reference, each forced by undefined behaviour there:
 *  - inter-molecular j start: the reference's src/frclong.c:86 pairs a molecule with
 *    itself for iMole >= 1 (NaN for any species with >= 3 molecules); here j starts at
 *    molecule iMole+1, which is what the loop bounds at :88 intend.
 *  - bonded terms of type NONE contribute nothing (the reference adds an uninitialised
 *    local, src/bndfrc.c:140-141, src/aglfrc.c:53-54, src/dihfrc.c:57-58, src/impfrc.c:47-48).
 *  - isSameMole starts as true (the reference leaves it uninitialised, src/frclong.c:224).
 *  - a solid-fluid site outside its table contributes nothing and raises flag bit 0
 *    (the reference keeps the previous site's values, src/frclong.c:1185-1189).
 */
#include "mspms_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.141592653589793      /* src/defs.h:203 */
#define ORC_R_RGAS 0.120272219        /* src/defs.h:201 */

static inline double mic(double d, double L) { return d - L * rint(d / L); }

int orc_natom(const orc_system *s) {
    int n = 0;
    for (int i = 0; i < s->nspecies; i++) n += s->sp[i].natom * s->sp[i].nmole;
    return n;
}

/* ---- pair kernels: src/ljfrc.c:21-71, src/elecfrc.c:17-60, :230-241 ---------------- */
void orc_ljfrc(const mg_params *p, double rijsq, double sigmaij, double epsilonij,
               double *uij, double *fij, double *uijshift) {
    double sw = 1.0;
    if (p->lj_switch && !(rijsq < p->rcutonsq)) {
        double a = p->rcutoffsq - rijsq;
        sw = a * a * (p->rcutoffsq + 2.0 * rijsq - 3.0 * p->rcutonsq) / p->roff2_minus_ron2_cube;
    }
    double rinv2 = 1.0 / rijsq;
    double s2 = sigmaij * sigmaij;
    double s6 = s2 * rinv2;
    s6 = s6 * s6 * s6;
    double s12 = s6 * s6;
    *uij = 4.0 * epsilonij * (s12 - s6);
    if (p->lj_switch) {
        if (rijsq < p->rcutonsq) {
            *fij = 24.0 * epsilonij * (2 * s12 - s6) * rinv2;
        } else {
            *fij = 24.0 * epsilonij * (2 * s12 - s6) * rinv2 * sw -
                   *uij * 12.0 * (p->rcutoffsq - rijsq) * (p->rcutonsq - rijsq) /
                       p->roff2_minus_ron2_cube;
            *uij *= sw;
        }
        *uijshift = 0.0;
    } else {
        *fij = 24.0 * epsilonij * (2 * s12 - s6) * rinv2;
        double sg6 = s2 * s2 * s2;
        *uijshift = epsilonij * sg6 * (sg6 * p->shift1 - 1.0);
    }
}

void orc_ewald_real(const mg_params *p, double rijsq, double chargeij, double *uij, double *fij) {
    double r = sqrt(rijsq);
    double bare = p->coulomb_prefactor * chargeij / r;
    *uij = bare * erfc(p->kappa * r);
    double kr = p->kappa * r;
    double damped = bare * erfc(kr);
    *fij = (damped + bare * 2.0 * kr * exp(-kr * kr) / sqrt(ORC_PI)) / rijsq;
}

void orc_ewald_excl(const mg_params *p, double rijsq, double chargeij, double *uij, double *fij) {
    double r = sqrt(rijsq);
    *uij = p->coulomb_prefactor * chargeij / r;
    *fij = -*uij / rijsq;
}

void orc_wolf_real(const mg_params *p, double rijsq, double chargeij, double *uij, double *fij) {
    double r = sqrt(rijsq);
    *uij = p->coulomb_prefactor * chargeij *
           (erfc(p->kappa * r) / r + p->wolfvcon1 + p->wolfvcon2 * (r - p->rcutoffelec));
    *fij = p->coulomb_prefactor * (chargeij / r) *
           (erfc(p->kappa * r) / rijsq + p->wolffcon1 * exp(-(p->kappa * r) * (p->kappa * r)) / r +
            p->wolffcon2);
}

static void orc_plain_coulomb(const mg_params *p, double rijsq, double chargeij, double *uij,
                              double *fij) {
    double r = sqrt(rijsq);
    *uij = p->coulomb_prefactor * chargeij / r;
    *fij = *uij / rijsq;
}

/* ---- accumulation helpers ------------------------------------------------------ */
typedef struct acc {
    double *fx, *fy, *fz;
    mg_energies *e;
} acc;

static inline void add_pair_force(acc *a, int ii, int jj, double fij, double rx, double ry,
                                  double rz) {
    double fxij = fij * rx, fyij = fij * ry, fzij = fij * rz;
    a->fx[ii] += fxij; a->fy[ii] += fyij; a->fz[ii] += fzij;
    a->fx[jj] -= fxij; a->fy[jj] -= fyij; a->fz[jj] -= fzij;
}

/* ---- plain Coulomb between two molecules, centre-of-mass cutoff
 *      (src/elecfrc.c:138-225, src/misc.c:72-103) --------------------------------------- */
static void mole_com(const mg_species *S, const double *x, const double *y, const double *z,
                     int iabs, double com[3], double *ex, double *fy, double *gz) {
    double mw = 0.0;
    for (int a = 0; a < S->natom; a++) mw += S->aw[a];
    com[0] = com[1] = com[2] = 0.0;
    for (int a = 0; a < S->natom; a++) {
        com[0] += x[iabs + a] * S->aw[a];
        com[1] += y[iabs + a] * S->aw[a];
        com[2] += z[iabs + a] * S->aw[a];
    }
    com[0] /= mw; com[1] /= mw; com[2] /= mw;
    for (int a = 0; a < S->natom; a++) {
        ex[iabs + a] = x[iabs + a] - com[0];
        fy[iabs + a] = y[iabs + a] - com[1];
        gz[iabs + a] = z[iabs + a] - com[2];
    }
}

static void xmole_coulomb(const orc_system *s, const mg_species *Si, int iabs,
                          const mg_species *Sj, int jabs, const double *x, const double *y,
                          const double *z, double *ex, double *fy, double *gz, acc *a) {
    const mg_params *p = &s->p;
    double ci[3], cj[3];
    mole_com(Si, x, y, z, iabs, ci, ex, fy, gz);
    mole_com(Sj, x, y, z, jabs, cj, ex, fy, gz);
    double rxcm = mic(ci[0] - cj[0], s->lx);
    double rycm = mic(ci[1] - cj[1], s->ly);
    double rzcm = mic(ci[2] - cj[2], s->lz);
    double rcmsq = rxcm * rxcm + rycm * rycm + rzcm * rzcm;
    if (!(rcmsq < p->rcutoffelecsq)) return;
    for (int m = 0; m < Si->natom; m++) {
        if (Si->ghost_type[m] == MG_GHOST_FULL) continue;
        int ii = iabs + m;
        for (int n = 0; n < Sj->natom; n++) {
            if (Sj->ghost_type[n] == MG_GHOST_FULL) continue;
            int jj = jabs + n;
            double rx = ex[ii] + rxcm - ex[jj];
            double ry = fy[ii] + rycm - fy[jj];
            double rz = gz[ii] + rzcm - gz[jj];
            double rsq = rx * rx + ry * ry + rz * rz;
            double r = sqrt(rsq);
            double u = p->coulomb_prefactor * Si->charge[m] * Sj->charge[n] / r;
            a->e->uelec += u;
            a->e->virial_inter += u;
            add_pair_force(a, ii, jj, u / rsq, rx, ry, rz);
        }
    }
}

/* ---- inter-molecular site pairs (src/frclong.c:52-220) ----------------------------- */
static void inter_pairs(const orc_system *s, const double *x, const double *y, const double *z,
                        acc *a, const orc_window *w, double *ex, double *fy, double *gz) {
    const mg_params *p = &s->p;
    int isum_atom = 0, isum_mole = 0;
    for (int is = 0; is < s->nspecies; is++) {
        const mg_species *Si = &s->sp[is];
        int jsum_atom = isum_atom, jsum_mole = isum_mole;
        for (int js = is; js < s->nspecies; js++) {
            const mg_species *Sj = &s->sp[js];
            int same = (is == js);
            int iabs = isum_atom;
            for (int im = 0; im < Si->nmole; im++, iabs += Si->natom) {
                int gmol = isum_mole + im;
                if (w && w->imol_end > w->imol_begin &&
                    (gmol < w->imol_begin || gmol >= w->imol_end))
                    continue;
                int jm0 = same ? im + 1 : 0;
                int jabs = same ? iabs + Sj->natom : jsum_atom;
                for (int jm = jm0; jm < Sj->nmole; jm++, jabs += Sj->natom) {
                    for (int m = 0; m < Si->natom; m++) {
                        if (Si->ghost_type[m] == MG_GHOST_FULL) continue;
                        int ii = iabs + m;
                        for (int n = 0; n < Sj->natom; n++) {
                            if (Sj->ghost_type[n] == MG_GHOST_FULL) continue;
                            int jj = jabs + n;
                            double rx = mic(x[ii] - x[jj], s->lx);
                            double ry = mic(y[ii] - y[jj], s->ly);
                            double rz = mic(z[ii] - z[jj], s->lz);
                            double rsq = rx * rx + ry * ry + rz * rz;
                            double u, f, us;
                            if (Si->ghost_type[m] != MG_GHOST_LJ && Sj->ghost_type[n] != MG_GHOST_LJ &&
                                rsq < p->rcutoffsq) {
                                double sig = 0.5 * (Si->sigma[m] + Sj->sigma[n]);
                                double eps = sqrt(Si->epsilon[m] * Sj->epsilon[n]);
                                orc_ljfrc(p, rsq, sig, eps, &u, &f, &us);
                                a->e->uvdw += u;
                                a->e->ushift += us;
                                a->e->virial_inter += f * rsq;
                                add_pair_force(a, ii, jj, f, rx, ry, rz);
                            }
                            if (p->charge_type != MG_ELEC_NONE) {
                                double qq = Si->charge[m] * Sj->charge[n];
                                if (p->charge_type == MG_ELEC_EWALD) {
                                    if (rsq < p->rcutoffelecsq) {
                                        orc_ewald_real(p, rsq, qq, &u, &f);
                                        a->e->ureal += u;
                                        add_pair_force(a, ii, jj, f, rx, ry, rz);
                                    }
                                } else if (p->charge_type == MG_ELEC_WOLF) {
                                    if (rsq < p->rcutoffelecsq) {
                                        orc_wolf_real(p, rsq, qq, &u, &f);
                                        a->e->ureal += u;
                                        a->e->virial_inter += f * rsq;
                                        add_pair_force(a, ii, jj, f, rx, ry, rz);
                                    }
                                }
                            }
                        }
                    }
                    if (p->charge_type == MG_ELEC_SIMPLE_COULOMB)
                        xmole_coulomb(s, Si, iabs, Sj, jabs, x, y, z, ex, fy, gz, a);
                }
            }
            jsum_atom += Sj->natom * Sj->nmole;
            jsum_mole += Sj->nmole;
        }
        isum_atom += Si->natom * Si->nmole;
        isum_mole += Si->nmole;
    }
}

long long orc_count_pairs(const orc_system *s, const double *x, const double *y,
                          const double *z, double r2) {
    long long cnt = 0;
    int n = orc_natom(s);
    int *mol = (int *)malloc(sizeof(int) * (size_t)n);
    int *ghost = (int *)malloc(sizeof(int) * (size_t)n);
    int a = 0, gm = 0;
    for (int is = 0; is < s->nspecies; is++)
        for (int im = 0; im < s->sp[is].nmole; im++, gm++)
            for (int m = 0; m < s->sp[is].natom; m++, a++) {
                mol[a] = gm;
                ghost[a] = s->sp[is].ghost_type[m];
            }
    for (int i = 0; i < n; i++) {
        if (ghost[i] == MG_GHOST_FULL) continue;
        for (int j = i + 1; j < n; j++) {
            if (ghost[j] == MG_GHOST_FULL || mol[j] == mol[i]) continue;
            double rx = mic(x[i] - x[j], s->lx);
            double ry = mic(y[i] - y[j], s->ly);
            double rz = mic(z[i] - z[j], s->lz);
            if (rx * rx + ry * ry + rz * rz < r2) cnt++;
        }
    }
    free(mol);
    free(ghost);
    return cnt;
}

/* ---- intra-molecular nonbonded corrections (src/frclong.c:222-982) ------------------ */
/* One 1-2 or 1-3 end pair (bond loop :233-409, angle loop :412-593). */
static void intra_excluded(const orc_system *s, const mg_species *S, int m, int n, int ii,
                           int jj, const double *x, const double *y, const double *z, acc *a,
                           int *isSameMole) {
    const mg_params *p = &s->p;
    double rx = x[ii] - x[jj], ry = y[ii] - y[jj], rz = z[ii] - z[jj];
    double u, f, us, rsq;
    if (fabs(rx) > s->lx * 0.5 || fabs(ry) > s->ly * 0.5 || fabs(rz) > s->lz * 0.5) {
        *isSameMole = 0;
        if (S->ghost_type[m] == MG_GHOST_FULL || S->ghost_type[n] == MG_GHOST_FULL) return;
    } else {
        *isSameMole = 1;
    }
    if (!*isSameMole) {
        /* the saved vector goes through an int (src/frclong.c:223, :278-280) */
        int rxo = (int)rx, ryo = (int)ry, rzo = (int)rz;
        rx = mic(rx, s->lx); ry = mic(ry, s->ly); rz = mic(rz, s->lz);
        rsq = rx * rx + ry * ry + rz * rz;
        if (S->ghost_type[m] != MG_GHOST_LJ && S->ghost_type[n] != MG_GHOST_LJ && rsq < p->rcutoffsq) {
            double sig = 0.5 * (S->sigma[m] + S->sigma[n]);
            double eps = sqrt(S->epsilon[m] * S->epsilon[n]);
            orc_ljfrc(p, rsq, sig, eps, &u, &f, &us);
            a->e->uvdw += u;
            a->e->virial_inter += f * rsq;
            add_pair_force(a, ii, jj, f, rx, ry, rz);
        }
        rx = rxo; ry = ryo; rz = rzo;
    }
    if (p->charge_type == MG_ELEC_EWALD || p->charge_type == MG_ELEC_WOLF) {
        int wolf = (p->charge_type == MG_ELEC_WOLF);
        double qq = S->charge[m] * S->charge[n];
        rsq = rx * rx + ry * ry + rz * rz;
        if (rsq < p->rcutoffelecsq) {
            orc_ewald_excl(p, rsq, qq, &u, &f);
            a->e->uexcl += u;
            if (wolf) a->e->virial_inter += f * rsq;
            add_pair_force(a, ii, jj, f, rx, ry, rz);
        }
        rx = mic(rx, s->lx); ry = mic(ry, s->ly); rz = mic(rz, s->lz);
        rsq = rx * rx + ry * ry + rz * rz;
        if (rsq < p->rcutoffelecsq) {
            if (wolf) {
                orc_wolf_real(p, rsq, qq, &u, &f);
                a->e->virial_inter += f * rsq;
            } else {
                orc_ewald_real(p, rsq, qq, &u, &f);
            }
            a->e->ureal += u;
            add_pair_force(a, ii, jj, f, rx, ry, rz);
        }
    }
}

/* One 1-4 end pair (dihedral loop :597-787, eps scaled by f0) or nbp pair
 * (:791-977, eps unscaled). isSameMole is read, never written, here: the
 * reference's "isSameMole == ..." statements at :622, :632, :813, :823 are no-ops. */
static void intra_14(const orc_system *s, const mg_species *S, int m, int n, int ii, int jj,
                     const double *x, const double *y, const double *z, acc *a, double epsscale,
                     int isSameMole) {
    const mg_params *p = &s->p;
    double rx = x[ii] - x[jj], ry = y[ii] - y[jj], rz = z[ii] - z[jj];
    double u, f, us, rsq;
    if (fabs(rx) > s->lx * 0.5 || fabs(ry) > s->ly * 0.5 || fabs(rz) > s->lz * 0.5) {
        if (S->ghost_type[m] == MG_GHOST_FULL || S->ghost_type[n] == MG_GHOST_FULL) return;
    }
    if (!isSameMole) {
        int rxo = (int)rx, ryo = (int)ry, rzo = (int)rz;
        rx = mic(rx, s->lx); ry = mic(ry, s->ly); rz = mic(rz, s->lz);
        rsq = rx * rx + ry * ry + rz * rz;
        if (S->ghost_type[m] != MG_GHOST_LJ && S->ghost_type[n] != MG_GHOST_LJ && rsq < p->rcutoffsq) {
            double sig = 0.5 * (S->sigma[m] + S->sigma[n]);
            double eps = sqrt(S->epsilon[m] * S->epsilon[n]);
            orc_ljfrc(p, rsq, sig, eps, &u, &f, &us);
            a->e->uvdw += u;
            a->e->virial_inter += f * rsq;
            add_pair_force(a, ii, jj, f, rx, ry, rz);
        }
        rx = rxo; ry = ryo; rz = rzo;
    } else {
        rsq = rx * rx + ry * ry + rz * rz;
        if (rsq < p->rcutoffsq) {
            double sig = 0.5 * (S->sigma[m] + S->sigma[n]);
            double eps = epsscale * sqrt(S->epsilon[m] * S->epsilon[n]);
            orc_ljfrc(p, rsq, sig, eps, &u, &f, &us);
            a->e->uvdw += u;
            a->e->virial_inter += f * rsq;
            add_pair_force(a, ii, jj, f, rx, ry, rz);
        }
    }
    if (p->charge_type == MG_ELEC_NONE) return;
    double qq = S->charge[m] * S->charge[n];
    rx = mic(rx, s->lx); ry = mic(ry, s->ly); rz = mic(rz, s->lz);
    rsq = rx * rx + ry * ry + rz * rz;
    if (!(rsq < p->rcutoffelecsq)) return;
    if (p->charge_type == MG_ELEC_EWALD) {
        orc_ewald_real(p, rsq, qq, &u, &f);
        a->e->ureal += u;
    } else if (p->charge_type == MG_ELEC_WOLF) {
        orc_wolf_real(p, rsq, qq, &u, &f);
        a->e->ureal += u;
        a->e->virial_inter += f * rsq;
    } else {
        orc_plain_coulomb(p, rsq, qq, &u, &f);
        a->e->uelec += u;
        a->e->virial_inter += f * rsq;
    }
    add_pair_force(a, ii, jj, f, rx, ry, rz);
}

/* Reference uniqueness flags (src/initvars.c:13-146), including its index use: a
 * dihedral/angle that shares end atoms with an angle/bond clears the flag of the entry
 * whose index equals the angle/bond index (:66, :86, :134). */
static void unique_flags(const mg_species *S, unsigned char *dih_u, unsigned char *agl_u) {
    int ndu = S->ndih > 0 ? S->ndih : 0;
    int nau = S->nangle > 0 ? S->nangle : 0;
    for (int i = 0; i < ndu; i++) dih_u[i] = 1;
    for (int i = 0; i < S->ndih - 1; i++) {
        if (!dih_u[i]) continue;
        for (int j = i + 1; j < S->ndih; j++) {
            if (!dih_u[j]) continue;
            const int *di = S->dih_idx + 4 * i, *dj = S->dih_idx + 4 * j;
            if ((di[0] == dj[0] && di[3] == dj[3]) || (di[0] == dj[3] && di[3] == dj[0])) dih_u[j] = 0;
        }
    }
    for (int i = 0; i < S->ndih; i++) {
        if (!dih_u[i]) continue;
        const int *di = S->dih_idx + 4 * i;
        for (int j = 0; j < S->nangle; j++) {
            const int *aj = S->angle_idx + 3 * j;
            if ((di[0] == aj[0] && di[3] == aj[2]) || (di[0] == aj[2] && di[3] == aj[0]))
                if (j < ndu) dih_u[j] = 0;
        }
    }
    for (int i = 0; i < S->ndih; i++) {
        if (!dih_u[i]) continue;
        const int *di = S->dih_idx + 4 * i;
        for (int j = 0; j < S->nbond; j++) {
            const int *bj = S->bond_idx + 2 * j;
            if ((di[0] == bj[0] && di[3] == bj[1]) || (di[0] == bj[1] && di[3] == bj[0]))
                if (j < ndu) dih_u[j] = 0;
        }
    }
    for (int i = 0; i < nau; i++) agl_u[i] = 1;
    for (int i = 0; i < S->nangle - 1; i++) {
        if (!agl_u[i]) continue;
        for (int j = i + 1; j < S->nangle; j++) {
            if (!agl_u[j]) continue;
            const int *ai = S->angle_idx + 3 * i, *aj = S->angle_idx + 3 * j;
            if ((ai[0] == aj[0] && ai[2] == aj[2]) || (ai[0] == aj[2] && ai[2] == aj[0])) agl_u[j] = 0;
        }
    }
    for (int i = 0; i < S->nangle; i++) {
        if (!agl_u[i]) continue;
        const int *ai = S->angle_idx + 3 * i;
        for (int j = 0; j < S->nbond; j++) {
            const int *bj = S->bond_idx + 2 * j;
            if ((ai[0] == bj[0] && ai[2] == bj[1]) || (ai[0] == bj[1] && ai[2] == bj[0]))
                if (j < nau) agl_u[j] = 0;
        }
    }
}

static void intra_pairs(const orc_system *s, const double *x, const double *y, const double *z,
                        acc *a) {
    int isum_atom = 0;
    int isSameMole = 1;
    for (int is = 0; is < s->nspecies; is++) {
        const mg_species *S = &s->sp[is];
        unsigned char dih_u[256], agl_u[256];
        unique_flags(S, dih_u, agl_u);
        for (int im = 0; im < S->nmole; im++, isum_atom += S->natom) {
            for (int b = 0; b < S->nbond; b++) {
                int m = S->bond_idx[2 * b], n = S->bond_idx[2 * b + 1];
                intra_excluded(s, S, m, n, isum_atom + m, isum_atom + n, x, y, z, a, &isSameMole);
            }
            for (int g = 0; g < S->nangle; g++) {
                if (!agl_u[g]) continue;
                int m = S->angle_idx[3 * g], n = S->angle_idx[3 * g + 2];
                intra_excluded(s, S, m, n, isum_atom + m, isum_atom + n, x, y, z, a, &isSameMole);
            }
            for (int d = 0; d < S->ndih; d++) {
                if (!dih_u[d]) continue;
                int m = S->dih_idx[4 * d], n = S->dih_idx[4 * d + 3];
                intra_14(s, S, m, n, isum_atom + m, isum_atom + n, x, y, z, a, s->p.f0, isSameMole);
            }
            for (int q = 0; q < S->nnbp; q++) {
                int src = (s->p.compat & MG_COMPAT_NBP_INDEX) ? S->ndih : q;
                int m = 0, n = 0;
                if (src < S->nnbp) { m = S->nbp_idx[2 * src]; n = S->nbp_idx[2 * src + 1]; }
                intra_14(s, S, m, n, isum_atom + m, isum_atom + n, x, y, z, a, 1.0, isSameMole);
            }
        }
    }
}

/* ---- per-site lookup --------------------------------------------------------------- */
static void site_of(const orc_system *s, int abs, int *spec, int *rel) {
    int base = 0;
    for (int i = 0; i < s->nspecies; i++) {
        int cnt = s->sp[i].natom * s->sp[i].nmole;
        if (abs < base + cnt) {
            *spec = i;
            *rel = (abs - base) % s->sp[i].natom;
            return;
        }
        base += cnt;
    }
    *spec = 0;
    *rel = 0;
}

/* ---- Ewald reciprocal space, self term, vacuum dipole (src/frclong.c:988-1129) ----- */
static double *site_charges(const orc_system *s) {
    int n = orc_natom(s);
    double *q = (double *)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; i++) {
        int sp, rel;
        site_of(s, i, &sp, &rel);
        q[i] = s->sp[sp].charge[rel];
    }
    return q;
}

/* The k-vector loop of src/frclong.c:996-1046 over the vectors numbered koff mod stride:
 * adds the forces into a and returns sum_k kvec |S(k)|^2 (not yet scaled). */
static double kspace_loop(const orc_system *s, const double *x, const double *y, const double *z,
                          const double *q, acc *a, int stride, int koff) {
    const mg_params *p = &s->p;
    int n = orc_natom(s);
    long long kcount = 0;
    double ufourier = 0.0;
    for (int kx = -p->kmax[0]; kx <= p->kmax[0]; kx++)
        for (int ky = -p->kmax[1]; ky <= p->kmax[1]; ky++)
            for (int kz = -p->kmax[2]; kz <= p->kmax[2]; kz++) {
                int ksq = kx * kx + ky * ky + kz * kz;
                if (!(ksq <= p->ksqmax && ksq != 0)) continue;
                if ((kcount++ % stride) != koff) continue;
                double rkx = p->twopi_lx * kx, rky = p->twopi_ly * ky, rkz = p->twopi_lz * kz;
                double rksq = rkx * rkx + rky * rky + rkz * rkz;
                double kvec = exp(-p->bfactor_ewald * rksq) / rksq;
                double sr = 0.0, si = 0.0;
                for (int i = 0; i < n; i++) {
                    double t = rkx * x[i] + rky * y[i] + rkz * z[i];
                    sr = sr + q[i] * cos(t);
                    si = si + q[i] * sin(t);
                }
                ufourier += kvec * (sr * sr + si * si);
                for (int i = 0; i < n; i++) {
                    double t = rkx * x[i] + rky * y[i] + rkz * z[i];
                    double fij = 2.0 * q[i] * (sr * sin(t) - si * cos(t)) * p->vfactor_ewald * kvec *
                                 p->coulomb_prefactor;
                    a->fx[i] += fij * rkx;
                    a->fy[i] += fij * rky;
                    a->fz[i] += fij * rkz;
                }
            }
    return ufourier;
}

/* src/frclong.c:1047-1129 after the k-vector loop: scaled Fourier energy, self term,
 * uelec, vacuum dipole, the Ewald virial. */
static void ewald_tail(const orc_system *s, const double *x, const double *y, const double *z,
                       const double *q, acc *a, double ufourier) {
    const mg_params *p = &s->p;
    int n = orc_natom(s);
    ufourier *= p->vfactor_ewald * p->coulomb_prefactor;
    a->e->ufourier = ufourier;
    double uself = 0.0;
    for (int i = 0; i < n; i++) uself += q[i] * q[i];
    uself *= p->coulomb_prefactor * sqrt(p->kappa * p->kappa / ORC_PI);
    a->e->uself = uself;
    a->e->uelec = a->e->ureal + a->e->ufourier - a->e->uself - a->e->uexcl;
    if (p->ewald_bc == MG_EWALD_BC_VACUUM) {
        double *ex = (double *)malloc(sizeof(double) * (size_t)n * 3);
        double *fy = ex + n, *gz = ex + 2 * n;
        int base = 0;
        for (int is = 0; is < s->nspecies; is++) {
            const mg_species *S = &s->sp[is];
            for (int im = 0; im < S->nmole; im++, base += S->natom) {
                double com[3];
                mole_com(S, x, y, z, base, com, ex, fy, gz);
                com[0] -= s->lx * rint(com[0] / s->lx);
                com[1] -= s->ly * rint(com[1] / s->ly);
                com[2] -= s->lz * rint(com[2] / s->lz);
                for (int k = base; k < base + S->natom; k++) {
                    ex[k] = ex[k] + com[0];
                    fy[k] = fy[k] + com[1];
                    gz[k] = gz[k] + com[2];
                }
            }
        }
        double qrx = 0.0, qry = 0.0, qrz = 0.0;
        for (int i = 0; i < n; i++) {
            qrx = qrx + q[i] * ex[i];
            qry = qry + q[i] * fy[i];
            qrz = qrz + q[i] * gz[i];
        }
        double uvac = qrx * qrx + qry * qry + qrz * qrz;
        uvac *= p->twopi_over_3v * p->coulomb_prefactor;
        a->e->uvacuum = uvac;
        for (int i = 0; i < n; i++) {
            double fij = -2.0 * p->twopi_over_3v * q[i] * p->coulomb_prefactor;
            a->fx[i] += fij * qrx;
            a->fy[i] += fij * qry;
            a->fz[i] += fij * qrz;
        }
        a->e->uelec += uvac;
        free(ex);
    }
    a->e->virial_inter += a->e->uelec;
}

static void ewald_kspace(const orc_system *s, const double *x, const double *y, const double *z,
                         acc *a, const orc_window *w) {
    double *q = site_charges(s);
    int stride = (w && w->k_stride > 1) ? w->k_stride : 1;
    int koff = (w && stride > 1 && w->k_offset > 0) ? w->k_offset % stride : 0;
    double ufourier = kspace_loop(s, x, y, z, q, a, stride, koff);
    ewald_tail(s, x, y, z, q, a, ufourier);
    free(q);
}

/* ---- solid-fluid models ------------------------------------------------------------- */
/* hypergeometric series (src/sffrc.c:1092-1116) */
static void hypergeo_series(double a, double b, double c, double zz, double rr, double *sumV,
                            double *sumF) {
    double zn = 1.0, an1 = 1.0;
    *sumV = 1.0;
    *sumF = 0.0;
    for (int i = 0; i <= 10; i++) {
        double an = (a + i) * (b + i) / ((c + i) * (1 + i));
        an1 = an1 * an;
        zn *= zz;
        *sumV = *sumV + an1 * zn;
        *sumF = *sumF - 2.0 * (i + 1.0) * an1 * zn / rr;
    }
}

/* cal_sf_hypergeo (src/sffrc.c:1120-1209): returns the energy term the caller adds */
static double sf_hypergeo(const orc_system *s, const mg_species *S, int rel, int ii,
                          const double *x, const double *y, acc *a) {
    double sig = 0.5 * (S->sigma[rel] + s->solid_sigma);
    double eps = sqrt(S->epsilon[rel] * s->solid_epsilon);
    double usum = 0.0, ulast = 0.0;
    double fxi = a->fx[ii], fyi = a->fy[ii];
    for (int t = 0; t < s->ntube; t++) {
        double rx = mic(x[ii] - s->tube_x[t], s->lx);
        double ry = mic(y[ii] - s->tube_y[t], s->ly);
        double rsq = rx * rx + ry * ry;
        double r = sqrt(rsq);
        double R = s->tube_r[t], Rsq = R * R;
        double hrep, hfrep, hatt, hfatt, u, f;
        if (r < R) {
            double ljc = s->const_3pisq_theta * eps * sig * sig;
            double k = sig * R / (Rsq - rsq);
            double zf = rsq / Rsq;
            hypergeo_series(-4.5, -4.5, 1.0, zf, r, &hrep, &hfrep);
            double k2 = k * k, k4 = k2 * k2, k10 = k4 * k4 * k2;
            double rep1 = 0.65625 * k10;
            double rep2 = -hfrep + hrep * (20.0 * r / (Rsq - rsq));
            hypergeo_series(-1.5, -1.5, 1.0, zf, r, &hatt, &hfatt);
            double att1 = -k4;
            double att2 = -hfatt + hatt * (8.0 * r / (Rsq - rsq));
            u = ljc * (rep1 * hrep + att1 * hatt);
            f = -ljc * (rep1 * rep2 + att1 * att2);
        } else {
            double ljc = s->const_3pisq_theta * eps * sig * sig * R;
            double k = sig * r / (rsq - Rsq);
            double zf = Rsq / rsq;
            hypergeo_series(-4.5, -4.5, 1.0, zf, r, &hrep, &hfrep);
            double k2 = k * k, k4 = k2 * k2, k10 = k4 * k4 * k2;
            double rep1 = 0.65625 * k10;
            double rep2 = hfrep / r + hrep * (-20.0 / (rsq - Rsq) + 9.0 / rsq);
            hypergeo_series(-1.5, -1.5, 1.0, zf, r, &hatt, &hfatt);
            double att1 = -k4;
            double att2 = hfatt / r + hatt * (-8.0 / (rsq - Rsq) + 3.0 / rsq);
            u = ljc * (rep1 * hrep + att1 * hatt) / r;
            f = -ljc * (rep1 * rep2 + att1 * att2);
        }
        fxi += f * rx / r;
        fyi += f * ry / r;
        ulast = u;
        usum += u;
    }
    a->fx[ii] = fxi;
    a->fy[ii] = fyi;
    return (s->p.compat & MG_COMPAT_HYPERGEO_LAST) ? ulast : usum;
}

/* cal_sf_atom_explicit (src/sffrc.c:1213-1314) */
static double sf_atom_explicit(const orc_system *s, const mg_species *S, int rel, int ii,
                               const double *x, const double *y, const double *z, acc *a) {
    const mg_params *p = &s->p;
    double sig = 0.5 * (S->sigma[rel] + s->solid_sigma);
    double eps = sqrt(S->epsilon[rel] * s->solid_epsilon);
    double usum = 0.0;
    double fxi = a->fx[ii], fyi = a->fy[ii], fzi = a->fz[ii];
    for (int j = 0; j < s->nsolid; j++) {
        double rx = mic(x[ii] - s->solid_x[j], s->lx);
        double ry = mic(y[ii] - s->solid_y[j], s->ly);
        double rz = mic(z[ii] - s->solid_z[j], s->lz);
        double rsq = rx * rx + ry * ry + rz * rz;
        if (!(rsq < p->rcutoffsq)) continue;
        double sw = 1.0;
        if (p->lj_switch && !(rsq < p->rcutonsq)) {
            double d = p->rcutoffsq - rsq;
            sw = d * d * (p->rcutoffsq + 2.0 * rsq - 3.0 * p->rcutonsq) / p->roff2_minus_ron2_cube;
        }
        double s2 = sig * sig / rsq;
        double s6 = s2 * s2 * s2;
        double s12 = s6 * s6;
        double d12 = s12 - s6;
        double ut = eps * d12;
        double f;
        if (p->lj_switch) {
            usum += ut * sw;
            if (rsq < p->rcutonsq)
                f = 24.0 * eps * (d12 + s12) / rsq;
            else
                f = 24.0 * eps * (d12 + s12) / rsq * sw -
                    4.0 * ut * 12.0 * (p->rcutoffsq - rsq) * (p->rcutonsq - rsq) / p->roff2_minus_ron2_cube;
        } else {
            usum += ut;
            f = 24.0 * eps * (d12 + s12) / rsq;
        }
        fxi += f * rx;
        fyi += f * ry;
        fzi += f * rz;
    }
    a->fx[ii] = fxi;
    a->fy[ii] = fyi;
    a->fz[ii] = fzi;
    return usum * 4.0;
}

/* ---- Tasos CForce_atom restated (mylibtasos/forces.f90:6-173) -------------------------- */
/* Hermite basis on the unit interval, scaled as in cubicauxiliary.f90:76-130:
 * V0 weight of the lower node value, V1 of the upper, D0/D1 of the node derivatives
 * (already multiplied by the spacing h); primes are d/dx in A^-1. */
typedef struct herm1 { double v0, v1, d0, d1, v0p, v1p, d0p, d1p; } herm1;

static herm1 herm_basis(double t, double h) {
    herm1 b;
    b.v1 = -(t * t * (2.0 * t - 3.0));          /* -f(t) */
    b.v0 = t * t * (2.0 * t - 3.0) + 1;          /* g(t) */
    b.d0 = h * (t * (t - 1) * (t - 1));          /* hx*w(t) */
    double u = 1 - t;
    b.d1 = -h * (u * (u - 1) * (u - 1));         /* -hx*w(1-t) */
    b.v1p = -(6.0 * t * (t - 1.0)) / h;          /* -fprime/h */
    b.v0p = (6.0 * t * (t - 1.0)) / h;           /* gprime/h */
    b.d0p = t * (3.0 * t - 4.0) + 1.0;           /* w1prime */
    b.d1p = -(-t * (3.0 * t - 2.0));             /* -w2prime */
    return b;
}

double orc_tasos_min_pe(const orc_tasos *g) {
    double m = 10e10;
    long long nn = (long long)g->nx * g->ny * g->nz;
    for (long long i = 0; i < nn; i++)
        if (g->values[8 * i] < m) m = g->values[8 * i];
    return m;
}

int orc_tasos_force(const orc_tasos *g, unsigned compat, double X, double Y, double Z, double *pe,
                    double force[3]) {
    /* PBCuc case 2 (mylibtasos/pbc.f90:80-84): only z is periodic */
    double xp = X, yp = Y, zp = Z - floor(Z / g->cuc) * g->cuc;
    int I1 = (int)floor(xp / g->hx + 1), J1 = (int)floor(yp / g->hy + 1), K1 = (int)floor(zp / g->hz + 1);
    int ngx = g->nx - 2, ngy = g->ny - 2, ngz = g->nz - 2;
    /* the reference tests < 0 (forces.f90:59) but index 0 is outside its arrays too */
    if (I1 < 1 || J1 < 1 || K1 < 1) return -9999;
    if (I1 > ngx + 1 || J1 > ngy + 1 || K1 > ngz + 1) return -9999;
    double tx = (xp - (I1 - 1) * g->hx) / g->hx;
    double ty = (yp - (J1 - 1) * g->hy) / g->hy;
    double tz = (zp - (K1 - 1) * g->hz) / g->hz;
    herm1 bx = herm_basis(tx, g->hx), by = herm_basis(ty, g->hy), bz = herm_basis(tz, g->hz);
    int i0 = I1 - 1, j0 = J1 - 1, k0 = K1 - 1;
    double val = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
    for (int c = 0; c < 8; c++) {
        int ci = c & 1, cj = (c >> 1) & 1, ck = (c >> 2) & 1;
        const double *rec = g->values + 8 * (((long long)(k0 + ck) * g->ny + (j0 + cj)) * g->nx + (i0 + ci));
        /* per-axis weights for this corner: value weight and derivative weight */
        double wx = ci ? bx.v1 : bx.v0, dx = ci ? bx.d1 : bx.d0;
        double wy = cj ? by.v1 : by.v0, dy = cj ? by.d1 : by.d0;
        double wz = ck ? bz.v1 : bz.v0, dz = ck ? bz.d1 : bz.d0;
        double wxp = ci ? bx.v1p : bx.v0p, dxp = ci ? bx.d1p : bx.d0p;
        double wyp = cj ? by.v1p : by.v0p, dyp = cj ? by.d1p : by.d0p;
        double wzp = ck ? bz.v1p : bz.v0p, dzp = ck ? bz.d1p : bz.d0p;
        /* Dxyz: the reference pairs corner (0,0,1)'s value with corner (1,1,0)'s basis and
         * vice versa (cubicauxiliary.f90:225-226 against forces.f90:158-159) */
        int tci = ci, tcj = cj, tck = ck;
        if ((compat & MG_COMPAT_TASOS_DXYZ) && ((c == 4) || (c == 3))) {
            tci = 1 - ci; tcj = 1 - cj; tck = 1 - ck;
        }
        double txd = tci ? bx.d1 : bx.d0, tyd = tcj ? by.d1 : by.d0, tzd = tck ? bz.d1 : bz.d0;
        double txdp = tci ? bx.d1p : bx.d0p, tydp = tcj ? by.d1p : by.d0p, tzdp = tck ? bz.d1p : bz.d0p;
        double F = rec[0], Dx = rec[1], Dy = rec[2], Dz = rec[3];
        double Dxy = rec[4], Dxz = rec[5], Dyz = rec[6], Dxyz = rec[7];
        val += F * wx * wy * wz + Dx * dx * wy * wz + Dy * wx * dy * wz + Dz * wx * wy * dz +
               Dxy * dx * dy * wz + Dxz * dx * wy * dz + Dyz * wx * dy * dz + Dxyz * txd * tyd * tzd;
        gx += F * wxp * wy * wz + Dx * dxp * wy * wz + Dy * wxp * dy * wz + Dz * wxp * wy * dz +
              Dxy * dxp * dy * wz + Dxz * dxp * wy * dz + Dyz * wxp * dy * dz + Dxyz * txdp * tyd * tzd;
        gy += F * wx * wyp * wz + Dx * dx * wyp * wz + Dy * wx * dyp * wz + Dz * wx * wyp * dz +
              Dxy * dx * dyp * wz + Dxz * dx * wyp * dz + Dyz * wx * dyp * dz + Dxyz * txd * tydp * tzd;
        gz += F * wx * wy * wzp + Dx * dx * wy * wzp + Dy * wx * dy * wzp + Dz * wx * wy * dzp +
              Dxy * dx * dy * wzp + Dxz * dx * wy * dzp + Dyz * wx * dy * dzp + Dxyz * txd * tyd * tzdp;
    }
    force[0] = -gx;
    force[1] = -gy;
    force[2] = -gz;
    if ((compat & MG_COMPAT_TASOS_PE_FLIP) && val < 1.5 * g->min_pe)
        *pe = -val;
    else
        *pe = val;
    return 0;
}

/* get_values_from_grid (src/sffrc.c:951-1089): 32-term polynomial in absolute A */
static int sf_myinterp(const orc_myinterp *g, double fx, double fy, double fz, double *usf,
                       double fsf[3]) {
    int ax = (int)((fx - g->xmin) / g->itvl_x);
    int ay = (int)((fy - g->ymin) / g->itvl_y);
    fz = fz - g->zmax * rint(fz / g->zmax);
    if (fz < 0) fz = g->zmax + fz;
    int az = (int)((fz - 0.0) / g->itvl_z);
    long long ncube = (long long)g->ncx * g->ncy * g->ncz;
    long long cube = (long long)ax * g->ncy * g->ncz + (long long)ay * g->ncz + az;
    if (cube < 0 || cube >= ncube || ax < 0 || ay < 0 || az < 0) return -1;
    double x = fx, y = fy, z = fz;
    double x2 = x * x, x3 = x2 * x, y2 = y * y, y3 = y2 * y, z2 = z * z, z3 = z2 * z;
    double v[32] = {1.0, x, y, z, x2, x * y, x * z, y2, y * z, z2,
                    x3, x2 * y, x * y2, x2 * z, x * z2, y3, y2 * z, y * z2, z3, x * y * z,
                    x3 * y, x2 * y2, x * y3, x3 * z, x2 * z2, x * z3, y3 * z, y2 * z2, y * z3,
                    x2 * y * z, x * y2 * z, x * y * z2};
    double out[4];
    for (int q = 0; q < 4; q++) {
        const double *c = g->coeff + (size_t)q * 32 * ncube;
        double acc = c[cube] * v[0];
        for (int t = 1; t < 32; t++) acc = acc + c[(size_t)t * ncube + cube] * v[t];
        out[q] = acc;
    }
    *usf = out[0];
    fsf[0] = out[1];
    fsf[1] = out[2];
    fsf[2] = out[3];
    return 0;
}

static int solid_fluid(const orc_system *s, const double *x, const double *y, const double *z,
                       acc *a) {
    const mg_params *p = &s->p;
    int flags = 0;
    int n = orc_natom(s);
    double usf = 0.0;
    for (int i = 0; i < n; i++) {
        int sp, rel;
        site_of(s, i, &sp, &rel);
        const mg_species *S = &s->sp[sp];
        if (S->ghost_type[rel] != MG_GHOST_NONE) continue;
        if (p->sf_type == MG_SF_HYPERGEO) {
            usf += sf_hypergeo(s, S, rel, i, x, y, a);
        } else if (p->sf_type == MG_SF_ATOM_EXPLICIT) {
            usf += sf_atom_explicit(s, S, rel, i, x, y, z, a);
        } else if (p->sf_type == MG_SF_TASOS) {
            int t = S->interp_type[rel];
            double pe, f[3];
            if (t < 1 || t > s->ntasos ||
                orc_tasos_force(&s->tasos[t - 1], p->compat, x[i] * p->sigma_base,
                                y[i] * p->sigma_base, z[i] * p->sigma_base, &pe, f) != 0) {
                flags |= 1;
                continue;
            }
            usf += pe / p->epsilon_base;
            a->fx[i] += f[0] * (p->sigma_base / p->epsilon_base);
            a->fy[i] += f[1] * (p->sigma_base / p->epsilon_base);
            a->fz[i] += f[2] * (p->sigma_base / p->epsilon_base);
        } else if (p->sf_type == MG_SF_MY_INTERP) {
            int t = S->interp_type[rel];
            double u, f[3];
            if (t < 0 || t >= s->nmyinterp ||
                sf_myinterp(&s->myinterp[t], x[i] * p->sigma_base, y[i] * p->sigma_base,
                            z[i] * p->sigma_base, &u, f) != 0) {
                flags |= 1;
                continue;
            }
            usf += u * ORC_R_RGAS / p->epsilon_base;
            a->fx[i] += f[0] * ORC_R_RGAS * p->sigma_base / p->epsilon_base;
            a->fy[i] += f[1] * ORC_R_RGAS * p->sigma_base / p->epsilon_base;
            a->fz[i] += f[2] * ORC_R_RGAS * p->sigma_base / p->epsilon_base;
        }
    }
    a->e->usflj = usf;
    return flags;
}

/* ---- frclong ------------------------------------------------------------------------ */
int orc_frclong(const orc_system *s, const double *x, const double *y, const double *z,
                double *fxl, double *fyl, double *fzl, mg_energies *e, const orc_window *w) {
    int n = orc_natom(s);
    for (int i = 0; i < n; i++) fxl[i] = fyl[i] = fzl[i] = 0.0;
    e->uvdw = e->ushift = e->uelec = e->ureal = e->uexcl = e->virial_inter = 0.0;
    e->ufourier = e->uself = e->uvacuum = e->usflj = e->uotherff = 0.0;
    acc a = {fxl, fyl, fzl, e};
    double *com_scratch = (double *)calloc((size_t)n * 3 + 3, sizeof(double));
    inter_pairs(s, x, y, z, &a, w, com_scratch, com_scratch + n, com_scratch + 2 * n);
    if (!(w && w->skip_intra)) intra_pairs(s, x, y, z, &a);
    free(com_scratch);
    e->ushift *= s->p.shift4;
    if (s->p.charge_type == MG_ELEC_EWALD) {
        ewald_kspace(s, x, y, z, &a, w);
    } else if (s->p.charge_type == MG_ELEC_WOLF) {
        double q2 = 0.0;
        for (int i = 0; i < n; i++) {
            int sp, rel;
            site_of(s, i, &sp, &rel);
            q2 += s->sp[sp].charge[rel] * s->sp[sp].charge[rel];
        }
        e->uself = q2 * (s->p.coulomb_prefactor * s->p.wolfvcon3);
        e->uelec = e->ureal - e->uself - e->uexcl;
    }
    int flags = solid_fluid(s, x, y, z, &a);
    e->uotherff = 0.0;
    e->uinter = e->uvdw + e->uelec + e->usflj + e->uotherff;
    return flags;
}

/* ---- frclong on several host threads ------------------------------------------------
 * The same terms as orc_frclong, with the two O(N^2)-class loops shared out: the
 * inter-molecular pair rows (src/frclong.c:56-218) in contiguous ranges of equal pair count
 * and the k-vectors (src/frclong.c:996-1046) dealt round robin. Each thread accumulates into
 * its own force block and energies; the blocks are added in thread order, then the serial
 * remainder (intra-molecular corrections, Ewald tail, Wolf self, solid-fluid) runs as in
 * orc_frclong. Only the order of the sums differs from the serial call.
 * With nslices > 1 the call evaluates slice `slice` of that work: the slice-th of nslices
 * row ranges of equal pair count and the k-vectors numbered slice mod nslices (the O(N)
 * remainder runs in every slice). The nslices slices together do the pair and k-vector work
 * of one full call exactly once, so they time a full call in measured parts. */
typedef struct mt_job {
    const orc_system *s;
    const double *x, *y, *z, *q;
    int imol_begin, imol_end; /* pair rows (global molecule index of the i-molecule) */
    int kstride, koff;        /* k-vectors koff mod kstride; kstride 0: none */
    double *f;                /* [3][n] */
    double *scratch;          /* [3][n] COM offsets of the plain-Coulomb model */
    mg_energies e;
    double ufourier;
} mt_job;

static void *mt_run(void *arg) {
    mt_job *j = (mt_job *)arg;
    int n = orc_natom(j->s);
    acc a = {j->f, j->f + n, j->f + 2 * n, &j->e};
    if (j->imol_end > j->imol_begin) {
        orc_window w = {j->imol_begin, j->imol_end, 1, 1, 0};
        inter_pairs(j->s, j->x, j->y, j->z, &a, &w, j->scratch, j->scratch + n, j->scratch + 2 * n);
    }
    if (j->kstride > 0) j->ufourier = kspace_loop(j->s, j->x, j->y, j->z, j->q, &a, j->kstride, j->koff);
    return NULL;
}

int orc_frclong_mt(const orc_system *s, const double *x, const double *y, const double *z,
                   double *fxl, double *fyl, double *fzl, mg_energies *e, int nthreads, int slice, int nslices) {
    if (nslices < 1) nslices = 1;
    if (slice < 0 || slice >= nslices) return -1;
    int n = orc_natom(s), T = nthreads < 1 ? 1 : nthreads, M = 0;
    for (int i = 0; i < s->nspecies; i++) M += s->sp[i].nmole;
    /* site pairs each i-molecule row examines, and cuts at equal shares of their sum */
    double *cum = (double *)malloc(sizeof(double) * (size_t)(M + 1));
    cum[0] = 0.0;
    int g = 0;
    for (int is = 0; is < s->nspecies; is++) {
        const mg_species *Si = &s->sp[is];
        double later = 0.0;
        for (int js = is + 1; js < s->nspecies; js++) later += (double)s->sp[js].nmole * s->sp[js].natom;
        for (int im = 0; im < Si->nmole; im++, g++)
            cum[g + 1] = cum[g] + (double)Si->natom * ((double)(Si->nmole - im - 1) * Si->natom + later);
    }
    /* rows of this slice: the slice-th of nslices ranges of equal pair count; then T
     * ranges of equal pair count within it */
    int r0 = 0, r1 = M;
    {
        double lo = cum[M] * slice / nslices, hi = cum[M] * (slice + 1) / nslices;
        while (r0 < M && cum[r0] < lo) r0++;
        r1 = r0;
        while (r1 < M && cum[r1] < hi) r1++;
        if (slice == nslices - 1) r1 = M;
        if (slice == 0) r0 = 0;
    }
    int *cut = (int *)malloc(sizeof(int) * (size_t)(T + 1));
    cut[0] = r0;
    for (int t = 1; t < T; t++) {
        double want = cum[r0] + (cum[r1] - cum[r0]) * t / T;
        int c = cut[t - 1];
        while (c < r1 && cum[c] < want) c++;
        cut[t] = c;
    }
    cut[T] = r1;
    free(cum);
    const int ewald = s->p.charge_type == MG_ELEC_EWALD;
    double *q = ewald ? site_charges(s) : NULL;
    mt_job *jobs = (mt_job *)calloc((size_t)T, sizeof(mt_job));
    pthread_t *tid = (pthread_t *)calloc((size_t)T, sizeof(pthread_t));
    int *started = (int *)calloc((size_t)T, sizeof(int));
    for (int t = 0; t < T; t++) {
        mt_job *j = &jobs[t];
        j->s = s;
        j->x = x; j->y = y; j->z = z; j->q = q;
        j->imol_begin = cut[t];
        j->imol_end = cut[t + 1];
        j->kstride = ewald ? T * nslices : 0;
        j->koff = slice + nslices * t;
        j->f = (double *)calloc((size_t)n * 3, sizeof(double));
        j->scratch = (double *)calloc((size_t)n * 3 + 3, sizeof(double));
        started[t] = T > 1 && pthread_create(&tid[t], NULL, mt_run, j) == 0;
        if (!started[t]) mt_run(j);
    }
    for (int t = 0; t < T; t++)
        if (started[t]) pthread_join(tid[t], NULL);
    for (int i = 0; i < n; i++) fxl[i] = fyl[i] = fzl[i] = 0.0;
    memset(e, 0, sizeof(*e));
    double ufourier = 0.0;
    for (int t = 0; t < T; t++) {
        const mt_job *j = &jobs[t];
        for (int i = 0; i < n; i++) {
            fxl[i] += j->f[i];
            fyl[i] += j->f[n + i];
            fzl[i] += j->f[2 * n + i];
        }
        e->uvdw += j->e.uvdw;
        e->ushift += j->e.ushift;
        e->ureal += j->e.ureal;
        e->uelec += j->e.uelec;
        e->virial_inter += j->e.virial_inter;
        ufourier += j->ufourier;
        free(j->f);
        free(j->scratch);
    }
    free(jobs);
    free(tid);
    free(started);
    free(cut);
    acc a = {fxl, fyl, fzl, e};
    e->ushift *= s->p.shift4;
    if (slice != 0) { /* the O(N) remainder belongs to slice 0 */
        if (ewald) e->ufourier = ufourier * s->p.vfactor_ewald * s->p.coulomb_prefactor;
        free(q);
        return 0;
    }
    intra_pairs(s, x, y, z, &a);
    if (ewald) {
        ewald_tail(s, x, y, z, q, &a, ufourier);
        free(q);
    } else if (s->p.charge_type == MG_ELEC_WOLF) {
        double q2 = 0.0;
        for (int i = 0; i < n; i++) {
            int sp, rel;
            site_of(s, i, &sp, &rel);
            q2 += s->sp[sp].charge[rel] * s->sp[sp].charge[rel];
        }
        e->uself = q2 * (s->p.coulomb_prefactor * s->p.wolfvcon3);
        e->uelec = e->ureal - e->uself - e->uexcl;
    }
    int flags = solid_fluid(s, x, y, z, &a);
    e->uotherff = 0.0;
    e->uinter = e->uvdw + e->uelec + e->usflj + e->uotherff;
    return flags;
}

/* ---- bonded terms (src/bndfrc.c, src/aglfrc.c, src/dihfrc.c, src/impfrc.c) ---------- */
static double bond_term(const mg_species *S, int b, int base, const double *x, const double *y,
                        const double *z, double *fx, double *fy, double *fz, double *vir) {
    int i1 = base + S->bond_idx[2 * b], i2 = base + S->bond_idx[2 * b + 1];
    double rx = x[i1] - x[i2], ry = y[i1] - y[i2], rz = z[i1] - z[i2];
    double rsq = rx * rx + ry * ry + rz * rz;
    double r = sqrt(rsq);
    const double *bp = S->bond_param + 3 * b;
    double u, f;
    switch (S->bond_type[b]) {
    case MG_BOND_HARMONIC: {
        double dr = r - bp[1];
        u = 0.5 * bp[0] * dr * dr;
        f = -bp[0] * dr / r;
        break;
    }
    case MG_BOND_MORSE: {
        double dr = r - bp[1];
        double ex = exp(-bp[2] * dr);
        double om = 1.0 - ex;
        u = bp[0] * om * om;
        f = -2.0 * bp[0] * bp[2] * om * ex / r;
        break;
    }
    case MG_BOND_FENE: {
        double rmax2 = bp[1] * bp[1];
        u = bp[0] * rmax2 * log(1.0 - rsq / rmax2);
        f = -2.0 * bp[0] * rmax2 / (rmax2 - rsq);
        break;
    }
    default:
        *vir = 0.0;
        return 0.0;
    }
    *vir = f * rsq;
    fx[i1] += f * rx; fy[i1] += f * ry; fz[i1] += f * rz;
    fx[i2] -= f * rx; fy[i2] -= f * ry; fz[i2] -= f * rz;
    return u;
}

static double angle_term(const mg_species *S, int g, int base, const double *x, const double *y,
                         const double *z, double *fx, double *fy, double *fz, double *vir) {
    int ia = base + S->angle_idx[3 * g], ib = base + S->angle_idx[3 * g + 1],
        ic = base + S->angle_idx[3 * g + 2];
    const double *ap = S->angle_param + 5 * g;
    *vir = 0.0;
    if (S->angle_type[g] == MG_ANGLE_HARMONIC) {
        double xab = x[ia] - x[ib], yab = y[ia] - y[ib], zab = z[ia] - z[ib];
        double xcb = x[ic] - x[ib], ycb = y[ic] - y[ib], zcb = z[ic] - z[ib];
        double rab = sqrt(xab * xab + yab * yab + zab * zab), irab = 1.0 / rab;
        xab *= irab; yab *= irab; zab *= irab;
        double rcb = sqrt(xcb * xcb + ycb * ycb + zcb * zcb), ircb = 1.0 / rcb;
        xcb *= ircb; ycb *= ircb; zcb *= ircb;
        double c = xab * xcb + yab * ycb + zab * zcb;
        double th = acos(c);
        double sn = fmax(1.0e-8, sqrt(1.0 - c * c));
        double dth = th - ap[1];
        double u = 0.5 * ap[0] * dth * dth;
        double gm = ap[0] * dth / sn;
        double fxa = gm * (xcb - xab * c) * irab, fya = gm * (ycb - yab * c) * irab,
               fza = gm * (zcb - zab * c) * irab;
        double fxc = gm * (xab - xcb * c) * ircb, fyc = gm * (yab - ycb * c) * ircb,
               fzc = gm * (zab - zcb * c) * ircb;
        fx[ia] += fxa; fy[ia] += fya; fz[ia] += fza;
        fx[ib] = fx[ib] - fxa - fxc; fy[ib] = fy[ib] - fya - fyc; fz[ib] = fz[ib] - fza - fzc;
        fx[ic] += fxc; fy[ic] += fyc; fz[ic] += fzc;
        return u;
    }
    if (S->angle_type[g] == MG_ANGLE_TR_WATER) {
        double v13x = x[ia] - x[ic], v13y = y[ia] - y[ic], v13z = z[ia] - z[ic];
        double v12x = x[ia] - x[ib], v12y = y[ia] - y[ib], v12z = z[ia] - z[ib];
        double v23x = x[ib] - x[ic], v23y = y[ib] - y[ic], v23z = z[ib] - z[ic];
        double r13 = sqrt(v13x * v13x + v13y * v13y + v13z * v13z);
        double r12 = sqrt(v12x * v12x + v12y * v12y + v12z * v12z);
        double r23 = sqrt(v23x * v23x + v23y * v23y + v23z * v23z);
        double d3 = r13 - ap[3], d1 = r12 - ap[4], d2 = r23 - ap[4];
        double kt = ap[0], krt = ap[1], krr = ap[2];
        double u = 0.5 * kt * d3 * d3 + krt * d3 * (d1 + d2) + krr * d1 * d2;
        double t1 = -kt * d3 / r13, t21 = -krt * d3 / r12, t22 = -krt * (d1 + d2) / r13,
               t3 = -krr * d2 / r12;
        double fxa = (t1 * v13x + t21 * v12x + t22 * v13x + t3 * v12x);
        double fya = (t1 * v13y + t21 * v12y + t22 * v13y + t3 * v12y);
        double fza = (t1 * v13z + t21 * v12z + t22 * v13z + t3 * v12z);
        fx[ia] += fxa; fy[ia] += fya; fz[ia] += fza;
        t21 = -krt * d3 / r23;
        t22 = krt * d3 / r12;
        double t31 = -krr * d1 / r23, t32 = krr * d2 / r12;
        double fxb = (t21 * v23x + t22 * v12x + t31 * v23x + t32 * v12x);
        double fyb = (t21 * v23y + t22 * v12y + t31 * v23y + t32 * v12y);
        double fzb = (t21 * v23z + t22 * v12z + t31 * v23z + t32 * v12z);
        fx[ib] += fxb; fy[ib] += fyb; fz[ib] += fzb;
        t1 = kt * d3 / r13;
        t21 = krt * d3 / r23;
        t22 = krt * (d1 + d2) / r13;
        t3 = krr * d1 / r23;
        double fxc = (t1 * v13x + t21 * v23x + t22 * v13x + t3 * v23x);
        double fyc = (t1 * v13y + t21 * v23y + t22 * v13y + t3 * v23y);
        double fzc = (t1 * v13z + t21 * v23z + t22 * v13z + t3 * v23z);
        fx[ic] += fxc; fy[ic] += fyc; fz[ic] += fzc;
        *vir = fxa * v12x + fya * v12y + fza * v12z;
        *vir = *vir - fxc * v23x - fyc * v23y - fzc * v23z;
        return u;
    }
    return 0.0;
}

/* CHARMM-style torsion geometry shared by the CHARMM dihedral and improper
 * (src/dihfrc.c:165-276, src/impfrc.c:49-182): applies the forces for a given
 * prefactor `temp`. */
typedef struct tors { double aa1, bb1, cc1, aa2, bb2, cc2, t1, t2, t3; double rxjk, ryjk, rzjk, rxij, ryij, rzij, rxjl, ryjl, rzjl; } tors;

static tors tors_geom(int i1, int i2, int i3, int i4, const double *x, const double *y, const double *z) {
    tors t;
    t.rxjk = x[i3] - x[i2]; t.ryjk = y[i3] - y[i2]; t.rzjk = z[i3] - z[i2];
    t.rxij = x[i1] - x[i2]; t.ryij = y[i1] - y[i2]; t.rzij = z[i1] - z[i2];
    t.aa1 = t.ryjk * t.rzij - t.rzjk * t.ryij;
    t.bb1 = t.rzjk * t.rxij - t.rxjk * t.rzij;
    t.cc1 = t.rxjk * t.ryij - t.rxij * t.ryjk;
    t.rxjl = x[i4] - x[i2]; t.ryjl = y[i4] - y[i2]; t.rzjl = z[i4] - z[i2];
    t.aa2 = t.ryjl * t.rzjk - t.rzjl * t.ryjk;
    t.bb2 = t.rzjl * t.rxjk - t.rxjl * t.rzjk;
    t.cc2 = t.rxjl * t.ryjk - t.rxjk * t.ryjl;
    t.t1 = sqrt(t.aa1 * t.aa1 + t.bb1 * t.bb1 + t.cc1 * t.cc1);
    t.t2 = sqrt(t.aa2 * t.aa2 + t.bb2 * t.bb2 + t.cc2 * t.cc2);
    t.t3 = (t.aa1 * t.aa2 + t.bb1 * t.bb2 + t.cc1 * t.cc2);
    return t;
}

static void tors_apply(const tors *T, double temp, int i1, int i2, int i3, int i4,
                       const double *x, const double *y, const double *z, double *fx, double *fy,
                       double *fz) {
    double aa1 = T->aa1, bb1 = T->bb1, cc1 = T->cc1, aa2 = T->aa2, bb2 = T->bb2, cc2 = T->cc2;
    double t1 = T->t1, t2 = T->t2, t3 = T->t3;
    double rxjk = T->rxjk, ryjk = T->ryjk, rzjk = T->rzjk;
    double rxij = T->rxij, ryij = T->ryij, rzij = T->rzij;
    double rxjl = T->rxjl, ryjl = T->ryjl, rzjl = T->rzjl;
    double f = temp / (t2 * t1 * t1);
    fx[i1] = fx[i1] + f * ((bb2 * rzjk - cc2 * ryjk) * t1 - t3 / t1 * (bb1 * rzjk - cc1 * ryjk));
    fy[i1] = fy[i1] + f * ((-aa2 * rzjk + cc2 * rxjk) * t1 - t3 / t1 * (-aa1 * rzjk + cc1 * rxjk));
    fz[i1] = fz[i1] + f * ((aa2 * ryjk - bb2 * rxjk) * t1 - t3 / t1 * (aa1 * ryjk - bb1 * rxjk));
    f = temp / (t1 * t1 * t2 * t2);
    double rxik = x[i1] - x[i3], ryik = y[i1] - y[i3], rzik = z[i1] - z[i3];
    double rxkl = x[i4] - x[i3], rykl = y[i4] - y[i3], rzkl = z[i4] - z[i3];
    fx[i2] = fx[i2] + f * ((bb2 * rzik - bb1 * rzkl - cc2 * ryik + cc1 * rykl) * t1 * t2 -
                           t3 * (t2 / t1 * (bb1 * rzik - cc1 * ryik) + t1 / t2 * (-bb2 * rzkl + cc2 * rykl)));
    fy[i2] = fy[i2] + f * ((-aa2 * rzik + aa1 * rzkl + cc2 * rxik - cc1 * rxkl) * t1 * t2 -
                           t3 * (t2 / t1 * (-aa1 * rzik + cc1 * rxik) + t1 / t2 * (aa2 * rzkl - cc2 * rxkl)));
    fz[i2] = fz[i2] + f * ((aa2 * ryik - aa1 * rykl - bb2 * rxik + bb1 * rxkl) * t1 * t2 -
                           t3 * (t2 / t1 * (aa1 * ryik - bb1 * rxik) + t1 / t2 * (-aa2 * rykl + bb2 * rxkl)));
    fx[i3] = fx[i3] + f * ((-bb2 * rzij + bb1 * rzjl + cc2 * ryij - cc1 * ryjl) * t1 * t2 -
                           t3 * (t2 / t1 * (-bb1 * rzij + cc1 * ryij) + t1 / t2 * (bb2 * rzjl - cc2 * ryjl)));
    fy[i3] = fy[i3] + f * ((aa2 * rzij - aa1 * rzjl - cc2 * rxij + cc1 * rxjl) * t1 * t2 -
                           t3 * (t2 / t1 * (aa1 * rzij - cc1 * rxij) + t1 / t2 * (-aa2 * rzjl + cc2 * rxjl)));
    fz[i3] = fz[i3] + f * ((-aa2 * ryij + aa1 * ryjl + bb2 * rxij - bb1 * rxjl) * t1 * t2 -
                           t3 * (t2 / t1 * (-aa1 * ryij + bb1 * rxij) + t1 / t2 * (aa2 * ryjl - bb2 * rxjl)));
    f = temp / (t1 * t2 * t2);
    fx[i4] = fx[i4] + f * ((-bb1 * rzjk + cc1 * ryjk) * t2 - t3 / t2 * (-bb2 * rzjk + cc2 * ryjk));
    fy[i4] = fy[i4] + f * ((aa1 * rzjk - cc1 * rxjk) * t2 - t3 / t2 * (aa2 * rzjk - cc2 * rxjk));
    fz[i4] = fz[i4] + f * ((-aa1 * ryjk + bb1 * rxjk) * t2 - t3 / t2 * (-aa2 * ryjk + bb2 * rxjk));
}

static double dih_term(const mg_species *S, int d, int base, const double *x, const double *y,
                       const double *z, double *fx, double *fy, double *fz, double *vir, int *err) {
    int ia = base + S->dih_idx[4 * d], ib = base + S->dih_idx[4 * d + 1],
        ic = base + S->dih_idx[4 * d + 2], id = base + S->dih_idx[4 * d + 3];
    const double *cp = S->dih_param + 4 * d;
    *vir = 0.0;
    if (S->dih_type[d] == MG_DIH_OPLS) {
        double xab = x[ia] - x[ib], yab = y[ia] - y[ib], zab = z[ia] - z[ib];
        double xbc = x[ib] - x[ic], ybc = y[ib] - y[ic], zbc = z[ib] - z[ic];
        double xcd = x[ic] - x[id], ycd = y[ic] - y[id], zcd = z[ic] - z[id];
        double rrbc = 1.0 / sqrt(xbc * xbc + ybc * ybc + zbc * zbc);
        double pbx = yab * zbc - zab * ybc, pby = zab * xbc - xab * zbc, pbz = xab * ybc - yab * xbc;
        double pb2 = pbx * pbx + pby * pby + pbz * pbz;
        double rpb1 = 1.0 / sqrt(pb2), rpb2 = rpb1 * rpb1;
        double pcx = ybc * zcd - zbc * ycd, pcy = zbc * xcd - xbc * zcd, pcz = xbc * ycd - ybc * xcd;
        double pc2 = pcx * pcx + pcy * pcy + pcz * pcz;
        double rpc1 = 1.0 / sqrt(pc2), rpc2 = rpc1 * rpc1;
        double pbpc = pbx * pcx + pby * pcy + pbz * pcz;
        double c = pbpc * rpb1 * rpc1;
        double sn = (xbc * (pcy * pbz - pcz * pby) + ybc * (pbx * pcz - pbz * pcx) +
                     zbc * (pcx * pby - pcy * pbx)) * (rpb1 * rpc1 * rrbc);
        double th = atan2(sn, c);
        sn = copysign(fmax(1.0e-8, fabs(sn)), sn);
        double rsn = 1.0 / sn;
        double v1 = cp[0], v2 = cp[1], v3 = cp[2], v4 = cp[3];
        double u = v1 + 0.5 * (v2 * (1.0 + cos(th)) + v3 * (1.0 - cos(2.0 * th)) + v4 * (1.0 + cos(3.0 * th)));
        double dop = -0.5 * (v2 * sin(th) - 2.0 * v3 * sin(2.0 * th) + 3.0 * v4 * sin(3.0 * th));
        double gm = dop * rpb1 * rpc1 * rsn;
        double fax = gm * ((-pcy * zbc + pcz * ybc) - pbpc * rpb2 * (-pby * zbc + pbz * ybc));
        double fay = gm * ((pcx * zbc - pcz * xbc) - pbpc * rpb2 * (pbx * zbc - pbz * xbc));
        double faz = gm * ((-pcx * ybc + pcy * xbc) - pbpc * rpb2 * (-pbx * ybc + pby * xbc));
        double fcx = gm * ((-pcy * zab + pcz * yab) - pbpc * rpb2 * (-pby * zab + pbz * yab));
        double fcy = gm * ((pcx * zab - pcz * xab) - pbpc * rpb2 * (pbx * zab - pbz * xab));
        double fcz = gm * ((-pcx * yab + pcy * xab) - pbpc * rpb2 * (-pbx * yab + pby * xab));
        double fbx = gm * ((-pby * zcd + pbz * ycd) - pbpc * rpc2 * (-pcy * zcd + pcz * ycd));
        double fby = gm * ((pbx * zcd - pbz * xcd) - pbpc * rpc2 * (pcx * zcd - pcz * xcd));
        double fbz = gm * ((-pbx * ycd + pby * xcd) - pbpc * rpc2 * (-pcx * ycd + pcy * xcd));
        double fdx = gm * ((-pby * zbc + pbz * ybc) - pbpc * rpc2 * (-pcy * zbc + pcz * ybc));
        double fdy = gm * ((pbx * zbc - pbz * xbc) - pbpc * rpc2 * (pcx * zbc - pcz * xbc));
        double fdz = gm * ((-pbx * ybc + pby * xbc) - pbpc * rpc2 * (-pcx * ybc + pcy * xbc));
        fx[ia] += fax; fy[ia] += fay; fz[ia] += faz;
        fx[ib] += (-fax - fcx + fbx); fy[ib] += (-fay - fcy + fby); fz[ib] += (-faz - fcz + fbz);
        fx[ic] += fcx - fbx - fdx; fy[ic] += fcy - fby - fdy; fz[ic] += fcz - fbz - fdz;
        fx[id] += fdx; fy[id] += fdy; fz[id] += fdz;
        return u;
    }
    if (S->dih_type[d] == MG_DIH_CHARMM) {
        double kphi = cp[0], np = cp[1], d0 = cp[2];
        if (!(fabs(kphi) >= 1.0e-8)) return 0.0;
        tors T = tors_geom(ia, ib, ic, id, x, y, z);
        double phi = T.t3 / (T.t1 * T.t2);
        double alpha = phi;
        phi = 180.0 - (acos(phi) * 180.0 / ORC_PI);
        double u = kphi * (1 + cos((np * phi - d0) / 180 * ORC_PI));
        double temp;
        if (fabs(sin(phi * ORC_PI / 180)) <= 1e-10)
            temp = -np * np * kphi * cos((np * phi - d0) * ORC_PI / 180) / alpha;
        else
            temp = np * kphi * sin((np * phi - d0) * ORC_PI / 180) / sin(phi * ORC_PI / 180);
        tors_apply(&T, temp, ia, ib, ic, id, x, y, z, fx, fy, fz);
        return u;
    }
    (void)err;
    return 0.0;
}

static double imp_term(const mg_species *S, int q, int base, const double *x, const double *y,
                       const double *z, double *fx, double *fy, double *fz, double *vir, int *err) {
    *vir = 0.0;
    if (S->imp_type[q] != MG_IMP_CHARMM) return 0.0;
    const double *ip = S->imp_param + 2 * q;
    if (!(fabs(ip[0]) >= 1e-5)) return 0.0;
    int i1 = base + S->imp_idx[4 * q], i2 = base + S->imp_idx[4 * q + 1],
        i3 = base + S->imp_idx[4 * q + 2], i4 = base + S->imp_idx[4 * q + 3];
    tors T = tors_geom(i1, i2, i3, i4, x, y, z);
    double phi = T.t3 / (T.t1 * T.t2);
    double alpha = phi;
    phi = 180 - (acos(phi) * 180 / ORC_PI);
    double u = ip[0] * (phi - ip[1]) * (phi - ip[1]);
    u *= (ORC_PI / 180) * (ORC_PI / 180);
    double a = acos(alpha) * 180 / ORC_PI;
    /* the reference exits on these degenerate geometries (src/impfrc.c:96-134) */
    if ((fabs(ip[1]) <= 1e-5 && fabs(a) <= 1e-20) || (fabs(ip[1] - 180) <= 1e-5 && fabs(a - 180) <= 1e-20) ||
        (fabs(ip[1]) <= 1e-5 && fabs(a - 180) <= 1e-20) || (fabs(ip[1] - 180) <= 1e-5 && fabs(a) <= 1e-20)) {
        *err = 1;
        return u;
    }
    double temp = -2.0 * ip[0] * (phi - ip[1]) * ORC_PI / 180 / sin(phi * ORC_PI / 180);
    tors_apply(&T, temp, i1, i2, i3, i4, x, y, z, fx, fy, fz);
    return u;
}

int orc_frcshort(const orc_system *s, const double *x, const double *y, const double *z,
                 double *fxs, double *fys, double *fzs, mg_energies *e) {
    int n = orc_natom(s);
    int err = 0;
    e->ubond = e->uangle = e->udih = e->uimp = e->virial_intra = 0.0;
    for (int i = 0; i < n; i++) fxs[i] = fys[i] = fzs[i] = 0.0;
    int base = 0;
    for (int is = 0; is < s->nspecies; is++) {
        const mg_species *S = &s->sp[is];
        for (int im = 0; im < S->nmole; im++, base += S->natom) {
            double v;
            for (int b = 0; b < S->nbond; b++) {
                e->ubond += bond_term(S, b, base, x, y, z, fxs, fys, fzs, &v);
                e->virial_intra += v;
            }
            for (int g = 0; g < S->nangle; g++) {
                e->uangle += angle_term(S, g, base, x, y, z, fxs, fys, fzs, &v);
                e->virial_intra += v;
            }
            for (int d = 0; d < S->ndih; d++) {
                e->udih += dih_term(S, d, base, x, y, z, fxs, fys, fzs, &v, &err);
                e->virial_intra += v;
            }
            for (int q = 0; q < S->nimp; q++) {
                e->uimp += imp_term(S, q, base, x, y, z, fxs, fys, fzs, &v, &err);
                e->virial_intra += v;
            }
        }
    }
    e->uintra = e->ubond + e->uangle + e->udih + e->uimp;
    return err;
}
