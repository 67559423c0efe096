/*
 * md_oracle.c - CPU restatement of the reference's integrators (TEST INFRASTRUCTURE:
 * the checker of mg_md_run, never on the product path).
 *
 *   vver()      src/md.c:22-85        velocity Verlet with RESPA inner steps
 *   vver_nh_3() src/nvtnh.c:11-271    Nose-Hoover RESPA step with implicit solves
 *
 * Loop order, operation order and the running sums follow the reference statement by
 * statement (build with -ffp-contract=off), calling the restated frclong()/frcshort()
 * of mspms_oracle.c for the forces. The solver's convergence test in the reference reads
 * vxn/vxo at index natom through a stale loop index (src/nvtnh.c:128-139, :228-236);
 * those entries are never written (zero), the velocity tests compare NaN and never fail,
 * so only the thermostat test decides, which is what is restated here.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mspms_oracle.h"

typedef struct md_work {
    int n;
    double *rmass, *fxl, *fyl, *fzl, *fxs, *fys, *fzs;
    double *vxn, *vyn, *vzn, *vxo, *vyo, *vzo, *bx, *by, *bz;
    mg_energies el, es;
} md_work;

static void forces_long(const orc_system *s, const double *x, const double *y, const double *z, md_work *w) {
    orc_frclong(s, x, y, z, w->fxl, w->fyl, w->fzl, &w->el, NULL);
}

static void forces_short(const orc_system *s, const double *x, const double *y, const double *z, md_work *w) {
    orc_frcshort(s, x, y, z, w->fxs, w->fys, w->fzs, &w->es);
}

/* implicit solve of one thermostat (src/nvtnh.c:67-156 with the inner names) */
static double nh_solve(md_work *w, const double *fx, const double *fy, const double *fz, double *vx, double *vy,
                       double *vz, double hstep, double dstep, double q, double g_treq, double *pst,
                       double *sumv2_out) {
    const int n = w->n;
    const double err = 1.0e-10;
    double sumv2 = 0.0;
    for (int ii = 0; ii < n; ii++) {
        const double r_mass = w->rmass[ii];
        w->vxn[ii] = vx[ii];
        w->vyn[ii] = vy[ii];
        w->vzn[ii] = vz[ii];
        sumv2 = sumv2 + (w->vxn[ii] * w->vxn[ii] + w->vyn[ii] * w->vyn[ii] + w->vzn[ii] * w->vzn[ii]) / r_mass;
    }
    double psn = *pst, pso = psn;
    int ready = 0, iter = 0;
    while (!ready && iter < 100) {
        iter++;
        pso = psn;
        double delps = 0.0;
        for (int ii = 0; ii < n; ii++) {
            const double r_mass = w->rmass[ii];
            double ri;
            w->vxo[ii] = w->vxn[ii];
            w->vyo[ii] = w->vyn[ii];
            w->vzo[ii] = w->vzn[ii];
            w->bx[ii] = -hstep * (fx[ii] * r_mass - pso * w->vxo[ii]) - (vx[ii] - w->vxo[ii]);
            ri = w->vxo[ii] * dstep / q / r_mass;
            delps = delps + ri * w->bx[ii];
            w->by[ii] = -hstep * (fy[ii] * r_mass - pso * w->vyo[ii]) - (vy[ii] - w->vyo[ii]);
            ri = w->vyo[ii] * dstep / q / r_mass;
            delps = delps + ri * w->by[ii];
            w->bz[ii] = -hstep * (fz[ii] * r_mass - pso * w->vzo[ii]) - (vz[ii] - w->vzo[ii]);
            ri = w->vzo[ii] * dstep / q / r_mass;
            delps = delps + ri * w->bz[ii];
        }
        const double di = -(pso * hstep + 1.0);
        delps = delps - di * ((-sumv2 + g_treq) * hstep / q - (*pst - pso));
        delps = delps / (-dstep * hstep * sumv2 / q + di);
        sumv2 = 0.0;
        for (int ii = 0; ii < n; ii++) {
            const double r_mass = w->rmass[ii];
            w->vxn[ii] = w->vxn[ii] + (w->bx[ii] + hstep * w->vxo[ii] * delps) / di;
            w->vyn[ii] = w->vyn[ii] + (w->by[ii] + hstep * w->vyo[ii] * delps) / di;
            w->vzn[ii] = w->vzn[ii] + (w->bz[ii] + hstep * w->vzo[ii] * delps) / di;
            sumv2 = sumv2 + (w->vxn[ii] * w->vxn[ii] + w->vyn[ii] * w->vyn[ii] + w->vzn[ii] * w->vzn[ii]) / r_mass;
        }
        psn = pso + delps;
        ready = !(fabs((psn - pso) / psn) > err);
    }
    for (int ii = 0; ii < n; ii++) {
        vx[ii] = w->vxn[ii];
        vy[ii] = w->vyn[ii];
        vz[ii] = w->vzn[ii];
    }
    *pst = psn;
    *sumv2_out = sumv2;
    return sumv2;
}

static void record(double *row, const mg_md_state *st, double uinter, double uintra, double ushift) {
    if (!row) return;
    row[0] = st->ukin;
    row[1] = uinter;
    row[2] = uintra;
    row[3] = ushift;
    row[4] = st->ps;
    row[5] = st->ss;
    row[6] = st->pss;
    row[7] = st->sss;
    row[8] = st->tinst;
    row[9] = st->unhts;
    row[10] = st->unhtss;
    row[11] = 0.0;
}

int orc_md_run(const orc_system *s, const mg_md_params *mp, int nsteps, double *xx, double *yy, double *zz,
               double *vx, double *vy, double *vz, mg_md_state *st, double *log) {
    const int n = orc_natom(s);
    md_work w;
    memset(&w, 0, sizeof(w));
    w.n = n;
    double *buf = (double *)calloc((size_t)n * 16, sizeof(double));
    if (!buf) return -1;
    double *p = buf;
    w.rmass = p; p += n;
    w.fxl = p; p += n; w.fyl = p; p += n; w.fzl = p; p += n;
    w.fxs = p; p += n; w.fys = p; p += n; w.fzs = p; p += n;
    w.vxn = p; p += n; w.vyn = p; p += n; w.vzn = p; p += n;
    w.vxo = p; p += n; w.vyo = p; p += n; w.vzo = p; p += n;
    w.bx = p; p += n; w.by = p; p += n; w.bz = p;
    for (int sp = 0, a = 0; sp < s->nspecies; sp++)
        for (int m = 0; m < s->sp[sp].nmole; m++)
            for (int k = 0; k < s->sp[sp].natom; k++) w.rmass[a++] = 1.0 / s->sp[sp].aw[k];

    const double delt = mp->delt, deltby2 = delt / 2.0, delts = delt / mp->nstep_inner, deltsby2 = delts / 2.0;
    const double delt_sqby2 = delt * delt / 2.0, delts_sqby2 = delts * delts / 2.0;
    const double treq = mp->treq, qq = mp->qq, qqs = mp->qqs, gg = mp->gg, ggs = mp->ggs;

    forces_long(s, xx, yy, zz, &w);
    forces_short(s, xx, yy, zz, &w);
    double ukin = 0.0;
    for (int ii = 0; ii < n; ii++) ukin += (vx[ii] * vx[ii] + vy[ii] * vy[ii] + vz[ii] * vz[ii]) / w.rmass[ii];
    st->ukin = ukin * 0.5;
    st->tinst = 2.0 * st->ukin / mp->nfree;
    record(log, st, w.el.uinter, w.es.uintra, w.el.ushift);

    for (int step = 1; step <= nsteps; step++) {
        if (mp->scheme == MG_MD_NVT_NH) {
            double sumv2 = 0.0;
            for (int ii = 0; ii < n; ii++) {
                const double r_mass = w.rmass[ii];
                vx[ii] = vx[ii] + deltby2 * (w.fxl[ii] * r_mass - st->ps * vx[ii]);
                vy[ii] = vy[ii] + deltby2 * (w.fyl[ii] * r_mass - st->ps * vy[ii]);
                vz[ii] = vz[ii] + deltby2 * (w.fzl[ii] * r_mass - st->ps * vz[ii]);
            }
            for (int ll = 0; ll < mp->nstep_inner; ll++) {
                sumv2 = 0.0;
                for (int ii = 0; ii < n; ii++) {
                    const double r_mass = w.rmass[ii];
                    sumv2 = sumv2 + (vx[ii] * vx[ii] + vy[ii] * vy[ii] + vz[ii] * vz[ii]) / r_mass;
                    vx[ii] = vx[ii] + deltsby2 * (w.fxs[ii] * r_mass - st->pss * vx[ii]);
                    vy[ii] = vy[ii] + deltsby2 * (w.fys[ii] * r_mass - st->pss * vy[ii]);
                    vz[ii] = vz[ii] + deltsby2 * (w.fzs[ii] * r_mass - st->pss * vz[ii]);
                    xx[ii] = xx[ii] + delts * vx[ii];
                    yy[ii] = yy[ii] + delts * vy[ii];
                    zz[ii] = zz[ii] + delts * vz[ii];
                }
                st->sss = st->sss + st->pss * delts + (sumv2 - ggs * treq) * delts_sqby2 / qqs;
                st->pss = st->pss + (sumv2 - ggs * treq) * deltsby2 / qqs;
                forces_short(s, xx, yy, zz, &w);
                nh_solve(&w, w.fxs, w.fys, w.fzs, vx, vy, vz, deltsby2, delts, qqs, ggs * treq, &st->pss, &sumv2);
                st->unhtss = (st->pss * st->pss * qqs) / 2.0 + ggs * treq * st->sss;
            }
            st->ss = st->ss + st->ps * delt + (sumv2 - gg * treq) * delt_sqby2 / qq;
            st->ps = st->ps + (sumv2 - gg * treq) * deltby2 / qq;
            forces_long(s, xx, yy, zz, &w);
            nh_solve(&w, w.fxl, w.fyl, w.fzl, vx, vy, vz, deltby2, delt, qq, gg * treq, &st->ps, &sumv2);
            st->ukin = sumv2 / 2.0;
            st->unhts = (st->ps * st->ps * qq) / 2.0 + gg * treq * st->ss;
            st->tinst = 2.0 * st->ukin / mp->nfree;
        } else {
            for (int ii = 0; ii < n; ii++) {
                const double r_mass = w.rmass[ii];
                vx[ii] += (deltby2 * w.fxl[ii] * r_mass);
                vy[ii] += (deltby2 * w.fyl[ii] * r_mass);
                vz[ii] += (deltby2 * w.fzl[ii] * r_mass);
            }
            for (int ll = 0; ll < mp->nstep_inner; ll++) {
                for (int ii = 0; ii < n; ii++) {
                    const double r_mass = w.rmass[ii];
                    vx[ii] += (deltsby2 * w.fxs[ii] * r_mass);
                    vy[ii] += (deltsby2 * w.fys[ii] * r_mass);
                    vz[ii] += (deltsby2 * w.fzs[ii] * r_mass);
                    xx[ii] = xx[ii] + delts * vx[ii];
                    yy[ii] = yy[ii] + delts * vy[ii];
                    zz[ii] = zz[ii] + delts * vz[ii];
                }
                forces_short(s, xx, yy, zz, &w);
                for (int ii = 0; ii < n; ii++) {
                    const double r_mass = w.rmass[ii];
                    vx[ii] += (deltsby2 * w.fxs[ii] * r_mass);
                    vy[ii] += (deltsby2 * w.fys[ii] * r_mass);
                    vz[ii] += (deltsby2 * w.fzs[ii] * r_mass);
                }
            }
            forces_long(s, xx, yy, zz, &w);
            ukin = 0.0;
            for (int ii = 0; ii < n; ii++) {
                const double r_mass = w.rmass[ii];
                vx[ii] += (deltby2 * w.fxl[ii] * r_mass);
                vy[ii] += (deltby2 * w.fyl[ii] * r_mass);
                vz[ii] += (deltby2 * w.fzl[ii] * r_mass);
                ukin += (vx[ii] * vx[ii] + vy[ii] * vy[ii] + vz[ii] * vz[ii]) / r_mass;
            }
            st->ukin = ukin * 0.5;
            st->tinst = 2.0 * st->ukin / mp->nfree;
        }
        record(log ? log + (size_t)step * MG_MD_LOG : NULL, st, w.el.uinter, w.es.uintra, w.el.ushift);
    }
    free(buf);
    return 0;
}

/* ---- the canonical HMC move of one replica (src/hmc.c:23-40, src/dispmd.c:12-103) ------ */
#include "../include/mg_philox.h"

/* velinit (src/initvars.c:151-229) of move mv of a replica with the Philox streams of the
 * engine: Gaussian velocities sqrt(T/m) g, the total momentum removed and, with rescale, the
 * kinetic energy set to exactly treq nfree / 2; returns that kinetic energy */
static double hmc_velinit(const mg_hmc_params *hp, int replica, int move, int n, double *vx, double *vy,
                          double *vz) {
    const uint32_t key[2] = {(uint32_t)(hp->seed & 0xffffffffull), (uint32_t)(hp->seed >> 32)};
    const uint32_t mv = (uint32_t)move;
    const double nfree = (double)(3 * n - hp->nconstraint);
    const double stdv = sqrt(hp->treq) / sqrt(hp->mass);
    double px = 0.0, py = 0.0, pz = 0.0, sysm = 0.0;
    for (int i = 0; i < n; i++) {
        const uint32_t c0[4] = {(uint32_t)i, mv, 0u, (uint32_t)replica}, c1[4] = {(uint32_t)i, mv, 1u, (uint32_t)replica};
        uint32_t w0[4], w1[4];
        double g0, g1, g2, g3;
        mg_philox4x32_10(c0, key, w0);
        mg_philox4x32_10(c1, key, w1);
        mg_gauss2(w0, &g0, &g1);
        mg_gauss2(w1, &g2, &g3);
        vx[i] = stdv * g0;
        vy[i] = stdv * g1;
        vz[i] = stdv * g2;
        px += vx[i] * hp->mass;
        py += vy[i] * hp->mass;
        pz += vz[i] * hp->mass;
        sysm += hp->mass;
    }
    px /= sysm;
    py /= sysm;
    pz /= sysm;
    double ukin = 0.0;
    for (int i = 0; i < n; i++) {
        vx[i] -= px;
        vy[i] -= py;
        vz[i] -= pz;
        ukin += hp->mass * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
    }
    ukin = 0.5 * ukin;
    if (hp->rescale) {
        const double tinst = 2.0 * ukin / nfree, scaling = sqrt(hp->treq / tinst);
        ukin = 0.0;
        for (int i = 0; i < n; i++) {
            vx[i] *= scaling;
            vy[i] *= scaling;
            vz[i] *= scaling;
            ukin += hp->mass * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
        }
        ukin = 0.5 * ukin;
    }
    return ukin;
}

int orc_hmc_velocities(const mg_hmc_params *hp, int replica, int move, int n, double *vx, double *vy, double *vz) {
    hmc_velinit(hp, replica, move, n, vx, vy, vz);
    return 0;
}

int orc_hmc_replica(const orc_system *s, const mg_hmc_params *hp, int replica, int move0, int nmoves, double *xx,
                    double *yy, double *zz, int *accepted, double *dh_log, double *energy) {
    const int n = orc_natom(s);
    double *buf = (double *)calloc((size_t)n * 6, sizeof(double));
    if (!buf) return -1;
    double *vx = buf, *vy = buf + n, *vz = buf + 2 * n, *ox = buf + 3 * n, *oy = buf + 4 * n, *oz = buf + 5 * n;
    const uint32_t key[2] = {(uint32_t)(hp->seed & 0xffffffffull), (uint32_t)(hp->seed >> 32)};
    mg_md_params mp;
    memset(&mp, 0, sizeof(mp));
    mp.scheme = MG_MD_NVE;
    mp.nstep_inner = 1;
    mp.delt = hp->delt;
    mp.treq = hp->treq;
    mp.nfree = 3 * n - hp->nconstraint;
    int acc = 0;
    double e_cur = 0.0;
    for (int m = 0; m < nmoves; m++) {
        const uint32_t mv = (uint32_t)(move0 + m);
        const double ukin = hmc_velinit(hp, replica, move0 + m, n, vx, vy, vz);
        for (int i = 0; i < n; i++) {
            ox[i] = xx[i];
            oy[i] = yy[i];
            oz[i] = zz[i];
        }
        /* frclong + frcshort, then md_move over vver: orc_md_run evaluates the forces at
         * the start and records U0 and U1 */
        double log[2 * MG_MD_LOG];
        mg_md_state st;
        memset(&st, 0, sizeof(st));
        double *lg = (double *)calloc((size_t)(hp->nstep_md + 1) * MG_MD_LOG, sizeof(double));
        if (!lg) {
            free(buf);
            return -1;
        }
        orc_md_run(s, &mp, hp->nstep_md, xx, yy, zz, vx, vy, vz, &st, lg);
        memcpy(log, lg, sizeof(double) * MG_MD_LOG);
        memcpy(log + MG_MD_LOG, lg + (size_t)hp->nstep_md * MG_MD_LOG, sizeof(double) * MG_MD_LOG);
        free(lg);
        /* md_move's difference, with the reference's +d ushift (src/dispmd.c:48-50) */
        const double du = (log[MG_MD_LOG + 1] - log[1]) + (log[MG_MD_LOG + 2] - log[2]) +
                          (log[MG_MD_LOG + 0] - ukin) + (log[MG_MD_LOG + 3] - log[3]);
        const double dh = du / hp->treq;
        const uint32_t ca[4] = {0u, mv, 2u, (uint32_t)replica};
        uint32_t wa[4];
        mg_philox4x32_10(ca, key, wa);
        const int accept = dh <= 0.0 || mg_u01(wa[0], wa[1]) < exp(-dh);
        if (!accept) {
            memcpy(xx, ox, sizeof(double) * n);
            memcpy(yy, oy, sizeof(double) * n);
            memcpy(zz, oz, sizeof(double) * n);
        }
        acc += accept;
        e_cur = accept ? log[MG_MD_LOG + 1] + log[MG_MD_LOG + 3] : log[1] + log[3];
        if (dh_log) dh_log[m] = dh;
    }
    *accepted = acc;
    *energy = e_cur;
    free(buf);
    return 0;
}

/* the generator itself, for its known-answer test */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    mg_philox4x32_10(ctr, key, out);
}

/* ---- simulated annealing (src/siman.c:62-182) -------------------------------------- *
 * Stages at T = t_initial / mu_t^k until the first stage below t_min has run; each stage
 * is velinit (src/initvars.c:151-229) with the Philox streams of the engine (counter =
 * (site, stage, 0 or 1, 0x5349)) in place of gaussran(), then n_tries vver_nh_3 steps
 * at treq = T, then the thermostat scalars are reset (src/siman.c:167-174). */
int orc_siman_run(const orc_system *s, const mg_siman_params *sp, double *xx, double *yy, double *zz, double *vx,
                  double *vy, double *vz, mg_md_state *st, int *nstages, double *stage_log) {
    const int n = orc_natom(s);
    double *aw = (double *)calloc((size_t)n, sizeof(double));
    double *lg = (double *)calloc((size_t)(sp->n_tries + 1) * MG_MD_LOG, sizeof(double));
    if (!aw || !lg) {
        free(aw);
        free(lg);
        return -1;
    }
    double sysm = 0.0;
    for (int q = 0, a = 0; q < s->nspecies; q++)
        for (int m = 0; m < s->sp[q].nmole; m++)
            for (int k = 0; k < s->sp[q].natom; k++) {
                aw[a] = s->sp[q].aw[k];
                sysm += aw[a];
                a++;
            }
    const uint32_t key[2] = {(uint32_t)(sp->seed & 0xffffffffull), (uint32_t)(sp->seed >> 32)};
    int nst = 0;
    double T = sp->t_initial;
    for (;;) {
        if (nst >= sp->max_stages) {
            free(aw);
            free(lg);
            return -2;
        }
        if (nst > 0) {
            st->ps = st->ss = st->pss = st->sss = 0.0;
            st->unhts = st->unhtss = 0.0;
        }
        double px = 0.0, py = 0.0, pz = 0.0;
        const double stdvtmp = sqrt(T);
        for (int i = 0; i < n; i++) {
            const uint32_t c0[4] = {(uint32_t)i, (uint32_t)nst, 0u, 0x5349u};
            const uint32_t c1[4] = {(uint32_t)i, (uint32_t)nst, 1u, 0x5349u};
            uint32_t w0[4], w1[4];
            double g0, g1, g2, g3;
            mg_philox4x32_10(c0, key, w0);
            mg_philox4x32_10(c1, key, w1);
            mg_gauss2(w0, &g0, &g1);
            mg_gauss2(w1, &g2, &g3);
            const double stdv = stdvtmp / sqrt(aw[i]);
            vx[i] = stdv * g0;
            vy[i] = stdv * g1;
            vz[i] = stdv * g2;
            px += vx[i] * aw[i];
            py += vy[i] * aw[i];
            pz += vz[i] * aw[i];
        }
        px /= sysm;
        py /= sysm;
        pz /= sysm;
        double ukin = 0.0;
        for (int i = 0; i < n; i++) {
            vx[i] -= px;
            vy[i] -= py;
            vz[i] -= pz;
            ukin += aw[i] * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
        }
        ukin = 0.5 * ukin;
        const double scaling = sqrt(T / (2.0 * ukin / sp->md.nfree));
        for (int i = 0; i < n; i++) {
            vx[i] *= scaling;
            vy[i] *= scaling;
            vz[i] *= scaling;
        }
        mg_md_params mp = sp->md;
        mp.treq = T;
        orc_md_run(s, &mp, sp->n_tries, xx, yy, zz, vx, vy, vz, st, lg);
        if (stage_log) {
            const double *r = lg + (size_t)sp->n_tries * MG_MD_LOG;
            double *o = stage_log + (size_t)nst * MG_SIMAN_LOG;
            o[0] = T;
            o[1] = r[0];
            o[2] = r[1];
            o[3] = r[2];
            o[4] = r[3];
            o[5] = r[8];
            o[6] = r[9];
            o[7] = r[10];
        }
        nst++;
        const int done = T < sp->t_min;
        T /= sp->mu_t;
        if (done) break;
    }
    *nstages = nst;
    free(aw);
    free(lg);
    return 0;
}

/* ---- NPT: npt_respa and npt_nh_operator (src/nptnh.c:10-234) ------------------------ */
typedef struct npt_scalars {
    double vts, vbs, rts, utsbs, ukin, tinst, pinst, pljlrc;
} npt_scalars;

/* sum over species pairs of the LJ pressure-correction terms (src/initvars.c:476-520)
 * divided by V^2 in the reference's order (src/misc.c:131-148) */
static double npt_pljlrc(const orc_system *s, int lj_lrc, double boxv) {
    if (!lj_lrc) return 0.0;
    const double pi = 3.141592653589793;
    const double t1 = (32.0 / 9.0) * pi * pow(s->p.rcutoff, -9.0), t2 = -(16.0 / 3.0) * pi * pow(s->p.rcutoff, -3.0);
    double p = 0.0;
    for (int m = 0; m < s->nspecies; m++)
        for (int nn = 0; nn < s->nspecies; nn++) {
            double term = 0.0;
            for (int i = 0; i < s->sp[m].natom; i++)
                for (int j = 0; j < s->sp[nn].natom; j++) {
                    const double sij = 0.5 * (s->sp[m].sigma[i] + s->sp[nn].sigma[j]);
                    const double eij = sqrt(s->sp[m].epsilon[i] * s->sp[nn].epsilon[j]);
                    term += (pow(sij, 9.0) * t1 + pow(sij, 3.0) * t2) * (eij * pow(sij, 3.0));
                }
            p += (term * s->sp[m].nmole * s->sp[nn].nmole / boxv / boxv);
        }
    return p;
}

static void npt_operator(const mg_npt_params *mp, int n, const double *rmass, double *vx, double *vy, double *vz,
                         double virial, double boxv, npt_scalars *c) {
    const double nfree = mp->nfree, treq = mp->treq, qts = mp->qts, qbs = mp->qbs, preq = mp->preq;
    const double N_plus1RT = (nfree + 1) * treq, one_3N = 1.0 + 3.0 / nfree;
    const double dt_outer2 = mp->delt / 2.0, dt_outer4 = mp->delt / 4.0, dt_outer8 = mp->delt / 8.0;
    double mvsq = 0.0;
    for (int ii = 0; ii < n; ii++) mvsq += (vx[ii] * vx[ii] + vy[ii] * vy[ii] + vz[ii] * vz[ii]) / rmass[ii];
    const double pdiff = virial + c->pljlrc * boxv * 3.0 - preq * boxv * 3.0;
    double Gts = (mvsq + qbs * c->vbs * c->vbs - N_plus1RT) / qts;
    c->vts = c->vts + dt_outer4 * Gts;
    const double BB = exp(-c->vts * dt_outer8);
    c->vbs = c->vbs * BB;
    double Gbs = (one_3N * mvsq + pdiff) / qbs;
    c->vbs = c->vbs + dt_outer4 * Gbs;
    c->vbs = c->vbs * BB;
    c->rts = c->rts + dt_outer2 * c->vts;
    const double AA = exp(-dt_outer2 * (c->vts + one_3N * c->vbs));
    for (int ii = 0; ii < n; ii++) {
        vx[ii] = vx[ii] * AA;
        vy[ii] = vy[ii] * AA;
        vz[ii] = vz[ii] * AA;
    }
    c->vbs = c->vbs * BB;
    mvsq = mvsq * AA * AA;
    Gbs = (one_3N * mvsq + pdiff) / qbs;
    c->vbs = c->vbs + dt_outer4 * Gbs;
    c->vbs = c->vbs * BB;
    Gts = (mvsq + qbs * c->vbs * c->vbs - N_plus1RT) / qts;
    c->vts = c->vts + dt_outer4 * Gts;
    c->utsbs = 0.5 * qbs * c->vbs * c->vbs + 0.5 * qts * c->vts * c->vts + (nfree + 1) * treq * c->rts + preq * boxv;
    c->ukin = mvsq / 2.0;
    c->tinst = 2.0 * c->ukin / nfree;
    const double pideal = n / boxv * c->tinst;
    c->pinst = pideal + virial / 3.0 / boxv + c->pljlrc;
}

static void npt_record(double *row, const npt_scalars *c, double uinter, double uintra, double ushift, double lx,
                       double boxv) {
    if (!row) return;
    const double r[12] = {c->ukin, uinter, uintra, ushift, c->vts, c->vbs, c->rts, c->utsbs, c->tinst, c->pinst,
                          lx, boxv};
    memcpy(row, r, sizeof(r));
}

int orc_npt_run(const orc_system *s0, const mg_npt_params *mp, int nsteps, double *xx, double *yy, double *zz,
                double *vx, double *vy, double *vz, double *box, mg_npt_state *st, double *log) {
    const int n = orc_natom(s0);
    orc_system s = *s0;
    s.lx = box[0];
    s.ly = box[1];
    s.lz = box[2];
    double *buf = (double *)calloc((size_t)n * 7, sizeof(double));
    if (!buf) return -1;
    double *rmass = buf, *fxl = buf + n, *fyl = buf + 2 * n, *fzl = buf + 3 * n, *fxs = buf + 4 * n,
           *fys = buf + 5 * n, *fzs = buf + 6 * n;
    for (int q = 0, a = 0; q < s.nspecies; q++)
        for (int m = 0; m < s.sp[q].nmole; m++)
            for (int k = 0; k < s.sp[q].natom; k++) rmass[a++] = 1.0 / s.sp[q].aw[k];
    const double pi = 3.141592653589793;
    const double deltby2 = mp->delt / 2.0, delts = mp->delt / mp->nstep_inner, deltsby2 = delts / 2.0;
    double boxv = s.lx * s.ly * s.lz;
    npt_scalars c;
    memset(&c, 0, sizeof(c));
    c.vts = st->vts;
    c.vbs = st->vbs;
    c.rts = st->rts;
    c.pljlrc = npt_pljlrc(&s, mp->lj_lrc, boxv);
    mg_energies el, es;
    orc_frclong(&s, xx, yy, zz, fxl, fyl, fzl, &el, NULL);
    orc_frcshort(&s, xx, yy, zz, fxs, fys, fzs, &es);
    {
        double mvsq = 0.0;
        for (int ii = 0; ii < n; ii++) mvsq += (vx[ii] * vx[ii] + vy[ii] * vy[ii] + vz[ii] * vz[ii]) / rmass[ii];
        c.ukin = mvsq / 2.0;
        c.tinst = 2.0 * c.ukin / mp->nfree;
        c.utsbs = 0.5 * mp->qbs * c.vbs * c.vbs + 0.5 * mp->qts * c.vts * c.vts + (mp->nfree + 1) * mp->treq * c.rts +
                  mp->preq * boxv;
        c.pinst = n / boxv * c.tinst + (el.virial_inter + es.virial_intra) / 3.0 / boxv + c.pljlrc;
    }
    npt_record(log, &c, el.uinter, es.uintra, el.ushift, s.lx, boxv);
    for (int step = 1; step <= nsteps; step++) {
        npt_operator(mp, n, rmass, vx, vy, vz, el.virial_inter + es.virial_intra, boxv, &c);
        for (int ii = 0; ii < n; ii++) {
            vx[ii] += (deltby2 * fxl[ii] * rmass[ii]);
            vy[ii] += (deltby2 * fyl[ii] * rmass[ii]);
            vz[ii] += (deltby2 * fzl[ii] * rmass[ii]);
        }
        for (int ll = 0; ll < mp->nstep_inner; ll++) {
            const double AA = exp(deltsby2 * c.vbs);
            for (int ii = 0; ii < n; ii++) {
                const double r_mass = rmass[ii];
                vx[ii] += (deltsby2 * fxs[ii] * r_mass);
                vy[ii] += (deltsby2 * fys[ii] * r_mass);
                vz[ii] += (deltsby2 * fzs[ii] * r_mass);
                xx[ii] = xx[ii] * AA;
                yy[ii] = yy[ii] * AA;
                zz[ii] = zz[ii] * AA;
                xx[ii] = xx[ii] + delts * vx[ii];
                yy[ii] = yy[ii] + delts * vy[ii];
                zz[ii] = zz[ii] + delts * vz[ii];
                xx[ii] = xx[ii] * AA;
                yy[ii] = yy[ii] * AA;
                zz[ii] = zz[ii] * AA;
            }
            const double expfactor = exp(delts * c.vbs);
            s.lx = s.lx * expfactor;
            s.ly = s.ly * expfactor;
            s.lz = s.lz * expfactor;
            boxv = s.lx * s.ly * s.lz;
            c.pljlrc = npt_pljlrc(&s, mp->lj_lrc, boxv);
            if (s.p.charge_type == MG_ELEC_EWALD) {
                s.p.vfactor_ewald = 2.0 * pi / boxv;
                s.p.twopi_lx = 2.0 * pi / s.lx;
                s.p.twopi_ly = 2.0 * pi / s.ly;
                s.p.twopi_lz = 2.0 * pi / s.lz;
                s.p.twopi_over_3v = 2.0 * pi / 3.0 / boxv;
            }
            orc_frcshort(&s, xx, yy, zz, fxs, fys, fzs, &es);
            for (int ii = 0; ii < n; ii++) {
                const double r_mass = rmass[ii];
                vx[ii] += (deltsby2 * fxs[ii] * r_mass);
                vy[ii] += (deltsby2 * fys[ii] * r_mass);
                vz[ii] += (deltsby2 * fzs[ii] * r_mass);
            }
        }
        orc_frclong(&s, xx, yy, zz, fxl, fyl, fzl, &el, NULL);
        for (int ii = 0; ii < n; ii++) {
            const double r_mass = rmass[ii];
            vx[ii] += (deltby2 * fxl[ii] * r_mass);
            vy[ii] += (deltby2 * fyl[ii] * r_mass);
            vz[ii] += (deltby2 * fzl[ii] * r_mass);
        }
        npt_operator(mp, n, rmass, vx, vy, vz, el.virial_inter + es.virial_intra, boxv, &c);
        npt_record(log ? log + (size_t)step * 12 : NULL, &c, el.uinter, es.uintra, el.ushift, s.lx, boxv);
    }
    box[0] = s.lx;
    box[1] = s.ly;
    box[2] = s.lz;
    st->vts = c.vts;
    st->vbs = c.vbs;
    st->rts = c.rts;
    st->utsbs = c.utsbs;
    st->ukin = c.ukin;
    st->tinst = c.tinst;
    st->pinst = c.pinst;
    free(buf);
    return 0;
}
