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
        /* velinit (src/initvars.c:151-229) with the Philox streams */
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
            ox[i] = xx[i];
            oy[i] = yy[i];
            oz[i] = zz[i];
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
            const double tinst = 2.0 * ukin / mp.nfree, scaling = sqrt(hp->treq / tinst);
            ukin = 0.0;
            for (int i = 0; i < n; i++) {
                vx[i] *= scaling;
                vy[i] *= scaling;
                vz[i] *= scaling;
                ukin += hp->mass * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
            }
            ukin = 0.5 * ukin;
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
