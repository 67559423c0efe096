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
