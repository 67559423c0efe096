/*
 * frc_gb300.c - drop-in replacement of mspms2's force layer on the GB300 engine.
 *
 * Linked into the reference program in place of src/frclong.c and src/frcshort.c (and
 * of the mylibtasos Fortran library), it provides
 *   int frclong(void)   (src/frclong.c:20)  - nonbonded forces into fxl/fyl/fzl
 *   int frcshort(void)  (src/frcshort.c:20) - bonded forces into fxs/fys/fzs
 * with the same globals read and written (src/molevars.h, src/vars.h), so md.c, hmc.c,
 * siman.c, nvtnh.c and nptnh.c call it unchanged. It also provides the four Fortran
 * entry points src/sffrc.c:149-222 and :1322-1337 call (initpotentialgrid_,
 * pass_grid_file_name_, read_grids_, cforce_atom_): they keep the Tasos tables for the
 * engine instead of a Fortran module.
 *
 * Build inside the reference tree (it includes the reference's mspms2.h):
 *   gcc -std=gnu99 -O2 -fcommon -I<reference>/src -I<this repo>/include -c frc_gb300.c
 * and link with -L<this repo>/mspms2_gb300 -lmspms2_gb300.
 *
 * Environment (read on the first call):
 *   MSPMS2_GB300_DEVICE     CUDA device ordinal (default 0)
 *   MSPMS2_GB300_PRECISION  "mixed" (default) or "fp64"
 *   MSPMS2_GB300_SKIN       Verlet skin in reduced length units (default 0: rebuild each call)
 *   MSPMS2_GB300_NOEXIT     if set, a failure sets frc_gb300_status instead of exit(1)
 *
 * Errors: like the reference, a failure prints a message to stderr and fpouts and exits
 * with status 1, unless MSPMS2_GB300_NOEXIT is set.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mspms2.h"
#include "mspms2_gb300.h"

int frc_gb300_status; /* last mg_status of the engine (0 = OK) */

static mg_ctx *g_ctx;
static int g_noexit;
static mg_params g_params_set;
static int g_have_params;
static double g_box_set[3];
static int g_topo_natom = -1, g_topo_nmole[NSPECIE_MAX];
static int g_sf_loaded;

static int fail(mg_status st, const char *what) {
    frc_gb300_status = st;
    fprintf(stderr, "frc_gb300: %s failed (status %d): %s\n", what, st, g_ctx ? mg_last_error(g_ctx) : "");
    if (fpouts) fprintf(fpouts, "frc_gb300: %s failed (status %d)\n", what, st);
    if (!g_noexit) exit(1);
    return st;
}

/* ---- Tasos tables: the Fortran entry points of src/sffrc.c:149-222 ------------------- */
#define TAS_MAX 12
static int tas_n, tas_ngx, tas_ngy, tas_ngz;
static double tas_hx, tas_hy, tas_hz, tas_cuc;
static char tas_file[TAS_MAX][256];
static double *tas_values[TAS_MAX];

/* grid size rule of mylibtasos/initialize.f90:97-104 with the 0.2 A spacing of
 * mylibtasos/global.f90:214 (ANINT: round half away from zero) */
void initpotentialgrid_(int *tnuatoms, double *auc, double *buc, double *cuc, int *na, int *nb, int *nc,
                        double *radius) {
    (void)na; (void)nb; (void)nc; (void)radius;
    const double spacing = 0.2;
    tas_n = *tnuatoms;
    tas_ngx = (int)lround(*auc / spacing);
    tas_ngy = (int)lround(*buc / spacing);
    tas_ngz = (int)lround(*cuc / spacing);
    tas_hx = *auc / tas_ngx;
    tas_hy = *buc / tas_ngy;
    tas_hz = *cuc / tas_ngz;
    tas_cuc = *cuc;
}

void pass_grid_file_name_(char *name, int *idx) {
    if (*idx >= 1 && *idx <= TAS_MAX) {
        strncpy(tas_file[*idx - 1], name, 255);
        tas_file[*idx - 1][255] = 0;
    }
}

/* text format of mylibtasos/grid.f90:81-93: one node per line (F, Dx, Dy, Dz, Dxy, Dxz,
 * Dyz, Dxyz), K outermost, then J, I innermost */
void read_grids_(int *nspecies) {
    long long nn = (long long)(tas_ngx + 2) * (tas_ngy + 2) * (tas_ngz + 2);
    for (int s = 0; s < *nspecies && s < TAS_MAX; s++) {
        FILE *fp = fopen(tas_file[s], "r");
        if (!fp) {
            fprintf(stderr, "frc_gb300: cannot open Tasos grid %s\n", tas_file[s]);
            exit(1);
        }
        double *v = (double *)malloc(sizeof(double) * 8 * (size_t)nn);
        for (long long i = 0; i < 8 * nn; i++)
            if (!v || fscanf(fp, "%lf", &v[i]) != 1) {
                fprintf(stderr, "frc_gb300: Tasos grid %s is short\n", tas_file[s]);
                exit(1);
            }
        fclose(fp);
        free(tas_values[s]);
        tas_values[s] = v;
    }
    g_sf_loaded = 0;
}

/* The per-site Fortran force is evaluated on the GPU inside frclong(); nothing else in
 * the program calls it. */
void cforce_atom_(int *atomid, double *x, double *y, double *z, double *pe, double *force) {
    (void)x; (void)y; (void)z; (void)pe; (void)force;
    fprintf(stderr, "frc_gb300: cforce_atom_ called outside frclong (AtomID %d)\n", *atomid);
    exit(1);
}

/* ---- globals -> engine ------------------------------------------------------------ */
static void fill_params(mg_params *p) {
    memset(p, 0, sizeof(*p));
    p->rcutoff = rcutoff;
    p->rcuton = rcuton;
    p->rcutoffelec = rcutoffelec;
    p->lj_switch = isLJswitchOn;
    p->f0 = f0;
    p->charge_type = iChargeType;
    p->kappa = kappa;
    p->kmax[0] = KMAXX;
    p->kmax[1] = KMAXY;
    p->kmax[2] = KMAXZ;
    p->ksqmax = KSQMAX;
    p->ewald_bc = fEwald_BC ? fEwald_BC : MG_EWALD_BC_TINFOIL;
    p->coulomb_prefactor = coulomb_prefactor;
    p->sf_type = iSF_type;
    p->sigma_base = sigma_base;
    p->epsilon_base = epsilon_base;
    p->compat = MG_COMPAT_ALL;
    p->respa_split = 0.0;
    /* the derived constants as the program holds them (a volume move does not refresh the
     * Ewald ones, src/volchg.c:30-77) */
    p->rcutoffsq = rcutoffsq;
    p->rcutonsq = rcutonsq;
    p->rcutoffelecsq = rcutoffelecsq;
    p->roff2_minus_ron2_cube = roff2_minus_ron2_cube;
    p->shift1 = shift1;
    p->shift4 = shift4;
    p->wolfvcon1 = wolfvcon1;
    p->wolfvcon2 = wolfvcon2;
    p->wolfvcon3 = wolfvcon3;
    p->wolffcon1 = wolffcon1;
    p->wolffcon2 = wolffcon2;
    p->bfactor_ewald = Bfactor_ewald;
    p->vfactor_ewald = Vfactor_ewald;
    p->twopi_lx = TWOPI_LX;
    p->twopi_ly = TWOPI_LY;
    p->twopi_lz = TWOPI_LZ;
    p->twopi_over_3v = twopi_over_3v;
}

/* SAMPLE_MOLECULE (src/molevars.h:40-73) -> mg_species; the index lists are copied
 * because the reference keeps nbp_idx as doubles and the parameters in separate arrays */
static int set_topology(void) {
    static mg_species sp[NSPECIE_MAX];
    static int *ibuf[NSPECIE_MAX];
    static double *dbuf[NSPECIE_MAX];
    for (int s = 0; s < nspecie; s++) {
        SAMPLE_MOLECULE *m = &sample_mole[s];
        int na = m->natom, nb = m->nbond, ng = m->nangle, nd = m->ndih, ni = m->nimp, nn = m->nnbp;
        free(ibuf[s]);
        free(dbuf[s]);
        ibuf[s] = (int *)malloc(sizeof(int) * (size_t)(2 * na + 3 * nb + 4 * ng + 5 * nd + 5 * ni + 2 * nn + 1));
        dbuf[s] = (double *)malloc(sizeof(double) * (size_t)(4 * na + 3 * nb + 5 * ng + 4 * nd + 2 * ni + 1));
        if (!ibuf[s] || !dbuf[s]) return fail(MG_ERR_ALLOC, "topology copy");
        int *ip = ibuf[s];
        double *dp = dbuf[s];
        mg_species *o = &sp[s];
        memset(o, 0, sizeof(*o));
        o->natom = na;
        o->nmole = nmole_per_specie[s];
        o->ghost_type = m->ghost_type;
        o->interp_type = m->interp_type;
        o->epsilon = m->epsilon;
        o->sigma = m->sigma;
        o->charge = m->charge;
        o->aw = m->aw;
        o->nbond = nb;
        o->bond_idx = &m->bnd_idx[0][0];
        o->bond_type = m->bnd_type;
        for (int k = 0; k < nb; k++) {
            dp[3 * k] = m->bnd_para_0[k];
            dp[3 * k + 1] = m->bnd_para_1[k];
            dp[3 * k + 2] = m->bnd_para_2[k];
        }
        o->bond_param = dp;
        dp += 3 * nb;
        o->nangle = ng;
        o->angle_idx = &m->agl_idx[0][0];
        o->angle_type = m->agl_type;
        for (int k = 0; k < ng; k++) {
            dp[5 * k] = m->agl_para_1[k];
            dp[5 * k + 1] = m->agl_para_2[k];
            dp[5 * k + 2] = m->agl_para_3[k];
            dp[5 * k + 3] = m->agl_para_4[k];
            dp[5 * k + 4] = m->agl_para_5[k];
        }
        o->angle_param = dp;
        dp += 5 * ng;
        o->ndih = nd;
        o->dih_idx = &m->dih_idx[0][0];
        o->dih_type = m->dih_type;
        for (int k = 0; k < nd; k++) {
            dp[4 * k] = m->dih_para_1[k];
            dp[4 * k + 1] = m->dih_para_2[k];
            dp[4 * k + 2] = m->dih_para_3[k];
            dp[4 * k + 3] = m->dih_para_4[k];
        }
        o->dih_param = dp;
        dp += 4 * nd;
        o->nimp = ni;
        o->imp_idx = &m->imp_idx[0][0];
        o->imp_type = m->imp_type;
        for (int k = 0; k < ni; k++) {
            dp[2 * k] = m->imp_para_0[k];
            dp[2 * k + 1] = m->imp_para_1[k];
        }
        o->imp_param = dp;
        o->nnbp = nn;
        for (int k = 0; k < nn; k++) {
            ip[2 * k] = (int)m->nbp_idx[k][0];
            ip[2 * k + 1] = (int)m->nbp_idx[k][1];
        }
        o->nbp_idx = ip;
        g_topo_nmole[s] = nmole_per_specie[s];
    }
    mg_status st = mg_set_topology(g_ctx, nspecie, sp);
    if (st) return fail(st, "mg_set_topology");
    g_topo_natom = natom;
    return 0;
}

/* my-interp coefficients (src/vars.h:321-448): 4 quantities x 32 terms, per cube */
#define MI_LIST(X) X(0) X(1) X(2) X(3) X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) \
    X(16) X(17) X(18) X(19) X(20) X(21) X(22) X(23) X(24) X(25) X(26) X(27) X(28) X(29) X(30) X(31)

static int set_myinterp(void) {
    for (int t = 0; t < NUNIQUE_ATOM_MAX; t++) {
        if (!ene0[t]) continue;
        size_t nc = (size_t)ncube_total;
        double *co = (double *)malloc(sizeof(double) * 128 * nc);
        if (!co) return fail(MG_ERR_ALLOC, "my-interp copy");
        const double *src[128];
        int k = 0;
#define MI_E(i) src[k++] = ene##i[t];
#define MI_X(i) src[k++] = fxa##i[t];
#define MI_Y(i) src[k++] = fya##i[t];
#define MI_Z(i) src[k++] = fza##i[t];
        MI_LIST(MI_E) MI_LIST(MI_X) MI_LIST(MI_Y) MI_LIST(MI_Z)
        for (int q = 0; q < 128; q++) memcpy(co + (size_t)q * nc, src[q], sizeof(double) * nc);
        mg_status st = mg_sf_myinterp_set(g_ctx, t, ncube_x, ncube_y, ncube_z, grid_itvl_x, grid_itvl_y,
                                          grid_itvl_z, xmin, ymin, zmax, co);
        free(co);
        if (st) return fail(st, "mg_sf_myinterp_set");
    }
    return 0;
}

static int set_solid_fluid(void) {
    mg_status st = MG_OK;
    switch (iSF_type) {
    case MG_SF_HYPERGEO:
        st = mg_sf_hypergeo_set(g_ctx, ntube, hgntc_xx, hgntc_yy, hgnt_radius, solid_sigma[0], solid_epsilon[0],
                                const_3pisq_theta);
        break;
    case MG_SF_ATOM_EXPLICIT:
        st = mg_sf_atom_explicit_set(g_ctx, solid_natom, solid_xx, solid_yy, solid_zz, solid_sigma[0],
                                     solid_epsilon[0]);
        break;
    case MG_SF_TASOS:
        for (int t = 0; t < tas_n && t < TAS_MAX; t++) {
            if (!tas_values[t]) continue;
            st = mg_sf_tasos_set_grid(g_ctx, t + 1, tas_ngx + 2, tas_ngy + 2, tas_ngz + 2, tas_hx, tas_hy, tas_hz,
                                      tas_cuc, tas_values[t]);
            if (st) break;
        }
        break;
    case MG_SF_MY_INTERP:
        return set_myinterp();
    default:
        break;
    }
    if (st) return fail(st, "solid-fluid tables");
    g_sf_loaded = 1;
    return 0;
}

static int ensure_engine(void) {
    if (!g_ctx) {
        mg_options opt;
        mg_options_default(&opt);
        const char *v;
        if ((v = getenv("MSPMS2_GB300_DEVICE"))) opt.device = atoi(v);
        if ((v = getenv("MSPMS2_GB300_PRECISION")) && !strcmp(v, "fp64")) opt.precision = MG_PREC_FP64;
        if ((v = getenv("MSPMS2_GB300_SKIN"))) opt.skin = atof(v);
        g_noexit = getenv("MSPMS2_GB300_NOEXIT") != NULL;
        mg_status st = mg_create(&g_ctx, &opt);
        if (st) return fail(st, "mg_create (an sm_103 GPU is required)");
    }
    mg_params p;
    fill_params(&p);
    if (!g_have_params || memcmp(&p, &g_params_set, sizeof(p)) != 0) {
        mg_status st = mg_set_params(g_ctx, &p);
        if (st) return fail(st, "mg_set_params");
        g_params_set = p;
        g_have_params = 1;
    }
    int topo = g_topo_natom != natom;
    for (int s = 0; s < nspecie && !topo; s++) topo = g_topo_nmole[s] != nmole_per_specie[s];
    if (topo && set_topology()) return frc_gb300_status;
    if (boxlx != g_box_set[0] || boxly != g_box_set[1] || boxlz != g_box_set[2]) {
        mg_status st = mg_set_box(g_ctx, boxlx, boxly, boxlz);
        if (st) return fail(st, "mg_set_box");
        g_box_set[0] = boxlx;
        g_box_set[1] = boxly;
        g_box_set[2] = boxlz;
    }
    if (!g_sf_loaded && iSF_type != MG_SF_NONE && set_solid_fluid()) return frc_gb300_status;
    return 0;
}

/* ---- the force calls ---------------------------------------------------------------- */
int frclong(void) {
    if (ensure_engine()) return 0;
    mg_energies e;
    mg_status st = mg_compute(g_ctx, xx, yy, zz, MG_TERMS_LONG, fxl, fyl, fzl, NULL, NULL, NULL, &e);
    frc_gb300_status = st;
    if (st) {
        fail(st, "mg_compute (long)");
        return 0;
    }
    uvdw = e.uvdw;
    ushift = e.ushift;
    ureal = e.ureal;
    uexcl = e.uexcl;
    ufourier = e.ufourier;
    uself = e.uself;
    uvacuum = e.uvacuum;
    uelec = e.uelec;
    usflj = e.usflj;
    uotherff = e.uotherff;
    uinter = e.uinter;
    virial_inter = e.virial_inter;
    return 0;
}

int frcshort(void) {
    if (ensure_engine()) return 0;
    mg_energies e;
    mg_status st = mg_compute(g_ctx, xx, yy, zz, MG_TERMS_SHORT, NULL, NULL, NULL, fxs, fys, fzs, &e);
    frc_gb300_status = st;
    if (st) {
        fail(st, "mg_compute (short)");
        return 0;
    }
    ubond = e.ubond;
    uangle = e.uangle;
    udih = e.udih;
    uimp = e.uimp;
    uintra = e.uintra;
    virial_intra = e.virial_intra;
    return 0;
}
