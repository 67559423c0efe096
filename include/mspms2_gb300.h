/*
 * mspms2_gb300.h - C ABI of the GB300 (sm_103a) nonbonded-force engine for mspms2.
 *
 * The engine evaluates, on one GPU, what the reference computes in
 *   frclong()  (src/frclong.c:20-1233)  - all nonbonded forces into fxl/fyl/fzl:
 *              LJ (src/ljfrc.c:21-71), Ewald real/exclusion and Wolf
 *              (src/elecfrc.c:17-60), plain Coulomb (src/elecfrc.c:138-241),
 *              Ewald reciprocal + self + vacuum dipole (src/frclong.c:988-1129),
 *              Wolf self (src/frclong.c:1130-1143), solid-fluid potentials
 *              (src/frclong.c:1145-1209, src/sffrc.c, the mylibtasos Fortran sources);
 *   frcshort() (src/frcshort.c:20-91)  - bonded forces into fxs/fys/fzs
 *              (src/bndfrc.c, src/aglfrc.c, src/dihfrc.c, src/impfrc.c).
 *
 * Plain C types only: pointers, sizes, doubles. Every call returns an mg_status
 * (0 = success); mg_last_error() gives a one-line description of the last failure
 * in the calling thread's most recently used context.
 *
 * Units are whatever the caller uses consistently; the reference passes its
 * reduced units (length sigma_base A, energy epsilon_base K). Only the tabulated
 * solid-fluid models convert to A/K internally, exactly like the reference
 * (src/sffrc.c:1322-1337, src/sffrc.c:951-965), using mg_params.sigma_base and
 * mg_params.epsilon_base.
 *
 * Threading: a context is used by one host thread at a time. Many contexts may
 * coexist (each owns its device buffers and CUDA stream).
 */
#ifndef MSPMS2_GB300_H_
#define MSPMS2_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MG_ABI_VERSION 1

#if defined(__GNUC__)
#define MG_API __attribute__((visibility("default")))
#else
#define MG_API
#endif

typedef int mg_status;
enum {
    MG_OK = 0,
    MG_ERR_INVALID = 1,      /* bad argument or inconsistent input */
    MG_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    MG_ERR_NO_DEVICE = 3,    /* no usable sm_103 device */
    MG_ERR_STATE = 4,        /* call order violated (e.g. compute before topology) */
    MG_ERR_OUT_OF_GRID = 5,  /* a site left a solid-fluid table (reference: AtomID=-9999,
                                mylibtasos/forces.f90:59-79; assert, src/sffrc.c:987) */
    MG_ERR_NONFINITE = 6,    /* a force or energy came out NaN/Inf */
    MG_ERR_CAPACITY = 7,     /* an internal list exceeded its capacity after retries */
    MG_ERR_UNSUPPORTED = 8,  /* a model option the engine does not implement */
    MG_ERR_ALLOC = 9         /* device or host allocation failed */
};

/* Precision of the pair/k-space/solid-fluid arithmetic. */
enum {
    MG_PREC_MIXED = 0,  /* FP32 pair, k-space and solid-fluid arithmetic; per-site forces and
                           energies carried as exact FP32 hi+lo pairs or FP64; structure
                           factors summed in FP32 per 512-site block, in FP64 across blocks */
    MG_PREC_FP64 = 1    /* every step in FP64 (the plain-FP64 GPU path) */
};

/* Model selectors; the numeric values are the reference's (src/defs.h:129-170). */
enum { MG_GHOST_NONE = 0, MG_GHOST_LJ = 1, MG_GHOST_FULL = 2 };
enum { MG_BOND_NONE = 0, MG_BOND_HARMONIC = 1, MG_BOND_MORSE = 2, MG_BOND_FENE = 3 };
enum { MG_ANGLE_NONE = 0, MG_ANGLE_HARMONIC = 1, MG_ANGLE_TR_WATER = 2 };
enum { MG_DIH_NONE = 0, MG_DIH_OPLS = 1, MG_DIH_CHARMM = 2 };
enum { MG_IMP_NONE = 0, MG_IMP_CHARMM = 1 };
enum { MG_SF_NONE = 0, MG_SF_HYPERGEO = 1, MG_SF_ATOM_EXPLICIT = 2, MG_SF_TASOS = 3,
       MG_SF_MY_INTERP = 4 };
enum { MG_ELEC_NONE = 0, MG_ELEC_EWALD = 1, MG_ELEC_WOLF = 2, MG_ELEC_SIMPLE_COULOMB = 3 };
enum { MG_EWALD_BC_TINFOIL = 1, MG_EWALD_BC_VACUUM = 2 };

/* Reference behaviours reproduced by default (mg_params.compat, bit flags).
 * Clearing a bit selects the corrected behaviour instead. */
enum {
    MG_COMPAT_NBP_INDEX = 1 << 0,   /* nbp pair read as nbp_idx[ndih] (src/frclong.c:793-794) */
    MG_COMPAT_TASOS_DXYZ = 1 << 1,  /* Dxyz weights of corners (i,j,k+1)/(i+1,j+1,k) swapped
                                       (mylibtasos/cubicauxiliary.f90:219-233 vs forces.f90:155-162) */
    MG_COMPAT_TASOS_PE_FLIP = 1 << 2, /* PE = -F if F < 1.5*minPE (mylibtasos/forces.f90:167-171) */
    MG_COMPAT_HYPERGEO_LAST = 1 << 3, /* hypergeo energy keeps the last tube only (src/sffrc.c:1201) */
    MG_COMPAT_ALL = 0xF
};

/* One molecular species: the reference's SAMPLE_MOLECULE template
 * (src/molevars.h:40-73) plus its molecule count (nmole_per_specie). Atoms of a
 * molecule are contiguous, molecules of a species are contiguous and species follow
 * each other in order, exactly as the reference lays out xx/yy/zz. */
typedef struct mg_species {
    int natom;                 /* sites per molecule */
    int nmole;                 /* molecules of this species */
    const int *ghost_type;     /* [natom] MG_GHOST_* */
    const int *interp_type;    /* [natom] solid-fluid table id (Tasos: 1-based AtomID;
                                  my-interp: 0-based, as after init_my_interp) */
    const double *epsilon;     /* [natom] */
    const double *sigma;       /* [natom] */
    const double *charge;      /* [natom] */
    const double *aw;          /* [natom] site mass (for centres of mass) */
    int nbond;
    const int *bond_idx;       /* [nbond*2] */
    const int *bond_type;      /* [nbond] */
    const double *bond_param;  /* [nbond*3]  Kb, Req, alpha */
    int nangle;
    const int *angle_idx;      /* [nangle*3] */
    const int *angle_type;     /* [nangle] */
    const double *angle_param; /* [nangle*5] agl_para_1..5 (Ktheta, Thetaeq, p3, p4, p5) */
    int ndih;
    const int *dih_idx;        /* [ndih*4] */
    const int *dih_type;       /* [ndih] */
    const double *dih_param;   /* [ndih*4]  c1..c4 */
    int nimp;
    const int *imp_idx;        /* [nimp*4] */
    const int *imp_type;       /* [nimp] */
    const double *imp_param;   /* [nimp*2]  komega, omega0 */
    int nnbp;
    const int *nbp_idx;        /* [nnbp*2] */
} mg_species;

/* Force-field parameters and the derived constants the reference keeps as globals
 * (src/vars.h). The derived block is taken as given so that a caller that keeps
 * stale constants (the reference's volume move does not refresh the Ewald box
 * constants, src/volchg.c:30-77) gets the reference's numbers; mg_params_derive()
 * fills it the way src/initvars.c:591-599 and :433-462 do. */
typedef struct mg_params {
    double rcutoff, rcuton, rcutoffelec;
    int lj_switch;              /* isLJswitchOn */
    double f0;                  /* 1-4 LJ scale */
    int charge_type;            /* MG_ELEC_* */
    double kappa;               /* Ewald/Wolf damping (reduced) */
    int kmax[3];                /* KMAXX, KMAXY, KMAXZ */
    int ksqmax;                 /* KSQMAX */
    int ewald_bc;               /* MG_EWALD_BC_* */
    double coulomb_prefactor;   /* reduced Coulomb constant */
    int sf_type;                /* MG_SF_* */
    double sigma_base, epsilon_base; /* unit scales used by the tabulated SF models */
    unsigned compat;            /* MG_COMPAT_* */
    double respa_split;         /* 0: reference split (short = bonded, long = nonbonded).
                                   > 0: distance split radius; short also gets the
                                   inter-molecular LJ/real-space pairs with r < respa_split */
    /* derived (set by mg_params_derive or copied from the reference globals) */
    double rcutoffsq, rcutonsq, rcutoffelecsq, roff2_minus_ron2_cube;
    double shift1, shift4;
    double wolfvcon1, wolfvcon2, wolfvcon3, wolffcon1, wolffcon2;
    double bfactor_ewald, vfactor_ewald, twopi_lx, twopi_ly, twopi_lz, twopi_over_3v;
} mg_params;

/* Energies and virials written by mg_compute; names and meanings follow the
 * reference globals (src/vars.h:164-205). uelec holds uewald/uwolf/ucoulomb. */
typedef struct mg_energies {
    double uvdw, ushift, ureal, uexcl, ufourier, uself, uvacuum, uelec;
    double usflj, uotherff, uinter, virial_inter;
    double ubond, uangle, udih, uimp, uintra, virial_intra;
} mg_energies;

enum { MG_TERMS_LONG = 1, MG_TERMS_SHORT = 2, MG_TERMS_ALL = 3 };

typedef struct mg_options {
    int device;          /* CUDA device ordinal */
    int precision;       /* MG_PREC_* */
    double skin;         /* Verlet skin added to the list radius (caller units); the list is
                            rebuilt when any site moved more than skin/2. 0 = rebuild each call */
    int deterministic;   /* nonzero: fixed-order reductions everywhere (default 1) */
} mg_options;

typedef struct mg_ctx mg_ctx;

/* Statistics of the last mg_compute (for measurement; no effect on results). */
typedef struct mg_stats {
    long long pairs_within_cutoff;  /* inter-molecular site pairs with r < cutoff, counted once */
    long long cluster_pairs;        /* i-cluster x j-cluster entries processed (full list) */
    long long nclusters;
    long long kvectors;             /* half-space k-vectors evaluated */
    int list_rebuilt;               /* 1 if the neighbour list was rebuilt in this call */
    int list_builds;                /* total builds since creation */
    double kernel_ms[8];            /* per-stage device times of the last call, if timing is on:
                                       0 list build + packing, 1 pair kernel, 2 intra+bonded,
                                       3 k-space phases + S(k) + its reduction, 4 k-space force,
                                       5 solid-fluid, 6 reductions and checks, 7 total */
    int kernel_launches;            /* kernels this library launched in the last call */
} mg_stats;

/* ---- lifecycle ---------------------------------------------------------- */
/* Every entry point checks its handles: a NULL context or required pointer returns
 * MG_ERR_INVALID (mg_destroy(NULL) is a no-op returning MG_OK; the two void helpers
 * below ignore a NULL struct). */
MG_API void mg_options_default(mg_options *opt);
MG_API mg_status mg_create(mg_ctx **ctx, const mg_options *opt);
MG_API mg_status mg_destroy(mg_ctx *ctx);
MG_API const char *mg_last_error(const mg_ctx *ctx);
MG_API int mg_abi_version(void);

/* ---- system description -------------------------------------------------- */
/* Fill the derived block of p from its primary fields and the box
 * (src/initvars.c:591-599, :433-455; coulomb_prefactor, :462, is a primary field). */
MG_API void mg_params_derive(mg_params *p, double lx, double ly, double lz);
/* Call mg_set_params first: the nbp bit of mg_params.compat is read here. */
MG_API mg_status mg_set_topology(mg_ctx *ctx, int nspecies, const mg_species *species);
MG_API mg_status mg_set_params(mg_ctx *ctx, const mg_params *p);
MG_API mg_status mg_set_box(mg_ctx *ctx, double lx, double ly, double lz);
/* Use the caller's CUDA stream (cudaStream_t passed as void*); NULL = the context's own. */
MG_API mg_status mg_set_stream(mg_ctx *ctx, void *stream);
MG_API mg_status mg_set_timing(mg_ctx *ctx, int enable);

/* ---- solid-fluid models (src/sffrc.c) ------------------------------------ */
/* Tasos tricubic-Hermite grid for AtomID `type` (1-based). `values` holds the
 * node records in the reference's Fortran order FG(I,J,K) with I fastest
 * (mylibtasos/grid.f90:81-93): 8 doubles per node (F, Dx, Dy, Dz, Dxy, Dxz, Dyz,
 * Dxyz), nx*ny*nz nodes (nx = ngx+2 ...). Grid spacing hx,hy,hz (A); cuc is the
 * z period used by the nanotube PBC (mylibtasos/pbc.f90:80-84). */
MG_API mg_status mg_sf_tasos_set_grid(mg_ctx *ctx, int type, int nx, int ny, int nz,
                               double hx, double hy, double hz, double cuc,
                               const double *values);
/* Hypergeometric smooth tubes (src/sffrc.c:16-78, 1092-1209), reduced units. */
MG_API mg_status mg_sf_hypergeo_set(mg_ctx *ctx, int ntube, const double *cx, const double *cy,
                             const double *radius, double solid_sigma, double solid_epsilon,
                             double const_3pisq_theta);
/* Explicit solid atoms (src/sffrc.c:81-142, 1213-1314), reduced units. */
MG_API mg_status mg_sf_atom_explicit_set(mg_ctx *ctx, int nsolid, const double *sx, const double *sy,
                                  const double *sz, double solid_sigma, double solid_epsilon);
/* "My interp" 32-term per-cube polynomials (src/sffrc.c:228-748, 951-1089) for table
 * `type` (0-based): coeff = [4][32][ncube] doubles (energy, fx, fy, fz), cube index
 * ix*ncy*ncz + iy*ncz + iz; lengths in A. */
MG_API mg_status mg_sf_myinterp_set(mg_ctx *ctx, int type, int ncx, int ncy, int ncz,
                             double itvl_x, double itvl_y, double itvl_z,
                             double xmin, double ymin, double zmax, const double *coeff);

/* ---- evaluation ---------------------------------------------------------- */
/* Host buffers. x/y/z: [natom] site positions (unwrapped, as the reference keeps them).
 * terms: MG_TERMS_*. Long forces go to fxl/fyl/fzl, short to fxs/fys/fzs (each
 * overwritten; a triple may be NULL when its terms are not requested). e may be NULL. */
MG_API mg_status mg_compute(mg_ctx *ctx, const double *x, const double *y, const double *z, int terms,
                     double *fxl, double *fyl, double *fzl,
                     double *fxs, double *fys, double *fzs, mg_energies *e);
/* Same with device pointers (inputs resident in HBM, outputs written on device). The
 * energies are written to host memory after the call completes. */
MG_API mg_status mg_compute_device(mg_ctx *ctx, const double *d_x, const double *d_y,
                            const double *d_z, int terms,
                            double *d_fxl, double *d_fyl, double *d_fzl,
                            double *d_fxs, double *d_fys, double *d_fzs, mg_energies *e);
MG_API mg_status mg_get_stats(const mg_ctx *ctx, mg_stats *s);

/* ---- autotuning (no reference counterpart) ------------------------------------- */
/* The launch geometry the engine picks per system: the cell size of the neighbour-list
 * grid (column width, as a factor of the default min((8 V/N)^(1/3), 0.75 r_list)), the
 * cluster size (the largest z extent of a cluster, as a factor of the column width;
 * clusters hold at most 8 sites) and the threads per site of the reciprocal-space force
 * pass (2, 4 or 8). Results are reproducible for a given geometry; two geometries sum in
 * different orders, so their results agree to rounding, not bit for bit. */
typedef struct mg_tuning {
    double cell_scale, zcap_scale;
    int kforce_threads;
    double ms_default, ms_tuned;  /* one evaluation with the default and the chosen geometry */
    int configs_tried;
} mg_tuning;
/* Times evaluations of `terms` at host positions x, y, z over a small set of geometries
 * (threads per site first, then cell size x cluster size) and keeps the fastest. */
MG_API mg_status mg_autotune(mg_ctx *ctx, const double *x, const double *y, const double *z, int terms,
                             mg_tuning *out);
/* Applies a geometry found before (scales within 0.5..2, threads 2, 4 or 8). */
MG_API mg_status mg_set_tuning(mg_ctx *ctx, const mg_tuning *t);
MG_API mg_status mg_get_tuning(const mg_ctx *ctx, mg_tuning *t);
/* Device status word of the last call: bit 0 out-of-grid, bit 1 non-finite result,
 * bit 2 list overflow, bit 3 column overflow. */
MG_API mg_status mg_get_device_flags(const mg_ctx *ctx, unsigned *flags);

/* ---- neighbour-list inspection (tests of the bit-exact list build) ----------- */
/* Copies the cluster layout and cluster-pair list of the last build:
 * grid[3] = (columns along x, columns along y, small-box flag), *zcap = the largest z
 * extent of a cluster, cluster_atoms[ncl*8] (site index or -1), pairs[npairs*2]
 * (i-cluster, j-cluster, grouped by i-cluster in search order), shifts[npairs*3] (the
 * periodic image of the j-cluster in box lengths). Pass NULL buffers to query ncl and
 * npairs. */
MG_API mg_status mg_debug_get_list(mg_ctx *ctx, int *ncl, long long *npairs, int *grid, double *zcap,
                            int *cluster_atoms, int *pairs, int *shifts);

/* ---- device-resident integration (src/md.c, src/nvtnh.c) -------------------- */
/* Schemes; the values are the reference's what_ensemble codes (src/defs.h:18-19). */
enum {
    MG_MD_NVE = 0,    /* vver(): velocity Verlet RESPA step (src/md.c:22-85) */
    MG_MD_NVT_NH = 1  /* vver_nh_3(): Nose-Hoover RESPA step with implicit thermostat
                         solves (src/nvtnh.c:11-271) */
};

/* Integration parameters, in the reference's reduced units and names (src/vars.h). */
typedef struct mg_md_params {
    int scheme;       /* MG_MD_* */
    int nstep_inner;  /* short-force steps per outer step (nstep_inner) */
    double delt;      /* outer step (delt after src/readins.c:73) */
    double treq;      /* target temperature */
    double qq, qqs;   /* thermostat masses, outer and inner (the MDNVT input section) */
    double gg, ggs;   /* thermostat degrees of freedom (the reference sets both to nfree) */
    int nfree;        /* 3*natom - nconstraint (src/initvars.c:588), for tinst */
} mg_md_params;

/* Thermostat scalars and the last step's kinetic quantities (src/vars.h:137-157). */
typedef struct mg_md_state {
    double ps, ss, pss, sss;          /* thermostat momenta and positions, outer and inner */
    double ukin, tinst, unhts, unhtss;
} mg_md_state;

/* Values recorded per step by mg_md_run, in this order: ukin, uinter, uintra, ushift,
 * ps, ss, pss, sss, tinst, unhts, unhtss, (unused). With a distance split
 * (mg_params.respa_split > 0) uinter and ushift are the sums of both buckets. */
#define MG_MD_LOG 12

/* Runs nsteps steps of the scheme on the device, like the reference's main loop does with
 * vver_nh_3() or vver() (src/mspms2.c:67-77): forces are evaluated first at the given
 * positions, then every step kicks, drifts and re-evaluates forces with the positions,
 * velocities and thermostat scalars kept in device memory. x/y/z and vx/vy/vz (host,
 * [natom]) hold the start and are overwritten with the end; state likewise. log, if not
 * NULL, receives (nsteps+1)*MG_MD_LOG doubles: the start, then every step. Site masses
 * are the topology's aw. */
MG_API mg_status mg_md_run(mg_ctx *ctx, const mg_md_params *p, int nsteps, double *x, double *y, double *z,
                           double *vx, double *vy, double *vz, mg_md_state *state, double *log);

/* ---- NPT (npt_respa, src/nptnh.c:10-234) ------------------------------------------ */
/* Isotropic Nose-Hoover thermostat + barostat around a RESPA step: the operator
 * npt_nh_operator() (src/nptnh.c:10-132) before and after the step, inner steps that
 * scale positions by exp(dt_inner/2 vbs) around the drift and the box by exp(dt_inner vbs),
 * with the LJ long-range correction (src/misc.c:131-148, terms of src/initvars.c:476-520
 * when lj_lrc is set) and the Ewald box constants refreshed every inner step. */
typedef struct mg_npt_params {
    int nstep_inner;
    double delt, treq, preq;  /* reduced: time, temperature, pressure (bar / pressure_base) */
    double qts, qbs;          /* thermostat and barostat masses (MDNPT section) */
    int nfree;                /* 3*natom - nconstraint */
    int lj_lrc;               /* isLJlrcOn: add the LJ long-range pressure correction */
} mg_npt_params;

typedef struct mg_npt_state {
    double vts, vbs, rts;     /* thermostat velocity, barostat velocity, thermostat position */
    double utsbs, ukin, tinst, pinst;
} mg_npt_state;

/* Values recorded per step by mg_npt_run: ukin, uinter, uintra, ushift, vts, vbs, rts,
 * utsbs, tinst, pinst, boxlx, boxv. Row 0 (the start) holds pinst of the start forces
 * (the reference leaves pinst unset until its first step). */
#define MG_NPT_LOG 12

/* Runs nsteps npt_respa steps on the device. x, y, z, vx, vy, vz [natom] and box[3] hold
 * the start and receive the end; the context's box and Ewald constants follow the box.
 * state holds vts, vbs, rts at the start (init_npt_respa, src/initvars.c:378-380, sets
 * vts = sqrt((nfree+1)/qts), vbs = sqrt((nfree+1)/qbs), rts = 0) and receives the end.
 * log, if not NULL, receives (nsteps+1)*MG_NPT_LOG doubles. */
MG_API mg_status mg_npt_run(mg_ctx *ctx, const mg_npt_params *p, int nsteps, double *x, double *y, double *z,
                            double *vx, double *vy, double *vz, double *box, mg_npt_state *state, double *log);

/* ---- batched simulated annealing of Lennard-Jones replicas -------------------- */
/* Many independent one-site LJ boxes of uneven size (reduced units, cubic boxes of at
 * least 2 rcutoff, no switch) through the reference's siman() schedule
 * (src/siman.c:62-182), all in one persistent launch: a thread block takes whole
 * replicas, largest first. Each stage of the schedule (as mg_siman_run: T = t_initial /
 * mu_t^k up to the first T below t_min) is velinit at T with the exact rescaling,
 * n_tries vver_nh_3 steps with one inner step (src/nvtnh.c:11-271; a one-site fluid has
 * no short forces) and the thermostat reset, gg = ggs = nfree = 3 natom - nconstraint.
 * Replica r draws its velocities from mg_siman_run's Philox streams with the seed
 * seed ^ (r * 0x9E3779B97F4A7C15), so mg_siman_run on that replica alone with that seed
 * gives the same run up to the FP32 pair forces used here. Positions in and out; log:
 * per replica and stage, MG_SIMAN_BATCH_LOG values at the stage end: T, ukin, uinter
 * (LJ), ushift (the shift energy of the pairs inside the cutoff), tinst. */
typedef struct mg_siman_batch_params {
    double eps, sigma, rcutoff, mass;
    double delt;                      /* outer step (one inner step) */
    double qq, qqs;                   /* Nose-Hoover masses */
    double t_initial, t_min, mu_t;
    int n_tries, max_stages;
    uint64_t seed;
    int nconstraint;
} mg_siman_batch_params;
#define MG_SIMAN_BATCH_LOG 5
MG_API mg_status mg_siman_batch(int device, const mg_siman_batch_params *p, int nrep, const int *natom,
                                const double *box, double *x, double *y, double *z, int *nstages,
                                double *stage_log);

/* ---- trajectory file (trajectory(), src/dumpxyz.c:37-66) ------------------------ */
/* Attaches a trajectory file in the reference's binary layout (trj.mspms) to the
 * context: the header is written now; mg_md_run and mg_npt_run then append the frame
 * before their first step (once per file, as src/mspms2.c:57-60 does) and a frame every
 * `every` steps counted across calls (src/mspms2.c:123-126); mg_siman_run counts one step
 * per stage, as the reference's loop does. Frames leave the device through two staging
 * buffers, a copy stream and a writer thread, so the integrator does not wait for the
 * file. atom_names: 5 bytes per template site, species by species (the reference's
 * atom_name fields; shorter names NUL-padded). Site masses are the topology's aw. */
MG_API mg_status mg_traj_open(mg_ctx *ctx, const char *path, int every, const char *atom_names);
/* Waits for the queued frames, closes the file and detaches it; *nframes (optional)
 * receives the number of frames written. */
MG_API mg_status mg_traj_close(mg_ctx *ctx, long long *nframes);

/* ---- checkpoint (saveit()/loadit(), src/loadsave.c:19-128) --------------------- */
#define MG_NCOUNTS 40 /* NCOUNTS_MAX (src/defs.h:77) */
typedef struct mg_checkpoint {
    int natom;
    double *x, *y, *z, *vx, *vy, *vz;            /* [natom], caller-owned */
    double qq, ps, gg, ss, qqs, pss, ggs, sss;   /* Nose-Hoover (MDNVT) */
    double vts, rts, vbs;                        /* NPT thermostat/barostat */
    double boxlx, boxly, boxlz, boxv;
    int equilibrium;                             /* bEquilibrium, stored as one byte */
    int nframe, istep;
    int counts[MG_NCOUNTS];
    double accum[MG_NCOUNTS];                    /* the reference writes NCOUNTS_MAX doubles
                                                    of its accum[NCOUNTS_MAX][8]: its first
                                                    five rows */
} mg_checkpoint;
/* Writes the file byte for byte as saveit() does. */
MG_API mg_status mg_checkpoint_save(const char *path, const mg_checkpoint *ck);
/* Reads it as loadit() does: the counters (equilibrium .. accum) only with
 * with_counters (a continued run, iStart_option CONTINUE). */
MG_API mg_status mg_checkpoint_load(const char *path, mg_checkpoint *ck, int with_counters);
/* Sets the context's box to the checkpoint's and drops everything the engine keeps for
 * the old box (cluster list, k-vector tables). The Ewald box constants stay as
 * mg_set_params gave them, as loadit() leaves its globals. */
MG_API mg_status mg_checkpoint_apply(mg_ctx *ctx, const mg_checkpoint *ck);

/* No reference counterpart: mg_md_run (and the stages of mg_siman_run) replay whole
 * integration steps as one captured CUDA graph when they can: after an eager first force
 * evaluation, one step is captured and replayed nsteps times, with the energies of every
 * force call logged on the device and read after the run. Results are identical to the
 * step-by-step path. The steps run step by step instead when a trajectory is attached,
 * when the thermostat solve cannot run as a cooperative launch, or when a replayed step
 * raised a flag that needs the host (list capacity, small box, non-finite force, a site
 * off its table); then the start state is restored and the run repeated step by step.
 * Enabled by default; mg_get_md_graphs reports how many steps the last run replayed. */
MG_API mg_status mg_set_md_graphs(mg_ctx *ctx, int enable);
MG_API mg_status mg_get_md_graphs(const mg_ctx *ctx, int *enabled, int *last_steps);

/* Reciprocal-space overlap: with Ewald, the phase tables, S(k) and k-space force passes of
 * an evaluation run on a second stream of the context, beside the neighbour list and pair
 * kernels, and are joined (forces added, energy rows copied) where the serial order adds
 * them, so that results are identical either way. Enabled by default. */
MG_API mg_status mg_set_kspace_overlap(mg_ctx *ctx, int enable);

/* Structure factors on the tensor cores (mixed precision, KMAXZ <= 30): the sum over sites
 * as TF32 MMAs with a 3-term split product and FP32 accumulation; off, the CUDA-core FP32
 * pass. Enabled by default; no effect on the FP64 path. The two agree to FP32 rounding. */
MG_API mg_status mg_set_kspace_tensor(mg_ctx *ctx, int enable);

/* Bound of each on-chip pipeline wait (mbarrier poll loop) of the tensor-core S(k) pass, in
 * polls, for every context and mg_ewald_recip_static call of the process from the next
 * launch on; a negative value restores the default (2^20 polls, well under a second). When a
 * wait runs out, the pass stops issuing MMAs, waits with the default bound for the ones it
 * issued, frees its tensor memory and returns: mg_compute and the integrators then fail with
 * MG_ERR_CUDA, and mg_ewald_recip_static returns NaN forces and energy. 0 makes the first
 * wait give up at once, which exercises that path without a fault (tests). No reference
 * counterpart: the reference has no device code. */
MG_API mg_status mg_set_wait_limit(long long polls);

/* ---- simulated annealing (siman, src/siman.c:62-182) ---------------------------- */
/* Stages at T = t_initial, t_initial/mu_t, t_initial/mu_t^2, ...; the run ends after the
 * first stage whose T is below t_min (the reference tests T < t_min after the stage). A
 * stage is velinit at T (src/initvars.c:151-229: Gaussian velocities sqrt(T/aw) g, total
 * momentum removed, rescaled to T exactly), forces, n_tries vver_nh_3 steps with
 * treq = T, then the thermostat scalars are reset to zero (src/siman.c:167-174). The
 * Gaussians come from Philox4x32-10 (include/mg_philox.h), key = seed, counter = (site,
 * stage, 0 or 1, 0x5349), in place of the reference's serial generator. */
typedef struct mg_siman_params {
    mg_md_params md;   /* scheme MG_MD_NVT_NH; md.treq is set per stage */
    double t_initial;  /* reduced temperature of the first stage */
    double t_min;      /* the last stage is the first one below t_min */
    double mu_t;       /* cooling divisor (> 1) */
    int n_tries;       /* vver_nh_3 steps per stage (iters_fixed_t only paces printing) */
    int max_stages;    /* rows of stage_log; a longer schedule is refused */
    uint64_t seed;
} mg_siman_params;

/* Values recorded per stage by mg_siman_run, at the end of the stage: T, ukin, uinter,
 * uintra, ushift, tinst, unhts, unhtss. */
#define MG_SIMAN_LOG 8

/* Number of stages of the schedule, or -1 if it is invalid or needs more than limit. */
MG_API int mg_siman_stage_count(double t_initial, double t_min, double mu_t, int limit);

/* Runs the whole schedule on the device. x, y, z hold the start and receive the end;
 * vx, vy, vz receive the final velocities; state holds the first stage's thermostat
 * scalars and receives the last; *nstages the number of stages run; stage_log, if not
 * NULL, nstages*MG_SIMAN_LOG doubles. */
MG_API mg_status mg_siman_run(mg_ctx *ctx, const mg_siman_params *p, double *x, double *y, double *z,
                              double *vx, double *vy, double *vz, mg_md_state *state, int *nstages,
                              double *stage_log);

/* ---- batched Hybrid Monte Carlo (src/hmc.c:23-40, src/dispmd.c:12-103) ------- */
/* Lennard-Jones replicas (one site type, cubic boxes, reduced units). */
typedef struct mg_hmc_params {
    double eps, sigma, rcutoff;  /* LJ parameters and cutoff (no switch) */
    double mass;                 /* site mass */
    double treq;                 /* temperature */
    double delt;                 /* velocity-Verlet step */
    int nstep_md;                /* steps per move (nstep_md_per_hmc) */
    unsigned long long seed;     /* key of the Philox streams (include/mg_philox.h) */
    int rescale;                 /* 1: rescale the drawn velocities to exactly treq, as the
                                    reference's velinit does (src/initvars.c:210-218);
                                    0: plain Maxwell-Boltzmann draws */
    int nconstraint;             /* nfree = 3 natom - nconstraint, for the rescaling */
} mg_hmc_params;

/* nmoves canonical HMC moves of every replica, all in one launch: per move Maxwell-
 * Boltzmann velocities with zero momentum (velinit, src/initvars.c:151-229), nstep_md
 * velocity-Verlet steps (vver, src/md.c:22-85) and the reference's Metropolis test on
 * dH = (dU + dK + dUshift)/T (src/dispmd.c:48-66). Replica r has natom[r] sites in a
 * cubic box box[r] >= 2 rcutoff; x/y/z hold all replicas one after another (host,
 * in/out). Random draws are keyed by (seed, replica, move0 + move, atom), so a run of
 * k moves followed by one with move0 = k equals one run of 2k moves. Out: accepted[r]
 * (moves accepted), energy[r] (potential energy plus shift energy of the final state),
 * dh_log[r*nmoves + m] if not NULL. Pair forces FP32, energies FP64. A replica's
 * positions and cell list must fit in shared memory (about 8000 sites); larger give
 * MG_ERR_CAPACITY. Allocates device memory for the call. */
MG_API mg_status mg_hmc_batch(int device, const mg_hmc_params *p, int nrep, const int *natom, const double *box,
                              double *x, double *y, double *z, int nmoves, int move0, int *accepted,
                              double *dh_log, double *energy);

/* ---- solid-fluid potential grids (tools/sfgridgen.c:71-354) ----------------- */
/* One unit cell of a solid, periodic in z only, and the solid-fluid Lennard-Jones
 * parameters (Lorentz-Berthelot mixing), in A and K. */
typedef struct mg_sfgrid_spec {
    int nsolid;                       /* solid atoms in the cell (at most 2048) */
    const double *sx, *sy, *sz;       /* their positions, A */
    double uclx, ucly, uclz;          /* cell lengths, A */
    double f_sigma, f_epsilon;        /* fluid site sigma (A), epsilon (K) */
    double s_sigma, s_epsilon;        /* solid atom sigma (A), epsilon (K) */
    double rcuton, rcutoff;           /* A */
    int lj_switch;                    /* energy switch between rcuton and rcutoff */
} mg_sfgrid_spec;

/* The grids tools/sfgridgen.c writes (the my-interp model's input): nodes x = i*itvl,
 * i < dims[0] = floor(uclx/itvl)+2 (likewise y, z), index i*dims[1]*dims[2] +
 * j*dims[2] + k. out = 13 arrays of dims[0]*dims[1]*dims[2] doubles: energy (J/mol),
 * dE/dx, dE/dy, dE/dz (J/mol/A), then the derivatives of the force -dE: xx xy xz yx yy
 * yz zx zy zz. out == NULL only returns dims. precision: MG_PREC_*. Allocates device
 * memory for the call. */
MG_API mg_status mg_sfgrid_sfgridgen(int device, const mg_sfgrid_spec *spec, double itvl, int precision,
                                     int *dims, double *out);
/* A Tasos table (mylibtasos/grid.f90:81-93) of nx*ny*nz nodes at (i*hx, j*hy, k*hz):
 * values[((k*ny + j)*nx + i)*8 + q] = F, Dx, Dy, Dz, Dxy, Dxz, Dyz, Dxyz for q = 0..7
 * (K, K/A, K/A^2, K/A^3), ready for mg_sf_tasos_set_grid. No reference counterpart: the
 * reference reads these tables from files made by a generator it does not include. */
MG_API mg_status mg_sfgrid_tasos(int device, const mg_sfgrid_spec *spec, int nx, int ny, int nz, double hx,
                                 double hy, double hz, int precision, double *values);
/* The same table evaluated on the context's device straight into its Tasos table `type`
 * (as mg_sfgrid_tasos at the context's precision followed by mg_sf_tasos_set_grid with
 * cell length cuc), with no copy through host memory. */
/* No reference counterpart: ctx uses the Tasos tables of src (same device and precision)
 * without a copy. Replicas of one system (annealing runs, for instance) then hold one copy
 * of tables that can reach gigabytes; the storage is freed with the last context holding
 * it. A later mg_sf_tasos_set_grid / mg_sf_tasos_generate on either context gives that
 * context a storage of its own for that table. */
MG_API mg_status mg_sf_tasos_share(mg_ctx *ctx, const mg_ctx *src);
MG_API mg_status mg_sf_tasos_generate(mg_ctx *ctx, int type, const mg_sfgrid_spec *spec, int nx, int ny, int nz,
                                      double hx, double hy, double hz, double cuc);

/* ---- reciprocal space without device allocation ---------------------------- */
/* No counterpart in the reference: an extra entry point of this library.
 *
 * Ewald reciprocal-space energy and forces (the k-space part of src/frclong.c:988-1048,
 * computed by the same kernels as mg_compute) for callers that may not allocate device
 * memory: code that runs inside a pre-sized memory pool or a latency-bounded loop, where
 * a cudaMalloc would either fail or stall every stream of the device. The call allocates
 * no memory, on the device or the host: its scratch is one fixed array of
 * MG_EWALD_STATIC_SCRATCH_BYTES per device inside this library's device code, which
 * exists from the moment that code is loaded on the device.
 *
 * Device pointers: d_x, d_y, d_z, d_q [natom] positions and charges; d_f [3*natom] the
 * forces (x block, then y, then z), overwritten; d_energy one double, overwritten with
 * the reciprocal energy (mg_energies.ufourier), or NULL. Of p the fields kmax, ksqmax,
 * coulomb_prefactor, bfactor_ewald, vfactor_ewald and twopi_l{x,y,z} are read.
 * precision: MG_PREC_*. stream: a cudaStream_t as void*, NULL = the default stream; the
 * call is asynchronous on it. err: optional buffer of err_len bytes for a one-line
 * message when the call fails.
 *
 * The first call for a device does the set-up: it looks up the scratch address with that
 * device current (which may load the device code there); make it before any stream
 * capture. Every call selects `device` for its duration and restores the caller's. A call
 * whose scratch would exceed the limit returns MG_ERR_CAPACITY and launches nothing.
 * Nothing in the scratch needs to start at zero: the k-vector tables are rebuilt on the
 * device whenever KMAX/KSQMAX differ from those of the tables in place (their key is kept
 * in the scratch), and the call clears its status word. Calls on one device share the
 * scratch: two calls that are not ordered on the device (issued from different threads, or
 * on streams not ordered by events) race on it and give wrong results.
 * On the mixed path the structure factors come from the tensor-core pass (KMAXZ <= 30).
 * If one of its bounded on-chip waits runs out (mg_set_wait_limit), every force of d_f and
 * *d_energy are NaN: the failure shows in the outputs, without a host synchronisation. */
#define MG_EWALD_STATIC_SCRATCH_BYTES (32u << 20)
MG_API mg_status mg_ewald_recip_static(int device, void *stream, int precision, int natom,
                                       const double *d_x, const double *d_y, const double *d_z,
                                       const double *d_q, const mg_params *p, double *d_f,
                                       double *d_energy, char *err, size_t err_len);
/* For tests, no reference counterpart: the number of row ranges the k-space force pass of
 * the last successful mg_ewald_recip_static call of the process split its rows into (their
 * partial forces live in the scratch left after the tables; 1 = no split, 0 = no call yet). */
MG_API int mg_ewald_recip_static_last_split(void);

/* ---- adjoint: parameter gradients of a force loss ----------------------------- */
/* No counterpart in the reference (which has no derivatives with respect to force-field
 * parameters): the backward pass for force matching and parameter fitting.
 *
 * For host positions x, y, z [natom] and g = dL/dF (gx, gy, gz [natom]) of a loss L of
 * the long forces F (those of mg_compute with MG_TERMS_LONG, i.e. of frclong()), writes
 *   grad_eps[k]   = dL/d epsilon_k,  grad_sigma[k] = dL/d sigma_k,  grad_q[k] = dL/d q_k
 * for every site class k, a class being one site of one species template (the template's
 * epsilon[a], sigma[a], charge[a]), numbered species by species and site by site:
 * k = natom(species 0) + ... + natom(species s-1) + a. *nclass gets the number of classes
 * (at most 16). The pair terms are recomputed from the list of the forward evaluation
 * that the call runs first (the forces themselves are not returned); every sum is in a
 * fixed order, so results are reproducible. An epsilon of zero has no derivative (the
 * mixing rule takes its square root): its entries are 0.
 * Supported: no LJ switch, no distance split, no solid-fluid term, electrostatics none,
 * Wolf, or Ewald with tin-foil boundaries; anything else returns MG_ERR_UNSUPPORTED. */
MG_API mg_status mg_adjoint_params(mg_ctx *ctx, const double *x, const double *y, const double *z,
                                   const double *gx, const double *gy, const double *gz,
                                   double *grad_eps, double *grad_sigma, double *grad_q, int *nclass);

/* No counterpart in the reference: one force-matching evaluation. For host positions
 * x, y, z and target forces tx, ty, tz [natom], computes the long forces F, the loss
 *   *loss = scale * sum over sites and components of (F - T)^2
 * (scale = 1 / (3 natom) gives the mean squared force error) and its gradient with
 * respect to the site-class parameters, as mg_adjoint_params does for g = 2 scale (F - T).
 * The residual and g stay on the device: one forward evaluation and one adjoint pass. */
MG_API mg_status mg_force_match(mg_ctx *ctx, const double *x, const double *y, const double *z,
                                const double *tx, const double *ty, const double *tz, double scale,
                                double *loss, double *grad_eps, double *grad_sigma, double *grad_q,
                                int *nclass);

/* No counterpart in the reference: Hessian-vector product of the long-range energy in
 * positions, h = H v = -(dF/dr) v with F the long forces of mg_compute (MG_TERMS_LONG),
 * for host positions x, y, z and displacements vx, vy, vz [natom]; hx, hy, hz [natom] are
 * overwritten. Computed analytically from the pair terms of the forward evaluation that
 * the call runs first and, for Ewald, from the structure factors weighted by q_j v_j.
 * Where the reference keeps an integer-truncated vector for a molecule that spans the
 * box, that term does not move with the sites and contributes nothing. Same model
 * restrictions as mg_adjoint_params. */
MG_API mg_status mg_adjoint_hvp(mg_ctx *ctx, const double *x, const double *y, const double *z,
                                const double *vx, const double *vy, const double *vz,
                                double *hx, double *hy, double *hz);

#ifdef __cplusplus
}
#endif
#endif /* MSPMS2_GB300_H_ */
