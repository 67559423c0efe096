// mg_internal.cuh - internal declarations of the GB300 nonbonded-force engine.
//
// Data layout in HBM (one context = one system on one GPU):
//   per site, reference order     x,y,z (FP64, unwrapped, as the caller keeps them),
//                                 static tables: molecule id, charge, LJ half-sigma and
//                                 sqrt(eps), flags, solid-fluid table id;
//   per cluster of 8 sites        site index (or -1), FP64 reference point, FP64 bounding box;
//   per cluster slot (8 per       packed pair-kernel operands rebuilt every call: position
//   cluster, list order)          offset from the cluster reference + charge (float4 or
//                                 double4), LJ (float2/double2), molecule id + flags (int);
//   cluster-pair list (CSR)       j-cluster index (int) + periodic shift (float4/double4)
//                                 per entry, row starts per i-cluster;
//   reciprocal space              per-site phase tables e^{2 pi i n u} (n = 0..kmax per axis,
//                                 complex FP32 or FP64), partial structure factors per site
//                                 block (FP32 or FP64), S(k) and force coefficients;
//   energies                      per-block partial sums (FP64) reduced in a fixed order.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/mspms2_gb300.h"

#define MG_CL 8             // sites per cluster
#define MG_MAX_COLUMN 2048  // sites per grid column the on-chip sort handles
#define MG_ZB 32            // z buckets per column of the cluster search

// device status word bits (mg_get_device_flags)
#define MG_FLAG_OUT_OF_GRID 1u
#define MG_FLAG_NONFINITE 2u
#define MG_FLAG_LIST_OVERFLOW 4u
#define MG_FLAG_COLUMN_OVERFLOW 8u
#define MG_FLAG_IMPROPER_DEGENERATE 16u
#define MG_FLAG_SMALL_BOX 32u  // a cluster pair needs two images: use the small-box list
#define MG_FLAG_WAIT_TIMEOUT 64u  // a bounded on-chip wait (mbarrier) gave up
#define MG_FLAG_MMA_UNDRAINED 128u  // ...and MMAs it had issued did not finish within the bound either
#define MG_FLAG_FIXED_RANGE 256u    // a pair force beyond the range of the fixed-point force sums

// per-site flags packed next to the molecule id
#define MG_SITE_LJ 1        // takes part in LJ (ghost type NONE)
#define MG_SITE_DEAD 2      // GHOST_FULL or padding: no nonbonded interaction at all

// energy component slots written by the kernels (partials reduced in fixed order)
enum {
    E_UVDW = 0, E_USHIFT, E_UREAL, E_VIR,            // long bucket of the pair kernel
    E_UVDW_S, E_USHIFT_S, E_UREAL_S, E_VIR_S,        // short bucket (distance split)
    E_UEXCL, E_UCOUL, E_UFOURIER, E_USFLJ,
    E_UBOND, E_UANGLE, E_UDIH, E_UIMP, E_VIR_INTRA,
    E_DIPX, E_DIPY, E_DIPZ,
    E_NPAIR,                                          // pairs within cutoff (x2, full list)
    E_NCOMP
};

struct MgError {
    mg_status code;
    std::string msg;
};

// ---- topology expanded for the device ------------------------------------------
// Intra-molecular nonbonded corrections of one species, in the reference's order
// (src/frclong.c:233-977): kind 0 = 1-2/1-3 end pair, 1 = 1-4 end pair (eps*f0),
// 2 = nbp pair (eps unscaled).
struct IntraPair {
    int m, n, kind;
};

struct BondedTerm {  // one bonded term of a species template
    int kind;        // 0 bond, 1 angle, 2 dihedral, 3 improper
    int type;
    int idx[4];
    double p[5];
};

struct SpeciesDev {
    int natom, nmole, first_site, first_mole;
    int intra_off, nintra;    // into d_intra
    int bonded_off, nbonded;  // into d_bonded
    double mw;
};

struct ParamsDev {  // everything the kernels need, by value
    mg_params p;
    double lx, ly, lz;
    double rlist;
};

// ---- solid-fluid tables ----------------------------------------------------------
struct TasosDev {
    int nx, ny, nz;
    double hx, hy, hz, cuc, min_pe;
    void *values;  // float or double, [nz][ny][nx][8]
};

struct MyInterpDev {
    int ncx, ncy, ncz;
    double itvl_x, itvl_y, itvl_z, xmin, ymin, zmax;
    double *coeff;  // [4][32][ncube]
};

// ---- context ----------------------------------------------------------------------
struct mg_ctx_s;
struct MgTraj;  // trajectory writer (mg_io.cu)

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
};

// launch geometry picked by mg_autotune (defaults until it runs)
struct MgTuning {
    double cell_scale = 1.0;   // list column width relative to the default
    double zcap_scale = 1.0;   // cluster z extent relative to the column width
    int kforce_threads = 4;    // threads per site in the k-space force pass (2, 4, 8)
    bool tuned = false;
};

struct mg_ctx {
    mg_options opt;
    MgTuning tune;
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    bool timing = false;
    cudaEvent_t ev[10];
    bool have_events = false;
    MgError err{MG_OK, ""};

    // topology
    bool have_topology = false;
    int natom = 0, nmole = 0, nspecies = 0;
    std::vector<SpeciesDev> species;
    std::vector<int> h_site_mol, h_site_species, h_site_rel;
    std::vector<std::vector<double>> h_tmpl_eps, h_tmpl_sig, h_tmpl_aw;  // per species template
    std::vector<double> h_site_q;
    double sum_q2 = 0.0;
    int max_mol_atoms = 0;
    bool has_nbp = false;

    // params / box
    bool have_params = false, have_box = false;
    mg_params params;
    double lx = 0, ly = 0, lz = 0;

    // device: static per-site tables
    DevBuf d_site_mol, d_site_q, d_site_hsig, d_site_seps, d_site_flags, d_site_interp;
    DevBuf d_species, d_intra, d_bonded, d_site_aw;
    // device: per-call state
    DevBuf d_x, d_y, d_z;                 // positions (when the host API is used)
    DevBuf d_fl, d_fs;                    // forces [3][n] each (host API)
    DevBuf d_xbuild;                      // positions at the last list build [3][n]
    DevBuf d_img;                         // image shifts of the build (FP64 [3][n])
    // clusters and list
    int ncx = 0, ncy = 0, ncol = 0, ncl = 0;
    long long npairs = 0;
    bool small_box = false;
    double list_lx = 0, list_ly = 0, list_lz = 0, list_rlist = 0;
    bool list_valid = false;
    int list_builds = 0, list_rebuilt = 0;
    DevBuf d_col_count, d_col_start, d_col_fill, d_col_cl_start, d_col_sorted;
    DevBuf d_col_bkt;  // per column and z bucket: the cluster range that can reach the bucket
    DevBuf d_cl_atom, d_cl_ref, d_cl_refh, d_cl_bb, d_cl_col, d_cl_bbf, d_col_ncl, d_counter;
    double zcap = 0;           // largest z extent of a cluster
    bool small_box_forced = false;
    int col_refine = 0;        // column-grid refinements after overflows
    int cl_cap = 0;            // cluster capacity
    long long pair_cap = 0;    // cluster-pair entry capacity
    DevBuf d_pair_start, d_pair_count, d_pair_j, d_pair_shift;
    // inner sub-list of the distance split (cluster pairs within respa_split + skin)
    DevBuf d_sub_start, d_sub_count, d_sub_j, d_sub_shift, d_sub_img;
    // mixed-precision pair kernel: 64-bit fixed-point forces per cluster slot
    // [bucket][3][slots] in units of 2^-fixed_bits (lowered by 16 when a force leaves the range)
    DevBuf d_facc;
    int fixed_bits = 32;
    bool sub_ready = false;
    DevBuf d_pack_pos, d_pack_lj, d_pack_info;
    DevBuf d_pack_xi, d_pack_qp;  // mixed pair kernel: (x, y, z, info bits), (q, half-sigma, sqrt-eps, 0)
    // integration (mg_md_run): velocities, solver work arrays, 1/mass, partial sums,
    // thermostat scalars, per-step records
    DevBuf d_md_v, d_md_work, d_md_rmass, d_md_part, d_md_dev, d_md_log;
    DevBuf d_md_glog;          // graph replay: energy log, saved start state, step counter
    bool md_graphs = true;     // run whole integrator steps as a replayed CUDA graph
    int md_graph_steps = 0;    // steps the last run replayed as a graph (0: eager)
    // adjoint (mg_adjoint_params): site classes and one carved scratch block
    DevBuf d_adj_class, d_adj, d_adj_g;
    MgTraj *traj = nullptr;  // attached trajectory file, if any
    // reciprocal space
    int nrows = 0, nslots = 0, kmaxx = 0, kmaxy = 0, kmaxz = 0;
    long long kvectors = 0;
    std::vector<int> h_rows;  // [nrows][4]: kx, ky, kzmax, half_only
    DevBuf d_rows, d_row_slot, d_phase, d_spart, d_scoef, d_tasks;
    std::vector<int> h_chunk_kz;  // kzmax of each chunk of the FP32 table force pass
    DevBuf d_fcoef, d_fpart;      // its coefficients and partial forces
    DevBuf d_kfb;                 // the tensor-core force pass's coefficient tiles and their kzmax
    DevBuf d_qf;                  // FP32 copy of the S(k) site weights
    // the reciprocal-space chain runs on its own stream beside the list and pair kernels,
    // into its own force buffer and energy rows, joined before the forces are summed
    bool kspace_overlap = true;
    bool kspace_tensor = true;  // S(k) on the tensor cores (FP32 path, KMAXZ <= 30)
    bool forked = false;          // the last evaluation ran that chain on kstream
    cudaStream_t kstream = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    DevBuf d_fk, d_erows_k;
    double *ew_rows = nullptr;    // energy rows of the chain while it is enqueued
    int ntasks = 0, sblocks_atoms = 0;
    double ewald_box[3] = {0, 0, 0};
    // energies
    DevBuf d_epart, d_eout, d_flags, d_meta, d_pair_img;
    int epart_rows = 0, epart_cap = 0;
    // solid-fluid
    std::vector<TasosDev> tasos;   // index = AtomID - 1
    // table storage, shared by the contexts mg_sf_tasos_share links (freed with the last)
    std::vector<std::shared_ptr<DevBuf>> tasos_buf;
    DevBuf d_tasos;
    std::vector<MyInterpDev> myinterp;
    std::vector<DevBuf> myinterp_buf;
    DevBuf d_myinterp;
    int ntube = 0, nsolid = 0;
    DevBuf d_tubes, d_solid;
    double solid_sigma = 0, solid_epsilon = 0, const_3pisq_theta = 0;
    // stats
    mg_stats stats;
    unsigned last_flags = 0;
    int launches = 0;  // kernels launched in the current call
};

// ---- helpers shared by host translation units --------------------------------------
mg_status mg_fail(mg_ctx *c, mg_status code, const std::string &msg);
long long mg_wait_limit();  // polls of each on-chip pipeline wait (mg_set_wait_limit)
bool mg_ewald_horner_force(const mg_ctx *c);  // k-space forces by the Horner pass (threads per site apply)
bool mg_ewald_sk_tensor(const mg_ctx *c);     // S(k) by the tensor-core pass
mg_status mg_ewald_fork(mg_ctx *c, const double *dx, const double *dy, const double *dz);
mg_status mg_ewald_join(mg_ctx *c, double *fl);
mg_status mg_cuda_fail(mg_ctx *c, cudaError_t e, const char *what);
bool mg_ensure(mg_ctx *c, DevBuf &b, size_t bytes);
// the storage of Tasos table `type` (1-based) that this context may write: a fresh buffer
// when the table has none or shares its buffer with another context
DevBuf &mg_tasos_storage(mg_ctx *c, int type);
// forces of the given terms at device positions into the context's [3][n] blocks fl/fs,
// repeating the call when the neighbour-list set-up has to grow (mg_host.cu)
mg_status mg_compute_forces(mg_ctx *c, const double *dx, const double *dy, const double *dz, int terms,
                            double *fl, double *fs, mg_energies *e);
// the launches of one evaluation only (no readback, no retry; mg_host.cu)
mg_status mg_enqueue_forces(mg_ctx *c, const double *dx, const double *dy, const double *dz, int terms, double *fl,
                            double *fs);
// the energies of a raw component vector E[E_NCOMP] as mg_compute reports them
void mg_assemble_energies(mg_ctx *c, const double *E, int want_long, int want_short, mg_energies *e);
void mg_free(DevBuf &b);

#define MG_CUDA(call)                                                \
    do {                                                             \
        cudaError_t _e = (call);                                     \
        if (_e != cudaSuccess) return mg_cuda_fail(c, _e, #call);    \
    } while (0)

// stage launchers (defined in the kernel translation units)
mg_status mg_list_update(mg_ctx *c, const double *dx, const double *dy, const double *dz);
mg_status mg_pack_clusters(mg_ctx *c, const double *dx, const double *dy, const double *dz);
mg_status mg_launch_pair(mg_ctx *c, int want_long, int want_short, double *fl, double *fs);
mg_status mg_launch_intra(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *fl);
mg_status mg_launch_bonded(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *fs);
mg_status mg_ewald_setup(mg_ctx *c);
mg_status mg_launch_ewald(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *fl);
// adjoint support (mg_ewald.cu), valid after a long-range evaluation at the same positions
mg_status mg_ewald_weighted_sk(mg_ctx *c, const double *w, double2 *out);
mg_status mg_ewald_field(mg_ctx *c, const double *ones, double *field);
mg_status mg_ewald_kgrad(mg_ctx *c, const double2 *SA, const double2 *ST, int nclass, double *rows, int *nblocks);
mg_status mg_ewald_jvp(mg_ctx *c, const double *v, const double2 *SW, void *coef_scratch, double *out);
mg_status mg_launch_vacuum(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *fl);
mg_status mg_launch_coulomb_mole(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *fl);
mg_status mg_launch_sf(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *fl);
mg_status mg_launch_reduce(mg_ctx *c);
mg_status mg_launch_check(mg_ctx *c, const double *f, int n);
bool mg_list_retry(mg_ctx *c, unsigned flags, const int *meta_host);
// trajectory frames of device-resident runs (mg_io.cu): the frame before the first step
// (once per file) and one frame every `every` steps
mg_status mg_traj_start(mg_ctx *c, const double *d_x);
mg_status mg_traj_tick(mg_ctx *c, const double *d_x);
void mg_traj_destroy(mg_ctx *c);

// Energy partial rows: every block of every stage writes one full row of E_NCOMP
// FP64 values (zeros outside its own components); rows are reserved in launch order
// and summed in that fixed order by mg_launch_reduce.
int mg_reserve_rows(mg_ctx *c, int nblocks);

// hi + lo += v exactly (Knuth's two-sum) in FP32, which keeps about 48 significant bits
// without FP64 instructions (far slower than FP32 on this part); a plain addition in FP64
template <typename R>
__device__ __forceinline__ void mg_acc2(R &hi, R &lo, R v) {
    if constexpr (std::is_same<R, float>::value) {
        const float s = hi + v, bp = s - hi, ap = s - bp;
        lo += (hi - ap) + (v - bp);
        hi = s;
    } else {
        hi += v;
    }
}

// per-block row writer: sums v[0..NC) over the block and stores them at row[ids[k]]. The
// warp sums are taken in T (FP32 values are summed across the warp in FP32, since FP64 is
// far slower on this part), the sums over warps in FP64, all in a fixed order.
template <int NC, typename T>
__device__ __forceinline__ void mg_block_row(T (&v)[NC], const int (&ids)[NC], double *rows, int row) {
    __shared__ double red[32][NC];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NC; k++) {
        T t = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[w][k] = (double)t;
    }
    __syncthreads();
    double *out = rows + (size_t)row * E_NCOMP;
    if (threadIdx.x < E_NCOMP) out[threadIdx.x] = 0.0;
    __syncthreads();
    if (threadIdx.x < NC) {
        double t = 0.0;
        for (int i = 0; i < nw; i++) t += red[i][threadIdx.x];
        out[ids[threadIdx.x]] = t;
    }
}
