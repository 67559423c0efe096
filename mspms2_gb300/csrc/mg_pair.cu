// mg_pair.cu - inter-molecular LJ + Ewald-real/Wolf site pairs over the cluster-pair
// list, the fixed-order energy reduction and the non-finite check.
//
// Physics of one site pair (identical to src/frclong.c:114-196 with src/ljfrc.c:21-71,
// src/elecfrc.c:17-33 and :48-60): pairs of different molecules, neither GHOST_FULL;
// LJ when neither is GHOST_LJ and r^2 < rcutoff^2 (Lorentz-Berthelot mixing, optional
// energy switch, shift energy eps*sigma^6*(sigma^6*shift1-1) accumulated for the caller's
// shift4 factor); Ewald real space or Wolf when r^2 < rcutoffelec^2. Ewald pairs add no
// pair virial (the reference adds the total Ewald energy instead, src/frclong.c:1128).
//
// Execution: one warp per i-cluster (8 sites). Lane l owns i-site l%8 and j-slots l/8
// and l/8+4 of each j-cluster. Four j-clusters (32 sites: one float4 position, one
// float2 LJ pair and one int per lane) are staged in shared memory per step with
// coalesced loads. The list is a full list (each pair seen from both clusters), so no
// j-force scatter or atomic is needed: a lane accumulates only its own i-site force in
// FP32 over at most 64 j-clusters, then flushes it into an FP32 hi+lo pair by an exact
// two-sum (about 48 significant bits, and no FP64 instruction, which is far slower than
// FP32 on this part); the four lanes of an i-site are combined in FP64 with warp
// shuffles at the end. A lane's energy sums stay in FP32 over its list, are summed
// across the warp in FP32 and across warps and blocks in FP64; they are halved for the
// double counting. The FP64 path accumulates in FP64 throughout. Every reduction has a
// fixed order, so results are bit-reproducible.
#include <math.h>

#include "mg_internal.cuh"

#define PAIR_WPB 4       // warps (i-clusters) per block
#define PAIR_FLUSH 16    // list steps (4 j-clusters each) between force flushes

namespace {

template <typename R>
struct RT;
// erfc(x) for x >= 0 from e^{-x^2}, which the force needs anyway, in the form of
// Abramowitz & Stegun 7.1.26: erfc(x) = t P(t) e^{-x^2}, t = 1 / (1 + 0.35 x), with P of
// degree 8 fitted by least squares to the relative error of e^{x^2} erfc(x) on [0, 6]
// (iteratively reweighted towards the minimax). Relative error of the fit 1.1e-7; of the
// FP32 evaluation below, about 5e-7 on [0, 5] (tests/test_pair_erfc.py).
__device__ __forceinline__ float erfc_from_exp(float x, float ex) {
    const float t = __frcp_rn(fmaf(0.35f, x, 1.0f));
    float p = 5.973472579e-02f;
    p = fmaf(p, t, -3.627256178e-01f);
    p = fmaf(p, t, 7.487209283e-01f);
    p = fmaf(p, t, -6.124998983e-01f);
    p = fmaf(p, t, 5.585650393e-01f);
    p = fmaf(p, t, -8.000170377e-03f);
    p = fmaf(p, t, 2.266547403e-01f);
    p = fmaf(p, t, 1.917381094e-01f);
    p = fmaf(p, t, 1.978120333e-01f);
    return t * p * ex;
}

template <>
struct RT<float> {
    typedef float4 V4;
    typedef float2 V2;
    __device__ static float rs(float x) { return rsqrtf(x); }
    __device__ static float erfc_ex(float x, float ex) { return erfc_from_exp(x, ex); }
    __device__ static float exp_(float x) { return expf(x); }
    __device__ static float rint_(float x) { return rintf(x); }
};
template <>
struct RT<double> {
    typedef double4 V4;
    typedef double2 V2;
    __device__ static double rs(double x) { return rsqrt(x); }
    __device__ static double erfc_ex(double x, double) { return erfc(x); }
    __device__ static double exp_(double x) { return exp(x); }
    __device__ static double rint_(double x) { return rint(x); }
};

struct PairArgs {
    int n;
    const int *meta;  // meta[0] = number of clusters of the current build
    const int *pair_start, *pair_cnt, *pair_j, *info, *cl_atom;
    const void *pair_shift, *pos, *lj;
    double *fl, *fs;
    double rc2, rce2, rs2, rmax2;
    double lx, ly, lz;
    double kappa, coul, shift1, ron2, roff2, sw_denom, rce, v1, v2, f1, f2;
    int ljsw, mode;  // mode bit 0: long bucket, bit 1: short bucket
    double *rows;
    int row0;
};

template <typename R, int ELEC, bool MIC, bool SPLIT>
__global__ void __launch_bounds__(PAIR_WPB * 32) k_pair(PairArgs A) {
    typedef typename RT<R>::V4 V4;
    typedef typename RT<R>::V2 V2;
    __shared__ V4 s_pos[PAIR_WPB][32];
    __shared__ V2 s_lj[PAIR_WPB][32];
    __shared__ int s_info[PAIR_WPB][32];
    __shared__ V4 s_shift[PAIR_WPB][4];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int I = blockIdx.x * PAIR_WPB + w;
    // force accumulators (hi + lo; long, short) and energies
    R fLh[3] = {0, 0, 0}, fLl[3] = {0, 0, 0}, fSh[3] = {0, 0, 0}, fSl[3] = {0, 0, 0};
    R eng[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // uvdw ushift ureal vir (long), same (short), npair
    if (I < A.meta[0]) {
        const V4 *pos = (const V4 *)A.pos;
        const V2 *lj = (const V2 *)A.lj;
        const V4 *shift = (const V4 *)A.pair_shift;
        const int il = lane & 7, js = lane >> 3;
        const V4 pi = pos[I * MG_CL + il];
        const V2 li = lj[I * MG_CL + il];
        const int infi = A.info[I * MG_CL + il];
        const R rc2 = (R)A.rc2, rce2 = (R)A.rce2, rs2 = (R)A.rs2, rmax2 = (R)A.rmax2;
        const R kap = (R)A.kappa, coul = (R)A.coul, shift1 = (R)A.shift1;
        const R ron2 = (R)A.ron2, roff2 = (R)A.roff2, swd = (R)A.sw_denom;
        const R lx = (R)A.lx, ly = (R)A.ly, lz = (R)A.lz;
        const R ilx = (R)(1.0 / A.lx), ily = (R)(1.0 / A.ly), ilz = (R)(1.0 / A.lz);
        const R two_over_sqrtpi = (R)1.1283791670955126;
        const R rce = (R)A.rce, v1 = (R)A.v1, v2 = (R)A.v2, f1 = (R)A.f1, f2 = (R)A.f2;
        const bool use_long = (A.mode & 1) != 0, use_short = (A.mode & 2) != 0;
        R ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0;
        R e_vdw = 0, e_sh = 0, e_re = 0, e_vir = 0, s_vdw = 0, s_sh = 0, s_re = 0, s_vir = 0;
        int npair = 0;
        const int e0 = A.pair_start[I], e1 = e0 + A.pair_cnt[I];
        int steps = 0;
        for (int e = e0; e < e1; e += 4) {
            const int me = e + (lane >> 3);
            __syncwarp();
            if (me < e1) {
                const int J = A.pair_j[me];
                s_pos[w][lane] = pos[J * MG_CL + (lane & 7)];
                s_lj[w][lane] = lj[J * MG_CL + (lane & 7)];
                s_info[w][lane] = A.info[J * MG_CL + (lane & 7)];
                if ((lane & 7) == 0) s_shift[w][lane >> 3] = shift[me];
            }
            __syncwarp();
            const int nc = min(4, e1 - e);
            for (int q = 0; q < nc; q++) {
                const V4 sh = s_shift[w][q];
                const R xi = pi.x + sh.x, yi = pi.y + sh.y, zi = pi.z + sh.z;
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int t = q * 8 + js + 4 * h;
                    const V4 pj = s_pos[w][t];
                    const int infj = s_info[w][t];
                    R dx = xi - pj.x, dy = yi - pj.y, dz = zi - pj.z;
                    if (MIC) {
                        dx -= lx * RT<R>::rint_(dx * ilx);
                        dy -= ly * RT<R>::rint_(dy * ily);
                        dz -= lz * RT<R>::rint_(dz * ilz);
                    }
                    const R r2 = dx * dx + dy * dy + dz * dz;
                    const bool valid = !((infi | infj) & MG_SITE_DEAD) && ((infi >> 2) != (infj >> 2)) && r2 < rmax2;
                    if (!valid) continue;
                    const bool inner = SPLIT && r2 < rs2;
                    if (SPLIT && !(inner ? use_short : use_long)) continue;
                    const R rinv = RT<R>::rs(r2);
                    const R rinv2 = rinv * rinv;
                    R f = 0, ulj = 0, ush = 0, uel = 0, vir = 0;
                    if ((infi & infj & MG_SITE_LJ) && r2 < rc2) {
                        const V2 lj_j = s_lj[w][t];
                        const R sig = li.x + lj_j.x, eps = li.y * lj_j.y;
                        const R sig2 = sig * sig;
                        R s6 = sig2 * rinv2;
                        s6 = s6 * s6 * s6;
                        const R s12 = s6 * s6;
                        ulj = (R)4 * eps * (s12 - s6);
                        R flj = (R)24 * eps * ((R)2 * s12 - s6) * rinv2;
                        if (A.ljsw) {
                            if (!(r2 < ron2)) {
                                const R d = roff2 - r2;
                                const R sw = d * d * (roff2 + (R)2 * r2 - (R)3 * ron2) / swd;
                                flj = flj * sw - ulj * (R)12 * d * (ron2 - r2) / swd;
                                ulj *= sw;
                            }
                        } else {
                            const R sg6 = sig2 * sig2 * sig2;
                            ush = eps * sg6 * (sg6 * shift1 - (R)1);
                        }
                        f += flj;
                        vir += flj * r2;
                    }
                    if (ELEC != 0 && r2 < rce2) {
                        const R qq = pi.w * pj.w;
                        const R r = r2 * rinv;
                        const R kr = kap * r;
                        const R ex = RT<R>::exp_(-kr * kr);
                        const R ec = RT<R>::erfc_ex(kr, ex);
                        if (ELEC == 1) {
                            const R bare = coul * qq * rinv;
                            uel = bare * ec;
                            f += (uel + bare * kr * ex * two_over_sqrtpi) * rinv2;
                        } else {
                            uel = coul * qq * (ec * rinv + v1 + v2 * (r - rce));
                            const R fe = coul * qq * rinv * (ec * rinv2 + f1 * ex * rinv + f2);
                            f += fe;
                            vir += fe * r2;
                        }
                    }
                    npair += 1;
                    if (inner) {
                        bx += f * dx; by += f * dy; bz += f * dz;
                        s_vdw += ulj; s_sh += ush; s_re += uel; s_vir += vir;
                    } else {
                        ax += f * dx; ay += f * dy; az += f * dz;
                        e_vdw += ulj; e_sh += ush; e_re += uel; e_vir += vir;
                    }
                }
            }
            if (++steps == PAIR_FLUSH) {  // per-lane energies stay in R until the end
                steps = 0;
                mg_acc2(fLh[0], fLl[0], ax);
                mg_acc2(fLh[1], fLl[1], ay);
                mg_acc2(fLh[2], fLl[2], az);
                ax = ay = az = 0;
                if (SPLIT) {
                    mg_acc2(fSh[0], fSl[0], bx);
                    mg_acc2(fSh[1], fSl[1], by);
                    mg_acc2(fSh[2], fSl[2], bz);
                    bx = by = bz = 0;
                }
            }
        }
        mg_acc2(fLh[0], fLl[0], ax);
        mg_acc2(fLh[1], fLl[1], ay);
        mg_acc2(fLh[2], fLl[2], az);
        mg_acc2(fSh[0], fSl[0], bx);
        mg_acc2(fSh[1], fSl[1], by);
        mg_acc2(fSh[2], fSl[2], bz);
        eng[0] = e_vdw; eng[1] = e_sh; eng[2] = e_re; eng[3] = e_vir;
        eng[4] = s_vdw; eng[5] = s_sh; eng[6] = s_re; eng[7] = s_vir;
        eng[8] = (R)npair;
        double fL[3], fS[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            fL[k] = (double)fLh[k] + (double)fLl[k];
            fS[k] = (double)fSh[k] + (double)fSl[k];
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            fL[k] += __shfl_xor_sync(0xffffffffu, fL[k], 8);
            fL[k] += __shfl_xor_sync(0xffffffffu, fL[k], 16);
            if (SPLIT) {
                fS[k] += __shfl_xor_sync(0xffffffffu, fS[k], 8);
                fS[k] += __shfl_xor_sync(0xffffffffu, fS[k], 16);
            }
        }
        if (js == 0) {
            const int a = A.cl_atom[I * MG_CL + il];
            if (a >= 0) {
                const int n = A.n;
                if (A.fl) {
                    A.fl[a] = fL[0];
                    A.fl[n + a] = fL[1];
                    A.fl[2 * n + a] = fL[2];
                }
                if (A.fs) {
                    A.fs[a] = fS[0];
                    A.fs[n + a] = fS[1];
                    A.fs[2 * n + a] = fS[2];
                }
            }
        }
#pragma unroll
        for (int k = 0; k < 8; k++) eng[k] *= (R)0.5;  // every pair was seen from both sides
    }
    const int ids[9] = {E_UVDW, E_USHIFT, E_UREAL, E_VIR, E_UVDW_S, E_USHIFT_S, E_UREAL_S, E_VIR_S, E_NPAIR};
    mg_block_row<9>(eng, ids, A.rows, A.row0 + blockIdx.x);
}

template <typename R, int ELEC>
void launch_pair_elec(const PairArgs &A, bool mic, bool split, unsigned blocks, cudaStream_t s) {
    if (mic) {
        if (split) k_pair<R, ELEC, true, true><<<blocks, PAIR_WPB * 32, 0, s>>>(A);
        else k_pair<R, ELEC, true, false><<<blocks, PAIR_WPB * 32, 0, s>>>(A);
    } else {
        if (split) k_pair<R, ELEC, false, true><<<blocks, PAIR_WPB * 32, 0, s>>>(A);
        else k_pair<R, ELEC, false, false><<<blocks, PAIR_WPB * 32, 0, s>>>(A);
    }
}

template <typename R>
void launch_pair(const PairArgs &A, int elec, bool mic, bool split, unsigned blocks, cudaStream_t s) {
    if (elec == 1) launch_pair_elec<R, 1>(A, mic, split, blocks, s);
    else if (elec == 2) launch_pair_elec<R, 2>(A, mic, split, blocks, s);
    else launch_pair_elec<R, 0>(A, mic, split, blocks, s);
}

// fixed-order reduction of the partial rows: one block per component
__global__ void k_reduce_rows(const double *__restrict__ rows, int nrows, double *__restrict__ out) {
    __shared__ double s[256];
    int comp = blockIdx.x;
    double t = 0.0;
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) t += rows[(size_t)r * E_NCOMP + comp];
    s[threadIdx.x] = t;
    __syncthreads();
    for (int o = blockDim.x >> 1; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[comp] = s[0];
}

__global__ void k_check(const double *__restrict__ f, int n3, unsigned *__restrict__ flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool bad = i < n3 && !isfinite(f[i]);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flags, MG_FLAG_NONFINITE);
}

}  // namespace

mg_status mg_launch_pair(mg_ctx *c, int want_long, int want_short, double *fl, double *fs) {
    const mg_params &p = c->params;
    PairArgs A;
    A.n = c->natom;
    A.meta = (const int *)c->d_meta.p;
    A.pair_start = (int *)c->d_pair_start.p;
    A.pair_cnt = (int *)c->d_pair_count.p;
    A.pair_j = (int *)c->d_pair_j.p;
    A.pair_shift = c->d_pair_shift.p;
    if (want_short && !want_long && c->sub_ready) {
        // the inner pass of the distance split walks only the inner sub-list
        A.pair_start = (int *)c->d_sub_start.p;
        A.pair_cnt = (int *)c->d_sub_count.p;
        A.pair_j = (int *)c->d_sub_j.p;
        A.pair_shift = c->d_sub_shift.p;
    }
    A.pos = c->d_pack_pos.p;
    A.lj = c->d_pack_lj.p;
    A.info = (int *)c->d_pack_info.p;
    A.cl_atom = (int *)c->d_cl_atom.p;
    A.fl = want_long ? fl : nullptr;
    A.fs = want_short ? fs : nullptr;
    int elec = p.charge_type == MG_ELEC_EWALD ? 1 : (p.charge_type == MG_ELEC_WOLF ? 2 : 0);
    A.rc2 = p.rcutoffsq;
    A.rce2 = p.rcutoffelecsq;
    bool split = p.respa_split > 0;
    A.rs2 = split ? p.respa_split * p.respa_split : 0.0;
    A.rmax2 = elec ? fmax(p.rcutoffsq, p.rcutoffelecsq) : p.rcutoffsq;
    if (split && !want_long) A.rmax2 = fmin(A.rmax2, A.rs2);
    A.lx = c->lx;
    A.ly = c->ly;
    A.lz = c->lz;
    A.kappa = p.kappa;
    A.coul = p.coulomb_prefactor;
    A.shift1 = p.shift1;
    A.ron2 = p.rcutonsq;
    A.roff2 = p.rcutoffsq;
    A.sw_denom = p.roff2_minus_ron2_cube;
    A.rce = p.rcutoffelec;
    A.v1 = p.wolfvcon1;
    A.v2 = p.wolfvcon2;
    A.f1 = p.wolffcon1;
    A.f2 = p.wolffcon2;
    A.ljsw = p.lj_switch;
    A.mode = (want_long ? 1 : 0) | (want_short ? 2 : 0);
    unsigned blocks = (unsigned)((c->cl_cap + PAIR_WPB - 1) / PAIR_WPB);
    if (blocks == 0) return MG_OK;
    A.rows = (double *)c->d_epart.p;
    A.row0 = mg_reserve_rows(c, blocks);
    if (A.row0 < 0) return mg_fail(c, MG_ERR_ALLOC, "energy partial rows exhausted");
    if (c->opt.precision == MG_PREC_FP64)
        launch_pair<double>(A, elec, c->small_box, split, blocks, c->stream);
    else
        launch_pair<float>(A, elec, c->small_box, split, blocks, c->stream);
    MG_CUDA(cudaGetLastError());
    c->launches += 1;
    return MG_OK;
}

int mg_reserve_rows(mg_ctx *c, int nblocks) {
    if (c->epart_rows + nblocks > c->epart_cap) return -1;
    int r = c->epart_rows;
    c->epart_rows += nblocks;
    return r;
}

mg_status mg_launch_reduce(mg_ctx *c) {
    if (c->epart_rows == 0) {
        MG_CUDA(cudaMemsetAsync(c->d_eout.p, 0, sizeof(double) * E_NCOMP, c->stream));
        return MG_OK;
    }
    k_reduce_rows<<<E_NCOMP, 256, 0, c->stream>>>((double *)c->d_epart.p, c->epart_rows, (double *)c->d_eout.p);
    MG_CUDA(cudaGetLastError());
    c->launches += 1;
    return MG_OK;
}

mg_status mg_launch_check(mg_ctx *c, const double *f, int n) {
    int n3 = 3 * n;
    k_check<<<(n3 + 255) / 256, 256, 0, c->stream>>>(f, n3, (unsigned *)c->d_flags.p);
    MG_CUDA(cudaGetLastError());
    c->launches += 1;
    return MG_OK;
}
