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
// Mixed precision (k_pair): Newton's third law over the half of the cluster-pair list with
// J >= I, one warp per i-cluster, each unordered site pair evaluated once in FP32 and its
// force written to a per-warp shared matrix (i-site x j-slot). The row sums are the
// i-forces (FP32 within two super-steps, then 64-bit fixed point in registers); the column
// sums are the j-forces, added as 64-bit fixed point to slot-ordered accumulators (integer
// adds, so the result does not depend on the order in which warps arrive); k_fixed_forces
// turns those into the FP64 force blocks. Energies and virials: FP32 over at most eight
// super-steps of one lane, then exact FP32 hi + lo pairs (two-sum: FP64 operations are slow
// on this part), converted to FP64 once per lane. Details at k_pair.
//
// FP64 (k_pair_full, the plain-FP64 path): the full list, each pair from both sides, FP64
// throughout and no atomics. Lane l owns i-site l % 8 and j-slots l / 8 and l / 8 + 4 of
// each j-cluster; four j-clusters are staged in shared memory per step.
//
// Every reduction has a fixed order, so results are bit-reproducible.
#include <math.h>

#include "mg_internal.cuh"

#define PAIR_WPB 4       // warps (i-clusters) per block
#define PAIR_FLUSH 16    // list steps of k_pair_full (4 j-clusters each) between force flushes

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
struct RT<double> {
    typedef double4 V4;
    typedef double2 V2;
    __device__ static double rs(double x) { return rsqrt(x); }
    __device__ static double erfc_ex(double x, double) { return erfc(x); }
    __device__ static double exp_(double x) { return exp(x); }
    __device__ static double rint_(double x) { return rint(x); }
};

struct PairFullArgs {
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
__global__ void __launch_bounds__(PAIR_WPB * 32) k_pair_full(PairFullArgs A) {
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

template <int ELEC>
void launch_pair_full_elec(const PairFullArgs &A, bool mic, bool split, unsigned blocks, cudaStream_t s) {
    if (mic) {
        if (split) k_pair_full<double, ELEC, true, true><<<blocks, PAIR_WPB * 32, 0, s>>>(A);
        else k_pair_full<double, ELEC, true, false><<<blocks, PAIR_WPB * 32, 0, s>>>(A);
    } else {
        if (split) k_pair_full<double, ELEC, false, true><<<blocks, PAIR_WPB * 32, 0, s>>>(A);
        else k_pair_full<double, ELEC, false, false><<<blocks, PAIR_WPB * 32, 0, s>>>(A);
    }
}

// ---------------------------------------------------------------------------------
// mixed precision: half list, fixed-point forces
// ---------------------------------------------------------------------------------
#define PAIR_SS 8       // j-cluster entries per super-step
#define PAIR_NJ (PAIR_SS * MG_CL)
#ifndef PAIR_WIN
#define PAIR_WIN 128    // list entries compacted per window (the kept ones: J >= I)
#endif
#define PAIR_FFLUSH 2   // super-steps between the FP64 flushes of a lane's i-force partials
#define PAIR_EFLUSH 8   // super-steps between the FP64 flushes of a lane's energy partials

struct PairArgs {
    int n;
    const int *meta;  // meta[0] = number of clusters of the current build
    const int *pair_start, *pair_cnt, *pair_j, *pair_img, *cl_atom;
    const float4 *pair_shift, *xi, *qp;
    unsigned long long *facc_l, *facc_s;  // 64-bit fixed-point forces per cluster slot [3][slots]
    long long fstride;                    // slots of one component block
    float fscale, flimit;                 // 2^bits and 2^(52 - bits): unit 2^-bits, largest value
    unsigned *flags;
    // the pair parameters, rounded to FP32 once on the host
    float rc2, rce2, rs2, rmax2;
    float lx, ly, lz, ilx, ily, ilz;
    float kappa, coul, shift1, ron2, roff2, sw_denom, rce, v1, v2, f1, f2;
    int ljsw, mode;  // mode bit 0: long bucket, bit 1: short bucket
    double *rows;
    int row0;
};

__device__ __forceinline__ int info_of(float v) { return __float_as_int(v); }

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}

// x rounded to the nearest integer (ties to even) as a 64-bit two's-complement integer, for
// |x| < 2^55, built from its two 32-bit halves with 32-bit integer and FP32 operations only
// (64-bit conversions and 64-bit integer work run on the FP64 pipe or its neighbours, which
// are slow on this part): x = m 2^e with a 24-bit integer mantissa m; for e >= 0 the value is
// m << e (lo = m << e, hi = the bits shifted out), for |x| < 2^23 adding 2^23 rounds x to an
// integer held in the low mantissa bits; a negative value is the complement plus one, with
// the carry from lo into hi.
__device__ __forceinline__ long long f2ll_rn(float x) {
    const unsigned u = __float_as_uint(x);
    const int e = (int)((u >> 23) & 255u) - 150;
    const unsigned m = (u & 0x7fffffu) | 0x800000u;
    const unsigned ec = (unsigned)min(max(e, 0), 31);
    const unsigned small = __float_as_uint(fabsf(x) + 8388608.0f) - 0x4B000000u;
    unsigned lo = e >= 0 ? m << ec : small;
    unsigned hi = e >= 0 ? __funnelshift_l(m, 0u, ec) : 0u;
    if (u >> 31) {
        lo = ~lo + 1u;
        hi = ~hi + (lo == 0u ? 1u : 0u);
    }
    return (long long)(((unsigned long long)hi << 32) | lo);
}

// force component -> 64-bit fixed point in units of 1/scale; false when out of range or not
// finite (the limit, 2^52 units, leaves room for 2048 contributions of that size in one sum)
__device__ __forceinline__ bool to_fixed(float v, long long &o, float scale, float limit) {
    o = f2ll_rn(v * scale);
    return fabsf(v) < limit;
}

struct PairOut {
    float fx, fy, fz, r2, ulj, ush, uel, vir;
};

// One site pair (i at pi + sh, j at pj) in FP32: LJ (Lorentz-Berthelot, energy switch or
// shift energy) where both sites take part in LJ and r^2 < rc^2, Ewald real space (ELEC 1) or
// Wolf (ELEC 2) where r^2 < rce^2. Terms that do not apply are multiplied by zero rather than
// branched around, since the lanes of a warp hold different pairs.
template <int ELEC, bool MIC>
__device__ __forceinline__ PairOut pair_math(const PairArgs &A, const float4 &pi, const float4 &qi, int infi,
                                             const float4 &pj, const float4 &qj, const float4 &sh) {
    PairOut o;
    float dx = (pi.x + sh.x) - pj.x, dy = (pi.y + sh.y) - pj.y, dz = (pi.z + sh.z) - pj.z;
    if (MIC) {
        dx -= A.lx * rintf(dx * A.ilx);
        dy -= A.ly * rintf(dy * A.ily);
        dz -= A.lz * rintf(dz * A.ilz);
    }
    const float r2 = dx * dx + dy * dy + dz * dz;
    const int infj = info_of(pj.w);
    const float rinv = rsqrtf(r2);
    const float rinv2 = rinv * rinv;
    const bool lj_on = (infi & infj & MG_SITE_LJ) && r2 < A.rc2;
    const float eps = lj_on ? qi.z * qj.z : 0.f;
    const float sig = qi.y + qj.y;
    const float sig2 = sig * sig;
    float s6 = sig2 * rinv2;
    s6 = s6 * s6 * s6;
    const float s12 = s6 * s6;
    float ulj = 4.f * eps * (s12 - s6);
    float flj = 24.f * eps * (2.f * s12 - s6) * rinv2;
    float ush = 0.f;
    if (A.ljsw) {  // uniform over the launch
        if (!(r2 < A.ron2)) {
            const float d = A.roff2 - r2;
            const float sw = d * d * (A.roff2 + 2.f * r2 - 3.f * A.ron2) / A.sw_denom;
            flj = flj * sw - ulj * 12.f * d * (A.ron2 - r2) / A.sw_denom;
            ulj *= sw;
        }
    } else {
        const float sg6 = sig2 * sig2 * sig2;
        ush = eps * sg6 * (sg6 * A.shift1 - 1.f);
    }
    float f = flj, vir = flj * r2, uel = 0.f;
    if (ELEC != 0) {
        const float qq = r2 < A.rce2 ? qi.x * qj.x : 0.f;
        const float rr = r2 * rinv;
        const float kr = A.kappa * rr;
        const float ex = expf(-kr * kr);
        const float ec = erfc_from_exp(kr, ex);
        if (ELEC == 1) {
            const float bare = A.coul * qq * rinv;
            uel = bare * ec;
            f += (uel + bare * kr * ex * 1.1283791670955126f) * rinv2;
        } else {
            uel = A.coul * qq * (ec * rinv + A.v1 + A.v2 * (rr - A.rce));
            const float fe = A.coul * qq * rinv * (ec * rinv2 + A.f1 * ex * rinv + A.f2);
            f += fe;
            vir += fe * r2;
        }
    }
    o.fx = f * dx;
    o.fy = f * dy;
    o.fz = f * dz;
    o.r2 = r2;
    o.ulj = ulj;
    o.ush = ush;
    o.uel = uel;
    o.vir = vir;
    return o;
}


template <int NB>
struct PairSmem {
    float4 xj[PAIR_WPB][2][PAIR_NJ];  // x, y, z (cluster-relative), info bits
    float4 qj[PAIR_WPB][2][PAIR_NJ];  // q, half-sigma, sqrt-eps
    float4 sh[PAIR_WPB][2][PAIR_SS];  // periodic shift of each entry
    float4 xs[PAIR_WPB][MG_CL];       // the i-cluster's sites, as xj and qj
    float4 qs[PAIR_WPB][MG_CL];
    // pair forces by (bucket, component, i-site a, j-slot jj ^ 4a): the column pass (one lane
    // per j-slot, the sites in turn) and the row pass (16-byte loads) read without bank
    // conflicts, and the XOR spreads the stores of a round, which hold the pairs of one or two
    // sites, over the banks
    float fm[PAIR_WPB][NB][3][MG_CL][PAIR_NJ];
    int ent[PAIR_WPB][PAIR_WIN];      // kept entries of the window
    int jf[PAIR_WPB][PAIR_WIN];       // their j-cluster << 1 | (self entry: only i-site < j-site)
    unsigned short plist[PAIR_WPB][MG_CL * PAIR_NJ];  // the super-step's pairs: i-site << 6 | j-slot
};

// One warp per i-cluster I over the half of its list with J >= I: each unordered site pair
// once (Newton's third law). A cluster's entry with itself is kept for the zero image (site
// pairs a < b) and, when the cluster meets its own periodic image, for one of the images
// +s / -s (all site pairs). Per window of PAIR_WIN list entries the kept ones are compacted
// into shared memory in list order; per super-step of PAIR_SS of them:
//   1. the j-rows (positions with info bits; charge and LJ rows; shifts) arrive by cp.async,
//      one super-step ahead;
//   2. lane (site a = lane & 7, q = lane >> 3) tests site a against j-slots 8e + 4h + q of each
//      entry e (distance, molecule, ghost flags, RESPA bucket, a < b on the zero-image self
//      entry);
//   3. the active pairs are listed for the whole warp, site after site, and lane l takes
//      pairs l, l + 32, ... (the busiest site no longer sets the number of rounds): the pair
//      force goes to fm[bucket][.][a][jj ^ 4a] (one writer per cell), the energies to the
//      lane's partials;
//   4. the row sums of fm are the i-forces of the super-step: site a's four lanes a quarter
//      of the row each, into the lane's FP32 partial (64-bit fixed point every PAIR_FFLUSH
//      super-steps);
//   5. the column sums of fm, in site order, are the j-forces of the super-step; they are
//      added as 64-bit fixed point (units 2^-fixed_bits) to the slot-ordered accumulators.
// At the end of the row the site's i-force (its four lanes' integers summed) goes to the same
// accumulators. A value outside the fixed-point range raises MG_FLAG_FIXED_RANGE: the host
// then repeats the call with a coarser unit.
template <int ELEC, bool MIC, bool SPLIT>
__global__ void __launch_bounds__(PAIR_WPB * 32) k_pair(PairArgs A) {
    constexpr int NB = SPLIT ? 2 : 1;  // force buckets
    extern __shared__ __align__(16) unsigned char smem_raw[];
    PairSmem<NB> &S = *reinterpret_cast<PairSmem<NB> *>(smem_raw);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int a = lane & 7, q = lane >> 3;
    const int I = blockIdx.x * PAIR_WPB + w;
    long long FL[3] = {0, 0, 0}, FS[3] = {0, 0, 0};  // i-force sums in fixed point
    // uvdw ushift ureal vir (long bucket), then short: exact FP32 hi + lo pairs (no FP64 in the loop)
    float Eh[8] = {0, 0, 0, 0, 0, 0, 0, 0}, El[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int npair = 0;
    bool range_ok = true;
    if (I < A.meta[0]) {
        const float4 pi = A.xi[I * MG_CL + a];
        const float4 qi = A.qp[I * MG_CL + a];
        const int infi = info_of(pi.w);
        const bool use_long = (A.mode & 1) != 0, use_short = (A.mode & 2) != 0;
        const int e0 = A.pair_start[I], ne = A.pair_cnt[I];
        // lanes whose pairs precede lane (a, q)'s in the warp's list: every lane of sites
        // a' < a, and the lanes q' < q of site a (lane = a + 8 q)
        const unsigned lmask = ((1u << a) - 1u) * 0x01010101u | (((1u << (8 * q)) - 1u) & (0x01010101u << a));
        float eL[4] = {0, 0, 0, 0}, eS[4] = {0, 0, 0, 0};  // energy partials since the last FP64 flush
        float ax = 0, ay = 0, az = 0, bx = 0, by = 0, bz = 0;  // i-force partials since the last flush
        int sstep = 0;
        if (q == 0) {
            S.xs[w][a] = pi;
            S.qs[w][a] = qi;
        }
        for (int r0 = 0; r0 < ne; r0 += PAIR_WIN) {
            // compact the kept entries of window [r0, r0 + PAIR_WIN) in list order
            int nk = 0;
            for (int k0 = 0; k0 < PAIR_WIN && r0 + k0 < ne; k0 += 32) {
                const int k = r0 + k0 + lane;
                bool keep = false;
                int jf = 0;
                if (k < ne) {
                    const int J = A.pair_j[e0 + k];
                    bool self0 = false;
                    keep = J > I;
                    if (J == I) {
                        const int img = A.pair_img[e0 + k];
                        const int ix = (img & 1023) - 512, iy = ((img >> 10) & 1023) - 512,
                                  iz = ((img >> 20) & 1023) - 512;
                        self0 = ix == 0 && iy == 0 && iz == 0;
                        keep = iz > 0 || (iz == 0 && (iy > 0 || (iy == 0 && ix >= 0)));
                    }
                    jf = (J << 1) | (self0 ? 1 : 0);
                }
                const unsigned bal = __ballot_sync(0xffffffffu, keep);
                if (keep) {
                    const int o = nk + __popc(bal & ((1u << lane) - 1u));
                    S.ent[w][o] = e0 + k;
                    S.jf[w][o] = jf;
                }
                nk += __popc(bal);
            }
            __syncwarp();
            const int nss = (nk + PAIR_SS - 1) / PAIR_SS;
            auto stage = [&](int ss, int buf) {
                const int cnt = min(PAIR_SS, nk - ss * PAIR_SS);
#pragma unroll
                for (int k = 0; k < PAIR_NJ / 32; k++) {
                    const int t = lane + 32 * k, e = t >> 3;
                    if (e < cnt) {
                        const int J = S.jf[w][ss * PAIR_SS + e] >> 1;
                        cp_async16(&S.xj[w][buf][t], &A.xi[J * MG_CL + (t & 7)]);
                        cp_async16(&S.qj[w][buf][t], &A.qp[J * MG_CL + (t & 7)]);
                    }
                }
                if (lane < cnt) cp_async16(&S.sh[w][buf][lane], &A.pair_shift[S.ent[w][ss * PAIR_SS + lane]]);
                asm volatile("cp.async.commit_group;" ::: "memory");
            };
            if (nss > 0) stage(0, 0);
            for (int ss = 0; ss < nss; ss++, sstep++) {
                const int b = ss & 1;
                if (ss + 1 < nss) {
                    stage(ss + 1, b ^ 1);
                    asm volatile("cp.async.wait_group 1;" ::: "memory");
                } else {
                    asm volatile("cp.async.wait_group 0;" ::: "memory");
                }
                {  // clear the pair-force matrix of this super-step
                    uint4 *fm = reinterpret_cast<uint4 *>(&S.fm[w][0][0][0][0]);
                    constexpr int NF = (int)(NB * 3 * MG_CL * PAIR_NJ * sizeof(float) / 16);
#pragma unroll 4
                    for (int k = lane; k < NF; k += 32) fm[k] = make_uint4(0u, 0u, 0u, 0u);
                }
                __syncwarp();
                const int cnt = min(PAIR_SS, nk - ss * PAIR_SS);
                // 1. test
                unsigned m = 0u;
#pragma unroll
                for (int e = 0; e < PAIR_SS; e++) {
                    if (e < cnt) {
                        const float4 sh = S.sh[w][b][e];
                        const bool self0 = (S.jf[w][ss * PAIR_SS + e] & 1) != 0;
                        const float xs = pi.x + sh.x, ys = pi.y + sh.y, zs = pi.z + sh.z;
#pragma unroll
                        for (int h = 0; h < 2; h++) {
                            const int slot = 4 * h + q;
                            const float4 pj = S.xj[w][b][8 * e + slot];
                            float dx = xs - pj.x, dy = ys - pj.y, dz = zs - pj.z;
                            if (MIC) {
                                dx -= A.lx * rintf(dx * A.ilx);
                                dy -= A.ly * rintf(dy * A.ily);
                                dz -= A.lz * rintf(dz * A.ilz);
                            }
                            const float r2 = dx * dx + dy * dy + dz * dz;
                            const int infj = info_of(pj.w);
                            bool ok = !((infi | infj) & MG_SITE_DEAD) && ((infi ^ infj) >> 2) != 0 && r2 < A.rmax2 &&
                                      !(self0 && slot <= a);
                            if (SPLIT) ok = ok && (r2 < A.rs2 ? use_short : use_long);
                            m |= (ok ? 1u : 0u) << (2 * e + h);
                        }
                    }
                }
                // 2. one list for the warp, site after site (lane q's slots after those of q' < q):
                //    lane (a, q)'s offset is the sum of the counts of the lanes in lmask (sites
                //    a' < a, and site a's lanes q' < q), taken bit by bit from five ballots of
                //    the counts (no chain of dependent shuffles); the stores are unrolled over
                //    the 16 possible slots
                const int c0 = __popc(m);
                int off = 0, tot = 0;
#pragma unroll
                for (int bit = 0; bit < 5; bit++) {
                    const unsigned bb = __ballot_sync(0xffffffffu, (c0 >> bit) & 1);
                    off += __popc(bb & lmask) << bit;
                    tot += __popc(bb) << bit;
                }
#pragma unroll
                for (int t = 0; t < 2 * PAIR_SS; t++)
                    if (m & (1u << t))
                        S.plist[w][off + __popc(m & ((1u << t) - 1u))] =
                            (unsigned short)((a << 6) | (8 * (t >> 1) + 4 * (t & 1) + q));
                __syncwarp();
                // 3. pairs: lane l takes pairs l, l + 32, ... of the list; the pair force goes into
                //    fm (one writer per cell), the energies into the lane's partials (two pairs
                //    a lane per round as independent chains ran slower: 0.39 against 0.37 ms)
                for (int k = lane; k < tot; k += 32) {
                    const int code = S.plist[w][k];
                    const int ia = code >> 6, jj = code & 63;
                    const float4 xa = S.xs[w][ia];
                    const PairOut o = pair_math<ELEC, MIC>(A, xa, S.qs[w][ia], info_of(xa.w), S.xj[w][b][jj],
                                                           S.qj[w][b][jj], S.sh[w][b][jj >> 3]);
                    const bool inner = SPLIT && o.r2 < A.rs2;
                    npair += 2;  // counted as in a full list
                    const int bk = inner ? 1 : 0, col = jj ^ (ia << 2);
                    S.fm[w][bk][0][ia][col] = o.fx;
                    S.fm[w][bk][1][ia][col] = o.fy;
                    S.fm[w][bk][2][ia][col] = o.fz;
                    if (inner) {
                        eS[0] += o.ulj; eS[1] += o.ush; eS[2] += o.uel; eS[3] += o.vir;
                    } else {
                        eL[0] += o.ulj; eL[1] += o.ush; eL[2] += o.uel; eL[3] += o.vir;
                    }
                }
                __syncwarp();
                // 4. i-forces of the super-step: the row sums of site a, its four lanes a quarter
                //    of the row each (16-byte loads, rotated by a so that the lanes of one load
                //    fall on different banks)
#pragma unroll
                for (int bk = 0; bk < NB; bk++) {
                    float v[3];
#pragma unroll
                    for (int c = 0; c < 3; c++) {
                        const float4 *row = reinterpret_cast<const float4 *>(S.fm[w][bk][c][a]);
                        float s = 0.f;
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const float4 f = row[4 * q + ((k + a) & 3)];
                            s += (f.x + f.y) + (f.z + f.w);
                        }
                        v[c] = s;
                    }
                    if (bk == 0) {
                        ax += v[0]; ay += v[1]; az += v[2];
                    } else {
                        bx += v[0]; by += v[1]; bz += v[2];
                    }
                }
                if ((sstep + 1) % PAIR_FFLUSH == 0) {
                    long long o;
                    range_ok &= to_fixed(ax, o, A.fscale, A.flimit); FL[0] += o;
                    range_ok &= to_fixed(ay, o, A.fscale, A.flimit); FL[1] += o;
                    range_ok &= to_fixed(az, o, A.fscale, A.flimit); FL[2] += o;
                    ax = ay = az = 0;
                    if (SPLIT) {
                        range_ok &= to_fixed(bx, o, A.fscale, A.flimit); FS[0] += o;
                        range_ok &= to_fixed(by, o, A.fscale, A.flimit); FS[1] += o;
                        range_ok &= to_fixed(bz, o, A.fscale, A.flimit); FS[2] += o;
                        bx = by = bz = 0;
                    }
                }
                if ((sstep + 1) % PAIR_EFLUSH == 0) {
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        mg_acc2(Eh[k], El[k], eL[k]);
                        eL[k] = 0;
                        if (SPLIT) {
                            mg_acc2(Eh[4 + k], El[4 + k], eS[k]);
                            eS[k] = 0;
                        }
                    }
                }
                __syncwarp();
                // 4. j-forces of the super-step: minus the column sums, in site order
                for (int t = lane; t < cnt * MG_CL; t += 32) {
                    const int J = S.jf[w][ss * PAIR_SS + (t >> 3)] >> 1;
                    const unsigned slot = (unsigned)(J * MG_CL + (t & 7));
#pragma unroll
                    for (int bk = 0; bk < NB; bk++) {
                        unsigned long long *acc = bk ? A.facc_s : A.facc_l;
#pragma unroll
                        for (int c = 0; c < 3; c++) {
                            float v = S.fm[w][bk][c][0][t];
#pragma unroll
                            for (int i = 1; i < MG_CL; i++) v += S.fm[w][bk][c][i][t ^ (i << 2)];
                            if (v != 0.f) {
                                long long o;
                                range_ok &= to_fixed(-v, o, A.fscale, A.flimit);
                                atomicAdd(acc + c * A.fstride + slot, (unsigned long long)o);
                            }
                        }
                    }
                }
                __syncwarp();  // buffer b and the matrix are free for the next super-step
            }
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {  // the last partials
            mg_acc2(Eh[k], El[k], eL[k]);
            if (SPLIT) mg_acc2(Eh[4 + k], El[4 + k], eS[k]);
        }
        {
            long long o;
            range_ok &= to_fixed(ax, o, A.fscale, A.flimit); FL[0] += o;
            range_ok &= to_fixed(ay, o, A.fscale, A.flimit); FL[1] += o;
            range_ok &= to_fixed(az, o, A.fscale, A.flimit); FL[2] += o;
            if (SPLIT) {
                range_ok &= to_fixed(bx, o, A.fscale, A.flimit); FS[0] += o;
                range_ok &= to_fixed(by, o, A.fscale, A.flimit); FS[1] += o;
                range_ok &= to_fixed(bz, o, A.fscale, A.flimit); FS[2] += o;
            }
        }
        // i-forces: the site's four lanes (integer sums, exact in any order)
#pragma unroll
        for (int k = 0; k < 3; k++) {
            FL[k] += __shfl_xor_sync(0xffffffffu, FL[k], 8);
            FL[k] += __shfl_xor_sync(0xffffffffu, FL[k], 16);
            if (SPLIT) {
                FS[k] += __shfl_xor_sync(0xffffffffu, FS[k], 8);
                FS[k] += __shfl_xor_sync(0xffffffffu, FS[k], 16);
            }
        }
        if (q == 0 && !(infi & MG_SITE_DEAD)) {
            const long long slot = (long long)I * MG_CL + a;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                if (FL[c] != 0) atomicAdd(A.facc_l + c * A.fstride + slot, (unsigned long long)FL[c]);
                if (SPLIT && FS[c] != 0) atomicAdd(A.facc_s + c * A.fstride + slot, (unsigned long long)FS[c]);
            }
        }
    }
    if (__any_sync(0xffffffffu, !range_ok) && lane == 0) atomicOr(A.flags, MG_FLAG_FIXED_RANGE);
    double eng[9];
#pragma unroll
    for (int k = 0; k < 8; k++) eng[k] = (double)Eh[k] + (double)El[k];
    eng[8] = (double)npair;
    const int ids[9] = {E_UVDW, E_USHIFT, E_UREAL, E_VIR, E_UVDW_S, E_USHIFT_S, E_UREAL_S, E_VIR_S, E_NPAIR};
    mg_block_row<9>(eng, ids, A.rows, A.row0 + blockIdx.x);
}

// The fixed-point slot accumulators into FP64 forces in site order (overwriting fl / fs, when
// given), clearing every accumulator for the next evaluation. All loads are issued before the
// stores.
__global__ void k_fixed_forces(const int *__restrict__ meta, const int *__restrict__ cl_atom, int n,
                               unsigned long long *__restrict__ facc_l, unsigned long long *__restrict__ facc_s,
                               long long fstride, double unit, double *__restrict__ fl, double *__restrict__ fs) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= fstride) return;
    const int at = s < (long long)meta[0] * MG_CL ? cl_atom[s] : -1;
    long long vl[3], vs[3] = {0, 0, 0};
#pragma unroll
    for (int c = 0; c < 3; c++) vl[c] = (long long)__ldcg(facc_l + c * fstride + s);
    if (facc_s) {
#pragma unroll
        for (int c = 0; c < 3; c++) vs[c] = (long long)__ldcg(facc_s + c * fstride + s);
    }
#pragma unroll
    for (int c = 0; c < 3; c++) {
        facc_l[c * fstride + s] = 0ull;
        if (facc_s) facc_s[c * fstride + s] = 0ull;
    }
    if (at < 0) return;
#pragma unroll
    for (int c = 0; c < 3; c++) {
        if (fl) fl[(size_t)c * n + at] = (double)vl[c] * unit;
        if (fs) fs[(size_t)c * n + at] = (double)vs[c] * unit;
    }
}

template <int ELEC, bool MIC, bool SPLIT>
cudaError_t launch_pair_one(const PairArgs &A, unsigned blocks, cudaStream_t s) {
    const int smem = (int)sizeof(PairSmem<SPLIT ? 2 : 1>);
    cudaError_t e = cudaFuncSetAttribute(k_pair<ELEC, MIC, SPLIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k_pair<ELEC, MIC, SPLIT><<<blocks, PAIR_WPB * 32, smem, s>>>(A);
    return cudaGetLastError();
}

template <int ELEC>
cudaError_t launch_pair_elec(const PairArgs &A, bool mic, bool split, unsigned blocks, cudaStream_t s) {
    if (mic) return split ? launch_pair_one<ELEC, true, true>(A, blocks, s) : launch_pair_one<ELEC, true, false>(A, blocks, s);
    return split ? launch_pair_one<ELEC, false, true>(A, blocks, s) : launch_pair_one<ELEC, false, false>(A, blocks, s);
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
    const int elec = p.charge_type == MG_ELEC_EWALD ? 1 : (p.charge_type == MG_ELEC_WOLF ? 2 : 0);
    const bool split = p.respa_split > 0;
    const double rs2 = split ? p.respa_split * p.respa_split : 0.0;
    double rmax2 = elec ? fmax(p.rcutoffsq, p.rcutoffelecsq) : p.rcutoffsq;
    if (split && !want_long) rmax2 = fmin(rmax2, rs2);
    // the inner pass of the distance split walks only the inner sub-list
    const bool sub = want_short && !want_long && c->sub_ready;
    const int *pstart = (const int *)(sub ? c->d_sub_start.p : c->d_pair_start.p);
    const int *pcnt = (const int *)(sub ? c->d_sub_count.p : c->d_pair_count.p);
    const int *pj = (const int *)(sub ? c->d_sub_j.p : c->d_pair_j.p);
    const void *pshift = sub ? c->d_sub_shift.p : c->d_pair_shift.p;
    const int *pimg = (const int *)(sub ? c->d_sub_img.p : c->d_pair_img.p);
    const unsigned blocks = (unsigned)((c->cl_cap + PAIR_WPB - 1) / PAIR_WPB);
    if (blocks == 0) return MG_OK;
    const int row0 = mg_reserve_rows(c, blocks);
    if (row0 < 0) return mg_fail(c, MG_ERR_ALLOC, "energy partial rows exhausted");
    const int mode = (want_long ? 1 : 0) | (want_short ? 2 : 0);
    if (c->opt.precision == MG_PREC_FP64) {  // the plain-FP64 path: full list, FP64 sums, no atomics
        PairFullArgs F;
        F.n = c->natom;
        F.meta = (const int *)c->d_meta.p;
        F.pair_start = pstart;
        F.pair_cnt = pcnt;
        F.pair_j = pj;
        F.info = (const int *)c->d_pack_info.p;
        F.cl_atom = (const int *)c->d_cl_atom.p;
        F.pair_shift = pshift;
        F.pos = c->d_pack_pos.p;
        F.lj = c->d_pack_lj.p;
        F.fl = want_long ? fl : nullptr;
        F.fs = want_short ? fs : nullptr;
        F.rc2 = p.rcutoffsq, F.rce2 = p.rcutoffelecsq, F.rs2 = rs2, F.rmax2 = rmax2;
        F.lx = c->lx, F.ly = c->ly, F.lz = c->lz;
        F.kappa = p.kappa, F.coul = p.coulomb_prefactor, F.shift1 = p.shift1, F.ron2 = p.rcutonsq;
        F.roff2 = p.rcutoffsq, F.sw_denom = p.roff2_minus_ron2_cube, F.rce = p.rcutoffelec;
        F.v1 = p.wolfvcon1, F.v2 = p.wolfvcon2, F.f1 = p.wolffcon1, F.f2 = p.wolffcon2;
        F.ljsw = p.lj_switch;
        F.mode = mode;
        F.rows = (double *)c->d_epart.p;
        F.row0 = row0;
        if (elec == 1) launch_pair_full_elec<1>(F, c->small_box, split, blocks, c->stream);
        else if (elec == 2) launch_pair_full_elec<2>(F, c->small_box, split, blocks, c->stream);
        else launch_pair_full_elec<0>(F, c->small_box, split, blocks, c->stream);
        MG_CUDA(cudaGetLastError());
        c->launches += 1;
        return MG_OK;
    }
    PairArgs A;
    A.n = c->natom;
    A.meta = (const int *)c->d_meta.p;
    A.pair_start = pstart;
    A.pair_cnt = pcnt;
    A.pair_j = pj;
    A.pair_img = pimg;
    A.pair_shift = (const float4 *)pshift;
    A.xi = (const float4 *)c->d_pack_xi.p;
    A.qp = (const float4 *)c->d_pack_qp.p;
    A.cl_atom = (const int *)c->d_cl_atom.p;
    // fixed-point force accumulators per cluster slot, one [3][slots] block per bucket: zero
    // when allocated, cleared again by k_fixed_forces after every use
    A.fstride = (long long)c->cl_cap * MG_CL;
    const size_t fbytes = sizeof(unsigned long long) * 3 * (size_t)A.fstride;
    if (c->d_facc.bytes < 2 * fbytes) {
        if (!mg_ensure(c, c->d_facc, 2 * fbytes)) return MG_ERR_ALLOC;
        MG_CUDA(cudaMemsetAsync(c->d_facc.p, 0, c->d_facc.bytes, c->stream));
    }
    A.facc_l = (unsigned long long *)c->d_facc.p;
    A.facc_s = A.facc_l + 3 * A.fstride;
    A.fscale = ldexpf(1.0f, c->fixed_bits);
    A.flimit = ldexpf(1.0f, 52 - c->fixed_bits);
    A.flags = (unsigned *)c->d_flags.p;
    A.rc2 = (float)p.rcutoffsq;
    A.rce2 = (float)p.rcutoffelecsq;
    A.rs2 = (float)rs2;
    A.rmax2 = (float)rmax2;
    A.lx = (float)c->lx;
    A.ly = (float)c->ly;
    A.lz = (float)c->lz;
    A.ilx = (float)(1.0 / c->lx);
    A.ily = (float)(1.0 / c->ly);
    A.ilz = (float)(1.0 / c->lz);
    A.kappa = (float)p.kappa;
    A.coul = (float)p.coulomb_prefactor;
    A.shift1 = (float)p.shift1;
    A.ron2 = (float)p.rcutonsq;
    A.roff2 = (float)p.rcutoffsq;
    A.sw_denom = (float)p.roff2_minus_ron2_cube;
    A.rce = (float)p.rcutoffelec;
    A.v1 = (float)p.wolfvcon1;
    A.v2 = (float)p.wolfvcon2;
    A.f1 = (float)p.wolffcon1;
    A.f2 = (float)p.wolffcon2;
    A.ljsw = p.lj_switch;
    A.mode = mode;
    A.rows = (double *)c->d_epart.p;
    A.row0 = row0;
    cudaError_t e;
    if (elec == 1) e = launch_pair_elec<1>(A, c->small_box, split, blocks, c->stream);
    else if (elec == 2) e = launch_pair_elec<2>(A, c->small_box, split, blocks, c->stream);
    else e = launch_pair_elec<0>(A, c->small_box, split, blocks, c->stream);
    MG_CUDA(e);
    // both buckets the kernel may have written are cleared, whether or not they are wanted
    const unsigned fblocks = (unsigned)((A.fstride + 255) / 256);
    k_fixed_forces<<<fblocks, 256, 0, c->stream>>>(A.meta, A.cl_atom, A.n, A.facc_l, split ? A.facc_s : nullptr,
                                                   A.fstride, ldexp(1.0, -c->fixed_bits), want_long ? fl : nullptr,
                                                   want_short ? fs : nullptr);
    MG_CUDA(cudaGetLastError());
    c->launches += 2;
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
