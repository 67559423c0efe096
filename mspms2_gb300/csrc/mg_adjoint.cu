// mg_adjoint.cu - derivatives of the long-range forces (those of frclong(),
// src/frclong.c:20) for fitting and second-order methods:
//   mg_adjoint_params: the gradient of a loss L(F) with respect to the force-field
//     parameters of every site class (species, site of the template): LJ epsilon, sigma
//     and the charge;
//   mg_adjoint_hvp: the Hessian-vector product in positions, H v = -(dF/dr) v.
//
// Every nonbonded force of the engine is a sum of pair terms phi_ij(r) u_ij (u_ij the pair
// vector r_i - r_j, or its minimum image) plus the reciprocal-space force. With
// g_i = dL/dF_i:
//   dL/dp = sum over ordered pairs (i, j) of (g_i . u_ij) dphi_ij/dp   + reciprocal part,
//   dF_i  = sum_j [ phi_ij w_ij + chi_ij (u_ij . w_ij) u_ij ]         + reciprocal part,
// with w_ij = v_i - v_j and chi = (dphi/dr)/r. The pair terms are recomputed here from the
// cluster-pair list of the forward evaluation (nothing is stored between the passes):
//   LJ: phi = 24 eps_ij (2 s^12 - s^6)/r^2, eps_ij = sqrt(eps_i eps_j) (x f0 for 1-4
//       pairs), sigma_ij = (sigma_i + sigma_j)/2 (src/ljfrc.c:21-71, src/frclong.c:127-130);
//   Ewald real space and Wolf: phi = C q_i q_j psi(r) (src/elecfrc.c:17-60);
//   intramolecular corrections: the engine's intramolecular kernel term by term, with its
//       treatment of molecules that span the box (src/frclong.c:222-982);
//   reciprocal space, F_i = q_i W_i with W_i = sum_k cf_k Im(conj(S_k) e^{ik.r_i}) k
//       (src/frclong.c:988-1048): dL/dq_c = sum_{i in c} g_i . W_i
//       + sum_k cf_k Im(conj(T^c_k) (k . A_k)), T^c_k = sum_{j in c} e^{ik.r_j},
//       A_k = sum_i q_i g_i e^{ik.r_i}; the position derivative is in mg_ewald.cu.
// Pair arithmetic is FP32 on the mixed path and FP64 on the FP64 path; every sum over
// pairs, blocks and k-vectors is FP64 in a fixed order, so results are reproducible.
#include <math.h>
#include <string.h>

#include <vector>

#include "mg_internal.cuh"

#define ADJ_MAXC 16  // site classes
#define ADJ_TPB 128

namespace {

template <typename R>
struct AdjT;
template <>
struct AdjT<float> {
    typedef float4 V4;
    typedef float2 V2;
    __device__ static float erfc_(float x) { return erfcf(x); }
    __device__ static float erf_(float x) { return erff(x); }
    __device__ static float exp_(float x) { return expf(x); }
    __device__ static float sqrt_(float x) { return sqrtf(x); }
    __device__ static float rint_(float x) { return rintf(x); }
};
template <>
struct AdjT<double> {
    typedef double4 V4;
    typedef double2 V2;
    __device__ static double erfc_(double x) { return erfc(x); }
    __device__ static double erf_(double x) { return erf(x); }
    __device__ static double exp_(double x) { return exp(x); }
    __device__ static double sqrt_(double x) { return sqrt(x); }
    __device__ static double rint_(double x) { return rint(x); }
};

// electrostatic pair forms, per unit C q_i q_j
enum { EL_EWALD = 1, EL_WOLF = 2, EL_EWALD_EXCL = 3, EL_WOLF_EXCL = 4, EL_BARE_EXCL = 5 };

struct ElecK {
    double kappa, f1, f2;
};

// psi = phi / (C q q) and chi = (dpsi/dr) / r of one electrostatic form
// (a = 2 kappa/sqrt(pi), e = exp(-kappa^2 r^2)):
//   1 Ewald real space        erfc/r^3 + a e/r^2
//   2 Wolf                    erfc/r^3 + f1 e/r^2 + f2/r
//   3 Ewald real + exclusion  -erf/r^3 + a e/r^2     (1-2/1-3 pair of a whole molecule)
//   4 Wolf + exclusion        -erf/r^3 + f1 e/r^2 + f2/r
//   5 bare exclusion          -1/r^3
template <typename R, bool CHI>
__device__ __forceinline__ void elec_form(const ElecK &K, int form, R r2, R &psi, R &chi) {
    typedef AdjT<R> T;
    const R r = T::sqrt_(r2), ir = (R)1 / r, ir2 = ir * ir, ir3 = ir2 * ir, ir4 = ir2 * ir2;
    if (form == EL_BARE_EXCL) {
        psi = -ir3;
        if (CHI) chi = (R)3 * ir4 * ir;
        return;
    }
    const R kap = (R)K.kappa, kr = kap * r, e = T::exp_(-kr * kr), a = (R)1.1283791670955126 * kap;
    const bool excl = form == EL_EWALD_EXCL || form == EL_WOLF_EXCL;
    // +erfc (real space) or -erf (real space with the exclusion); d/dr of both is -a e
    const R ef = excl ? -T::erf_(kr) : T::erfc_(kr);
    const R f1 = (form == EL_EWALD || form == EL_EWALD_EXCL) ? a : (R)K.f1;
    const R f2 = (form == EL_EWALD || form == EL_EWALD_EXCL) ? (R)0 : (R)K.f2;
    psi = ef * ir3 + f1 * e * ir2 + f2 * ir;
    if (CHI) {
        const R d = -(R)3 * ef * ir4 - a * e * ir3 - f1 * e * ((R)2 * kap * kap * ir + (R)2 * ir3) - f2 * ir2;
        chi = d * ir;
    }
}

// LJ force coefficient phi, its sigma derivative and chi = (dphi/dr)/r
template <typename R>
__device__ __forceinline__ void lj_form(R r2, R sig, R eps, R &phi, R &dphi_dsig, R &chi) {
    const R ir2 = (R)1 / r2, s2 = sig * sig * ir2, s6 = s2 * s2 * s2, s12 = s6 * s6;
    phi = (R)24 * eps * ((R)2 * s12 - s6) * ir2;
    dphi_dsig = (R)24 * eps * ((R)24 * s12 - (R)6 * s6) * ir2 / sig;
    chi = (R)24 * eps * ((R)8 * s6 - (R)28 * s12) * ir2 * ir2;
}

struct Grad3 {
    double e[ADJ_MAXC], s[ADJ_MAXC], q[ADJ_MAXC];
};

// (g . u) times the parameter derivatives of an LJ term; eps_ij = se_i se_j scale, so
// d eps_ij / d eps_i = eps_ij / (2 eps_i); d sigma_ij / d sigma_i = 1/2
template <typename R>
__device__ __forceinline__ void grad_lj(Grad3 &G, R t, R r2, R hs_i, R hs_j, R se_i, R se_j, R scale, int ci,
                                        int cj) {
    const R eps = se_i * se_j * scale;
    if (eps == (R)0) return;
    R phi, dps, chi;
    lj_form<R>(r2, hs_i + hs_j, eps, phi, dps, chi);
    G.e[ci] += (double)((R)0.5 * t * phi / (se_i * se_i));
    G.e[cj] += (double)((R)0.5 * t * phi / (se_j * se_j));
    G.s[ci] += (double)((R)0.5 * t * dps);
    G.s[cj] += (double)((R)0.5 * t * dps);
}

template <typename R>
__device__ __forceinline__ void grad_elec(Grad3 &G, const ElecK &K, int form, R coul, R t, R r2, R q_i, R q_j,
                                          int ci, int cj) {
    R psi, chi;
    elec_form<R, false>(K, form, r2, psi, chi);
    const R c = coul * t * psi;
    G.q[ci] += (double)(c * q_j);
    G.q[cj] += (double)(c * q_i);
}

__device__ void write_rows(const Grad3 &G, int nclass, double *rows) {
    __shared__ double red[ADJ_TPB];
    for (int p = 0; p < 3 * nclass; p++) {
        const int k = p % nclass;
        red[threadIdx.x] = p < nclass ? G.e[k] : (p < 2 * nclass ? G.s[k] : G.q[k]);
        __syncthreads();
        for (int o = ADJ_TPB / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) rows[(size_t)blockIdx.x * 3 * nclass + p] = red[0];
        __syncthreads();
    }
}

struct AdjArgs {
    int n, nclass;
    const int *meta, *pair_start, *pair_cnt, *pair_j, *info, *cl_atom;
    const void *pos, *lj, *shift;
    const int *site_class;  // [n]
    const double *g;        // [3][n]: dL/dF (adjoint) or v (product)
    double rc2, rce2, rmax2, lx, ly, lz, coul;
    ElecK K;
    int elec;  // 0 none, EL_EWALD, EL_WOLF
    int mic;
    double *rows;  // adjoint: [blocks][3 * nclass]
    double *out;   // product: [3][n]
};

// one thread per i-slot over its cluster's list (a full list: every ordered pair once)
template <typename R>
__global__ void __launch_bounds__(ADJ_TPB) k_adj_pair(AdjArgs A) {
    typedef typename AdjT<R>::V4 V4;
    typedef typename AdjT<R>::V2 V2;
    Grad3 G;
    for (int c = 0; c < ADJ_MAXC; c++) G.e[c] = G.s[c] = G.q[c] = 0.0;
    const int slot = blockIdx.x * ADJ_TPB + threadIdx.x;
    const int I = slot / MG_CL;
    if (I < A.meta[0]) {
        const int a = A.cl_atom[slot];
        const V4 *pos = (const V4 *)A.pos;
        const V2 *lj = (const V2 *)A.lj;
        const V4 *shift = (const V4 *)A.shift;
        if (a >= 0) {
            const int infi = A.info[slot];
            const V4 pi = pos[slot];
            const V2 li = lj[slot];
            const int ci = A.site_class[a];
            const R gx = (R)A.g[a], gy = (R)A.g[A.n + a], gz = (R)A.g[2 * A.n + a];
            const R lx = (R)A.lx, ly = (R)A.ly, lz = (R)A.lz, coul = (R)A.coul;
            const int e0 = A.pair_start[I], e1 = e0 + A.pair_cnt[I];
            for (int e = e0; e < e1; e++) {
                const int J = A.pair_j[e];
                const V4 sh = shift[e];
                for (int jl = 0; jl < MG_CL; jl++) {
                    const int sj = J * MG_CL + jl;
                    const int b = A.cl_atom[sj];
                    if (b < 0) continue;
                    const int infj = A.info[sj];
                    const V4 pj = pos[sj];
                    R dx = pi.x + sh.x - pj.x, dy = pi.y + sh.y - pj.y, dz = pi.z + sh.z - pj.z;
                    if (A.mic) {
                        dx -= lx * AdjT<R>::rint_(dx / lx);
                        dy -= ly * AdjT<R>::rint_(dy / ly);
                        dz -= lz * AdjT<R>::rint_(dz / lz);
                    }
                    const R r2 = dx * dx + dy * dy + dz * dz;
                    if (((infi | infj) & MG_SITE_DEAD) || (infi >> 2) == (infj >> 2) || !(r2 < (R)A.rmax2)) continue;
                    const R t = gx * dx + gy * dy + gz * dz;
                    const int cj = A.site_class[b];
                    if ((infi & infj & MG_SITE_LJ) && r2 < (R)A.rc2) {
                        const V2 lj_j = lj[sj];
                        grad_lj<R>(G, t, r2, li.x, lj_j.x, li.y, lj_j.y, (R)1, ci, cj);
                    }
                    if (A.elec && r2 < (R)A.rce2) grad_elec<R>(G, A.K, A.elec, coul, t, r2, pi.w, pj.w, ci, cj);
                }
            }
        }
    }
    write_rows(G, A.nclass, A.rows);
}

struct IntraArgs {
    int n, nmole, nspecies, nclass;
    const SpeciesDev *species;
    const IntraPair *intra;
    const int *sflags, *site_class;
    const double *x, *y, *z, *q, *hsig, *seps, *g;
    double lx, ly, lz, rc2, rce2, f0, coul;
    ElecK K;
    int elec;
    double *rows;  // adjoint
    double *out;   // product
};

__device__ __forceinline__ double mic_d(double d, double L) { return d - L * rint(d / L); }

// The engine's intramolecular term list for one molecule, in its order, calling back for
// every term with its vector, whether that vector moves with the sites (false for the
// integer-truncated vector the reference keeps once a molecule is found to span the box,
// src/frclong.c:223, :278-312) and the term's form: 0 = LJ with an eps scale, else an
// electrostatic form.
template <typename R, typename Fn>
__device__ __forceinline__ void intra_terms(const IntraArgs &A, int mol, Fn &&fn) {
    int sp = 0;
    while (sp + 1 < A.nspecies && mol >= A.species[sp + 1].first_mole) sp++;
    const SpeciesDev S = A.species[sp];
    const int base = S.first_site + (mol - S.first_mole) * S.natom;
    int same = 1;
    for (int k = 0; k < S.nintra; k++) {
        const IntraPair ip = A.intra[S.intra_off + k];
        const int ii = base + ip.m, jj = base + ip.n;
        const int gi = A.sflags[ii], gj = A.sflags[jj];
        const bool full = ((gi | gj) & MG_SITE_DEAD) != 0;
        const bool ljok = (gi & (MG_SITE_LJ | MG_SITE_DEAD)) && (gj & (MG_SITE_LJ | MG_SITE_DEAD));
        double dx = A.x[ii] - A.x[jj], dy = A.y[ii] - A.y[jj], dz = A.z[ii] - A.z[jj];
        const bool straddle = fabs(dx) > A.lx * 0.5 || fabs(dy) > A.ly * 0.5 || fabs(dz) > A.lz * 0.5;
        bool moves = true;
        if (ip.kind == 0) {
            if (straddle) {
                same = 0;
                if (full) continue;
            } else {
                same = 1;
            }
        } else if (straddle && full) {
            continue;
        }
        if (!same) {
            const double mx = mic_d(dx, A.lx), my = mic_d(dy, A.ly), mz = mic_d(dz, A.lz);
            const R r2 = (R)(mx * mx + my * my + mz * mz);
            if (ljok && r2 < (R)A.rc2) fn(ii, jj, mx, my, mz, r2, true, 0, (R)1);
            dx = (double)(int)dx;
            dy = (double)(int)dy;
            dz = (double)(int)dz;
            moves = false;
        } else if (ip.kind != 0) {
            const R r2 = (R)(dx * dx + dy * dy + dz * dz);
            if (r2 < (R)A.rc2) fn(ii, jj, dx, dy, dz, r2, true, 0, ip.kind == 1 ? (R)A.f0 : (R)1);
        }
        if (A.elec == 0) continue;
        if (ip.kind == 0 && same) {
            const R r2 = (R)(dx * dx + dy * dy + dz * dz);
            if (r2 < (R)A.rce2)
                fn(ii, jj, dx, dy, dz, r2, moves, A.elec == EL_EWALD ? EL_EWALD_EXCL : EL_WOLF_EXCL, (R)0);
            continue;
        }
        if (ip.kind == 0) {
            const R r2 = (R)(dx * dx + dy * dy + dz * dz);
            if (r2 < (R)A.rce2) fn(ii, jj, dx, dy, dz, r2, moves, EL_BARE_EXCL, (R)0);
        }
        const double mx = mic_d(dx, A.lx), my = mic_d(dy, A.ly), mz = mic_d(dz, A.lz);
        const R r2 = (R)(mx * mx + my * my + mz * mz);
        if (r2 < (R)A.rce2) fn(ii, jj, mx, my, mz, r2, moves, A.elec, (R)0);
    }
}

template <typename R>
__global__ void __launch_bounds__(ADJ_TPB) k_adj_intra(IntraArgs A) {
    Grad3 G;
    for (int c = 0; c < ADJ_MAXC; c++) G.e[c] = G.s[c] = G.q[c] = 0.0;
    const int mol = blockIdx.x * ADJ_TPB + threadIdx.x;
    if (mol < A.nmole) {
        const int n = A.n;
        intra_terms<R>(A, mol, [&](int ii, int jj, double ux, double uy, double uz, R r2, bool, int form, R scale) {
            const R t = (R)(A.g[ii] - A.g[jj]) * (R)ux + (R)(A.g[n + ii] - A.g[n + jj]) * (R)uy +
                        (R)(A.g[2 * n + ii] - A.g[2 * n + jj]) * (R)uz;
            const int ci = A.site_class[ii], cj = A.site_class[jj];
            if (form == 0)
                grad_lj<R>(G, t, r2, (R)A.hsig[ii], (R)A.hsig[jj], (R)A.seps[ii], (R)A.seps[jj], scale, ci, cj);
            else
                grad_elec<R>(G, A.K, form, (R)A.coul, t, r2, (R)A.q[ii], (R)A.q[jj], ci, cj);
        });
    }
    write_rows(G, A.nclass, A.rows);
}

// per-class sums of g_i . W_i (reciprocal-space field term of the charge gradient)
__global__ void __launch_bounds__(ADJ_TPB) k_adj_field(int n, int nclass, const int *__restrict__ site_class,
                                                     const double *__restrict__ g, const double *__restrict__ w,
                                                     double *__restrict__ rows) {
    __shared__ double red[ADJ_TPB];
    const int a = blockIdx.x * ADJ_TPB + threadIdx.x;
    double v = 0.0;
    int c = -1;
    if (a < n) {
        c = site_class[a];
        v = g[a] * w[a] + g[n + a] * w[n + a] + g[2 * n + a] * w[2 * n + a];
    }
    for (int k = 0; k < nclass; k++) {
        red[threadIdx.x] = c == k ? v : 0.0;
        __syncthreads();
        for (int o = ADJ_TPB / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) rows[(size_t)blockIdx.x * nclass + k] = red[0];
        __syncthreads();
    }
}

// site weights for the structure factors: q_i g_i,d (d = 0..2), then (nclass > 0) the
// class indicators 1[class(i) = c] and a row of ones
__global__ void k_adj_weights(int n, int nclass, const int *__restrict__ site_class, const double *__restrict__ q,
                              const double *__restrict__ g, double *__restrict__ w) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    for (int d = 0; d < 3; d++) w[(size_t)d * n + a] = q[a] * g[(size_t)d * n + a];
    if (nclass == 0) return;
    for (int c = 0; c < nclass; c++) w[(size_t)(3 + c) * n + a] = site_class[a] == c ? 1.0 : 0.0;
    w[(size_t)(3 + nclass) * n + a] = 1.0;  // unit charges for the field pass
}

// ---- Hessian-vector product: directional derivative of the pair forces -----------------
// dF_i += phi w + chi (u . w) u for every term, w = v_i - v_j
template <typename R>
__device__ __forceinline__ void jvp_term(R phi, R chi, R ux, R uy, R uz, R wx, R wy, R wz, R &fx, R &fy, R &fz) {
    const R uw = chi * (ux * wx + uy * wy + uz * wz);
    fx += phi * wx + uw * ux;
    fy += phi * wy + uw * uy;
    fz += phi * wz + uw * uz;
}

template <typename R>
__global__ void __launch_bounds__(ADJ_TPB) k_hvp_pair(AdjArgs A) {
    typedef typename AdjT<R>::V4 V4;
    typedef typename AdjT<R>::V2 V2;
    const int slot = blockIdx.x * ADJ_TPB + threadIdx.x;
    const int I = slot / MG_CL;
    if (I >= A.meta[0]) return;
    const int a = A.cl_atom[slot];
    if (a < 0) return;
    const V4 *pos = (const V4 *)A.pos;
    const V2 *lj = (const V2 *)A.lj;
    const V4 *shift = (const V4 *)A.shift;
    const int n = A.n;
    const int infi = A.info[slot];
    const V4 pi = pos[slot];
    const V2 li = lj[slot];
    const R vx = (R)A.g[a], vy = (R)A.g[n + a], vz = (R)A.g[2 * n + a];
    const R lx = (R)A.lx, ly = (R)A.ly, lz = (R)A.lz, coul = (R)A.coul;
    double F[3] = {0, 0, 0};
    const int e0 = A.pair_start[I], e1 = e0 + A.pair_cnt[I];
    for (int e = e0; e < e1; e++) {
        const int J = A.pair_j[e];
        const V4 sh = shift[e];
        R fx = 0, fy = 0, fz = 0;
        for (int jl = 0; jl < MG_CL; jl++) {
            const int sj = J * MG_CL + jl;
            const int b = A.cl_atom[sj];
            if (b < 0) continue;
            const int infj = A.info[sj];
            const V4 pj = pos[sj];
            R dx = pi.x + sh.x - pj.x, dy = pi.y + sh.y - pj.y, dz = pi.z + sh.z - pj.z;
            if (A.mic) {
                dx -= lx * AdjT<R>::rint_(dx / lx);
                dy -= ly * AdjT<R>::rint_(dy / ly);
                dz -= lz * AdjT<R>::rint_(dz / lz);
            }
            const R r2 = dx * dx + dy * dy + dz * dz;
            if (((infi | infj) & MG_SITE_DEAD) || (infi >> 2) == (infj >> 2) || !(r2 < (R)A.rmax2)) continue;
            R phi = 0, chi = 0;
            if ((infi & infj & MG_SITE_LJ) && r2 < (R)A.rc2) {
                const V2 lj_j = lj[sj];
                R p, ds, c;
                lj_form<R>(r2, li.x + lj_j.x, li.y * lj_j.y, p, ds, c);
                phi += p;
                chi += c;
            }
            if (A.elec && r2 < (R)A.rce2) {
                R p, c;
                elec_form<R, true>(A.K, A.elec, r2, p, c);
                const R cq = coul * pi.w * pj.w;
                phi += cq * p;
                chi += cq * c;
            }
            jvp_term<R>(phi, chi, dx, dy, dz, vx - (R)A.g[b], vy - (R)A.g[n + b], vz - (R)A.g[2 * n + b], fx, fy, fz);
        }
        F[0] += (double)fx;
        F[1] += (double)fy;
        F[2] += (double)fz;
    }
    A.out[a] += F[0];
    A.out[n + a] += F[1];
    A.out[2 * n + a] += F[2];
}

template <typename R>
__global__ void __launch_bounds__(ADJ_TPB) k_hvp_intra(IntraArgs A) {
    const int mol = blockIdx.x * ADJ_TPB + threadIdx.x;
    if (mol >= A.nmole) return;
    const int n = A.n;
    const double *v = A.g;
    intra_terms<R>(A, mol, [&](int ii, int jj, double ux, double uy, double uz, R r2, bool moves, int form, R scale) {
        if (!moves) return;  // a truncated vector does not change with the positions
        R phi, chi;
        if (form == 0) {
            R ds;
            lj_form<R>(r2, (R)(A.hsig[ii] + A.hsig[jj]), (R)(A.seps[ii] * A.seps[jj]) * scale, phi, ds, chi);
        } else {
            elec_form<R, true>(A.K, form, r2, phi, chi);
            const R cq = (R)A.coul * (R)A.q[ii] * (R)A.q[jj];
            phi *= cq;
            chi *= cq;
        }
        R fx = 0, fy = 0, fz = 0;
        jvp_term<R>(phi, chi, (R)ux, (R)uy, (R)uz, (R)(v[ii] - v[jj]), (R)(v[n + ii] - v[n + jj]),
                    (R)(v[2 * n + ii] - v[2 * n + jj]), fx, fy, fz);
        A.out[ii] += (double)fx;
        A.out[n + ii] += (double)fy;
        A.out[2 * n + ii] += (double)fz;
        A.out[jj] -= (double)fx;
        A.out[n + jj] -= (double)fy;
        A.out[2 * n + jj] -= (double)fz;
    });
}

}  // namespace

// ---- host --------------------------------------------------------------------------
// Site classes: (species, site of its template), numbered species by species.
static int adj_classes(mg_ctx *c, std::vector<int> &cls) {
    std::vector<int> first(c->nspecies + 1, 0);
    for (int s = 0; s < c->nspecies; s++) first[s + 1] = first[s] + c->species[s].natom;
    cls.resize(c->natom);
    for (int a = 0; a < c->natom; a++) cls[a] = first[c->h_site_species[a]] + c->h_site_rel[a];
    return first[c->nspecies];
}

// checks the model, uploads the positions and the site classes and runs the forward
// long-range evaluation whose list, packed clusters, phase tables and S(k) the passes reuse
static mg_status adj_forward(mg_ctx *c, const double *x, const double *y, const double *z, int *nclass) {
    if (!c->have_topology || !c->have_params || !c->have_box)
        return mg_fail(c, MG_ERR_STATE, "set topology, params and box before computing");
    const mg_params &p = c->params;
    if (p.lj_switch || p.respa_split > 0 || p.sf_type != MG_SF_NONE ||
        !(p.charge_type == MG_ELEC_NONE || p.charge_type == MG_ELEC_WOLF ||
          (p.charge_type == MG_ELEC_EWALD && p.ewald_bc == MG_EWALD_BC_TINFOIL)))
        return mg_fail(c, MG_ERR_UNSUPPORTED,
                       "derivatives: LJ switch, distance split, solid-fluid, plain Coulomb and vacuum Ewald "
                       "are not supported");
    std::vector<int> cls;
    *nclass = adj_classes(c, cls);
    if (*nclass > ADJ_MAXC) return mg_fail(c, MG_ERR_UNSUPPORTED, "derivatives: more than 16 site classes");
    cudaSetDevice(c->device);
    const int n = c->natom;
    const size_t nb = sizeof(double) * n;
    if (!mg_ensure(c, c->d_x, 3 * nb) || !mg_ensure(c, c->d_fl, 3 * nb) || !mg_ensure(c, c->d_fs, 3 * nb) ||
        !mg_ensure(c, c->d_adj_class, sizeof(int) * n))
        return MG_ERR_ALLOC;
    cudaStream_t s = c->stream;
    double *dx = (double *)c->d_x.p, *dy = dx + n, *dz = dy + n;
    MG_CUDA(cudaMemcpyAsync(dx, x, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(dy, y, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(dz, z, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(c->d_adj_class.p, cls.data(), sizeof(int) * n, cudaMemcpyHostToDevice, s));
    // the host vector must outlive the copy
    MG_CUDA(cudaStreamSynchronize(s));
    return mg_compute_forces(c, dx, dy, dz, MG_TERMS_LONG, (double *)c->d_fl.p, (double *)c->d_fs.p, nullptr);
}

static ElecK elec_k(const mg_params &p) {
    ElecK K;
    K.kappa = p.kappa;
    K.f1 = p.wolffcon1;
    K.f2 = p.wolffcon2;
    return K;
}

static AdjArgs pair_args(mg_ctx *c, const double *g) {
    const mg_params &p = c->params;
    const int elec = p.charge_type == MG_ELEC_EWALD ? EL_EWALD : (p.charge_type == MG_ELEC_WOLF ? EL_WOLF : 0);
    AdjArgs A;
    A.n = c->natom;
    A.nclass = 0;
    A.meta = (const int *)c->d_meta.p;
    A.pair_start = (const int *)c->d_pair_start.p;
    A.pair_cnt = (const int *)c->d_pair_count.p;
    A.pair_j = (const int *)c->d_pair_j.p;
    A.info = (const int *)c->d_pack_info.p;
    A.cl_atom = (const int *)c->d_cl_atom.p;
    A.pos = c->d_pack_pos.p;
    A.lj = c->d_pack_lj.p;
    A.shift = c->d_pair_shift.p;
    A.site_class = (const int *)c->d_adj_class.p;
    A.g = g;
    A.rc2 = p.rcutoffsq;
    A.rce2 = p.rcutoffelecsq;
    A.rmax2 = elec ? fmax(p.rcutoffsq, p.rcutoffelecsq) : p.rcutoffsq;
    A.lx = c->lx;
    A.ly = c->ly;
    A.lz = c->lz;
    A.coul = p.coulomb_prefactor;
    A.K = elec_k(p);
    A.elec = elec;
    A.mic = c->small_box ? 1 : 0;
    A.rows = nullptr;
    A.out = nullptr;
    return A;
}

static IntraArgs intra_args(mg_ctx *c, const double *g) {
    const mg_params &p = c->params;
    const int n = c->natom;
    IntraArgs B;
    B.n = n;
    B.nmole = c->nmole;
    B.nspecies = c->nspecies;
    B.nclass = 0;
    B.species = (const SpeciesDev *)c->d_species.p;
    B.intra = (const IntraPair *)c->d_intra.p;
    B.sflags = (const int *)c->d_site_flags.p;
    B.site_class = (const int *)c->d_adj_class.p;
    B.x = (const double *)c->d_x.p;
    B.y = B.x + n;
    B.z = B.y + n;
    B.q = (const double *)c->d_site_q.p;
    B.hsig = (const double *)c->d_site_hsig.p;
    B.seps = (const double *)c->d_site_seps.p;
    B.g = g;
    B.lx = c->lx;
    B.ly = c->ly;
    B.lz = c->lz;
    B.rc2 = p.rcutoffsq;
    B.rce2 = p.rcutoffelecsq;
    B.f0 = p.f0;
    B.coul = p.coulomb_prefactor;
    B.K = elec_k(p);
    B.elec = p.charge_type == MG_ELEC_EWALD ? EL_EWALD : (p.charge_type == MG_ELEC_WOLF ? EL_WOLF : 0);
    B.rows = nullptr;
    B.out = nullptr;
    return B;
}

// the parameter passes for g = dL/dF ([3][n], on the device) after adj_forward; waits for
// the stream and writes the per-class sums
static mg_status adj_params_dev(mg_ctx *c, int nclass, const double *g, double *grad_eps, double *grad_sigma,
                                double *grad_q) {
    mg_status st = MG_OK;
    const mg_params &p = c->params;
    const int n = c->natom;
    cudaStream_t s = c->stream;
    const bool ewald = p.charge_type == MG_ELEC_EWALD && c->nrows > 0;
    const unsigned pblocks = (unsigned)(((size_t)c->cl_cap * MG_CL + ADJ_TPB - 1) / ADJ_TPB);
    const unsigned iblocks = (unsigned)((c->nmole + ADJ_TPB - 1) / ADJ_TPB);
    const unsigned fblocks = ewald ? (unsigned)((n + ADJ_TPB - 1) / ADJ_TPB) : 0;
    const size_t ns = ewald ? (size_t)c->nslots : 0;
    const unsigned kblocks = (unsigned)((ns + 255) / 256);
    // scratch in 8-byte units: weights, field, SA, ST, then the block rows
    const size_t o_w = 0, o_f = o_w + (ewald ? (4 + (size_t)nclass) * n : 0);
    const size_t o_sa = o_f + (ewald ? 3 * (size_t)n : 0), o_st = o_sa + 2 * 3 * ns;
    const size_t o_rp = o_st + 2 * (size_t)nclass * ns, o_ri = o_rp + (size_t)pblocks * 3 * nclass;
    const size_t o_rf = o_ri + (size_t)iblocks * 3 * nclass, o_rk = o_rf + (size_t)fblocks * nclass;
    const size_t total = o_rk + (size_t)kblocks * nclass;
    if (!mg_ensure(c, c->d_adj, sizeof(double) * total)) return MG_ERR_ALLOC;
    double *W = (double *)c->d_adj.p;
    const bool fp64 = c->opt.precision == MG_PREC_FP64;
    if (pblocks) {
        AdjArgs A = pair_args(c, g);
        A.nclass = nclass;
        A.rows = W + o_rp;
        if (fp64) k_adj_pair<double><<<pblocks, ADJ_TPB, 0, s>>>(A);
        else k_adj_pair<float><<<pblocks, ADJ_TPB, 0, s>>>(A);
        MG_CUDA(cudaGetLastError());
    }
    if (iblocks) {
        IntraArgs B = intra_args(c, g);
        B.nclass = nclass;
        B.rows = W + o_ri;
        if (fp64) k_adj_intra<double><<<iblocks, ADJ_TPB, 0, s>>>(B);
        else k_adj_intra<float><<<iblocks, ADJ_TPB, 0, s>>>(B);
        MG_CUDA(cudaGetLastError());
    }
    int kb = 0;
    if (ewald) {
        double *w = W + o_w, *field = W + o_f;
        double2 *SA = (double2 *)(W + o_sa), *ST = (double2 *)(W + o_st);
        k_adj_weights<<<(n + 255) / 256, 256, 0, s>>>(n, nclass, (const int *)c->d_adj_class.p,
                                                       (const double *)c->d_site_q.p, g, w);
        MG_CUDA(cudaGetLastError());
        if ((st = mg_ewald_field(c, w + (size_t)(3 + nclass) * n, field))) return st;
        k_adj_field<<<fblocks, ADJ_TPB, 0, s>>>(n, nclass, (const int *)c->d_adj_class.p, g, field, W + o_rf);
        MG_CUDA(cudaGetLastError());
        for (int d = 0; d < 3; d++)
            if ((st = mg_ewald_weighted_sk(c, w + (size_t)d * n, SA + (size_t)d * ns))) return st;
        for (int k = 0; k < nclass; k++)
            if ((st = mg_ewald_weighted_sk(c, w + (size_t)(3 + k) * n, ST + (size_t)k * ns))) return st;
        if ((st = mg_ewald_kgrad(c, SA, ST, nclass, W + o_rk, &kb))) return st;
    }
    std::vector<double> h(total - o_rp);
    if (!h.empty())
        MG_CUDA(cudaMemcpyAsync(h.data(), W + o_rp, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < nclass; k++) grad_eps[k] = grad_sigma[k] = grad_q[k] = 0.0;
    const double *rp = h.data(), *ri = rp + (o_ri - o_rp), *rf = rp + (o_rf - o_rp), *rk = rp + (o_rk - o_rp);
    for (unsigned b = 0; b < pblocks; b++)
        for (int k = 0; k < nclass; k++) {
            grad_eps[k] += rp[(size_t)b * 3 * nclass + k];
            grad_sigma[k] += rp[(size_t)b * 3 * nclass + nclass + k];
            grad_q[k] += rp[(size_t)b * 3 * nclass + 2 * nclass + k];
        }
    for (unsigned b = 0; b < iblocks; b++)
        for (int k = 0; k < nclass; k++) {
            grad_eps[k] += ri[(size_t)b * 3 * nclass + k];
            grad_sigma[k] += ri[(size_t)b * 3 * nclass + nclass + k];
            grad_q[k] += ri[(size_t)b * 3 * nclass + 2 * nclass + k];
        }
    for (unsigned b = 0; b < fblocks; b++)
        for (int k = 0; k < nclass; k++) grad_q[k] += rf[(size_t)b * nclass + k];
    for (int b = 0; b < kb; b++)
        for (int k = 0; k < nclass; k++) grad_q[k] += rk[(size_t)b * nclass + k];
    return MG_OK;
}

extern "C" mg_status mg_adjoint_params(mg_ctx *c, const double *x, const double *y, const double *z,
                                       const double *gx, const double *gy, const double *gz, double *grad_eps,
                                       double *grad_sigma, double *grad_q, int *nclass_out) {
    if (!c || !x || !y || !z || !gx || !gy || !gz || !grad_eps || !grad_sigma || !grad_q) return MG_ERR_INVALID;
    int nclass = 0;
    mg_status st = adj_forward(c, x, y, z, &nclass);
    if (nclass_out) *nclass_out = nclass;
    if (st) return st;
    const int n = c->natom;
    const size_t nb = sizeof(double) * n;
    if (!mg_ensure(c, c->d_adj_g, 6 * nb)) return MG_ERR_ALLOC;
    double *g = (double *)c->d_adj_g.p;
    cudaStream_t s = c->stream;
    MG_CUDA(cudaMemcpyAsync(g, gx, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(g + n, gy, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(g + 2 * n, gz, nb, cudaMemcpyHostToDevice, s));
    return adj_params_dev(c, nclass, g, grad_eps, grad_sigma, grad_q);
}

namespace {
// residual of force matching: g = 2 scale (F - T) and per-block sums of (F - T)^2
__global__ void __launch_bounds__(256) k_fm_residual(int n3, const double *__restrict__ f,
                                                     const double *__restrict__ t, double scale,
                                                     double *__restrict__ g, double *__restrict__ rows) {
    __shared__ double red[256];
    const int i = blockIdx.x * 256 + threadIdx.x;
    double d2 = 0.0;
    if (i < n3) {
        const double d = f[i] - t[i];
        g[i] = 2.0 * scale * d;
        d2 = d * d;
    }
    red[threadIdx.x] = d2;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) rows[blockIdx.x] = red[0];
}
}  // namespace

extern "C" mg_status mg_force_match(mg_ctx *c, const double *x, const double *y, const double *z,
                                    const double *tx, const double *ty, const double *tz, double scale,
                                    double *loss, double *grad_eps, double *grad_sigma, double *grad_q,
                                    int *nclass_out) {
    if (!c || !x || !y || !z || !tx || !ty || !tz || !loss || !grad_eps || !grad_sigma || !grad_q)
        return MG_ERR_INVALID;
    int nclass = 0;
    mg_status st = adj_forward(c, x, y, z, &nclass);
    if (nclass_out) *nclass_out = nclass;
    if (st) return st;
    const int n = c->natom;
    const size_t nb = sizeof(double) * n;
    const unsigned rb = (unsigned)((3 * (size_t)n + 255) / 256);
    if (!mg_ensure(c, c->d_adj_g, 6 * nb + sizeof(double) * rb)) return MG_ERR_ALLOC;
    double *g = (double *)c->d_adj_g.p, *t = g + 3 * n, *rows = t + 3 * n;
    cudaStream_t s = c->stream;
    MG_CUDA(cudaMemcpyAsync(t, tx, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(t + n, ty, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(t + 2 * n, tz, nb, cudaMemcpyHostToDevice, s));
    k_fm_residual<<<rb, 256, 0, s>>>(3 * n, (const double *)c->d_fl.p, t, scale, g, rows);
    MG_CUDA(cudaGetLastError());
    std::vector<double> h(rb);
    MG_CUDA(cudaMemcpyAsync(h.data(), rows, sizeof(double) * rb, cudaMemcpyDeviceToHost, s));
    // adj_params_dev waits for the stream, which completes the copy above
    if ((st = adj_params_dev(c, nclass, g, grad_eps, grad_sigma, grad_q))) return st;
    double sum = 0.0;
    for (unsigned b = 0; b < rb; b++) sum += h[b];
    *loss = scale * sum;
    return MG_OK;
}

extern "C" mg_status mg_adjoint_hvp(mg_ctx *c, const double *x, const double *y, const double *z,
                                    const double *vx, const double *vy, const double *vz, double *hx, double *hy,
                                    double *hz) {
    if (!c || !x || !y || !z || !vx || !vy || !vz || !hx || !hy || !hz) return MG_ERR_INVALID;
    int nclass = 0;
    mg_status st = adj_forward(c, x, y, z, &nclass);
    if (st) return st;
    const mg_params &p = c->params;
    const int n = c->natom;
    const size_t nb = sizeof(double) * n;
    cudaStream_t s = c->stream;
    const bool ewald = p.charge_type == MG_ELEC_EWALD && c->nrows > 0;
    const size_t ns = ewald ? (size_t)c->nslots : 0;
    // scratch in 8-byte units: v, out, weights, SW, coefficients
    const size_t o_v = 0, o_out = 3 * (size_t)n, o_w = o_out + 3 * (size_t)n;
    const size_t o_sw = o_w + (ewald ? 3 * (size_t)n : 0), o_cf = o_sw + 2 * 3 * ns, total = o_cf + 2 * ns;
    if (!mg_ensure(c, c->d_adj, sizeof(double) * total)) return MG_ERR_ALLOC;
    double *W = (double *)c->d_adj.p;
    double *v = W + o_v, *out = W + o_out;
    MG_CUDA(cudaMemcpyAsync(v, vx, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(v + n, vy, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(v + 2 * n, vz, nb, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemsetAsync(out, 0, 3 * nb, s));
    const bool fp64 = c->opt.precision == MG_PREC_FP64;
    const unsigned pblocks = (unsigned)(((size_t)c->cl_cap * MG_CL + ADJ_TPB - 1) / ADJ_TPB);
    const unsigned iblocks = (unsigned)((c->nmole + ADJ_TPB - 1) / ADJ_TPB);
    if (pblocks) {
        AdjArgs A = pair_args(c, v);
        A.out = out;
        if (fp64) k_hvp_pair<double><<<pblocks, ADJ_TPB, 0, s>>>(A);
        else k_hvp_pair<float><<<pblocks, ADJ_TPB, 0, s>>>(A);
        MG_CUDA(cudaGetLastError());
    }
    if (iblocks) {
        IntraArgs B = intra_args(c, v);
        B.out = out;
        if (fp64) k_hvp_intra<double><<<iblocks, ADJ_TPB, 0, s>>>(B);
        else k_hvp_intra<float><<<iblocks, ADJ_TPB, 0, s>>>(B);
        MG_CUDA(cudaGetLastError());
    }
    if (ewald) {
        double *w = W + o_w;
        double2 *SW = (double2 *)(W + o_sw);
        k_adj_weights<<<(n + 255) / 256, 256, 0, s>>>(n, 0, nullptr, (const double *)c->d_site_q.p, v, w);
        MG_CUDA(cudaGetLastError());
        for (int d = 0; d < 3; d++)
            if ((st = mg_ewald_weighted_sk(c, w + (size_t)d * n, SW + (size_t)d * ns))) return st;
        if ((st = mg_ewald_jvp(c, v, SW, W + o_cf, out))) return st;
    }
    MG_CUDA(cudaMemcpyAsync(hx, out, nb, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(hy, out + n, nb, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(hz, out + 2 * n, nb, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    // H v = -(dF/dr) v
    for (int a = 0; a < n; a++) {
        hx[a] = -hx[a];
        hy[a] = -hy[a];
        hz[a] = -hz[a];
    }
    return MG_OK;
}
