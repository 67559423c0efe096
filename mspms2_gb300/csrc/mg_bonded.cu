// mg_bonded.cu - per-molecule kernels: intra-molecular nonbonded corrections
// (src/frclong.c:222-982), bonded terms (src/frcshort.c:20-91 with src/bndfrc.c,
// src/aglfrc.c, src/dihfrc.c, src/impfrc.c), plain Coulomb between molecules with a
// centre-of-mass cutoff (src/elecfrc.c:138-225) and the vacuum-boundary dipole term of
// the Ewald sum (src/frclong.c:1065-1126).
//
// One thread owns one molecule and walks its template lists in the reference's order,
// so forces go to that molecule's sites without atomics and every sum has a fixed order.
// Site-pair vectors are formed in FP64 from the unwrapped positions and the arithmetic
// then runs in R (FP32 in the mixed path, FP64 in the FP64 path).
#include <math.h>

#include "mg_internal.cuh"

namespace {

template <typename R>
struct M;
template <>
struct M<float> {
    __device__ static float sqrt_(float x) { return sqrtf(x); }
    __device__ static float erfc_(float x) { return erfcf(x); }
    __device__ static float erf_(float x) { return erff(x); }
    __device__ static float exp_(float x) { return expf(x); }
    __device__ static float log_(float x) { return logf(x); }
    __device__ static float acos_(float x) { return acosf(x); }
    __device__ static float atan2_(float y, float x) { return atan2f(y, x); }
    __device__ static float cos_(float x) { return cosf(x); }
    __device__ static float sin_(float x) { return sinf(x); }
};
template <>
struct M<double> {
    __device__ static double sqrt_(double x) { return sqrt(x); }
    __device__ static double erfc_(double x) { return erfc(x); }
    __device__ static double erf_(double x) { return erf(x); }
    __device__ static double exp_(double x) { return exp(x); }
    __device__ static double log_(double x) { return log(x); }
    __device__ static double acos_(double x) { return acos(x); }
    __device__ static double atan2_(double y, double x) { return atan2(y, x); }
    __device__ static double cos_(double x) { return cos(x); }
    __device__ static double sin_(double x) { return sin(x); }
};

struct MolArgs {
    int nspecies, nmole, n;
    const SpeciesDev *species;
    const IntraPair *intra;
    const BondedTerm *bonded;
    const double *x, *y, *z;
    const double *q, *hsig, *seps, *aw;
    const int *sflags;
    double *f;  // [3][n]
    mg_params p;
    double lx, ly, lz;
    double *rows;
    int row0;
    unsigned *flags;
    const double *dipole;  // total dipole (vacuum force pass)
    double *com;           // [3][nmole]   (plain Coulomb)
    double *ex;            // [3][n]
};

__device__ __forceinline__ int species_of(const MolArgs &A, int mol) {
    int s = 0;
    while (s + 1 < A.nspecies && mol >= A.species[s + 1].first_mole) s++;
    return s;
}

__device__ __forceinline__ double mic(double d, double L) { return d - L * rint(d / L); }

// LJ between two sites with the reference's mixing and optional switch (src/ljfrc.c)
template <typename R>
__device__ __forceinline__ void lj_pair(const mg_params &p, R r2, R sig, R eps, R &u, R &f) {
    R rinv2 = (R)1 / r2;
    R s6 = sig * sig * rinv2;
    s6 = s6 * s6 * s6;
    R s12 = s6 * s6;
    u = (R)4 * eps * (s12 - s6);
    f = (R)24 * eps * ((R)2 * s12 - s6) * rinv2;
    if (p.lj_switch && !(r2 < (R)p.rcutonsq)) {
        R d = (R)p.rcutoffsq - r2;
        R swd = (R)p.roff2_minus_ron2_cube;
        R sw = d * d * ((R)p.rcutoffsq + (R)2 * r2 - (R)3 * (R)p.rcutonsq) / swd;
        f = f * sw - u * (R)12 * d * ((R)p.rcutonsq - r2) / swd;
        u *= sw;
    }
}

template <typename R>
__device__ __forceinline__ void ewald_real(const mg_params &p, R r2, R qq, R &u, R &f) {
    R r = M<R>::sqrt_(r2);
    R bare = (R)p.coulomb_prefactor * qq / r;
    R kr = (R)p.kappa * r;
    u = bare * M<R>::erfc_(kr);
    f = (u + bare * (R)2 * kr * M<R>::exp_(-kr * kr) * (R)0.5641895835477563) / r2;
}

template <typename R>
__device__ __forceinline__ void wolf_real(const mg_params &p, R r2, R qq, R &u, R &f) {
    R r = M<R>::sqrt_(r2);
    R kr = (R)p.kappa * r;
    R ec = M<R>::erfc_(kr);
    u = (R)p.coulomb_prefactor * qq * (ec / r + (R)p.wolfvcon1 + (R)p.wolfvcon2 * (r - (R)p.rcutoffelec));
    f = (R)p.coulomb_prefactor * (qq / r) * (ec / r2 + (R)p.wolffcon1 * M<R>::exp_(-kr * kr) / r + (R)p.wolffcon2);
}

__device__ __forceinline__ void addf(double *f, int n, int i, int j, double fx, double fy, double fz) {
    f[i] += fx; f[n + i] += fy; f[2 * n + i] += fz;
    f[j] -= fx; f[n + j] -= fy; f[2 * n + j] -= fz;
}

// energies: 0 uvdw, 1 ureal, 2 uexcl, 3 ucoul, 4 virial
template <typename R>
__global__ void k_intra(MolArgs A) {
    double eng[5] = {0, 0, 0, 0, 0};
    int mol = blockIdx.x * blockDim.x + threadIdx.x;
    if (mol < A.nmole) {
        const mg_params &p = A.p;
        const SpeciesDev S = A.species[species_of(A, mol)];
        const int base = S.first_site + (mol - S.first_mole) * S.natom;
        const int n = A.n;
        const int ct = p.charge_type;
        int same = 1;  // isSameMole of src/frclong.c:224 (starts true, see the oracle notes)
        for (int k = 0; k < S.nintra; k++) {
            const IntraPair ip = A.intra[S.intra_off + k];
            const int ii = base + ip.m, jj = base + ip.n;
            const int gi = A.sflags[ii], gj = A.sflags[jj];
            const bool full = ((gi | gj) & MG_SITE_DEAD) != 0;
            const bool ljok = (gi & (MG_SITE_LJ | MG_SITE_DEAD)) && (gj & (MG_SITE_LJ | MG_SITE_DEAD));
            double dx = A.x[ii] - A.x[jj], dy = A.y[ii] - A.y[jj], dz = A.z[ii] - A.z[jj];
            const bool straddle = fabs(dx) > A.lx * 0.5 || fabs(dy) > A.ly * 0.5 || fabs(dz) > A.lz * 0.5;
            const R sig = (R)(A.hsig[ii] + A.hsig[jj]);
            const R eps = (R)(A.seps[ii] * A.seps[jj]);
            const R qq = (R)(A.q[ii] * A.q[jj]);
            R u, f;
            if (ip.kind == 0) {  // 1-2 / 1-3 end pair
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
                // LJ of the minimum image; the unwrapped vector is kept through an int
                // (src/frclong.c:223, :278-312)
                double ox = (double)(int)dx, oy = (double)(int)dy, oz = (double)(int)dz;
                double mx = mic(dx, A.lx), my = mic(dy, A.ly), mz = mic(dz, A.lz);
                R r2 = (R)(mx * mx + my * my + mz * mz);
                if (ljok && r2 < (R)p.rcutoffsq) {
                    R eps_un = (R)(A.seps[ii] * A.seps[jj]);
                    lj_pair<R>(p, r2, sig, eps_un, u, f);
                    eng[0] += u;
                    eng[4] += (double)(f * r2);
                    addf(A.f, n, ii, jj, (double)f * mx, (double)f * my, (double)f * mz);
                }
                dx = ox; dy = oy; dz = oz;
            } else if (ip.kind != 0) {
                R r2 = (R)(dx * dx + dy * dy + dz * dz);
                if (r2 < (R)p.rcutoffsq) {
                    R e2 = ip.kind == 1 ? (R)p.f0 * eps : eps;
                    lj_pair<R>(p, r2, sig, e2, u, f);
                    eng[0] += u;
                    eng[4] += (double)(f * r2);
                    addf(A.f, n, ii, jj, (double)f * dx, (double)f * dy, (double)f * dz);
                }
            }
            if (ct == MG_ELEC_NONE) continue;
            if (ip.kind == 0 && same && (ct == MG_ELEC_EWALD || ct == MG_ELEC_WOLF)) {
                // Not straddling: the exclusion and the real-space term use the same vector
                // (the minimum image changes nothing), and their forces, each ~C q q / r^2,
                // nearly cancel. They are combined through erf = 1 - erfc before rounding;
                // the two energies are still accumulated separately.
                R r2 = (R)(dx * dx + dy * dy + dz * dz);
                if (!(r2 < (R)p.rcutoffelecsq)) continue;
                R r = M<R>::sqrt_(r2);
                R kr = (R)p.kappa * r;
                R bare = (R)p.coulomb_prefactor * qq / r;
                R ex = M<R>::exp_(-kr * kr), ef = M<R>::erf_(kr), ec = M<R>::erfc_(kr);
                R fsum;
                if (ct == MG_ELEC_EWALD) {
                    eng[1] += bare * ec;
                    fsum = bare * ((R)2 * kr * ex * (R)0.5641895835477563 - ef) / r2;
                } else {
                    eng[1] += (R)p.coulomb_prefactor * qq *
                              (ec / r + (R)p.wolfvcon1 + (R)p.wolfvcon2 * (r - (R)p.rcutoffelec));
                    fsum = bare * (-ef / r2 + (R)p.wolffcon1 * ex / r + (R)p.wolffcon2);
                    eng[4] += (double)(fsum * r2);
                }
                eng[2] += bare;
                addf(A.f, n, ii, jj, (double)fsum * dx, (double)fsum * dy, (double)fsum * dz);
                continue;
            }
            if (ip.kind == 0) {
                if (ct != MG_ELEC_EWALD && ct != MG_ELEC_WOLF) continue;
                R r2 = (R)(dx * dx + dy * dy + dz * dz);
                if (r2 < (R)p.rcutoffelecsq) {  // exclusion, no minimum image (src/elecfrc.c:35-46)
                    R r = M<R>::sqrt_(r2);
                    u = (R)p.coulomb_prefactor * qq / r;
                    f = -u / r2;
                    eng[2] += u;
                    if (ct == MG_ELEC_WOLF) eng[4] += (double)(f * r2);
                    addf(A.f, n, ii, jj, (double)f * dx, (double)f * dy, (double)f * dz);
                }
            }
            double mx = mic(dx, A.lx), my = mic(dy, A.ly), mz = mic(dz, A.lz);
            R r2 = (R)(mx * mx + my * my + mz * mz);
            if (!(r2 < (R)p.rcutoffelecsq)) continue;
            if (ct == MG_ELEC_EWALD) {
                ewald_real<R>(p, r2, qq, u, f);
                eng[1] += u;
            } else if (ct == MG_ELEC_WOLF) {
                wolf_real<R>(p, r2, qq, u, f);
                eng[1] += u;
                eng[4] += (double)(f * r2);
            } else {
                if (ip.kind == 0) continue;
                R r = M<R>::sqrt_(r2);
                u = (R)p.coulomb_prefactor * qq / r;
                f = u / r2;
                eng[3] += u;
                eng[4] += (double)(f * r2);
            }
            addf(A.f, n, ii, jj, (double)f * mx, (double)f * my, (double)f * mz);
        }
    }
    const int ids[5] = {E_UVDW, E_UREAL, E_UEXCL, E_UCOUL, E_VIR};
    mg_block_row<5>(eng, ids, A.rows, A.row0 + blockIdx.x);
}

// ---- bonded ---------------------------------------------------------------------------
template <typename R>
__device__ void tors_apply(R temp, const R v[9], const R (&rjk)[3], const R (&rij)[3], const R (&rjl)[3],
                           const R (&rik)[3], const R (&rkl)[3], R (&F)[4][3]) {
    const R aa1 = v[0], bb1 = v[1], cc1 = v[2], aa2 = v[3], bb2 = v[4], cc2 = v[5], t1 = v[6], t2 = v[7], t3 = v[8];
    const R rxjk = rjk[0], ryjk = rjk[1], rzjk = rjk[2], rxij = rij[0], ryij = rij[1], rzij = rij[2];
    const R rxjl = rjl[0], ryjl = rjl[1], rzjl = rjl[2], rxik = rik[0], ryik = rik[1], rzik = rik[2];
    const R rxkl = rkl[0], rykl = rkl[1], rzkl = rkl[2];
    R f = temp / (t2 * t1 * t1);
    F[0][0] = f * ((bb2 * rzjk - cc2 * ryjk) * t1 - t3 / t1 * (bb1 * rzjk - cc1 * ryjk));
    F[0][1] = f * ((-aa2 * rzjk + cc2 * rxjk) * t1 - t3 / t1 * (-aa1 * rzjk + cc1 * rxjk));
    F[0][2] = f * ((aa2 * ryjk - bb2 * rxjk) * t1 - t3 / t1 * (aa1 * ryjk - bb1 * rxjk));
    f = temp / (t1 * t1 * t2 * t2);
    F[1][0] = f * ((bb2 * rzik - bb1 * rzkl - cc2 * ryik + cc1 * rykl) * t1 * t2 -
                   t3 * (t2 / t1 * (bb1 * rzik - cc1 * ryik) + t1 / t2 * (-bb2 * rzkl + cc2 * rykl)));
    F[1][1] = f * ((-aa2 * rzik + aa1 * rzkl + cc2 * rxik - cc1 * rxkl) * t1 * t2 -
                   t3 * (t2 / t1 * (-aa1 * rzik + cc1 * rxik) + t1 / t2 * (aa2 * rzkl - cc2 * rxkl)));
    F[1][2] = f * ((aa2 * ryik - aa1 * rykl - bb2 * rxik + bb1 * rxkl) * t1 * t2 -
                   t3 * (t2 / t1 * (aa1 * ryik - bb1 * rxik) + t1 / t2 * (-aa2 * rykl + bb2 * rxkl)));
    F[2][0] = f * ((-bb2 * rzij + bb1 * rzjl + cc2 * ryij - cc1 * ryjl) * t1 * t2 -
                   t3 * (t2 / t1 * (-bb1 * rzij + cc1 * ryij) + t1 / t2 * (bb2 * rzjl - cc2 * ryjl)));
    F[2][1] = f * ((aa2 * rzij - aa1 * rzjl - cc2 * rxij + cc1 * rxjl) * t1 * t2 -
                   t3 * (t2 / t1 * (aa1 * rzij - cc1 * rxij) + t1 / t2 * (-aa2 * rzjl + cc2 * rxjl)));
    F[2][2] = f * ((-aa2 * ryij + aa1 * ryjl + bb2 * rxij - bb1 * rxjl) * t1 * t2 -
                   t3 * (t2 / t1 * (-aa1 * ryij + bb1 * rxij) + t1 / t2 * (aa2 * ryjl - bb2 * rxjl)));
    f = temp / (t1 * t2 * t2);
    F[3][0] = f * ((-bb1 * rzjk + cc1 * ryjk) * t2 - t3 / t2 * (-bb2 * rzjk + cc2 * ryjk));
    F[3][1] = f * ((aa1 * rzjk - cc1 * rxjk) * t2 - t3 / t2 * (aa2 * rzjk - cc2 * rxjk));
    F[3][2] = f * ((-aa1 * ryjk + bb1 * rxjk) * t2 - t3 / t2 * (-aa2 * ryjk + bb2 * rxjk));
}

// energies: 0 ubond, 1 uangle, 2 udih, 3 uimp, 4 virial_intra
template <typename R>
__global__ void k_bonded(MolArgs A) {
    double eng[5] = {0, 0, 0, 0, 0};
    int mol = blockIdx.x * blockDim.x + threadIdx.x;
    if (mol < A.nmole) {
        const SpeciesDev S = A.species[species_of(A, mol)];
        const int base = S.first_site + (mol - S.first_mole) * S.natom;
        const int n = A.n;
        double *fx = A.f, *fy = A.f + n, *fz = A.f + 2 * n;
        const R pi = (R)3.141592653589793;
        for (int k = 0; k < S.nbonded; k++) {
            const BondedTerm T = A.bonded[S.bonded_off + k];
            const int a0 = base + T.idx[0], a1 = base + T.idx[1], a2 = base + T.idx[2], a3 = base + T.idx[3];
            if (T.kind == 0) {
                // the bond length and its stretch r - r0 are formed in FP64: near equilibrium
                // the stretch is a few ulps of r in FP32
                const double dxd = A.x[a0] - A.x[a1], dyd = A.y[a0] - A.y[a1], dzd = A.z[a0] - A.z[a1];
                const double r2d = dxd * dxd + dyd * dyd + dzd * dzd, rd = sqrt(r2d);
                R rx = (R)dxd, ry = (R)dyd, rz = (R)dzd;
                R r2 = (R)r2d, r = (R)rd, u, f;
                if (T.type == MG_BOND_HARMONIC) {
                    R dr = (R)(rd - T.p[1]);
                    u = (R)0.5 * (R)T.p[0] * dr * dr;
                    f = -(R)T.p[0] * dr / r;
                } else if (T.type == MG_BOND_MORSE) {
                    R dr = (R)(rd - T.p[1]);
                    R ex = M<R>::exp_(-(R)T.p[2] * dr);
                    R om = (R)1 - ex;
                    u = (R)T.p[0] * om * om;
                    f = -(R)2 * (R)T.p[0] * (R)T.p[2] * om * ex / r;
                } else if (T.type == MG_BOND_FENE) {
                    R rm2 = (R)T.p[1] * (R)T.p[1];
                    u = (R)T.p[0] * rm2 * M<R>::log_((R)1 - r2 / rm2);
                    f = -(R)2 * (R)T.p[0] * rm2 / (rm2 - r2);
                } else {
                    continue;
                }
                eng[0] += u;
                eng[4] += (double)(f * r2);
                fx[a0] += f * rx; fy[a0] += f * ry; fz[a0] += f * rz;
                fx[a1] -= f * rx; fy[a1] -= f * ry; fz[a1] -= f * rz;
            } else if (T.kind == 1) {
                if (T.type == MG_ANGLE_HARMONIC) {
                    R xab = (R)(A.x[a0] - A.x[a1]), yab = (R)(A.y[a0] - A.y[a1]), zab = (R)(A.z[a0] - A.z[a1]);
                    R xcb = (R)(A.x[a2] - A.x[a1]), ycb = (R)(A.y[a2] - A.y[a1]), zcb = (R)(A.z[a2] - A.z[a1]);
                    R irab = (R)1 / M<R>::sqrt_(xab * xab + yab * yab + zab * zab);
                    xab *= irab; yab *= irab; zab *= irab;
                    R ircb = (R)1 / M<R>::sqrt_(xcb * xcb + ycb * ycb + zcb * zcb);
                    xcb *= ircb; ycb *= ircb; zcb *= ircb;
                    R c = xab * xcb + yab * ycb + zab * zcb;
                    R th = M<R>::acos_(c);
                    R sn = fmax((R)1.0e-8, M<R>::sqrt_((R)1 - c * c));
                    R dth = th - (R)T.p[1];
                    eng[1] += (double)((R)0.5 * (R)T.p[0] * dth * dth);
                    R gm = (R)T.p[0] * dth / sn;
                    R fxa = gm * (xcb - xab * c) * irab, fya = gm * (ycb - yab * c) * irab, fza = gm * (zcb - zab * c) * irab;
                    R fxc = gm * (xab - xcb * c) * ircb, fyc = gm * (yab - ycb * c) * ircb, fzc = gm * (zab - zcb * c) * ircb;
                    fx[a0] += fxa; fy[a0] += fya; fz[a0] += fza;
                    fx[a1] -= (double)fxa + (double)fxc; fy[a1] -= (double)fya + (double)fyc; fz[a1] -= (double)fza + (double)fzc;
                    fx[a2] += fxc; fy[a2] += fyc; fz[a2] += fzc;
                } else if (T.type == MG_ANGLE_TR_WATER) {
                    const double w13x = A.x[a0] - A.x[a2], w13y = A.y[a0] - A.y[a2], w13z = A.z[a0] - A.z[a2];
                    const double w12x = A.x[a0] - A.x[a1], w12y = A.y[a0] - A.y[a1], w12z = A.z[a0] - A.z[a1];
                    const double w23x = A.x[a1] - A.x[a2], w23y = A.y[a1] - A.y[a2], w23z = A.z[a1] - A.z[a2];
                    R v13x = (R)w13x, v13y = (R)w13y, v13z = (R)w13z;
                    R v12x = (R)w12x, v12y = (R)w12y, v12z = (R)w12z;
                    R v23x = (R)w23x, v23y = (R)w23y, v23z = (R)w23z;
                    // lengths and stretches in FP64 (see the bond case)
                    const double l13 = sqrt(w13x * w13x + w13y * w13y + w13z * w13z);
                    const double l12 = sqrt(w12x * w12x + w12y * w12y + w12z * w12z);
                    const double l23 = sqrt(w23x * w23x + w23y * w23y + w23z * w23z);
                    R r13 = (R)l13, r12 = (R)l12, r23 = (R)l23;
                    R d3 = (R)(l13 - T.p[3]), d1 = (R)(l12 - T.p[4]), d2 = (R)(l23 - T.p[4]);
                    R kt = (R)T.p[0], krt = (R)T.p[1], krr = (R)T.p[2];
                    eng[1] += (double)((R)0.5 * kt * d3 * d3 + krt * d3 * (d1 + d2) + krr * d1 * d2);
                    R t1 = -kt * d3 / r13, t21 = -krt * d3 / r12, t22 = -krt * (d1 + d2) / r13, t3 = -krr * d2 / r12;
                    R fxa = t1 * v13x + t21 * v12x + t22 * v13x + t3 * v12x;
                    R fya = t1 * v13y + t21 * v12y + t22 * v13y + t3 * v12y;
                    R fza = t1 * v13z + t21 * v12z + t22 * v13z + t3 * v12z;
                    fx[a0] += fxa; fy[a0] += fya; fz[a0] += fza;
                    t21 = -krt * d3 / r23;
                    t22 = krt * d3 / r12;
                    R t31 = -krr * d1 / r23, t32 = krr * d2 / r12;
                    fx[a1] += t21 * v23x + t22 * v12x + t31 * v23x + t32 * v12x;
                    fy[a1] += t21 * v23y + t22 * v12y + t31 * v23y + t32 * v12y;
                    fz[a1] += t21 * v23z + t22 * v12z + t31 * v23z + t32 * v12z;
                    t1 = kt * d3 / r13;
                    t21 = krt * d3 / r23;
                    t22 = krt * (d1 + d2) / r13;
                    t3 = krr * d1 / r23;
                    R fxc = t1 * v13x + t21 * v23x + t22 * v13x + t3 * v23x;
                    R fyc = t1 * v13y + t21 * v23y + t22 * v13y + t3 * v23y;
                    R fzc = t1 * v13z + t21 * v23z + t22 * v13z + t3 * v23z;
                    fx[a2] += fxc; fy[a2] += fyc; fz[a2] += fzc;
                    eng[4] += (double)(fxa * v12x + fya * v12y + fza * v12z) - (double)(fxc * v23x + fyc * v23y + fzc * v23z);
                }
            } else if (T.kind == 2 && T.type == MG_DIH_OPLS) {
                R xab = (R)(A.x[a0] - A.x[a1]), yab = (R)(A.y[a0] - A.y[a1]), zab = (R)(A.z[a0] - A.z[a1]);
                R xbc = (R)(A.x[a1] - A.x[a2]), ybc = (R)(A.y[a1] - A.y[a2]), zbc = (R)(A.z[a1] - A.z[a2]);
                R xcd = (R)(A.x[a2] - A.x[a3]), ycd = (R)(A.y[a2] - A.y[a3]), zcd = (R)(A.z[a2] - A.z[a3]);
                R rrbc = (R)1 / M<R>::sqrt_(xbc * xbc + ybc * ybc + zbc * zbc);
                R pbx = yab * zbc - zab * ybc, pby = zab * xbc - xab * zbc, pbz = xab * ybc - yab * xbc;
                R rpb1 = (R)1 / M<R>::sqrt_(pbx * pbx + pby * pby + pbz * pbz), rpb2 = rpb1 * rpb1;
                R pcx = ybc * zcd - zbc * ycd, pcy = zbc * xcd - xbc * zcd, pcz = xbc * ycd - ybc * xcd;
                R rpc1 = (R)1 / M<R>::sqrt_(pcx * pcx + pcy * pcy + pcz * pcz), rpc2 = rpc1 * rpc1;
                R pbpc = pbx * pcx + pby * pcy + pbz * pcz;
                R c = pbpc * rpb1 * rpc1;
                R sn = (xbc * (pcy * pbz - pcz * pby) + ybc * (pbx * pcz - pbz * pcx) + zbc * (pcx * pby - pcy * pbx)) *
                       (rpb1 * rpc1 * rrbc);
                R th = M<R>::atan2_(sn, c);
                sn = copysign(fmax((R)1.0e-8, fabs(sn)), sn);
                R rsn = (R)1 / sn;
                R v1 = (R)T.p[0], v2 = (R)T.p[1], v3 = (R)T.p[2], v4 = (R)T.p[3];
                eng[2] += (double)(v1 + (R)0.5 * (v2 * ((R)1 + M<R>::cos_(th)) + v3 * ((R)1 - M<R>::cos_((R)2 * th)) +
                                                  v4 * ((R)1 + M<R>::cos_((R)3 * th))));
                R dop = -(R)0.5 * (v2 * M<R>::sin_(th) - (R)2 * v3 * M<R>::sin_((R)2 * th) + (R)3 * v4 * M<R>::sin_((R)3 * th));
                R gm = dop * rpb1 * rpc1 * rsn;
                R fax = gm * ((-pcy * zbc + pcz * ybc) - pbpc * rpb2 * (-pby * zbc + pbz * ybc));
                R fay = gm * ((pcx * zbc - pcz * xbc) - pbpc * rpb2 * (pbx * zbc - pbz * xbc));
                R faz = gm * ((-pcx * ybc + pcy * xbc) - pbpc * rpb2 * (-pbx * ybc + pby * xbc));
                R fcx = gm * ((-pcy * zab + pcz * yab) - pbpc * rpb2 * (-pby * zab + pbz * yab));
                R fcy = gm * ((pcx * zab - pcz * xab) - pbpc * rpb2 * (pbx * zab - pbz * xab));
                R fcz = gm * ((-pcx * yab + pcy * xab) - pbpc * rpb2 * (-pbx * yab + pby * xab));
                R fbx = gm * ((-pby * zcd + pbz * ycd) - pbpc * rpc2 * (-pcy * zcd + pcz * ycd));
                R fby = gm * ((pbx * zcd - pbz * xcd) - pbpc * rpc2 * (pcx * zcd - pcz * xcd));
                R fbz = gm * ((-pbx * ycd + pby * xcd) - pbpc * rpc2 * (-pcx * ycd + pcy * xcd));
                R fdx = gm * ((-pby * zbc + pbz * ybc) - pbpc * rpc2 * (-pcy * zbc + pcz * ybc));
                R fdy = gm * ((pbx * zbc - pbz * xbc) - pbpc * rpc2 * (pcx * zbc - pcz * xbc));
                R fdz = gm * ((-pbx * ybc + pby * xbc) - pbpc * rpc2 * (-pcx * ybc + pcy * xbc));
                fx[a0] += fax; fy[a0] += fay; fz[a0] += faz;
                fx[a1] += (-fax - fcx + fbx); fy[a1] += (-fay - fcy + fby); fz[a1] += (-faz - fcz + fbz);
                fx[a2] += fcx - fbx - fdx; fy[a2] += fcy - fby - fdy; fz[a2] += fcz - fbz - fdz;
                fx[a3] += fdx; fy[a3] += fdy; fz[a3] += fdz;
            } else if ((T.kind == 2 && T.type == MG_DIH_CHARMM) || (T.kind == 3 && T.type == MG_IMP_CHARMM)) {
                R kk = (R)T.p[0];
                if (T.kind == 2 && !(fabs(T.p[0]) >= 1.0e-8)) continue;
                if (T.kind == 3 && !(fabs(T.p[0]) >= 1e-5)) continue;
                R rjk[3] = {(R)(A.x[a2] - A.x[a1]), (R)(A.y[a2] - A.y[a1]), (R)(A.z[a2] - A.z[a1])};
                R rij[3] = {(R)(A.x[a0] - A.x[a1]), (R)(A.y[a0] - A.y[a1]), (R)(A.z[a0] - A.z[a1])};
                R rjl[3] = {(R)(A.x[a3] - A.x[a1]), (R)(A.y[a3] - A.y[a1]), (R)(A.z[a3] - A.z[a1])};
                R rik[3] = {(R)(A.x[a0] - A.x[a2]), (R)(A.y[a0] - A.y[a2]), (R)(A.z[a0] - A.z[a2])};
                R rkl[3] = {(R)(A.x[a3] - A.x[a2]), (R)(A.y[a3] - A.y[a2]), (R)(A.z[a3] - A.z[a2])};
                R v[9];
                v[0] = rjk[1] * rij[2] - rjk[2] * rij[1];
                v[1] = rjk[2] * rij[0] - rjk[0] * rij[2];
                v[2] = rjk[0] * rij[1] - rij[0] * rjk[1];
                v[3] = rjl[1] * rjk[2] - rjl[2] * rjk[1];
                v[4] = rjl[2] * rjk[0] - rjl[0] * rjk[2];
                v[5] = rjl[0] * rjk[1] - rjk[0] * rjl[1];
                v[6] = M<R>::sqrt_(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
                v[7] = M<R>::sqrt_(v[3] * v[3] + v[4] * v[4] + v[5] * v[5]);
                v[8] = v[0] * v[3] + v[1] * v[4] + v[2] * v[5];
                R al = v[8] / (v[6] * v[7]);
                R phi = (R)180 - (M<R>::acos_(al) * (R)180 / pi);
                R temp, u;
                if (T.kind == 2) {
                    R np = (R)T.p[1], d0 = (R)T.p[2];
                    u = kk * ((R)1 + M<R>::cos_((np * phi - d0) / (R)180 * pi));
                    if (fabs(M<R>::sin_(phi * pi / (R)180)) <= (R)1e-10)
                        temp = -np * np * kk * M<R>::cos_((np * phi - d0) * pi / (R)180) / al;
                    else
                        temp = np * kk * M<R>::sin_((np * phi - d0) * pi / (R)180) / M<R>::sin_(phi * pi / (R)180);
                    eng[2] += u;
                } else {
                    R w0 = (R)T.p[1];
                    u = kk * (phi - w0) * (phi - w0) * ((pi / (R)180) * (pi / (R)180));
                    R a = M<R>::acos_(al) * (R)180 / pi;
                    if ((fabs(w0) <= (R)1e-5 && (fabs(a) <= (R)1e-20 || fabs(a - (R)180) <= (R)1e-20)) ||
                        (fabs(w0 - (R)180) <= (R)1e-5 && (fabs(a - (R)180) <= (R)1e-20 || fabs(a) <= (R)1e-20))) {
                        atomicOr(A.flags, MG_FLAG_IMPROPER_DEGENERATE);
                        continue;
                    }
                    temp = -(R)2 * kk * (phi - w0) * pi / (R)180 / M<R>::sin_(phi * pi / (R)180);
                    eng[3] += u;
                }
                R F[4][3];
                tors_apply<R>(temp, v, rjk, rij, rjl, rik, rkl, F);
                const int at[4] = {a0, a1, a2, a3};
                for (int r = 0; r < 4; r++) {
                    fx[at[r]] += F[r][0];
                    fy[at[r]] += F[r][1];
                    fz[at[r]] += F[r][2];
                }
            }
        }
    }
    const int ids[5] = {E_UBOND, E_UANGLE, E_UDIH, E_UIMP, E_VIR_INTRA};
    mg_block_row<5>(eng, ids, A.rows, A.row0 + blockIdx.x);
}

// ---- centres of mass (src/misc.c:72-103) ----------------------------------------------
__global__ void k_com(MolArgs A, int wrap) {
    int mol = blockIdx.x * blockDim.x + threadIdx.x;
    double dip[3] = {0, 0, 0};
    if (mol < A.nmole) {
        const SpeciesDev S = A.species[species_of(A, mol)];
        const int base = S.first_site + (mol - S.first_mole) * S.natom;
        double c[3] = {0, 0, 0};
        for (int a = 0; a < S.natom; a++) {
            c[0] += A.x[base + a] * A.aw[base + a];
            c[1] += A.y[base + a] * A.aw[base + a];
            c[2] += A.z[base + a] * A.aw[base + a];
        }
        c[0] /= S.mw; c[1] /= S.mw; c[2] /= S.mw;
        double w[3] = {c[0], c[1], c[2]};
        if (wrap) {
            w[0] -= A.lx * rint(w[0] / A.lx);
            w[1] -= A.ly * rint(w[1] / A.ly);
            w[2] -= A.lz * rint(w[2] / A.lz);
        }
        const int n = A.n;
        for (int a = 0; a < S.natom; a++) {
            double ex = A.x[base + a] - c[0], ey = A.y[base + a] - c[1], ez = A.z[base + a] - c[2];
            if (A.ex) {
                A.ex[base + a] = ex;
                A.ex[n + base + a] = ey;
                A.ex[2 * n + base + a] = ez;
            }
            double q = A.q[base + a];
            dip[0] += q * (ex + w[0]);
            dip[1] += q * (ey + w[1]);
            dip[2] += q * (ez + w[2]);
        }
        if (A.com) {
            A.com[mol] = c[0];
            A.com[A.nmole + mol] = c[1];
            A.com[2 * A.nmole + mol] = c[2];
        }
    }
    if (A.rows) {
        const int ids[3] = {E_DIPX, E_DIPY, E_DIPZ};
        mg_block_row<3>(dip, ids, A.rows, A.row0 + blockIdx.x);
    }
}

__global__ void k_vacuum_force(MolArgs A, int nrows_dip, const double *__restrict__ dip_rows) {
    // total dipole in fixed order (every thread sums the same rows)
    __shared__ double m[3];
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int r = 0; r < nrows_dip; r++) t += dip_rows[(size_t)r * E_NCOMP + E_DIPX + threadIdx.x];
        m[threadIdx.x] = t;
    }
    __syncthreads();
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A.n) return;
    double fij = -2.0 * A.p.twopi_over_3v * A.q[a] * A.p.coulomb_prefactor;
    A.f[a] += fij * m[0];
    A.f[A.n + a] += fij * m[1];
    A.f[2 * A.n + a] += fij * m[2];
}

// plain Coulomb between molecules whose centres of mass are closer than rcutoffelec;
// full molecule loop per thread (each pair seen from both sides, energies halved)
template <typename R>
__global__ void k_coulomb_mole(MolArgs A) {
    double eng[2] = {0, 0};
    int mi = blockIdx.x * blockDim.x + threadIdx.x;
    if (mi < A.nmole) {
        const int n = A.n, M_ = A.nmole;
        const SpeciesDev Si = A.species[species_of(A, mi)];
        const int bi = Si.first_site + (mi - Si.first_mole) * Si.natom;
        const double cx = A.com[mi], cy = A.com[M_ + mi], cz = A.com[2 * M_ + mi];
        for (int mj = 0; mj < M_; mj++) {
            if (mj == mi) continue;
            double rx = mic(cx - A.com[mj], A.lx), ry = mic(cy - A.com[M_ + mj], A.ly), rz = mic(cz - A.com[2 * M_ + mj], A.lz);
            if (!(rx * rx + ry * ry + rz * rz < A.p.rcutoffelecsq)) continue;
            const SpeciesDev Sj = A.species[species_of(A, mj)];
            const int bj = Sj.first_site + (mj - Sj.first_mole) * Sj.natom;
            for (int a = 0; a < Si.natom; a++) {
                int ii = bi + a;
                if (A.sflags[ii] & MG_SITE_DEAD) continue;
                double fx = 0, fy = 0, fz = 0;
                for (int b = 0; b < Sj.natom; b++) {
                    int jj = bj + b;
                    if (A.sflags[jj] & MG_SITE_DEAD) continue;
                    R dx = (R)(A.ex[ii] + rx - A.ex[jj]), dy = (R)(A.ex[n + ii] + ry - A.ex[n + jj]),
                      dz = (R)(A.ex[2 * n + ii] + rz - A.ex[2 * n + jj]);
                    R r2 = dx * dx + dy * dy + dz * dz;
                    R u = (R)A.p.coulomb_prefactor * (R)(A.q[ii] * A.q[jj]) / M<R>::sqrt_(r2);
                    R f = u / r2;
                    eng[0] += 0.5 * (double)u;
                    eng[1] += 0.5 * (double)u;
                    fx += f * dx; fy += f * dy; fz += f * dz;
                }
                A.f[ii] += fx;
                A.f[n + ii] += fy;
                A.f[2 * n + ii] += fz;
            }
        }
    }
    const int ids[2] = {E_UCOUL, E_VIR};
    mg_block_row<2>(eng, ids, A.rows, A.row0 + blockIdx.x);
}

MolArgs mol_args(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *f) {
    MolArgs A;
    A.nspecies = c->nspecies;
    A.nmole = c->nmole;
    A.n = c->natom;
    A.species = (SpeciesDev *)c->d_species.p;
    A.intra = (IntraPair *)c->d_intra.p;
    A.bonded = (BondedTerm *)c->d_bonded.p;
    A.x = dx;
    A.y = dy;
    A.z = dz;
    A.q = (double *)c->d_site_q.p;
    A.hsig = (double *)c->d_site_hsig.p;
    A.seps = (double *)c->d_site_seps.p;
    A.aw = (double *)c->d_site_aw.p;
    A.sflags = (int *)c->d_site_flags.p;
    A.f = f;
    A.p = c->params;
    A.lx = c->lx;
    A.ly = c->ly;
    A.lz = c->lz;
    A.rows = (double *)c->d_epart.p;
    A.row0 = 0;
    A.flags = (unsigned *)c->d_flags.p;
    A.dipole = nullptr;
    A.com = nullptr;
    A.ex = nullptr;
    return A;
}

}  // namespace

#define MOL_THREADS 128

mg_status mg_launch_intra(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *fl) {
    MolArgs A = mol_args(c, dx, dy, dz, fl);
    unsigned blocks = (unsigned)((c->nmole + MOL_THREADS - 1) / MOL_THREADS);
    A.row0 = mg_reserve_rows(c, blocks);
    if (A.row0 < 0) return mg_fail(c, MG_ERR_ALLOC, "energy partial rows exhausted");
    if (c->opt.precision == MG_PREC_FP64)
        k_intra<double><<<blocks, MOL_THREADS, 0, c->stream>>>(A);
    else
        k_intra<float><<<blocks, MOL_THREADS, 0, c->stream>>>(A);
    MG_CUDA(cudaGetLastError());
    c->launches += 1;
    return MG_OK;
}

mg_status mg_launch_bonded(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *fs) {
    MolArgs A = mol_args(c, dx, dy, dz, fs);
    unsigned blocks = (unsigned)((c->nmole + MOL_THREADS - 1) / MOL_THREADS);
    A.row0 = mg_reserve_rows(c, blocks);
    if (A.row0 < 0) return mg_fail(c, MG_ERR_ALLOC, "energy partial rows exhausted");
    if (c->opt.precision == MG_PREC_FP64)
        k_bonded<double><<<blocks, MOL_THREADS, 0, c->stream>>>(A);
    else
        k_bonded<float><<<blocks, MOL_THREADS, 0, c->stream>>>(A);
    MG_CUDA(cudaGetLastError());
    c->launches += 1;
    return MG_OK;
}

mg_status mg_launch_vacuum(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *fl) {
    MolArgs A = mol_args(c, dx, dy, dz, fl);
    unsigned blocks = (unsigned)((c->nmole + MOL_THREADS - 1) / MOL_THREADS);
    A.row0 = mg_reserve_rows(c, blocks);
    if (A.row0 < 0) return mg_fail(c, MG_ERR_ALLOC, "energy partial rows exhausted");
    k_com<<<blocks, MOL_THREADS, 0, c->stream>>>(A, 1);
    const double *dip_rows = (double *)c->d_epart.p + (size_t)A.row0 * E_NCOMP;
    k_vacuum_force<<<(c->natom + 255) / 256, 256, 0, c->stream>>>(A, (int)blocks, dip_rows);
    MG_CUDA(cudaGetLastError());
    c->launches += 2;
    return MG_OK;
}

mg_status mg_launch_coulomb_mole(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *fl) {
    MolArgs A = mol_args(c, dx, dy, dz, fl);
    if (!mg_ensure(c, c->d_spart, sizeof(double) * 3 * ((size_t)c->nmole + c->natom))) return MG_ERR_ALLOC;
    A.com = (double *)c->d_spart.p;
    A.ex = A.com + 3 * (size_t)c->nmole;
    A.rows = nullptr;
    unsigned blocks = (unsigned)((c->nmole + MOL_THREADS - 1) / MOL_THREADS);
    k_com<<<blocks, MOL_THREADS, 0, c->stream>>>(A, 0);
    A.rows = (double *)c->d_epart.p;
    A.row0 = mg_reserve_rows(c, blocks);
    if (A.row0 < 0) return mg_fail(c, MG_ERR_ALLOC, "energy partial rows exhausted");
    if (c->opt.precision == MG_PREC_FP64)
        k_coulomb_mole<double><<<blocks, MOL_THREADS, 0, c->stream>>>(A);
    else
        k_coulomb_mole<float><<<blocks, MOL_THREADS, 0, c->stream>>>(A);
    MG_CUDA(cudaGetLastError());
    c->launches += 2;
    return MG_OK;
}
