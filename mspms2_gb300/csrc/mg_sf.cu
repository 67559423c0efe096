// mg_sf.cu - solid-fluid potentials (src/frclong.c:1145-1209), one thread per site,
// applied to sites of ghost type NONE only.
//
//  Tasos   tricubic Hermite interpolation on an 8-value-per-node grid
//          (mylibtasos/forces.f90:6-173, cubicinterpolation.f90:9-116,
//          cubicauxiliary.f90:76-573). Positions go to A by sigma_base
//          (src/sffrc.c:1322-1337); only z is periodic (mylibtasos/pbc.f90:80-84). The
//          reference pairs the Dxyz value of corner (i,j,k+1) with the basis of corner
//          (i+1,j+1,k) and vice versa in both the value and the gradient; with
//          MG_COMPAT_TASOS_DXYZ the same pairing is used here. PE is negated when below
//          1.5*minPE (forces.f90:167-171) under MG_COMPAT_TASOS_PE_FLIP. Tables are FP32
//          in the mixed path (8 values x 4 B = one 32-byte sector per node), FP64 otherwise.
//  hypergeo  smooth tubes by the 11-term hypergeometric series (src/sffrc.c:1092-1209);
//          x and y forces only; the energy keeps the last tube under
//          MG_COMPAT_HYPERGEO_LAST (src/sffrc.c:1201).
//  explicit  LJ against listed solid atoms with the minimum image, cutoff and optional
//          switch (src/sffrc.c:1213-1314).
//  my-interp 32-term polynomial per cube in absolute A, J/mol (src/sffrc.c:951-1089);
//          evaluated in FP64 in both paths because its terms cancel strongly.
#include <math.h>

#include "mg_internal.cuh"

namespace {

struct SfArgs {
    int n, ntasos, nmy, ntube, nsolid;
    const double *x, *y, *z;
    const int *sflags, *interp;
    const double *hsig, *seps;  // 0.5*sigma and sqrt(eps) per site
    const TasosDev *tasos;
    const MyInterpDev *my;
    const double *tubes, *solid;
    double solid_sigma, solid_epsilon, c3pt;
    mg_params p;
    double lx, ly, lz;
    double *f;
    double *rows;
    int row0;
    unsigned *flags;
};

template <typename R>
struct Herm {
    R v0, v1, d0, d1, v0p, v1p, d0p, d1p;
};

template <typename R>
__device__ __forceinline__ Herm<R> herm(R t, R h) {
    Herm<R> b;
    R u = (R)1 - t;
    b.v1 = -(t * t * ((R)2 * t - (R)3));
    b.v0 = t * t * ((R)2 * t - (R)3) + (R)1;
    b.d0 = h * (t * (t - (R)1) * (t - (R)1));
    b.d1 = -h * (u * (u - (R)1) * (u - (R)1));
    b.v1p = -((R)6 * t * (t - (R)1)) / h;
    b.v0p = ((R)6 * t * (t - (R)1)) / h;
    b.d0p = t * ((R)3 * t - (R)4) + (R)1;
    b.d1p = t * ((R)3 * t - (R)2);
    return b;
}

template <typename R>
__device__ bool tasos_eval(const TasosDev &g, unsigned compat, double X, double Y, double Z, double &pe, double fo[3]) {
    double zp = Z - floor(Z / g.cuc) * g.cuc;
    int I1 = (int)floor(X / g.hx + 1), J1 = (int)floor(Y / g.hy + 1), K1 = (int)floor(zp / g.hz + 1);
    if (I1 < 1 || J1 < 1 || K1 < 1 || I1 > g.nx - 1 || J1 > g.ny - 1 || K1 > g.nz - 1) return false;
    const R tx = (R)((X - (I1 - 1) * g.hx) / g.hx), ty = (R)((Y - (J1 - 1) * g.hy) / g.hy),
            tz = (R)((zp - (K1 - 1) * g.hz) / g.hz);
    const Herm<R> bx = herm<R>(tx, (R)g.hx), by = herm<R>(ty, (R)g.hy), bz = herm<R>(tz, (R)g.hz);
    const R *vals = (const R *)g.values;
    const int i0 = I1 - 1, j0 = J1 - 1, k0 = K1 - 1;
    const bool swap = (compat & MG_COMPAT_TASOS_DXYZ) != 0;
    R val = 0, gx = 0, gy = 0, gz = 0;
#pragma unroll
    for (int c = 0; c < 8; c++) {
        const int ci = c & 1, cj = (c >> 1) & 1, ck = (c >> 2) & 1;
        const R *rec = vals + 8 * (((size_t)(k0 + ck) * g.ny + (j0 + cj)) * g.nx + (i0 + ci));
        const R wx = ci ? bx.v1 : bx.v0, dx = ci ? bx.d1 : bx.d0, wxp = ci ? bx.v1p : bx.v0p, dxp = ci ? bx.d1p : bx.d0p;
        const R wy = cj ? by.v1 : by.v0, dy = cj ? by.d1 : by.d0, wyp = cj ? by.v1p : by.v0p, dyp = cj ? by.d1p : by.d0p;
        const R wz = ck ? bz.v1 : bz.v0, dz = ck ? bz.d1 : bz.d0, wzp = ck ? bz.v1p : bz.v0p, dzp = ck ? bz.d1p : bz.d0p;
        const bool sw = swap && (c == 3 || c == 4);
        const int ti = sw ? 1 - ci : ci, tj = sw ? 1 - cj : cj, tk = sw ? 1 - ck : ck;
        const R txd = ti ? bx.d1 : bx.d0, tyd = tj ? by.d1 : by.d0, tzd = tk ? bz.d1 : bz.d0;
        const R txdp = ti ? bx.d1p : bx.d0p, tydp = tj ? by.d1p : by.d0p, tzdp = tk ? bz.d1p : bz.d0p;
        const R F = rec[0], Dx = rec[1], Dy = rec[2], Dz = rec[3], Dxy = rec[4], Dxz = rec[5], Dyz = rec[6], Dxyz = rec[7];
        val += F * wx * wy * wz + Dx * dx * wy * wz + Dy * wx * dy * wz + Dz * wx * wy * dz + Dxy * dx * dy * wz +
               Dxz * dx * wy * dz + Dyz * wx * dy * dz + Dxyz * txd * tyd * tzd;
        gx += F * wxp * wy * wz + Dx * dxp * wy * wz + Dy * wxp * dy * wz + Dz * wxp * wy * dz + Dxy * dxp * dy * wz +
              Dxz * dxp * wy * dz + Dyz * wxp * dy * dz + Dxyz * txdp * tyd * tzd;
        gy += F * wx * wyp * wz + Dx * dx * wyp * wz + Dy * wx * dyp * wz + Dz * wx * wyp * dz + Dxy * dx * dyp * wz +
              Dxz * dx * wyp * dz + Dyz * wx * dyp * dz + Dxyz * txd * tydp * tzd;
        gz += F * wx * wy * wzp + Dx * dx * wy * wzp + Dy * wx * dy * wzp + Dz * wx * wy * dzp + Dxy * dx * dy * wzp +
              Dxz * dx * wy * dzp + Dyz * wx * dy * dzp + Dxyz * txd * tyd * tzdp;
    }
    fo[0] = -(double)gx;
    fo[1] = -(double)gy;
    fo[2] = -(double)gz;
    pe = ((compat & MG_COMPAT_TASOS_PE_FLIP) && (double)val < 1.5 * g.min_pe) ? -(double)val : (double)val;
    return true;
}

template <typename R>
__device__ __forceinline__ void hyper_series(R a, R zz, R rr, R &sv, R &sf) {
    R zn = 1, an1 = 1;
    sv = 1;
    sf = 0;
#pragma unroll
    for (int i = 0; i <= 10; i++) {
        R an = (a + (R)i) * (a + (R)i) / (((R)1 + (R)i) * ((R)1 + (R)i));
        an1 = an1 * an;
        zn *= zz;
        sv = sv + an1 * zn;
        sf = sf - (R)2 * ((R)i + (R)1) * an1 * zn / rr;
    }
}

template <typename R>
__global__ void k_sf(SfArgs A) {
    double e[1] = {0.0};
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < A.n && (A.sflags[a] & 4)) {
        const mg_params &p = A.p;
        const double x = A.x[a], y = A.y[a], z = A.z[a];
        if (p.sf_type == MG_SF_TASOS) {
            const int t = A.interp[a];
            double pe, fo[3];
            if (t < 1 || t > A.ntasos || A.tasos[t - 1].values == nullptr ||
                !tasos_eval<R>(A.tasos[t - 1], p.compat, x * p.sigma_base, y * p.sigma_base, z * p.sigma_base, pe, fo)) {
                atomicOr(A.flags, MG_FLAG_OUT_OF_GRID);
            } else {
                e[0] = pe / p.epsilon_base;
                const double s = p.sigma_base / p.epsilon_base;
                A.f[a] += fo[0] * s;
                A.f[A.n + a] += fo[1] * s;
                A.f[2 * A.n + a] += fo[2] * s;
            }
        } else if (p.sf_type == MG_SF_HYPERGEO) {
            const R sig = (R)(A.hsig[a] + 0.5 * A.solid_sigma);
            const R eps = (R)(A.seps[a] * sqrt(A.solid_epsilon));
            R usum = 0, ulast = 0;
            double fx = 0, fy = 0;
            for (int t = 0; t < A.ntube; t++) {
                double dxd = x - A.tubes[3 * t], dyd = y - A.tubes[3 * t + 1];
                dxd -= A.lx * rint(dxd / A.lx);
                dyd -= A.ly * rint(dyd / A.ly);
                const R rx = (R)dxd, ry = (R)dyd;
                const R rsq = rx * rx + ry * ry, r = sqrt(rsq);
                const R Rt = (R)A.tubes[3 * t + 2], Rsq = Rt * Rt;
                R hr, hfr, ha, hfa, u, f;
                if (r < Rt) {
                    const R ljc = (R)A.c3pt * eps * sig * sig;
                    const R k = sig * Rt / (Rsq - rsq), zf = rsq / Rsq;
                    hyper_series<R>((R)-4.5, zf, r, hr, hfr);
                    const R k2 = k * k, k4 = k2 * k2, k10 = k4 * k4 * k2;
                    const R rep1 = (R)0.65625 * k10, rep2 = -hfr + hr * ((R)20 * r / (Rsq - rsq));
                    hyper_series<R>((R)-1.5, zf, r, ha, hfa);
                    const R att1 = -k4, att2 = -hfa + ha * ((R)8 * r / (Rsq - rsq));
                    u = ljc * (rep1 * hr + att1 * ha);
                    f = -ljc * (rep1 * rep2 + att1 * att2);
                } else {
                    const R ljc = (R)A.c3pt * eps * sig * sig * Rt;
                    const R k = sig * r / (rsq - Rsq), zf = Rsq / rsq;
                    hyper_series<R>((R)-4.5, zf, r, hr, hfr);
                    const R k2 = k * k, k4 = k2 * k2, k10 = k4 * k4 * k2;
                    const R rep1 = (R)0.65625 * k10, rep2 = hfr / r + hr * (-(R)20 / (rsq - Rsq) + (R)9 / rsq);
                    hyper_series<R>((R)-1.5, zf, r, ha, hfa);
                    const R att1 = -k4, att2 = hfa / r + ha * (-(R)8 / (rsq - Rsq) + (R)3 / rsq);
                    u = ljc * (rep1 * hr + att1 * ha) / r;
                    f = -ljc * (rep1 * rep2 + att1 * att2);
                }
                fx += (double)(f * rx / r);
                fy += (double)(f * ry / r);
                usum += u;
                ulast = u;
            }
            A.f[a] += fx;
            A.f[A.n + a] += fy;
            e[0] = (double)((p.compat & MG_COMPAT_HYPERGEO_LAST) ? ulast : usum);
        } else if (p.sf_type == MG_SF_ATOM_EXPLICIT) {
            const R sig = (R)(A.hsig[a] + 0.5 * A.solid_sigma);
            const R eps = (R)(A.seps[a] * sqrt(A.solid_epsilon));
            const R rc2 = (R)p.rcutoffsq, ron2 = (R)p.rcutonsq, swd = (R)p.roff2_minus_ron2_cube;
            double usum = 0, fx = 0, fy = 0, fz = 0;
            for (int j = 0; j < A.nsolid; j++) {
                double dxd = x - A.solid[3 * j], dyd = y - A.solid[3 * j + 1], dzd = z - A.solid[3 * j + 2];
                dxd -= A.lx * rint(dxd / A.lx);
                dyd -= A.ly * rint(dyd / A.ly);
                dzd -= A.lz * rint(dzd / A.lz);
                const R rx = (R)dxd, ry = (R)dyd, rz = (R)dzd;
                const R r2 = rx * rx + ry * ry + rz * rz;
                if (!(r2 < rc2)) continue;
                const R s2 = sig * sig / r2, s6 = s2 * s2 * s2, s12 = s6 * s6, d12 = s12 - s6;
                const R ut = eps * d12;
                R f = (R)24 * eps * (d12 + s12) / r2;
                R uu = ut;
                if (p.lj_switch && !(r2 < ron2)) {
                    const R d = rc2 - r2;
                    const R sw = d * d * (rc2 + (R)2 * r2 - (R)3 * ron2) / swd;
                    f = f * sw - (R)4 * ut * (R)12 * d * (ron2 - r2) / swd;
                    uu = ut * sw;
                }
                usum += (double)uu;
                fx += (double)(f * rx);
                fy += (double)(f * ry);
                fz += (double)(f * rz);
            }
            A.f[a] += fx;
            A.f[A.n + a] += fy;
            A.f[2 * A.n + a] += fz;
            e[0] = usum * 4.0;
        } else if (p.sf_type == MG_SF_MY_INTERP) {
            const int t = A.interp[a];
            bool ok = t >= 0 && t < A.nmy && A.my[t].coeff != nullptr;
            if (ok) {
                const MyInterpDev &g = A.my[t];
                double fxx = x * p.sigma_base, fyy = y * p.sigma_base, fzz = z * p.sigma_base;
                int ax = (int)((fxx - g.xmin) / g.itvl_x), ay = (int)((fyy - g.ymin) / g.itvl_y);
                fzz = fzz - g.zmax * rint(fzz / g.zmax);
                if (fzz < 0) fzz = g.zmax + fzz;
                int az = (int)(fzz / g.itvl_z);
                long long ncube = (long long)g.ncx * g.ncy * g.ncz;
                long long cube = (long long)ax * g.ncy * g.ncz + (long long)ay * g.ncz + az;
                ok = ax >= 0 && ay >= 0 && az >= 0 && cube < ncube;
                if (ok) {
                    const double X = fxx, Y = fyy, Zc = fzz;
                    const double x2 = X * X, x3 = x2 * X, y2 = Y * Y, y3 = y2 * Y, z2 = Zc * Zc, z3 = z2 * Zc;
                    const double v[32] = {1.0, X, Y, Zc, x2, X * Y, X * Zc, y2, Y * Zc, z2, x3, x2 * Y, X * y2, x2 * Zc,
                                          X * z2, y3, y2 * Zc, Y * z2, z3, X * Y * Zc, x3 * Y, x2 * y2, X * y3, x3 * Zc,
                                          x2 * z2, X * z3, y3 * Zc, y2 * z2, Y * z3, x2 * Y * Zc, X * y2 * Zc, X * Y * z2};
                    double out[4];
                    for (int qd = 0; qd < 4; qd++) {
                        const double *cf = g.coeff + (size_t)qd * 32 * ncube;
                        double acc = cf[cube] * v[0];
                        for (int k = 1; k < 32; k++) acc = acc + cf[(size_t)k * ncube + cube] * v[k];
                        out[qd] = acc;
                    }
                    const double rr = 0.120272219;  // R_RGAS (src/defs.h:201): J/mol -> K
                    e[0] = out[0] * rr / p.epsilon_base;
                    const double s = rr * p.sigma_base / p.epsilon_base;
                    A.f[a] += out[1] * s;
                    A.f[A.n + a] += out[2] * s;
                    A.f[2 * A.n + a] += out[3] * s;
                }
            }
            if (!ok) atomicOr(A.flags, MG_FLAG_OUT_OF_GRID);
        }
    }
    const int ids[1] = {E_USFLJ};
    mg_block_row<1>(e, ids, A.rows, A.row0 + blockIdx.x);
}

}  // namespace

mg_status mg_launch_sf(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *fl) {
    SfArgs A;
    A.n = c->natom;
    A.ntasos = (int)c->tasos.size();
    A.nmy = (int)c->myinterp.size();
    A.ntube = c->ntube;
    A.nsolid = c->nsolid;
    A.x = dx;
    A.y = dy;
    A.z = dz;
    A.sflags = (int *)c->d_site_flags.p;
    A.interp = (int *)c->d_site_interp.p;
    A.hsig = (double *)c->d_site_hsig.p;
    A.seps = (double *)c->d_site_seps.p;
    A.tasos = (TasosDev *)c->d_tasos.p;
    A.my = (MyInterpDev *)c->d_myinterp.p;
    A.tubes = (double *)c->d_tubes.p;
    A.solid = (double *)c->d_solid.p;
    A.solid_sigma = c->solid_sigma;
    A.solid_epsilon = c->solid_epsilon;
    A.c3pt = c->const_3pisq_theta;
    A.p = c->params;
    A.lx = c->lx;
    A.ly = c->ly;
    A.lz = c->lz;
    A.f = fl;
    A.rows = (double *)c->d_epart.p;
    A.flags = (unsigned *)c->d_flags.p;
    if (c->params.sf_type == MG_SF_HYPERGEO && c->ntube == 0) return MG_OK;
    unsigned blocks = (unsigned)((c->natom + 127) / 128);
    A.row0 = mg_reserve_rows(c, blocks);
    if (A.row0 < 0) return mg_fail(c, MG_ERR_ALLOC, "energy partial rows exhausted");
    if (c->opt.precision == MG_PREC_FP64)
        k_sf<double><<<blocks, 128, 0, c->stream>>>(A);
    else
        k_sf<float><<<blocks, 128, 0, c->stream>>>(A);
    MG_CUDA(cudaGetLastError());
    c->launches += 1;
    return MG_OK;
}
