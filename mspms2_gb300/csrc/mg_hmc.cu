// mg_hmc.cu - batched Hybrid Monte Carlo of Lennard-Jones replicas in one persistent
// launch: the reference's hmc() canonical move (src/hmc.c:23-40) with md_move()
// (src/dispmd.c:12-103) over vver() steps (src/md.c:22-85), for many independent boxes.
//
// One thread block runs whole replicas, taking the next one (largest first) from a work
// counter. Per move it
//   1. draws Maxwell-Boltzmann velocities sqrt(T)/sqrt(m) N(0,1) per component from the
//      counter-based generator of include/mg_philox.h, removes the total momentum and,
//      like the reference (velinit, src/initvars.c:151-229), optionally rescales them
//      to exactly T; K0 = sum m v^2 / 2;
//   2. evaluates forces and energy U0 (frclong) and runs nstep velocity-Verlet steps
//      (a half kick, then per step: drift, forces, a full kick, the last one a half kick);
//   3. takes dH = (dU + dK + dUshift) / T, the reference's sum with its +dUshift
//      (src/dispmd.c:48-50), and accepts when dH <= 0 or a uniform draw < exp(-dH),
//      otherwise restores the positions.
// FP64 positions and velocities live in global memory (L2-resident for the whole batch);
// FP32 copies of the positions, wrapped into the box, and a cell list live in shared
// memory. Pair forces are FP32; energies, kinetic energies and dH are FP64. Cells of at
// least rcutoff with three or more per axis give a 27-cell scan; smaller boxes use all
// pairs with the minimum image. Each cell's atoms are kept in index order, so every sum
// has a fixed order and a run is reproducible.
#include <math.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "../../include/mg_philox.h"
#include "mg_internal.cuh"

#define HMC_TPB 512
#ifndef HMC_UNROLL
#define HMC_UNROLL 4     // j candidates per step of the force loop
#endif
constexpr int kHmcUnroll = HMC_UNROLL;
#ifndef HMC_MINB
#define HMC_MINB 1       // resident blocks per SM the replica kernels are compiled for
#endif

namespace {

struct HmcArgs {
    int nrep;
    const int *order, *natom, *offset;
    const double *box;
    double *x, *y, *z, *vx, *vy, *vz, *ox, *oy, *oz;
    int *counter;
    int nmoves, move0, nstep;
    double eps, sig2, rc, rc2, shift_pair, mass, treq, dt;
    int rescale, nconstraint;
    uint32_t key0, key1;
    int *accepted;
    double *dh_log, *energy;
    int nmax, ncmax;
};

// fixed-order block sum of three doubles (thread 0 gets the result)
__device__ __forceinline__ void block_sum3(double &a, double &b, double &c) {
    __shared__ double red[3][HMC_TPB];
    red[0][threadIdx.x] = a;
    red[1][threadIdx.x] = b;
    red[2][threadIdx.x] = c;
    __syncthreads();
    for (int o = HMC_TPB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            red[0][threadIdx.x] += red[0][threadIdx.x + o];
            red[1][threadIdx.x] += red[1][threadIdx.x + o];
            red[2][threadIdx.x] += red[2][threadIdx.x + o];
        }
        __syncthreads();
    }
    a = red[0][0];
    b = red[1][0];
    c = red[2][0];
    __syncthreads();
}

struct Smem {
    float4 *pos;  // [nmax] wrapped FP32 positions sorted by cell (index order inside a cell); w = atom index
    int *list;    // [nmax] cell of each atom while the cells are built
    int *start;   // [ncmax + 1] first sorted slot of each cell
    int *cnt;     // [ncmax]
};

__device__ __forceinline__ int cell_of(float v, float inv_w, int nc) {
    int c = (int)(v * inv_w);
    return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

// coordinate w wrapped into [0, L) in FP32: the image count in FP32, the subtraction as one
// FP64 FMA (FP64 runs at a small fraction of the FP32 rate on this part); a count off by
// one at the boundary leaves a rounding outside [0, L), folded back here
__device__ __forceinline__ float wrapf(double w, double L, float Lf, float iLf) {
    const float nf = floorf((float)w * iLf);
    float t = (float)fma(-(double)nf, L, w);
    if (t >= Lf) t -= Lf;
    if (t < 0.f) t = 0.f;
    return t;
}

// Wrapped FP32 positions of the replica into shared memory, sorted by cell with index order
// inside each cell (fixed order for every sum); without cells (nc == 0), in index order.
__device__ __forceinline__ void load_positions(const HmcArgs &A, const Smem &S, int off, int n, double L, int nc) {
    const float Lf = (float)L, iLf = (float)(1.0 / L), inv_w = nc > 0 ? (float)(nc / L) : 0.f;
    if (nc == 0) {
        for (int i = threadIdx.x; i < n; i += HMC_TPB)
            S.pos[i] = make_float4(wrapf(A.x[off + i], L, Lf, iLf), wrapf(A.y[off + i], L, Lf, iLf),
                                   wrapf(A.z[off + i], L, Lf, iLf), __int_as_float(i));
        __syncthreads();
        return;
    }
    const int ncell = nc * nc * nc;
    for (int c = threadIdx.x; c < ncell; c += HMC_TPB) S.cnt[c] = 0;
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += HMC_TPB) {
        const float px = wrapf(A.x[off + i], L, Lf, iLf), py = wrapf(A.y[off + i], L, Lf, iLf);
        const float pz = wrapf(A.z[off + i], L, Lf, iLf);
        const int cell = (cell_of(pz, inv_w, nc) * nc + cell_of(py, inv_w, nc)) * nc + cell_of(px, inv_w, nc);
        S.list[i] = cell;
        atomicAdd(&S.cnt[cell], 1);
    }
    __syncthreads();
    // exclusive scan of the counts by warp 0 (lanes own consecutive chunks)
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x, chunk = (ncell + 31) / 32;
        const int b = lane * chunk, e = min(ncell, b + chunk);
        int sum = 0;
        for (int c = b; c < e; c++) sum += S.cnt[c];
        int incl = sum;
        for (int o = 1; o < 32; o <<= 1) {
            int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        int run = incl - sum;
        for (int c = b; c < e; c++) {
            S.start[c] = run;
            run += S.cnt[c];
            S.cnt[c] = 0;  // reused as the fill counter
        }
        if (lane == 31) S.start[ncell] = incl;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += HMC_TPB) {
        const int cell = S.list[i];
        const int k = S.start[cell] + atomicAdd(&S.cnt[cell], 1);
        S.pos[k] = make_float4(wrapf(A.x[off + i], L, Lf, iLf), wrapf(A.y[off + i], L, Lf, iLf),
                               wrapf(A.z[off + i], L, Lf, iLf), __int_as_float(i));
    }
    __syncthreads();
    for (int c = threadIdx.x; c < ncell; c += HMC_TPB) {  // index order inside each cell
        const int b = S.start[c], e = S.start[c + 1];
        for (int k = b + 1; k < e; k++) {
            const float4 v = S.pos[k];
            const int vi = __float_as_int(v.w);
            int m = k - 1;
            while (m >= b && __float_as_int(S.pos[m].w) > vi) {
                S.pos[m + 1] = S.pos[m];
                m--;
            }
            S.pos[m + 1] = v;
        }
    }
    // chunks of 32 slots per (y, z) row of cells, as a prefix over the rows (S.cnt[0..nc^2])
    if (threadIdx.x == 0) {
        int t = 0;
        for (int r = 0; r < nc * nc; r++) {
            S.cnt[r] = t;
            t += (S.start[r * nc + nc] - S.start[r * nc] + 31) / 32;
        }
        S.cnt[nc * nc] = t;
    }
    __syncthreads();
}

// LJ force and pair energy (each pair is seen from both sides)
__device__ __forceinline__ void lj_add(float dx, float dy, float dz, float sig2, float eps, float rc2, float &fx,
                                       float &fy, float &fz, float &e, int &np) {
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (!(r2 < rc2)) return;
    const float ir2 = __frcp_rn(r2);
    const float s2 = sig2 * ir2, s6 = s2 * s2 * s2, s12 = s6 * s6;
    e += 4.f * eps * (s12 - s6);
    const float f = 24.f * eps * (2.f * s12 - s6) * ir2;
    fx += f * dx;
    fy += f * dy;
    fz += f * dz;
    np += 1;
}

// Forces on every atom of the replica, warp-cooperatively: a warp takes up to 32 atoms of
// one (y, z) row of cells (consecutive sorted slots, one atom per lane) and all lanes walk
// the same j-atoms, those of the 9 neighbour rows over the chunk's x cells +-1, so that
// each j load is a broadcast and the lanes do not diverge. y and z images come from the
// row offsets; x takes the minimum image per pair (correct for any chunk, L >= 2 rc). j
// order is fixed (rows, then cells in x, then slots), so every sum has a fixed order.
// fn(i, fx, fy, fz, e, np) receives each atom's force, LJ energy and pair count.
template <typename F>
__device__ __forceinline__ void replica_forces(const HmcArgs &A, const Smem &S, int n, double L, int nc, F &&fn) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int NW = HMC_TPB / 32;
    const float Lf = (float)L, iL = (float)(1.0 / L), sig2 = (float)A.sig2, eps = (float)A.eps;
    const float rc2 = (float)A.rc2;
    if (nc == 0) {  // all pairs, minimum image
        for (int base = wid * 32; base < n; base += NW * 32) {
            const int k = base + lane;
            const bool act = k < n;
            const float4 pi = S.pos[act ? k : base];
            float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
            int np = 0;
            for (int j = 0; j < n; j++) {
                const float4 pj = S.pos[j];
                float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                dx -= Lf * rintf(dx * iL);
                dy -= Lf * rintf(dy * iL);
                dz -= Lf * rintf(dz * iL);
                if (j != k) lj_add(dx, dy, dz, sig2, eps, rc2, fx, fy, fz, e, np);
            }
            if (act) fn(__float_as_int(pi.w), fx, fy, fz, e, np);
        }
        return;
    }
    const float inv_w = (float)(nc / L);
    const int nchunk = S.cnt[nc * nc];
    int r = 0;
    for (int t = wid; t < nchunk; t += NW) {  // chunks dealt to the warps in order
        while (S.cnt[r + 1] <= t) r++;
        const int y = r % nc, z = r / nc;
        const int re = S.start[r * nc + nc];
        {
            const int base = S.start[r * nc] + 32 * (t - S.cnt[r]);
            const int k = base + lane, klast = min(base + 32, re) - 1;
            const bool act = k < re;
            const float4 pi = S.pos[act ? k : base];
            const int xlo = cell_of(S.pos[base].x, inv_w, nc), xhi = cell_of(S.pos[klast].x, inv_w, nc);
            const int m = min(xhi - xlo + 3, nc);      // cells of the x range
            const int xs = (xlo - 1 + nc) % nc;       // its first cell
            const int run1 = min(m, nc - xs);         // cells before the wrap
            float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
            int np = 0;
            for (int dz = -1; dz <= 1; dz++) {
                int uz = z + dz;
                const float sz = uz < 0 ? -Lf : (uz >= nc ? Lf : 0.f);
                uz = (uz + nc) % nc;
                for (int dy = -1; dy <= 1; dy++) {
                    int uy = y + dy;
                    const float sy = uy < 0 ? -Lf : (uy >= nc ? Lf : 0.f);
                    uy = (uy + nc) % nc;
                    const int c0 = (uz * nc + uy) * nc;
                    for (int run = 0; run < 2; run++) {
                        const int ca = run == 0 ? c0 + xs : c0, cb = run == 0 ? c0 + xs + run1 : c0 + (m - run1);
                        const int jb = S.start[ca], je = S.start[cb];
#pragma unroll kHmcUnroll
                        for (int j = jb; j < je; j++) {
                            const float4 pj = S.pos[j];
                            float dx = pi.x - pj.x;
                            dx -= Lf * rintf(dx * iL);
                            const float dyy = pi.y - (pj.y + sy), dzz = pi.z - (pj.z + sz);
                            if (j != k) lj_add(dx, dyy, dzz, sig2, eps, rc2, fx, fy, fz, e, np);
                        }
                    }
                }
            }
            if (act) fn(__float_as_int(pi.w), fx, fy, fz, e, np);
        }
    }
}

// forces at the shared-memory positions, v += f h / m; optional energy (U, pair count)
__device__ __forceinline__ void force_kick(const HmcArgs &A, const Smem &S, int off, int n, double L, int nc, double h,
                                           double *u_out, double *np_out) {
    double esum = 0.0, nsum = 0.0, unused = 0.0;
    const double hm = h / A.mass;
    replica_forces(A, S, n, L, nc, [&](int i, float fx, float fy, float fz, float e, int np) {
        A.vx[off + i] += hm * (double)fx;
        A.vy[off + i] += hm * (double)fy;
        A.vz[off + i] += hm * (double)fz;
        esum += (double)e;
        nsum += (double)np;
    });
    if (u_out) {
        block_sum3(esum, nsum, unused);
        *u_out = 0.5 * esum;
        *np_out = 0.5 * nsum;
    }
}

__global__ void __launch_bounds__(HMC_TPB, HMC_MINB) k_hmc(HmcArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem S;
    S.pos = (float4 *)smem_raw;
    S.list = (int *)(S.pos + A.nmax);
    S.start = S.list + A.nmax;
    S.cnt = S.start + A.ncmax + 1;
    __shared__ int s_rep;
    const uint32_t key[2] = {A.key0, A.key1};
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_rep = atomicAdd(A.counter, 1);
        __syncthreads();
        const int k = s_rep;
        if (k >= A.nrep) break;
        const int r = A.order[k], n = A.natom[r], off = A.offset[r];
        const double L = A.box[r];
        int nc = (int)floor(L / A.rc);
        if (nc < 3) nc = 0;
        int acc = 0;
        double u_cur = 0.0;
        for (int m = 0; m < A.nmoves; m++) {
            const uint32_t mv = (uint32_t)(A.move0 + m);
            // 1. velocities (velinit) and the saved positions
            const double sd = sqrt(A.treq) / sqrt(A.mass);
            double px = 0, py = 0, pz = 0;
            for (int i = threadIdx.x; i < n; i += HMC_TPB) {
                const uint32_t c0[4] = {(uint32_t)i, mv, 0u, (uint32_t)r}, c1[4] = {(uint32_t)i, mv, 1u, (uint32_t)r};
                uint32_t w0[4], w1[4];
                mg_philox4x32_10(c0, key, w0);
                mg_philox4x32_10(c1, key, w1);
                double g0, g1, g2, g3;
                mg_gauss2(w0, &g0, &g1);
                mg_gauss2(w1, &g2, &g3);
                const double v0 = sd * g0, v1 = sd * g1, v2 = sd * g2;
                A.vx[off + i] = v0;
                A.vy[off + i] = v1;
                A.vz[off + i] = v2;
                px += v0 * A.mass;
                py += v1 * A.mass;
                pz += v2 * A.mass;
                A.ox[off + i] = A.x[off + i];
                A.oy[off + i] = A.y[off + i];
                A.oz[off + i] = A.z[off + i];
            }
            block_sum3(px, py, pz);
            const double sysm = A.mass * n;
            px /= sysm;
            py /= sysm;
            pz /= sysm;
            double k0 = 0, d0 = 0, d1 = 0;
            for (int i = threadIdx.x; i < n; i += HMC_TPB) {
                const double v0 = A.vx[off + i] - px, v1 = A.vy[off + i] - py, v2 = A.vz[off + i] - pz;
                A.vx[off + i] = v0;
                A.vy[off + i] = v1;
                A.vz[off + i] = v2;
                k0 += A.mass * (v0 * v0 + v1 * v1 + v2 * v2);
            }
            block_sum3(k0, d0, d1);
            k0 *= 0.5;
            if (A.rescale) {  // to exactly treq (src/initvars.c:208-227)
                const double tinst = 2.0 * k0 / (3.0 * n - A.nconstraint);
                const double scaling = sqrt(A.treq / tinst);
                k0 = d0 = d1 = 0;
                for (int i = threadIdx.x; i < n; i += HMC_TPB) {
                    const double v0 = A.vx[off + i] * scaling, v1 = A.vy[off + i] * scaling;
                    const double v2 = A.vz[off + i] * scaling;
                    A.vx[off + i] = v0;
                    A.vy[off + i] = v1;
                    A.vz[off + i] = v2;
                    k0 += A.mass * (v0 * v0 + v1 * v1 + v2 * v2);
                }
                block_sum3(k0, d0, d1);
                k0 *= 0.5;
            }
            // 2. trajectory
            double u0, n0, u1 = 0, n1 = 0;
            load_positions(A, S, off, n, L, nc);
            force_kick(A, S, off, n, L, nc, 0.5 * A.dt, &u0, &n0);
            for (int s = 1; s <= A.nstep; s++) {
                __syncthreads();
                for (int i = threadIdx.x; i < n; i += HMC_TPB) {
                    A.x[off + i] += A.dt * A.vx[off + i];
                    A.y[off + i] += A.dt * A.vy[off + i];
                    A.z[off + i] += A.dt * A.vz[off + i];
                }
                __syncthreads();
                load_positions(A, S, off, n, L, nc);
                const bool last = s == A.nstep;
                force_kick(A, S, off, n, L, nc, last ? 0.5 * A.dt : A.dt, last ? &u1 : nullptr, last ? &n1 : nullptr);
            }
            __syncthreads();
            double k1 = 0, e0 = 0, e1 = 0;
            for (int i = threadIdx.x; i < n; i += HMC_TPB) {
                const double v0 = A.vx[off + i], v1 = A.vy[off + i], v2 = A.vz[off + i];
                k1 += A.mass * (v0 * v0 + v1 * v1 + v2 * v2);
            }
            block_sum3(k1, e0, e1);
            k1 *= 0.5;
            // 3. Metropolis test on the reference's energy difference
            const double dh = ((u1 - u0) + (k1 - k0) + A.shift_pair * (n1 - n0)) / A.treq;
            const uint32_t ca[4] = {0u, mv, 2u, (uint32_t)r};
            uint32_t wa[4];
            mg_philox4x32_10(ca, key, wa);
            const double ua = mg_u01(wa[0], wa[1]);
            const bool accept = dh <= 0.0 || ua < exp(-dh);
            if (!accept) {
                for (int i = threadIdx.x; i < n; i += HMC_TPB) {
                    A.x[off + i] = A.ox[off + i];
                    A.y[off + i] = A.oy[off + i];
                    A.z[off + i] = A.oz[off + i];
                }
            }
            acc += accept ? 1 : 0;
            u_cur = accept ? u1 + A.shift_pair * n1 : u0 + A.shift_pair * n0;
            if (threadIdx.x == 0 && A.dh_log) A.dh_log[(size_t)r * A.nmoves + m] = dh;
        }
        if (threadIdx.x == 0) {
            A.accepted[r] = acc;
            A.energy[r] = u_cur;
        }
    }
}

// ---- batched simulated annealing (siman, src/siman.c:62-182) --------------------------
struct SimanArgs {
    int nrep, total;
    const int *order, *natom, *offset;
    const double *box;
    double *x, *y, *z, *vx, *vy, *vz;   // [total]
    double *f, *vn, *vo, *b;            // [3][total] each: forces, solver work arrays
    int *counter;
    int nst, n_tries, nconstraint;
    double eps, sig2, rc, rc2, shift_pair, mass, dt, qq, qqs, t_initial, mu_t;
    uint64_t seed;
    double *log;                        // [nrep][nst][MG_SIMAN_BATCH_LOG]
    int nmax, ncmax;
};

// FP32 LJ forces (shared-memory positions) into f, with the pair energy and pair count
__device__ __forceinline__ void siman_forces(const SimanArgs &A, const HmcArgs &H, const Smem &S, int off, int n,
                                             double L, int nc, double &u, double &np) {
    const int total = A.total;
    double esum = 0.0, nsum = 0.0, unused = 0.0;
    replica_forces(H, S, n, L, nc, [&](int i, float fx, float fy, float fz, float e, int cnt) {
        A.f[off + i] = (double)fx;
        A.f[total + off + i] = (double)fy;
        A.f[2 * (size_t)total + off + i] = (double)fz;
        esum += (double)e;
        nsum += (double)cnt;
    });
    __syncthreads();
    block_sum3(esum, nsum, unused);
    u = 0.5 * esum;
    np = 0.5 * nsum;
}

// The implicit Nose-Hoover solve of src/nvtnh.c:67-156 (inner) and :165-252 (outer) for
// the block's replica, in the same arithmetic as the engine's solver kernels: Newton
// iterations on the thermostat momentum with fixed-order block sums, at most 100, the
// reference's test on the momentum alone. f == nullptr: zero forces (the short forces of
// a one-site fluid). Returns the new momentum; sumv2 = sum m v^2 of the new velocities.
__device__ double siman_nh_solve(const SimanArgs &A, int off, int n, const double *f, double h, double dt, double q,
                                 double g_treq, double ps_pred, double &sumv2) {
    const size_t total = (size_t)A.total;
    const double r = 1.0 / A.mass;
    double t0 = 0.0, d0 = 0.0, d1 = 0.0;
    for (int i = threadIdx.x; i < n; i += HMC_TPB) {
        const double v[3] = {A.vx[off + i], A.vy[off + i], A.vz[off + i]};
        double s2 = 0.0;
        for (int d = 0; d < 3; d++) {
            A.vn[d * total + off + i] = v[d];
            s2 += v[d] * v[d];
        }
        t0 += s2 / r;
    }
    block_sum3(t0, d0, d1);
    sumv2 = t0;
    double psn = ps_pred;
    for (int iter = 1; iter <= 100; iter++) {
        double ds = 0.0, e0 = 0.0, e1 = 0.0;
        for (int i = threadIdx.x; i < n; i += HMC_TPB) {
            const double v[3] = {A.vx[off + i], A.vy[off + i], A.vz[off + i]};
            for (int d = 0; d < 3; d++) {
                const size_t k = d * total + off + i;
                const double vo = A.vn[k];
                A.vo[k] = vo;
                const double fd = f ? f[k] : 0.0;
                const double b = -h * (fd * r - psn * vo) - (v[d] - vo);
                A.b[k] = b;
                const double ri = vo * dt / q / r;
                ds += ri * b;
            }
        }
        block_sum3(ds, e0, e1);
        const double pso = psn, di = -(pso * h + 1.0);
        double delps = ds - di * ((-sumv2 + g_treq) * h / q - (ps_pred - pso));
        delps = delps / (-dt * h * sumv2 / q + di);
        double s2 = 0.0;
        e0 = e1 = 0.0;
        for (int i = threadIdx.x; i < n; i += HMC_TPB) {
            double m2 = 0.0;
            for (int d = 0; d < 3; d++) {
                const size_t k = d * total + off + i;
                const double vn = A.vn[k] + (A.b[k] + h * A.vo[k] * delps) / di;
                A.vn[k] = vn;
                m2 += vn * vn;
            }
            s2 += m2 / r;
        }
        block_sum3(s2, e0, e1);
        sumv2 = s2;
        psn = pso + delps;
        if (!(fabs((psn - pso) / psn) > 1.0e-10)) break;
    }
    for (int i = threadIdx.x; i < n; i += HMC_TPB) {
        A.vx[off + i] = A.vn[off + i];
        A.vy[off + i] = A.vn[total + off + i];
        A.vz[off + i] = A.vn[2 * total + off + i];
    }
    __syncthreads();
    return psn;
}

// One block runs whole replicas (largest first, from a work counter): every stage of the
// schedule is velinit at T, forces, n_tries vver_nh_3 steps with one inner step (a
// one-site fluid has no short forces) and the thermostat reset.
__global__ void __launch_bounds__(HMC_TPB, HMC_MINB) k_siman_batch(SimanArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Smem S;
    S.pos = (float4 *)smem_raw;
    S.list = (int *)(S.pos + A.nmax);
    S.start = S.list + A.nmax;
    S.cnt = S.start + A.ncmax + 1;
    __shared__ int s_rep;
    HmcArgs H;  // what the shared-memory position and force helpers read
    H.x = A.x;
    H.y = A.y;
    H.z = A.z;
    H.sig2 = A.sig2;
    H.eps = A.eps;
    H.rc2 = A.rc2;
    const size_t total = (size_t)A.total;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_rep = atomicAdd(A.counter, 1);
        __syncthreads();
        const int kr = s_rep;
        if (kr >= A.nrep) break;
        const int rep = A.order[kr], n = A.natom[rep], off = A.offset[rep];
        const double L = A.box[rep];
        int nc = (int)floor(L / A.rc);
        if (nc < 3) nc = 0;
        const uint64_t seed = A.seed ^ ((uint64_t)rep * 0x9E3779B97F4A7C15ull);
        const uint32_t key[2] = {(uint32_t)(seed & 0xffffffffull), (uint32_t)(seed >> 32)};
        const double nfree = 3.0 * n - A.nconstraint, mass = A.mass, r = 1.0 / mass;
        const double dt = A.dt, h = dt / 2.0, dts = dt, hs = dts / 2.0, dt_sqby2 = dt * dt / 2.0;
        const double dts_sqby2 = dts * dts / 2.0;
        double T = A.t_initial;
        for (int k = 0; k < A.nst; k++) {
            double ps = 0.0, ss = 0.0, pss = 0.0, sss = 0.0;  // stage 0 from zero, later ones reset
            // velinit at T (src/initvars.c:151-229) on the Philox streams of mg_siman_run
            const double stdv = sqrt(T) / sqrt(mass);
            double px = 0.0, py = 0.0, pz = 0.0;
            for (int i = threadIdx.x; i < n; i += HMC_TPB) {
                const uint32_t c0[4] = {(uint32_t)i, (uint32_t)k, 0u, 0x5349u};
                const uint32_t c1[4] = {(uint32_t)i, (uint32_t)k, 1u, 0x5349u};
                uint32_t w0[4], w1[4];
                double g0, g1, g2, g3;
                mg_philox4x32_10(c0, key, w0);
                mg_philox4x32_10(c1, key, w1);
                mg_gauss2(w0, &g0, &g1);
                mg_gauss2(w1, &g2, &g3);
                const double v0 = stdv * g0, v1 = stdv * g1, v2 = stdv * g2;
                A.vx[off + i] = v0;
                A.vy[off + i] = v1;
                A.vz[off + i] = v2;
                px += v0 * mass;
                py += v1 * mass;
                pz += v2 * mass;
            }
            block_sum3(px, py, pz);
            const double sysm = mass * n;
            px /= sysm;
            py /= sysm;
            pz /= sysm;
            double ukin = 0.0, d0 = 0.0, d1 = 0.0;
            for (int i = threadIdx.x; i < n; i += HMC_TPB) {
                const double v0 = A.vx[off + i] - px, v1 = A.vy[off + i] - py, v2 = A.vz[off + i] - pz;
                A.vx[off + i] = v0;
                A.vy[off + i] = v1;
                A.vz[off + i] = v2;
                ukin += mass * (v0 * v0 + v1 * v1 + v2 * v2);
            }
            block_sum3(ukin, d0, d1);
            ukin = 0.5 * ukin;
            const double scaling = sqrt(T / (2.0 * ukin / nfree));
            for (int i = threadIdx.x; i < n; i += HMC_TPB) {
                A.vx[off + i] *= scaling;
                A.vy[off + i] *= scaling;
                A.vz[off + i] *= scaling;
            }
            __syncthreads();
            const double g_treq = nfree * T;  // gg = ggs = nfree (src/siman.c:167-174)
            double u = 0.0, np = 0.0, sumv2 = 0.0;
            load_positions(H, S, off, n, L, nc);
            siman_forces(A, H, S, off, n, L, nc, u, np);
            for (int st = 1; st <= A.n_tries; st++) {  // vver_nh_3 (src/nvtnh.c:11-271)
                double sv = 0.0;
                for (int i = threadIdx.x; i < n; i += HMC_TPB) {  // outer half kick
                    for (int d = 0; d < 3; d++) {
                        double *vd = d == 0 ? A.vx : (d == 1 ? A.vy : A.vz);
                        const double v = vd[off + i];
                        vd[off + i] = v + h * (A.f[d * total + off + i] * r - ps * v);
                    }
                }
                __syncthreads();
                for (int i = threadIdx.x; i < n; i += HMC_TPB) {  // inner step: no short forces
                    double s2 = 0.0;
                    double *pos[3] = {A.x, A.y, A.z};
                    for (int d = 0; d < 3; d++) {
                        double *vd = d == 0 ? A.vx : (d == 1 ? A.vy : A.vz);
                        double v = vd[off + i];
                        s2 += v * v;
                        v = v + hs * (0.0 * r - pss * v);
                        vd[off + i] = v;
                        pos[d][off + i] = pos[d][off + i] + dts * v;
                    }
                    sv += s2 / r;
                }
                d0 = d1 = 0.0;
                block_sum3(sv, d0, d1);
                sss = sss + pss * dts + (sv - g_treq) * dts_sqby2 / A.qqs;
                pss = pss + (sv - g_treq) * hs / A.qqs;
                pss = siman_nh_solve(A, off, n, nullptr, hs, dts, A.qqs, g_treq, pss, sumv2);
                ss = ss + ps * dt + (sumv2 - g_treq) * dt_sqby2 / A.qq;
                ps = ps + (sumv2 - g_treq) * h / A.qq;
                load_positions(H, S, off, n, L, nc);
                siman_forces(A, H, S, off, n, L, nc, u, np);
                ps = siman_nh_solve(A, off, n, A.f, h, dt, A.qq, g_treq, ps, sumv2);
            }
            if (threadIdx.x == 0) {
                double *o = A.log + ((size_t)rep * A.nst + k) * MG_SIMAN_BATCH_LOG;
                o[0] = T;
                o[1] = sumv2 / 2.0;  // ukin at the stage end
                o[2] = u;            // uinter (LJ)
                o[3] = A.shift_pair * np;
                o[4] = sumv2 / nfree;
            }
            T /= A.mu_t;
        }
    }
}

}  // namespace

extern "C" mg_status mg_siman_batch(int device, const mg_siman_batch_params *p, int nrep, const int *natom,
                                    const double *box, double *x, double *y, double *z, int *nstages,
                                    double *stage_log) {
    if (!p || nrep <= 0 || !natom || !box || !x || !y || !z || !nstages || !stage_log) return MG_ERR_INVALID;
    if (!(p->eps >= 0) || !(p->sigma > 0) || !(p->rcutoff > 0) || !(p->mass > 0) || !(p->delt > 0) ||
        !(p->qq > 0) || !(p->qqs > 0) || p->n_tries < 0 || p->nconstraint < 0)
        return MG_ERR_INVALID;
    const int nst = mg_siman_stage_count(p->t_initial, p->t_min, p->mu_t, p->max_stages);
    if (nst < 0) return MG_ERR_CAPACITY;
    int nmax = 0, ncmax = 0;
    long long total = 0;
    for (int r = 0; r < nrep; r++) {
        if (natom[r] < 2 || !(box[r] >= 2.0 * p->rcutoff) || 3 * natom[r] <= p->nconstraint) return MG_ERR_INVALID;
        nmax = std::max(nmax, natom[r]);
        int nc = (int)floor(box[r] / p->rcutoff);
        if (nc >= 3) ncmax = std::max(ncmax, nc * nc * nc);
        total += natom[r];
    }
    if (total > 0x7fffffffLL) return MG_ERR_CAPACITY;
    const size_t smem = 16 * (size_t)nmax + 4 * (size_t)nmax + 4 * (2 * (size_t)ncmax + 1) + 16;
    if (smem > 200 * 1024) return MG_ERR_CAPACITY;  // one replica's positions and cells stay on chip
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return MG_ERR_NO_DEVICE;
    }
    int major = 0, minor = 0, nsm = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    if (major != 10 || minor != 3) return MG_ERR_NO_DEVICE;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return MG_ERR_CUDA;
    }
    std::vector<int> offset(nrep), order(nrep);
    long long o = 0;
    for (int r = 0; r < nrep; r++) {
        offset[r] = (int)o;
        o += natom[r];
    }
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return natom[a] > natom[b]; });
    const size_t nb = sizeof(double) * (size_t)total;
    std::vector<void *> bufs;
    auto dalloc = [&](size_t bytes) -> void * {
        void *q = nullptr;
        if (cudaMalloc(&q, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        bufs.push_back(q);
        return q;
    };
    mg_status st = MG_OK;
    cudaStream_t s = nullptr;
    const size_t nlog = (size_t)nrep * nst * MG_SIMAN_BATCH_LOG;
    double *d_state = (double *)dalloc(18 * nb);
    int *d_int = (int *)dalloc(sizeof(int) * (3 * (size_t)nrep + 1));
    double *d_box = (double *)dalloc(sizeof(double) * nrep);
    double *d_log = (double *)dalloc(sizeof(double) * nlog);
    if (!d_state || !d_int || !d_box || !d_log || cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) {
        st = MG_ERR_ALLOC;
    } else {
        SimanArgs A;
        A.nrep = nrep;
        A.total = (int)total;
        int *d_order = d_int, *d_natom = d_int + nrep, *d_offset = d_int + 2 * nrep;
        A.counter = d_int + 3 * nrep;
        A.order = d_order;
        A.natom = d_natom;
        A.offset = d_offset;
        A.box = d_box;
        A.x = d_state;
        A.y = A.x + total;
        A.z = A.y + total;
        A.vx = A.z + total;
        A.vy = A.vx + total;
        A.vz = A.vy + total;
        A.f = A.vz + total;
        A.vn = A.f + 3 * total;
        A.vo = A.vn + 3 * total;
        A.b = A.vo + 3 * total;
        A.nst = nst;
        A.n_tries = p->n_tries;
        A.nconstraint = p->nconstraint;
        A.eps = p->eps;
        A.sig2 = p->sigma * p->sigma;
        A.rc = p->rcutoff;
        A.rc2 = p->rcutoff * p->rcutoff;
        // shift energy of one pair inside the cutoff, as for mg_hmc_batch
        const double shift1 = pow(1.0 / p->rcutoff, 6.0), sig6 = pow(p->sigma, 6.0);
        A.shift_pair = p->eps * sig6 * (sig6 * shift1 - 1.0) * (4.0 * shift1);
        A.mass = p->mass;
        A.dt = p->delt;
        A.qq = p->qq;
        A.qqs = p->qqs;
        A.t_initial = p->t_initial;
        A.mu_t = p->mu_t;
        A.seed = p->seed;
        A.log = d_log;
        A.nmax = nmax;
        A.ncmax = ncmax;
        cudaMemcpyAsync(d_order, order.data(), sizeof(int) * nrep, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_natom, natom, sizeof(int) * nrep, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_offset, offset.data(), sizeof(int) * nrep, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(A.counter, 0, sizeof(int), s);
        cudaMemcpyAsync(d_box, box, sizeof(double) * nrep, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(A.x, x, nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(A.y, y, nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(A.z, z, nb, cudaMemcpyHostToDevice, s);
        if (cudaFuncSetAttribute(k_siman_batch, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
            st = MG_ERR_CUDA;
        } else {
            int per_sm = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_siman_batch, HMC_TPB, smem);
            const int blocks = std::max(1, std::min(nrep, nsm * std::max(per_sm, 1)));
            k_siman_batch<<<blocks, HMC_TPB, smem, s>>>(A);
            cudaMemcpyAsync(x, A.x, nb, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(y, A.y, nb, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(z, A.z, nb, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(stage_log, d_log, sizeof(double) * nlog, cudaMemcpyDeviceToHost, s);
            if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) st = MG_ERR_CUDA;
        }
    }
    cudaGetLastError();
    for (void *q : bufs) cudaFree(q);
    if (s) cudaStreamDestroy(s);
    cudaSetDevice(prev);
    *nstages = nst;
    return st;
}

extern "C" mg_status mg_hmc_batch(int device, const mg_hmc_params *p, int nrep, const int *natom, const double *box,
                                  double *x, double *y, double *z, int nmoves, int move0, int *accepted,
                                  double *dh_log, double *energy) {
    if (!p || nrep <= 0 || nmoves < 0 || move0 < 0 || !natom || !box || !x || !y || !z || !accepted || !energy)
        return MG_ERR_INVALID;
    if (!(p->eps >= 0) || !(p->sigma > 0) || !(p->rcutoff > 0) || !(p->mass > 0) || !(p->treq > 0) ||
        !(p->delt > 0) || p->nstep_md < 1 || p->nconstraint < 0)
        return MG_ERR_INVALID;
    int nmax = 0, ncmax = 0;
    long long total = 0;
    for (int r = 0; r < nrep; r++) {
        if (natom[r] < 2 || !(box[r] >= 2.0 * p->rcutoff)) return MG_ERR_INVALID;  // minimum image needs L >= 2 rc
        nmax = std::max(nmax, natom[r]);
        int nc = (int)floor(box[r] / p->rcutoff);
        if (nc >= 3) ncmax = std::max(ncmax, nc * nc * nc);
        total += natom[r];
    }
    const size_t smem = 16 * (size_t)nmax + 4 * (size_t)nmax + 4 * (2 * (size_t)ncmax + 1) + 16;
    if (smem > 200 * 1024) return MG_ERR_CAPACITY;  // one replica's positions and cells stay on chip
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return MG_ERR_NO_DEVICE;
    }
    int major = 0, minor = 0, nsm = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    if (major != 10 || minor != 3) return MG_ERR_NO_DEVICE;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return MG_ERR_CUDA;
    }
    std::vector<int> offset(nrep), order(nrep);
    long long o = 0;
    for (int r = 0; r < nrep; r++) {
        offset[r] = (int)o;
        o += natom[r];
    }
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return natom[a] > natom[b]; });
    const size_t nb = sizeof(double) * (size_t)total;
    std::vector<void *> bufs;
    auto dalloc = [&](size_t bytes) -> void * {
        void *q = nullptr;
        if (cudaMalloc(&q, bytes ? bytes : 16) != cudaSuccess) return nullptr;
        bufs.push_back(q);
        return q;
    };
    mg_status st = MG_OK;
    cudaStream_t s = nullptr;
    double *d_state = (double *)dalloc(9 * nb);
    int *d_int = (int *)dalloc(sizeof(int) * (3 * (size_t)nrep + 2 * (size_t)nrep + 1));
    double *d_box = (double *)dalloc(sizeof(double) * nrep);
    double *d_dh = (double *)dalloc(sizeof(double) * (size_t)nrep * std::max(nmoves, 1));
    double *d_energy = (double *)dalloc(sizeof(double) * nrep);
    if (!d_state || !d_int || !d_box || !d_dh || !d_energy || cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) {
        st = MG_ERR_ALLOC;
    } else {
        HmcArgs A;
        A.nrep = nrep;
        int *d_order = d_int, *d_natom = d_int + nrep, *d_offset = d_int + 2 * nrep, *d_acc = d_int + 3 * nrep;
        A.counter = d_int + 5 * nrep;
        A.order = d_order;
        A.natom = d_natom;
        A.offset = d_offset;
        A.box = d_box;
        A.x = d_state;
        A.y = A.x + total;
        A.z = A.y + total;
        A.vx = A.z + total;
        A.vy = A.vx + total;
        A.vz = A.vy + total;
        A.ox = A.vz + total;
        A.oy = A.ox + total;
        A.oz = A.oy + total;
        A.nmoves = nmoves;
        A.move0 = move0;
        A.nstep = p->nstep_md;
        A.eps = p->eps;
        A.sig2 = p->sigma * p->sigma;
        A.rc = p->rcutoff;
        A.rc2 = p->rcutoff * p->rcutoff;
        // shift energy of one pair inside the cutoff: eps sig^6 (sig^6 shift1 - 1) shift4,
        // shift1 = (1/rcutoff)^6, shift4 = 4 shift1 (src/initvars.c:591-599, src/frclong.c)
        const double shift1 = pow(1.0 / p->rcutoff, 6.0), sig6 = pow(p->sigma, 6.0);
        A.shift_pair = p->eps * sig6 * (sig6 * shift1 - 1.0) * (4.0 * shift1);
        A.mass = p->mass;
        A.treq = p->treq;
        A.dt = p->delt;
        A.rescale = p->rescale;
        A.nconstraint = p->nconstraint;
        A.key0 = (uint32_t)(p->seed & 0xffffffffull);
        A.key1 = (uint32_t)(p->seed >> 32);
        A.accepted = d_acc;
        A.dh_log = d_dh;
        A.energy = d_energy;
        A.nmax = nmax;
        A.ncmax = ncmax;
        cudaMemcpyAsync(d_order, order.data(), sizeof(int) * nrep, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_natom, natom, sizeof(int) * nrep, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(d_offset, offset.data(), sizeof(int) * nrep, cudaMemcpyHostToDevice, s);
        cudaMemsetAsync(A.counter, 0, sizeof(int), s);
        cudaMemcpyAsync(d_box, box, sizeof(double) * nrep, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(A.x, x, nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(A.y, y, nb, cudaMemcpyHostToDevice, s);
        cudaMemcpyAsync(A.z, z, nb, cudaMemcpyHostToDevice, s);
        if (cudaFuncSetAttribute(k_hmc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
            st = MG_ERR_CUDA;
        } else {
            int per_sm = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hmc, HMC_TPB, smem);
            const int blocks = std::max(1, std::min(nrep, nsm * std::max(per_sm, 1)));
            k_hmc<<<blocks, HMC_TPB, smem, s>>>(A);
            cudaMemcpyAsync(x, A.x, nb, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(y, A.y, nb, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(z, A.z, nb, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(accepted, d_acc, sizeof(int) * nrep, cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(energy, d_energy, sizeof(double) * nrep, cudaMemcpyDeviceToHost, s);
            if (dh_log && nmoves > 0)
                cudaMemcpyAsync(dh_log, d_dh, sizeof(double) * (size_t)nrep * nmoves, cudaMemcpyDeviceToHost, s);
            if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) st = MG_ERR_CUDA;
        }
    }
    cudaGetLastError();
    for (void *q : bufs) cudaFree(q);
    if (s) cudaStreamDestroy(s);
    cudaSetDevice(prev);
    return st;
}
