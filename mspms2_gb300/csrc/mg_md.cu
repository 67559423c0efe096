// mg_md.cu - device-resident integration: the reference's velocity Verlet RESPA step
// (vver, src/md.c:22-85) and its Nose-Hoover RESPA step with implicit thermostat
// solves (vver_nh_3, src/nvtnh.c:11-271).
//
// Positions, velocities, forces and the thermostat scalars stay on the device for the
// whole run; the host only orders the kernels, evaluates forces through the same path
// as mg_compute_device and, once per batch of solver iterations, reads whether the
// thermostat solve has converged. Sums over sites (sum m v^2 and the solver's delps)
// are block partials reduced by one block in a fixed order, so a run is reproducible.
//
// Arithmetic follows the reference expression by expression in FP64 (r_mass = 1/aw,
// f*r_mass, v^2/r_mass, ...). Reference behaviours kept:
//  - the solver's convergence test reads the velocity arrays at index natom (a stale
//    loop index, src/nvtnh.c:128-139 and :228-236), which the reference never writes,
//    so only the thermostat test |(ps_new - ps_old)/ps_new| <= 1e-10 decides; at most
//    100 iterations;
//  - the thermostat predictor of the outer step uses sum m v^2 of the last inner solve.
#include <math.h>

#include <vector>

#include <cooperative_groups.h>

#include "mg_internal.cuh"
#include "../../include/mg_philox.h"

#define MD_TPB 256       // threads per block of the site kernels
#define MD_ITER_BATCH 4  // solver iterations launched between convergence reads
#define MD_MAX_ITER 100  // the reference's iteration limit
#define MD_ERR 1.0e-10   // the reference's convergence tolerance

namespace {

// thermostat scalars and solver state, in device memory
struct MdDev {
    double ps, ss, pss, sss;  // thermostat momenta and positions (outer, inner)
    double sumv2;             // the reference's running sum m v^2
    double psn, pso, delps, di;
    double ukin, tinst, unhts, unhtss;
    double vel[4];            // velinit: momentum shift (x, y, z) and the rescaling factor
    int ready, iter;
};

struct MdArgs {
    int n;
    double *x, *y, *z;            // positions [n] each
    double *v;                    // velocities [3][n]
    double *vn, *vo, *b;          // solver work arrays [3][n]
    const double *rmass;          // 1/aw per site
    const double *fl, *fs;        // long and short forces [3][n]
    double *part;                 // block partial sums
    MdDev *s;
};

// sum of the block's values in a fixed order, written to part[blockIdx.x]
__device__ __forceinline__ void block_partial(double v, double *part) {
    __shared__ double red[MD_TPB];
    red[threadIdx.x] = v;
    __syncthreads();
    for (int o = MD_TPB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// fixed-order sum of nb block partials by one block
__device__ double sum_partials(const double *part, int nb) {
    __shared__ double red[MD_TPB];
    double t = 0.0;
    for (int i = threadIdx.x; i < nb; i += MD_TPB) t += part[i];
    red[threadIdx.x] = t;
    __syncthreads();
    for (int o = MD_TPB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    return red[0];
}

__global__ void k_md_rmass(int n, const double *__restrict__ aw, double *__restrict__ rmass) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < n) rmass[a] = 1.0 / aw[a];
}

// v += h (f r_mass - ps v) (ps = 0: plain kick); optional partial of sum m v^2 after it
__global__ void k_md_kick(MdArgs A, const double *__restrict__ f, double h, int thermo, int want_sum) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    double m2 = 0.0;
    if (a < A.n) {
        const double r = A.rmass[a], ps = thermo ? A.s->ps : 0.0;
        const int n = A.n;
        for (int d = 0; d < 3; d++) {
            double v = A.v[d * n + a];
            v = thermo ? v + h * (f[d * n + a] * r - ps * v) : v + h * f[d * n + a] * r;
            A.v[d * n + a] = v;
            m2 += v * v;
        }
        m2 /= r;
    }
    if (want_sum) block_partial(m2, A.part);
}

// inner step opening: partial of sum m v^2 (velocities before the kick), then
// v += hs (fs r_mass - pss v), x += dts v  (pss = 0 without thermostat)
__global__ void k_md_inner_drift(MdArgs A, double hs, double dts, int thermo) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    double m2 = 0.0;
    if (a < A.n) {
        const double r = A.rmass[a], pss = thermo ? A.s->pss : 0.0;
        const int n = A.n;
        double *pos[3] = {A.x, A.y, A.z};
        double s = 0.0;
        for (int d = 0; d < 3; d++) {
            double v = A.v[d * n + a];
            s += v * v;
            v = thermo ? v + hs * (A.fs[d * n + a] * r - pss * v) : v + hs * A.fs[d * n + a] * r;
            A.v[d * n + a] = v;
            pos[d][a] = pos[d][a] + dts * v;
        }
        m2 = s / r;
    }
    if (thermo) block_partial(m2, A.part);
}

// inner thermostat predictor (src/nvtnh.c:56-57)
__global__ void k_md_inner_predict(MdArgs A, int nb, double ggs_treq, double dts, double dts_sqby2, double hs,
                                   double qqs) {
    const double sumv2 = sum_partials(A.part, nb);
    if (threadIdx.x != 0) return;
    MdDev *s = A.s;
    s->sumv2 = sumv2;
    s->sss = s->sss + s->pss * dts + (sumv2 - ggs_treq) * dts_sqby2 / qqs;
    s->pss = s->pss + (sumv2 - ggs_treq) * hs / qqs;
}

// outer thermostat predictor (src/nvtnh.c:162-163), from the last inner solve's sum
__global__ void k_md_outer_predict(MdDev *s, double gg_treq, double dt, double dt_sqby2, double h, double qq) {
    s->ss = s->ss + s->ps * dt + (s->sumv2 - gg_treq) * dt_sqby2 / qq;
    s->ps = s->ps + (s->sumv2 - gg_treq) * h / qq;
}

// ---- implicit thermostat solve (src/nvtnh.c:67-156 inner, :165-252 outer) ----------
struct NhArgs {
    const double *f;  // the forces of this solve
    double h, dt, q, g_treq;
    int inner;        // 1: pss (inner thermostat), 0: ps (outer)
};

__device__ __forceinline__ double &nh_ps(MdDev *s, int inner) { return inner ? s->pss : s->ps; }

// vn = v and its sum m v^2; the scalar kernel below starts the iteration
__global__ void k_nh_start(MdArgs A) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    double m2 = 0.0;
    if (a < A.n) {
        const int n = A.n;
        double s = 0.0;
        for (int d = 0; d < 3; d++) {
            const double v = A.v[d * n + a];
            A.vn[d * n + a] = v;
            s += v * v;
        }
        m2 = s / A.rmass[a];
    }
    block_partial(m2, A.part);
}

__global__ void k_nh_start_scalar(MdArgs A, int nb, int inner) {
    const double sumv2 = sum_partials(A.part, nb);
    if (threadIdx.x != 0) return;
    A.s->sumv2 = sumv2;
    A.s->psn = nh_ps(A.s, inner);
    A.s->ready = 0;
    A.s->iter = 0;
}

// vo = vn; b = -h (f r_mass - pso vo) - (v - vo); partial of sum (vo dt / q / r_mass) b
__global__ void k_nh_residual(MdArgs A, NhArgs N) {
    if (A.s->ready) return;
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    double t = 0.0;
    if (a < A.n) {
        const int n = A.n;
        const double r = A.rmass[a], pso = A.s->psn;
        for (int d = 0; d < 3; d++) {
            const double vo = A.vn[d * n + a];
            A.vo[d * n + a] = vo;
            const double b = -N.h * (N.f[d * n + a] * r - pso * vo) - (A.v[d * n + a] - vo);
            A.b[d * n + a] = b;
            const double ri = vo * N.dt / N.q / r;
            t += ri * b;
        }
    }
    block_partial(t, A.part);
}

// Newton step of the thermostat momentum (src/nvtnh.c:99-102, :206-208)
__global__ void k_nh_step_scalar(MdArgs A, NhArgs N, int nb) {
    if (A.s->ready) return;
    double delps = sum_partials(A.part, nb);
    if (threadIdx.x != 0) return;
    MdDev *s = A.s;
    const double pso = s->psn, ps = nh_ps(s, N.inner);
    const double di = -(pso * N.h + 1.0);
    delps = delps - di * ((-s->sumv2 + N.g_treq) * N.h / N.q - (ps - pso));
    delps = delps / (-N.dt * N.h * s->sumv2 / N.q + di);
    s->pso = pso;
    s->delps = delps;
    s->di = di;
}

// vn += (b + h vo delps) / di and its sum m v^2
__global__ void k_nh_update(MdArgs A, NhArgs N) {
    if (A.s->ready) return;
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    double m2 = 0.0;
    if (a < A.n) {
        const int n = A.n;
        const double delps = A.s->delps, di = A.s->di;
        double s = 0.0;
        for (int d = 0; d < 3; d++) {
            const double vn = A.vn[d * n + a] + (A.b[d * n + a] + N.h * A.vo[d * n + a] * delps) / di;
            A.vn[d * n + a] = vn;
            s += vn * vn;
        }
        m2 = s / A.rmass[a];
    }
    block_partial(m2, A.part);
}

// new momentum and the reference's convergence test (thermostat only, see the header)
__global__ void k_nh_check_scalar(MdArgs A, int nb) {
    if (A.s->ready) return;
    const double sumv2 = sum_partials(A.part, nb);
    if (threadIdx.x != 0) return;
    MdDev *s = A.s;
    s->sumv2 = sumv2;
    s->psn = s->pso + s->delps;
    s->iter += 1;
    const bool converged = !(fabs((s->psn - s->pso) / s->psn) > MD_ERR);
    s->ready = (converged || s->iter >= MD_MAX_ITER) ? 1 : 0;
}

// v = vn; the thermostat takes the solved momentum
__global__ void k_nh_finish(MdArgs A, int inner) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < 3 * A.n) A.v[a] = A.vn[a];
    if (a == 0) nh_ps(A.s, inner) = A.s->psn;
}

// The whole implicit solve in one cooperative launch: the same arithmetic as the kernel
// sequence above (k_nh_start ... k_nh_finish), with grid-wide barriers in place of kernel
// boundaries and no host round trip per batch of iterations. Each block walks the same
// 256-site chunks ("virtual blocks") the separate kernels use and every block sums the
// partials in the same fixed order, so the result is identical for any grid size. Two
// partial buffers alternate, so two barriers per iteration order every read before the
// next write. The loop stops at the reference's 100 iterations like the host loop does.
__device__ __forceinline__ void block_partial_at(double v, double *part, int idx) {
    __shared__ double red2[MD_TPB];
    red2[threadIdx.x] = v;
    __syncthreads();
    for (int o = MD_TPB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) red2[threadIdx.x] += red2[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[idx] = red2[0];
    __syncthreads();
}

__global__ void __launch_bounds__(MD_TPB) k_nh_solve_coop(MdArgs A, NhArgs N, int nb) {
    cooperative_groups::grid_group grid = cooperative_groups::this_grid();
    double *pa = A.part, *pb = A.part + nb;
    const int n = A.n;
    for (int vb = blockIdx.x; vb < nb; vb += gridDim.x) {  // vn = v and sum m v^2
        const int a = vb * MD_TPB + threadIdx.x;
        double m2 = 0.0;
        if (a < n) {
            double s = 0.0;
            for (int d = 0; d < 3; d++) {
                const double v = A.v[d * n + a];
                A.vn[d * n + a] = v;
                s += v * v;
            }
            m2 = s / A.rmass[a];
        }
        block_partial_at(m2, pa, vb);
    }
    grid.sync();
    double sumv2 = sum_partials(pa, nb);
    __syncthreads();
    const double ps = nh_ps(A.s, N.inner);  // the predicted momentum, fixed during the solve
    double psn = ps, pso = ps, delps = 0.0, di = 0.0;
    int iter = 0;
    bool ready = false;
    while (!ready) {
        for (int vb = blockIdx.x; vb < nb; vb += gridDim.x) {  // residual (k_nh_residual)
            const int a = vb * MD_TPB + threadIdx.x;
            double t = 0.0;
            if (a < n) {
                const double r = A.rmass[a];
                for (int d = 0; d < 3; d++) {
                    const double vo = A.vn[d * n + a];
                    A.vo[d * n + a] = vo;
                    const double b = -N.h * (N.f[d * n + a] * r - psn * vo) - (A.v[d * n + a] - vo);
                    A.b[d * n + a] = b;
                    const double ri = vo * N.dt / N.q / r;
                    t += ri * b;
                }
            }
            block_partial_at(t, pb, vb);
        }
        grid.sync();
        double dl = sum_partials(pb, nb);  // Newton step (k_nh_step_scalar)
        __syncthreads();
        pso = psn;
        di = -(pso * N.h + 1.0);
        dl = dl - di * ((-sumv2 + N.g_treq) * N.h / N.q - (ps - pso));
        dl = dl / (-N.dt * N.h * sumv2 / N.q + di);
        delps = dl;
        for (int vb = blockIdx.x; vb < nb; vb += gridDim.x) {  // update (k_nh_update)
            const int a = vb * MD_TPB + threadIdx.x;
            double m2 = 0.0;
            if (a < n) {
                double s = 0.0;
                for (int d = 0; d < 3; d++) {
                    const double vn = A.vn[d * n + a] + (A.b[d * n + a] + N.h * A.vo[d * n + a] * delps) / di;
                    A.vn[d * n + a] = vn;
                    s += vn * vn;
                }
                m2 = s / A.rmass[a];
            }
            block_partial_at(m2, pa, vb);
        }
        grid.sync();
        sumv2 = sum_partials(pa, nb);  // check (k_nh_check_scalar)
        __syncthreads();
        psn = pso + delps;
        iter += 1;
        const bool converged = !(fabs((psn - pso) / psn) > MD_ERR);
        ready = converged || iter >= MD_MAX_ITER;
    }
    for (int i = blockIdx.x * MD_TPB + threadIdx.x; i < 3 * n; i += gridDim.x * MD_TPB) A.v[i] = A.vn[i];
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        MdDev *s = A.s;
        s->sumv2 = sumv2;
        s->psn = psn;
        s->pso = pso;
        s->delps = delps;
        s->di = di;
        s->iter = iter;
        s->ready = 1;
        nh_ps(s, N.inner) = psn;
    }
}

// The same solve for the mixed path, reduced to one unknown. Given ps_new the per-site
// equation vn (1 + h ps_new) = v + h f r is linear, so the joint Newton iteration above
// converges to the root of the scalar equation
//   G(p) = p - ps - (h/q) (K0 / (1 + h p)^2 - g treq) = 0,  K0 = sum m (v + h f r)^2,
// and vn = (v + h f r) / (1 + h p). One pass forms v + h f r and K0, Newton on p runs in
// registers (each block the same steps, so no grid-wide work per iteration), one pass
// scales the velocities and sums m vn^2. Same convergence test and iteration limit as the
// reference's solve; the root agrees with the joint iteration's to rounding.
__global__ void __launch_bounds__(MD_TPB) k_nh_solve_scalar(MdArgs A, NhArgs N, int nb) {
    cooperative_groups::grid_group grid = cooperative_groups::this_grid();
    double *pa = A.part, *pb = A.part + nb;
    const int n = A.n;
    for (int vb = blockIdx.x; vb < nb; vb += gridDim.x) {  // w = v + h f r and sum m w^2
        const int a = vb * MD_TPB + threadIdx.x;
        double m2 = 0.0;
        if (a < n) {
            const double r = A.rmass[a];
            double s = 0.0;
            for (int d = 0; d < 3; d++) {
                const double w = A.v[d * n + a] + N.h * N.f[d * n + a] * r;
                A.vn[d * n + a] = w;
                s += w * w;
            }
            m2 = s / r;
        }
        block_partial_at(m2, pa, vb);
    }
    grid.sync();
    const double K0 = sum_partials(pa, nb);
    __syncthreads();
    const double ps = nh_ps(A.s, N.inner);
    double p = ps, pold = ps, dp = 0.0;
    int iter = 0;
    bool ready = false;
    while (!ready) {
        const double ix = 1.0 / (1.0 + N.h * p), ix2 = ix * ix;
        const double G = p - ps - (N.h / N.q) * (K0 * ix2 - N.g_treq);
        const double dG = 1.0 + 2.0 * N.h * N.h * K0 * ix2 * ix / N.q;
        dp = -G / dG;
        pold = p;
        p = pold + dp;
        iter += 1;
        ready = !(fabs(dp / p) > MD_ERR) || iter >= MD_MAX_ITER;
    }
    const double scale = 1.0 / (1.0 + N.h * p);
    for (int vb = blockIdx.x; vb < nb; vb += gridDim.x) {  // vn = w / (1 + h p) and sum m vn^2
        const int a = vb * MD_TPB + threadIdx.x;
        double m2 = 0.0;
        if (a < n) {
            double s = 0.0;
            for (int d = 0; d < 3; d++) {
                const double vn = A.vn[d * n + a] * scale;
                A.vn[d * n + a] = vn;
                A.v[d * n + a] = vn;
                s += vn * vn;
            }
            m2 = s / A.rmass[a];
        }
        block_partial_at(m2, pb, vb);
    }
    grid.sync();
    const double sumv2 = sum_partials(pb, nb);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        MdDev *s = A.s;
        s->sumv2 = sumv2;
        s->psn = p;
        s->pso = pold;
        s->delps = dp;
        s->di = -(pold * N.h + 1.0);
        s->iter = iter;
        s->ready = 1;
        nh_ps(s, N.inner) = p;
    }
}

// end-of-step scalars: thermostat energies, kinetic energy and temperature
__global__ void k_md_step_scalars(MdDev *s, int nb_unused, double qq, double qqs, double gg_treq,
                                  double ggs_treq, double nfree, int thermo, double *log_row) {
    (void)nb_unused;
    if (thermo) {
        s->unhtss = (s->pss * s->pss * qqs) / 2.0 + ggs_treq * s->sss;
        s->ukin = s->sumv2 / 2.0;
        s->unhts = (s->ps * s->ps * qq) / 2.0 + gg_treq * s->ss;
    }
    s->tinst = 2.0 * s->ukin / nfree;
    if (log_row) {
        log_row[0] = s->ukin;
        log_row[4] = s->ps;
        log_row[5] = s->ss;
        log_row[6] = s->pss;
        log_row[7] = s->sss;
        log_row[8] = s->tinst;
        log_row[9] = s->unhts;
        log_row[10] = s->unhtss;
    }
}

// ---- graph replay of whole steps ---------------------------------------------------
// The step's record row chosen by a device step counter (so that one captured step can
// be replayed), then the counter moves on; otherwise k_md_step_scalars.
__global__ void k_set_one(int *p) { *p = 1; }

__global__ void k_graph_row(MdDev *s, double qq, double qqs, double gg_treq, double ggs_treq, double nfree,
                            int thermo, double *dlog, int *counter) {
    if (thermo) {
        s->unhtss = (s->pss * s->pss * qqs) / 2.0 + ggs_treq * s->sss;
        s->ukin = s->sumv2 / 2.0;
        s->unhts = (s->ps * s->ps * qq) / 2.0 + gg_treq * s->ss;
    }
    s->tinst = 2.0 * s->ukin / nfree;
    double *row = dlog + (size_t)(*counter) * MG_MD_LOG;
    row[0] = s->ukin;
    row[4] = s->ps;
    row[5] = s->ss;
    row[6] = s->pss;
    row[7] = s->sss;
    row[8] = s->tinst;
    row[9] = s->unhts;
    row[10] = s->unhtss;
    *counter += 1;
}

// the raw energy components of one force call into the device log (slot `slot` of the
// current step) and its error flags into a word that keeps them for the whole run
__global__ void k_graph_energy(const double *__restrict__ eout, const unsigned *__restrict__ flags,
                               double *__restrict__ elog, const int *__restrict__ counter, int calls, int slot,
                               unsigned *__restrict__ sticky) {
    const int t = threadIdx.x;
    const size_t row = ((size_t)(*counter) * calls + slot) * E_NCOMP;
    if (t < E_NCOMP) elog[row + t] = eout[t];
    if (t == 0) *sticky |= flags[0];
}

// sum m v^2 / 2 of the current velocities into ukin (plain velocity Verlet, src/md.c:66-79)
__global__ void k_md_ukin_scalar(MdArgs A, int nb) {
    const double sumv2 = sum_partials(A.part, nb);
    if (threadIdx.x == 0) A.s->ukin = sumv2 * 0.5;
}

// ---- velinit (src/initvars.c:151-229) on counter-based streams ------------------------
// v = sqrt(treq / aw) g with g standard normal (Philox4x32-10, key = seed, counter =
// (site, stage, purpose 0/1, tag)); partials [4][nb] of aw v (x, y, z) and of aw
__global__ void k_vel_draw(MdArgs A, const double *__restrict__ aw, double treq, uint32_t k0, uint32_t k1,
                           uint32_t stage, uint32_t tag, int nb) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    double p[4] = {0.0, 0.0, 0.0, 0.0};
    if (a < A.n) {
        const uint32_t key[2] = {k0, k1};
        const uint32_t c0[4] = {(uint32_t)a, stage, 0u, tag}, c1[4] = {(uint32_t)a, stage, 1u, tag};
        uint32_t w0[4], w1[4];
        double g0, g1, g2, g3;
        mg_philox4x32_10(c0, key, w0);
        mg_philox4x32_10(c1, key, w1);
        mg_gauss2(w0, &g0, &g1);
        mg_gauss2(w1, &g2, &g3);
        const double m = aw[a], stdv = sqrt(treq) / sqrt(m);
        const double v[3] = {stdv * g0, stdv * g1, stdv * g2};
        for (int d = 0; d < 3; d++) {
            A.v[d * A.n + a] = v[d];
            p[d] = v[d] * m;
        }
        p[3] = m;
    }
    for (int k = 0; k < 4; k++) block_partial(p[k], A.part + (size_t)k * nb);
}

// momentum per unit mass of the system (the reference's px /= system_mass)
__global__ void k_vel_momentum(MdArgs A, int nb) {
    __shared__ double red[MD_TPB];
    double out[4];
    for (int k = 0; k < 4; k++) {
        double t = 0.0;
        for (int i = threadIdx.x; i < nb; i += MD_TPB) t += A.part[(size_t)k * nb + i];
        red[threadIdx.x] = t;
        __syncthreads();
        for (int o = MD_TPB / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        out[k] = red[0];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int d = 0; d < 3; d++) A.s->vel[d] = out[d] / out[3];
}

// v -= P/M; partial of aw v^2
__global__ void k_vel_shift(MdArgs A, const double *__restrict__ aw) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    double m2 = 0.0;
    if (a < A.n) {
        double s2 = 0.0;
        for (int d = 0; d < 3; d++) {
            const double v = A.v[d * A.n + a] - A.s->vel[d];
            A.v[d * A.n + a] = v;
            s2 += v * v;
        }
        m2 = aw[a] * s2;
    }
    block_partial(m2, A.part);
}

// ukin, tinst and the factor that rescales the temperature to treq exactly
__global__ void k_vel_scale_scalar(MdArgs A, int nb, double treq, double nfree) {
    const double s2 = sum_partials(A.part, nb);
    if (threadIdx.x != 0) return;
    const double ukin = 0.5 * s2, tinst = 2.0 * ukin / nfree;
    A.s->vel[3] = sqrt(treq / tinst);
}

// v *= scaling; partial of aw v^2 (the recomputed kinetic energy)
__global__ void k_vel_scale(MdArgs A, const double *__restrict__ aw) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    double m2 = 0.0;
    if (a < A.n) {
        const double sc = A.s->vel[3];
        double s2 = 0.0;
        for (int d = 0; d < 3; d++) {
            const double v = A.v[d * A.n + a] * sc;
            A.v[d * A.n + a] = v;
            s2 += v * v;
        }
        m2 = aw[a] * s2;
    }
    block_partial(m2, A.part);
}

// ---- NPT (src/nptnh.c) ------------------------------------------------------------
// partial of sum v^2 / r_mass (the operator's mvsq, src/nptnh.c:22-28)
__global__ void k_npt_mvsq(MdArgs A) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    double m2 = 0.0;
    if (a < A.n) {
        const int n = A.n;
        m2 = (A.v[a] * A.v[a] + A.v[n + a] * A.v[n + a] + A.v[2 * n + a] * A.v[2 * n + a]) / A.rmass[a];
    }
    block_partial(m2, A.part);
}

__global__ void k_npt_mvsq_scalar(MdArgs A, int nb) {
    const double t = sum_partials(A.part, nb);
    if (threadIdx.x == 0) A.s->sumv2 = t;
}

// v *= AA (src/nptnh.c:89-94)
__global__ void k_npt_scale_v(MdArgs A, double aa) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < 3 * A.n) A.v[a] = A.v[a] * aa;
}

// inner step of npt_respa (src/nptnh.c:155-176): v += hs fs r_mass, x = ((x AA) + dts v) AA
__global__ void k_npt_inner(MdArgs A, double hs, double dts, double aa) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A.n) return;
    const double r = A.rmass[a];
    const int n = A.n;
    double *pos[3] = {A.x, A.y, A.z};
    for (int d = 0; d < 3; d++) {
        const double v = A.v[d * n + a] + (hs * A.fs[d * n + a] * r);
        A.v[d * n + a] = v;
        double x = pos[d][a] * aa;
        x = x + dts * v;
        pos[d][a] = x * aa;
    }
}

// the thermostat scalars a new annealing stage starts from (src/siman.c:167-174)
__global__ void k_siman_reset(MdDev *s) {
    s->ps = s->ss = s->pss = s->sss = 0.0;
    s->unhts = s->unhtss = 0.0;
}

}  // namespace

// ---------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------
namespace {

struct MdRun {
    mg_ctx *c;
    MdArgs A;
    int nb;  // site blocks
    cudaStream_t s;
    int coop_grid = 0;  // blocks of the cooperative solve (0: the device cannot run it)
};

mg_status nh_solve(MdRun &R, const double *f, double h, double dt, double q, double g_treq, int inner) {
    mg_ctx *c = R.c;
    NhArgs N;
    N.f = f;
    N.h = h;
    N.dt = dt;
    N.q = q;
    N.g_treq = g_treq;
    N.inner = inner;
    if (R.coop_grid > 0) {
        int nb = R.nb;
        void *args[] = {(void *)&R.A, (void *)&N, (void *)&nb};
        // the FP64 path keeps the reference's joint iteration; the mixed path solves for ps alone
        const void *fn = c->opt.precision == MG_PREC_FP64 ? (const void *)k_nh_solve_coop : (const void *)k_nh_solve_scalar;
        MG_CUDA(cudaLaunchCooperativeKernel(fn, dim3(R.coop_grid), dim3(MD_TPB), args, 0, R.s));
        c->launches += 1;
        return MG_OK;
    }
    k_nh_start<<<R.nb, MD_TPB, 0, R.s>>>(R.A);
    k_nh_start_scalar<<<1, MD_TPB, 0, R.s>>>(R.A, R.nb, inner);
    c->launches += 2;
    for (int it = 0; it < MD_MAX_ITER; it += MD_ITER_BATCH) {
        for (int k = 0; k < MD_ITER_BATCH; k++) {
            k_nh_residual<<<R.nb, MD_TPB, 0, R.s>>>(R.A, N);
            k_nh_step_scalar<<<1, MD_TPB, 0, R.s>>>(R.A, N, R.nb);
            k_nh_update<<<R.nb, MD_TPB, 0, R.s>>>(R.A, N);
            k_nh_check_scalar<<<1, MD_TPB, 0, R.s>>>(R.A, R.nb);
        }
        c->launches += 4 * MD_ITER_BATCH;
        int ready = 0;
        MG_CUDA(cudaMemcpyAsync(&ready, &R.A.s->ready, sizeof(int), cudaMemcpyDeviceToHost, R.s));
        MG_CUDA(cudaStreamSynchronize(R.s));
        if (ready) break;
    }
    k_nh_finish<<<(3 * R.A.n + MD_TPB - 1) / MD_TPB, MD_TPB, 0, R.s>>>(R.A, inner);
    c->launches += 1;
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}

}  // namespace

namespace {

// buffers and the MdRun of an integration with log_rows per-step records
mg_status md_prepare(mg_ctx *c, size_t log_rows, MdRun &R) {
    const int n = c->natom;
    const size_t nb3 = sizeof(double) * 3 * (size_t)n;
    const int nb = (n + MD_TPB - 1) / MD_TPB;
    if (!mg_ensure(c, c->d_x, nb3) || !mg_ensure(c, c->d_fl, nb3) || !mg_ensure(c, c->d_fs, nb3) ||
        !mg_ensure(c, c->d_md_v, nb3) || !mg_ensure(c, c->d_md_work, 3 * nb3) ||
        !mg_ensure(c, c->d_md_rmass, sizeof(double) * n) ||
        !mg_ensure(c, c->d_md_part, sizeof(double) * (4 * (size_t)nb + 4)) ||
        !mg_ensure(c, c->d_md_dev, sizeof(MdDev)) ||
        !mg_ensure(c, c->d_md_log, sizeof(double) * MG_MD_LOG * log_rows))
        return MG_ERR_ALLOC;
    R.c = c;
    R.nb = nb;
    R.s = c->stream;
    {  // the cooperative solve needs every block of its grid resident at once
        int coop = 0, sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, c->device);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->device);
        int per_sm2 = 0;
        if (coop && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_nh_solve_coop, MD_TPB, 0) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, k_nh_solve_scalar, MD_TPB, 0) == cudaSuccess &&
            std::min(per_sm, per_sm2) > 0)
            R.coop_grid = std::min(nb, std::min(per_sm, per_sm2) * sms);
        cudaGetLastError();
    }
    MdArgs &A = R.A;
    double *w = (double *)c->d_md_work.p;
    A.n = n;
    A.x = (double *)c->d_x.p;
    A.y = A.x + n;
    A.z = A.y + n;
    A.v = (double *)c->d_md_v.p;
    A.vn = w;
    A.vo = w + 3 * (size_t)n;
    A.b = w + 6 * (size_t)n;
    A.rmass = (const double *)c->d_md_rmass.p;
    A.fl = (const double *)c->d_fl.p;
    A.fs = (const double *)c->d_fs.p;
    A.part = (double *)c->d_md_part.p;
    A.s = (MdDev *)c->d_md_dev.p;
    k_md_rmass<<<nb, MD_TPB, 0, R.s>>>(n, (const double *)c->d_site_aw.p, (double *)c->d_md_rmass.p);
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}

// nsteps of the scheme from the device state of R: forces at the start (as the reference
// evaluates them before its loop), the step-0 record and one record per step (device
// rows dlog; uinter, uintra and ushift of every row in hlog)
#define MD_GRAPH_FALLBACK 1000  // the graph path did not run the steps: run them eagerly

// Steps 1..nsteps by replaying one captured step. The device state at the start
// (positions, velocities, thermostat scalars) is saved first; if the capture cannot be
// made or a step of the replay raised a flag the eager loop handles (list or column
// capacity, small box, non-finite force, a site off its table), the start state is
// restored and MD_GRAPH_FALLBACK returned.
mg_status md_graph_steps(MdRun &R, const mg_md_params *mp, int nsteps, double *dlog, double *hlog) {
    mg_ctx *c = R.c;
    MdArgs &A = R.A;
    const int nb = R.nb, n = A.n;
    cudaStream_t s = R.s;
    double *dx = A.x, *dy = A.y, *dz = A.z;
    double *fl = (double *)c->d_fl.p, *fs = (double *)c->d_fs.p;
    const bool nh = mp->scheme == MG_MD_NVT_NH;
    const double dt = mp->delt, h = dt / 2.0, dts = dt / mp->nstep_inner, hs = dts / 2.0;
    const double dt_sqby2 = dt * dt / 2.0, dts_sqby2 = dts * dts / 2.0;
    const double gg_treq = mp->gg * mp->treq, ggs_treq = mp->ggs * mp->treq;
    const int calls = mp->nstep_inner + 1;
    const size_t elog_n = ((size_t)nsteps + 1) * calls * E_NCOMP;
    const size_t save_n = 6 * (size_t)n + (sizeof(MdDev) + 7) / 8;
    if (!mg_ensure(c, c->d_md_glog, sizeof(double) * (elog_n + save_n) + 64)) return MG_ERR_ALLOC;
    double *elog = (double *)c->d_md_glog.p, *save = elog + elog_n;
    int *counter = (int *)(save + save_n);
    unsigned *sticky = (unsigned *)(counter + 1);
    MG_CUDA(cudaMemcpyAsync(save, dx, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, s));
    MG_CUDA(cudaMemcpyAsync(save + 3 * (size_t)n, A.v, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, s));
    MG_CUDA(cudaMemcpyAsync(save + 6 * (size_t)n, A.s, sizeof(MdDev), cudaMemcpyDeviceToDevice, s));
    MG_CUDA(cudaMemsetAsync(counter, 0, 64, s));
    k_set_one<<<1, 1, 0, s>>>(counter);
    auto restore = [&]() -> mg_status {
        MG_CUDA(cudaMemcpyAsync(dx, save, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, s));
        MG_CUDA(cudaMemcpyAsync(A.v, save + 3 * (size_t)n, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, s));
        MG_CUDA(cudaMemcpyAsync(A.s, save + 6 * (size_t)n, sizeof(MdDev), cudaMemcpyDeviceToDevice, s));
        MG_CUDA(cudaStreamSynchronize(s));
        c->list_valid = false;
        return MD_GRAPH_FALLBACK;
    };
    // capture one step (the launches of the eager loop, in its order)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    mg_status st = MG_OK;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return restore();
    }
    k_md_kick<<<nb, MD_TPB, 0, s>>>(A, fl, h, nh ? 1 : 0, 0);
    for (int ll = 0; ll < mp->nstep_inner && !st; ll++) {
        k_md_inner_drift<<<nb, MD_TPB, 0, s>>>(A, hs, dts, nh ? 1 : 0);
        if (nh) k_md_inner_predict<<<1, MD_TPB, 0, s>>>(A, nb, ggs_treq, dts, dts_sqby2, hs, mp->qqs);
        if ((st = mg_enqueue_forces(c, dx, dy, dz, MG_TERMS_SHORT, fl, fs))) break;
        k_graph_energy<<<1, 32 * ((E_NCOMP + 31) / 32), 0, s>>>((const double *)c->d_eout.p,
                                                                (const unsigned *)c->d_flags.p, elog, counter, calls,
                                                                ll, sticky);
        if (nh) {
            if ((st = nh_solve(R, fs, hs, dts, mp->qqs, ggs_treq, 1))) break;
        } else {
            k_md_kick<<<nb, MD_TPB, 0, s>>>(A, fs, hs, 0, 0);
        }
    }
    if (!st) {
        if (nh) k_md_outer_predict<<<1, 1, 0, s>>>(A.s, gg_treq, dt, dt_sqby2, h, mp->qq);
        st = mg_enqueue_forces(c, dx, dy, dz, MG_TERMS_LONG, fl, fs);
    }
    if (!st) {
        k_graph_energy<<<1, 32 * ((E_NCOMP + 31) / 32), 0, s>>>((const double *)c->d_eout.p,
                                                                (const unsigned *)c->d_flags.p, elog, counter, calls,
                                                                mp->nstep_inner, sticky);
        if (nh) {
            st = nh_solve(R, fl, h, dt, mp->qq, gg_treq, 0);
            if (!st)
                k_graph_row<<<1, 1, 0, s>>>(A.s, mp->qq, mp->qqs, gg_treq, ggs_treq, (double)mp->nfree, 1, dlog,
                                            counter);
        } else {
            k_md_kick<<<nb, MD_TPB, 0, s>>>(A, fl, h, 0, 1);
            k_md_ukin_scalar<<<1, MD_TPB, 0, s>>>(A, nb);
            k_graph_row<<<1, 1, 0, s>>>(A.s, mp->qq, mp->qqs, gg_treq, ggs_treq, (double)mp->nfree, 0, dlog,
                                        counter);
        }
    }
    const cudaError_t ce = cudaStreamEndCapture(s, &graph);
    cudaGetLastError();
    if (st || ce != cudaSuccess || !graph ||
        cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
        cudaGetLastError();
        if (graph) cudaGraphDestroy(graph);
        return restore();
    }
    bool launched = true;
    for (int step = 1; step <= nsteps && launched; step++) launched = cudaGraphLaunch(exec, s) == cudaSuccess;
    unsigned flags = 0;
    std::vector<double> E((size_t)(nsteps + 1) * calls * E_NCOMP);
    if (launched) {
        MG_CUDA(cudaMemcpyAsync(&flags, sticky, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaMemcpyAsync(E.data(), elog, sizeof(double) * E.size(), cudaMemcpyDeviceToHost, s));
        launched = cudaStreamSynchronize(s) == cudaSuccess;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    c->launches += 1;
    const unsigned bad = MG_FLAG_OUT_OF_GRID | MG_FLAG_NONFINITE | MG_FLAG_LIST_OVERFLOW | MG_FLAG_COLUMN_OVERFLOW |
                         MG_FLAG_SMALL_BOX | MG_FLAG_IMPROPER_DEGENERATE | MG_FLAG_WAIT_TIMEOUT |
                         MG_FLAG_MMA_UNDRAINED | MG_FLAG_FIXED_RANGE;
    if (!launched || (flags & bad)) {
        cudaGetLastError();
        return restore();
    }
    // the energies of every step, as the eager loop records them
    for (int step = 1; step <= nsteps; step++) {
        mg_energies el, es;
        mg_assemble_energies(c, &E[((size_t)step * calls + mp->nstep_inner) * E_NCOMP], 1, 0, &el);
        mg_assemble_energies(c, &E[((size_t)step * calls + mp->nstep_inner - 1) * E_NCOMP], 0, 1, &es);
        hlog[(size_t)step * MG_MD_LOG + 1] = el.uinter + es.uinter;
        hlog[(size_t)step * MG_MD_LOG + 2] = es.uintra;
        hlog[(size_t)step * MG_MD_LOG + 3] = el.ushift + es.ushift;
    }
    c->md_graph_steps = nsteps;
    return MG_OK;
}

mg_status md_loop(MdRun &R, const mg_md_params *mp, int nsteps, double *dlog, double *hlog, bool traj_steps) {
    mg_ctx *c = R.c;
    MdArgs &A = R.A;
    const int nb = R.nb;
    cudaStream_t s = R.s;
    double *dx = A.x, *dy = A.y, *dz = A.z;
    double *fl = (double *)c->d_fl.p, *fs = (double *)c->d_fs.p;
    const bool nh = mp->scheme == MG_MD_NVT_NH;
    const double dt = mp->delt, h = dt / 2.0, dts = dt / mp->nstep_inner, hs = dts / 2.0;
    const double dt_sqby2 = dt * dt / 2.0, dts_sqby2 = dts * dts / 2.0;
    const double gg_treq = mp->gg * mp->treq, ggs_treq = mp->ggs * mp->treq;
    MG_CUDA(cudaMemsetAsync(dlog, 0, sizeof(double) * MG_MD_LOG * ((size_t)nsteps + 1), s));
    mg_energies e;
    mg_status st = mg_compute_forces(c, dx, dy, dz, MG_TERMS_ALL, fl, fs, &e);
    if (st) return st;
    // with a distance split the short call also returns the inner pairs' share of
    // uinter and ushift; the record holds the sum of both buckets
    double uinter_l = e.uinter, uinter_s = 0.0, ushift_l = e.ushift, ushift_s = 0.0, uintra = e.uintra;
    // step 0 record: kinetic energy of the given velocities
    k_nh_start<<<nb, MD_TPB, 0, s>>>(A);
    k_md_ukin_scalar<<<1, MD_TPB, 0, s>>>(A, nb);
    k_md_step_scalars<<<1, 1, 0, s>>>(A.s, nb, mp->qq, mp->qqs, gg_treq, ggs_treq, (double)mp->nfree, 0, dlog);
    hlog[1] = uinter_l;
    hlog[2] = uintra;
    hlog[3] = ushift_l;
    c->md_graph_steps = 0;
    // whole steps as a replayed graph where possible: no trajectory frames to hand to the
    // host between steps, and the thermostat solve as one cooperative launch
    if (c->md_graphs && nsteps >= 2 && !(traj_steps && c->traj) && (!nh || R.coop_grid > 0)) {
        st = md_graph_steps(R, mp, nsteps, dlog, hlog);
        if (st != MD_GRAPH_FALLBACK) return st;
        // the start state is back: forces at the start again, then the eager loop
        if ((st = mg_compute_forces(c, dx, dy, dz, MG_TERMS_ALL, fl, fs, &e))) return st;
    }
    for (int step = 1; step <= nsteps; step++) {
        k_md_kick<<<nb, MD_TPB, 0, s>>>(A, fl, h, nh ? 1 : 0, 0);
        for (int ll = 0; ll < mp->nstep_inner; ll++) {
            k_md_inner_drift<<<nb, MD_TPB, 0, s>>>(A, hs, dts, nh ? 1 : 0);
            if (nh) k_md_inner_predict<<<1, MD_TPB, 0, s>>>(A, nb, ggs_treq, dts, dts_sqby2, hs, mp->qqs);
            MG_CUDA(cudaGetLastError());
            if ((st = mg_compute_forces(c, dx, dy, dz, MG_TERMS_SHORT, fl, fs, &e))) return st;
            uintra = e.uintra;
            uinter_s = e.uinter;
            ushift_s = e.ushift;
            if (nh) {
                if ((st = nh_solve(R, fs, hs, dts, mp->qqs, ggs_treq, 1))) return st;
            } else {
                k_md_kick<<<nb, MD_TPB, 0, s>>>(A, fs, hs, 0, 0);
            }
        }
        if (nh) k_md_outer_predict<<<1, 1, 0, s>>>(A.s, gg_treq, dt, dt_sqby2, h, mp->qq);
        MG_CUDA(cudaGetLastError());
        if ((st = mg_compute_forces(c, dx, dy, dz, MG_TERMS_LONG, fl, fs, &e))) return st;
        uinter_l = e.uinter;
        ushift_l = e.ushift;
        double *row = dlog + (size_t)step * MG_MD_LOG;
        if (nh) {
            if ((st = nh_solve(R, fl, h, dt, mp->qq, gg_treq, 0))) return st;
            k_md_step_scalars<<<1, 1, 0, s>>>(A.s, nb, mp->qq, mp->qqs, gg_treq, ggs_treq, (double)mp->nfree, 1, row);
        } else {
            k_md_kick<<<nb, MD_TPB, 0, s>>>(A, fl, h, 0, 1);
            k_md_ukin_scalar<<<1, MD_TPB, 0, s>>>(A, nb);
            k_md_step_scalars<<<1, 1, 0, s>>>(A.s, nb, mp->qq, mp->qqs, gg_treq, ggs_treq, (double)mp->nfree, 0, row);
        }
        MG_CUDA(cudaGetLastError());
        hlog[(size_t)step * MG_MD_LOG + 1] = uinter_l + uinter_s;
        hlog[(size_t)step * MG_MD_LOG + 2] = uintra;
        hlog[(size_t)step * MG_MD_LOG + 3] = ushift_l + ushift_s;
        if (traj_steps && (st = mg_traj_tick(c, dx))) return st;
    }
    return MG_OK;
}

// merges the device rows with the host-side energies into the caller's log
void md_merge_log(const double *dl, const double *hlog, size_t rows, double *log) {
    for (size_t r = 0; r < rows; r++) {
        double *o = log + r * MG_MD_LOG;
        const double *d = dl + r * MG_MD_LOG;
        for (int k = 0; k < MG_MD_LOG; k++) o[k] = d[k];
        o[1] = hlog[r * MG_MD_LOG + 1];
        o[2] = hlog[r * MG_MD_LOG + 2];
        o[3] = hlog[r * MG_MD_LOG + 3];
    }
}

mg_status md_check(mg_ctx *c, const mg_md_params *mp) {
    if (mp->scheme != MG_MD_NVE && mp->scheme != MG_MD_NVT_NH)
        return mg_fail(c, MG_ERR_INVALID, "unknown integration scheme");
    if (mp->nstep_inner < 1 || !(mp->delt > 0) || !(mp->nfree > 0))
        return mg_fail(c, MG_ERR_INVALID, "nstep_inner, delt and nfree must be positive");
    if (mp->scheme == MG_MD_NVT_NH && !(mp->qq > 0 && mp->qqs > 0))
        return mg_fail(c, MG_ERR_INVALID, "thermostat masses must be positive");
    if (!c->have_topology || !c->have_params || !c->have_box)
        return mg_fail(c, MG_ERR_STATE, "set topology, params and box before integrating");
    return MG_OK;
}

}  // namespace

extern "C" mg_status mg_md_run(mg_ctx *c, const mg_md_params *mp, int nsteps, double *x, double *y, double *z,
                               double *vx, double *vy, double *vz, mg_md_state *state, double *log) {
    if (!c || !mp || !state || nsteps < 0 || !x || !y || !z || !vx || !vy || !vz) return MG_ERR_INVALID;
    mg_status st = md_check(c, mp);
    if (st) return st;
    cudaSetDevice(c->device);
    const int n = c->natom;
    MdRun R;
    if ((st = md_prepare(c, (size_t)nsteps + 1, R))) return st;
    cudaStream_t s = R.s;
    double *dlog = (double *)c->d_md_log.p;
    const size_t nb1 = sizeof(double) * n;
    MG_CUDA(cudaMemcpyAsync(R.A.x, x, nb1, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(R.A.y, y, nb1, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(R.A.z, z, nb1, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(R.A.v, vx, nb1, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(R.A.v + n, vy, nb1, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(R.A.v + 2 * n, vz, nb1, cudaMemcpyHostToDevice, s));
    MdDev h0 = {};
    h0.ps = state->ps;
    h0.ss = state->ss;
    h0.pss = state->pss;
    h0.sss = state->sss;
    h0.unhts = state->unhts;
    h0.unhtss = state->unhtss;
    MG_CUDA(cudaMemcpyAsync(c->d_md_dev.p, &h0, sizeof(MdDev), cudaMemcpyHostToDevice, s));
    std::vector<double> hlog(MG_MD_LOG * ((size_t)nsteps + 1), 0.0);
    if ((st = mg_traj_start(c, R.A.x))) return st;
    if ((st = md_loop(R, mp, nsteps, dlog, hlog.data(), true))) return st;
    MG_CUDA(cudaMemcpyAsync(x, R.A.x, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(y, R.A.y, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(z, R.A.z, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(vx, R.A.v, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(vy, R.A.v + n, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(vz, R.A.v + 2 * n, nb1, cudaMemcpyDeviceToHost, s));
    MdDev hf;
    MG_CUDA(cudaMemcpyAsync(&hf, c->d_md_dev.p, sizeof(MdDev), cudaMemcpyDeviceToHost, s));
    std::vector<double> dl(hlog.size());
    MG_CUDA(cudaMemcpyAsync(dl.data(), dlog, sizeof(double) * dl.size(), cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    MG_CUDA(cudaGetLastError());
    state->ps = hf.ps;
    state->ss = hf.ss;
    state->pss = hf.pss;
    state->sss = hf.sss;
    state->ukin = hf.ukin;
    state->tinst = hf.tinst;
    state->unhts = hf.unhts;
    state->unhtss = hf.unhtss;
    if (log) md_merge_log(dl.data(), hlog.data(), (size_t)nsteps + 1, log);
    return MG_OK;
}

// ---------------------------------------------------------------------------------
// simulated annealing (src/siman.c:62-182): stages at T = t_initial / mu_t^k, each a
// velinit at T, forces, n_tries Nose-Hoover RESPA steps and a reset of the thermostat
// scalars; the run ends after the first stage whose T is below t_min.
// ---------------------------------------------------------------------------------
#define MG_SIMAN_TAG 0x5349u  // fourth Philox counter word of the annealing velocities

extern "C" int mg_siman_stage_count(double t_initial, double t_min, double mu_t, int limit) {
    if (!(t_initial > 0) || !(mu_t > 1.0) || !(t_min >= 0) || limit < 1) return -1;
    double T = t_initial;
    for (int k = 0; k < limit; k++) {
        if (T < t_min) return k + 1;
        T /= mu_t;
    }
    return -1;
}

extern "C" mg_status mg_siman_run(mg_ctx *c, const mg_siman_params *sp, double *x, double *y, double *z,
                                  double *vx, double *vy, double *vz, mg_md_state *state, int *nstages,
                                  double *stage_log) {
    if (!c || !sp || !state || !nstages || !x || !y || !z || !vx || !vy || !vz) return MG_ERR_INVALID;
    if (sp->md.scheme != MG_MD_NVT_NH) return mg_fail(c, MG_ERR_INVALID, "annealing runs the Nose-Hoover scheme");
    if (sp->n_tries < 0) return mg_fail(c, MG_ERR_INVALID, "n_tries must not be negative");
    mg_md_params mp = sp->md;
    mp.treq = sp->t_initial;
    mg_status st = md_check(c, &mp);
    if (st) return st;
    const int nst = mg_siman_stage_count(sp->t_initial, sp->t_min, sp->mu_t, sp->max_stages);
    if (nst < 0)
        return mg_fail(c, MG_ERR_CAPACITY, "the schedule needs more than max_stages stages (or is invalid)");
    cudaSetDevice(c->device);
    const int n = c->natom;
    MdRun R;
    if ((st = md_prepare(c, (size_t)sp->n_tries + 1, R))) return st;
    cudaStream_t s = R.s;
    double *dlog = (double *)c->d_md_log.p;
    const size_t nb1 = sizeof(double) * n;
    MG_CUDA(cudaMemcpyAsync(R.A.x, x, nb1, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(R.A.y, y, nb1, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(R.A.z, z, nb1, cudaMemcpyHostToDevice, s));
    MdDev h0 = {};
    h0.ps = state->ps;
    h0.ss = state->ss;
    h0.pss = state->pss;
    h0.sss = state->sss;
    h0.unhts = state->unhts;
    h0.unhtss = state->unhtss;
    MG_CUDA(cudaMemcpyAsync(c->d_md_dev.p, &h0, sizeof(MdDev), cudaMemcpyHostToDevice, s));
    const double *aw = (const double *)c->d_site_aw.p;
    const uint32_t k0 = (uint32_t)(sp->seed & 0xffffffffull), k1 = (uint32_t)(sp->seed >> 32);
    std::vector<double> hlog(MG_MD_LOG * ((size_t)sp->n_tries + 1), 0.0), last(MG_MD_LOG);
    double T = sp->t_initial;
    for (int k = 0; k < nst; k++) {
        mp.treq = T;
        if (k > 0) k_siman_reset<<<1, 1, 0, s>>>(R.A.s);
        k_vel_draw<<<R.nb, MD_TPB, 0, s>>>(R.A, aw, T, k0, k1, (uint32_t)k, MG_SIMAN_TAG, R.nb);
        k_vel_momentum<<<1, MD_TPB, 0, s>>>(R.A, R.nb);
        k_vel_shift<<<R.nb, MD_TPB, 0, s>>>(R.A, aw);
        k_vel_scale_scalar<<<1, MD_TPB, 0, s>>>(R.A, R.nb, T, (double)mp.nfree);
        k_vel_scale<<<R.nb, MD_TPB, 0, s>>>(R.A, aw);
        MG_CUDA(cudaGetLastError());
        c->launches += 6;
        if ((st = md_loop(R, &mp, sp->n_tries, dlog, hlog.data(), false))) return st;
        if ((st = mg_traj_tick(c, R.A.x))) return st;  // one step of the reference's loop per stage
        MG_CUDA(cudaMemcpyAsync(last.data(), dlog + (size_t)sp->n_tries * MG_MD_LOG, sizeof(double) * MG_MD_LOG,
                                cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaStreamSynchronize(s));
        if (stage_log) {
            double *o = stage_log + (size_t)k * MG_SIMAN_LOG;
            const double *hl = hlog.data() + (size_t)sp->n_tries * MG_MD_LOG;
            o[0] = T;
            o[1] = last[0];   // ukin
            o[2] = hl[1];     // uinter
            o[3] = hl[2];     // uintra
            o[4] = hl[3];     // ushift
            o[5] = last[8];   // tinst
            o[6] = last[9];   // unhts
            o[7] = last[10];  // unhtss
        }
        T /= sp->mu_t;
    }
    MG_CUDA(cudaMemcpyAsync(x, R.A.x, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(y, R.A.y, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(z, R.A.z, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(vx, R.A.v, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(vy, R.A.v + n, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(vz, R.A.v + 2 * n, nb1, cudaMemcpyDeviceToHost, s));
    MdDev hf;
    MG_CUDA(cudaMemcpyAsync(&hf, c->d_md_dev.p, sizeof(MdDev), cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    MG_CUDA(cudaGetLastError());
    state->ps = hf.ps;
    state->ss = hf.ss;
    state->pss = hf.pss;
    state->sss = hf.sss;
    state->ukin = hf.ukin;
    state->tinst = hf.tinst;
    state->unhts = hf.unhts;
    state->unhtss = hf.unhtss;
    *nstages = nst;
    return MG_OK;
}

// ---------------------------------------------------------------------------------
// NPT: npt_respa (src/nptnh.c:134-234) around npt_nh_operator (src/nptnh.c:10-132). The
// operator's scalar updates are a handful of FP64 operations on the host, in the
// reference's order, from sum m v^2 reduced on the device; the host also owns the box,
// which changes every inner step (list, k-vectors and Ewald constants follow it).
// ---------------------------------------------------------------------------------
namespace {

struct NptScalars {
    double vts, vbs, rts, utsbs, ukin, tinst, pinst, pljlrc;
};

// the LJ long-range pressure correction (src/misc.c:131-148) with the species-pair terms
// of src/initvars.c:476-520
double npt_pljlrc(const mg_ctx *c, int lj_lrc, double boxv) {
    if (!lj_lrc) return 0.0;
    const double pi = 3.141592653589793, rc = c->params.rcutoff;
    const double t1 = (32.0 / 9.0) * pi * pow(rc, -9.0), t2 = -(16.0 / 3.0) * pi * pow(rc, -3.0);
    double p = 0.0;
    for (int m = 0; m < c->nspecies; m++)
        for (int nn = 0; nn < c->nspecies; nn++) {
            double term = 0.0;
            for (size_t i = 0; i < c->h_tmpl_sig[m].size(); i++)
                for (size_t j = 0; j < c->h_tmpl_sig[nn].size(); j++) {
                    const double sij = 0.5 * (c->h_tmpl_sig[m][i] + c->h_tmpl_sig[nn][j]);
                    const double eij = sqrt(c->h_tmpl_eps[m][i] * c->h_tmpl_eps[nn][j]);
                    term += (pow(sij, 9.0) * t1 + pow(sij, 3.0) * t2) * (eij * pow(sij, 3.0));
                }
            p += (term * c->species[m].nmole * c->species[nn].nmole / boxv / boxv);
        }
    return p;
}

mg_status npt_operator(MdRun &R, const mg_npt_params *mp, double virial, double boxv, NptScalars &q) {
    mg_ctx *c = R.c;
    k_npt_mvsq<<<R.nb, MD_TPB, 0, R.s>>>(R.A);
    k_npt_mvsq_scalar<<<1, MD_TPB, 0, R.s>>>(R.A, R.nb);
    double mvsq = 0.0;
    MG_CUDA(cudaMemcpyAsync(&mvsq, &R.A.s->sumv2, sizeof(double), cudaMemcpyDeviceToHost, R.s));
    MG_CUDA(cudaStreamSynchronize(R.s));
    const double nfree = mp->nfree, treq = mp->treq, qts = mp->qts, qbs = mp->qbs, preq = mp->preq;
    const double N_plus1RT = (nfree + 1) * treq, one_3N = 1.0 + 3.0 / nfree;
    const double dt_outer2 = mp->delt / 2.0, dt_outer4 = mp->delt / 4.0, dt_outer8 = mp->delt / 8.0;
    const double pdiff = virial + q.pljlrc * boxv * 3.0 - preq * boxv * 3.0;
    double Gts = (mvsq + qbs * q.vbs * q.vbs - N_plus1RT) / qts;
    q.vts = q.vts + dt_outer4 * Gts;
    const double BB = exp(-q.vts * dt_outer8);
    q.vbs = q.vbs * BB;
    double Gbs = (one_3N * mvsq + pdiff) / qbs;
    q.vbs = q.vbs + dt_outer4 * Gbs;
    q.vbs = q.vbs * BB;
    q.rts = q.rts + dt_outer2 * q.vts;
    const double AA = exp(-dt_outer2 * (q.vts + one_3N * q.vbs));
    k_npt_scale_v<<<(3 * R.A.n + MD_TPB - 1) / MD_TPB, MD_TPB, 0, R.s>>>(R.A, AA);
    MG_CUDA(cudaGetLastError());
    c->launches += 3;
    q.vbs = q.vbs * BB;
    mvsq = mvsq * AA * AA;
    Gbs = (one_3N * mvsq + pdiff) / qbs;
    q.vbs = q.vbs + dt_outer4 * Gbs;
    q.vbs = q.vbs * BB;
    Gts = (mvsq + qbs * q.vbs * q.vbs - N_plus1RT) / qts;
    q.vts = q.vts + dt_outer4 * Gts;
    q.utsbs = 0.5 * qbs * q.vbs * q.vbs + 0.5 * qts * q.vts * q.vts + (nfree + 1) * treq * q.rts + preq * boxv;
    q.ukin = mvsq / 2.0;
    q.tinst = 2.0 * q.ukin / nfree;
    q.pinst = R.A.n / boxv * q.tinst + virial / 3.0 / boxv + q.pljlrc;
    return MG_OK;
}

// the new box and the box constants the reference refreshes (src/nptnh.c:178-199)
void npt_set_box(mg_ctx *c, double lx, double ly, double lz) {
    const double pi = 3.141592653589793;
    c->lx = lx;
    c->ly = ly;
    c->lz = lz;
    c->list_valid = false;
    const double boxv = lx * ly * lz;
    if (c->params.charge_type == MG_ELEC_EWALD) {
        c->params.vfactor_ewald = 2.0 * pi / boxv;
        c->params.twopi_lx = 2.0 * pi / lx;
        c->params.twopi_ly = 2.0 * pi / ly;
        c->params.twopi_lz = 2.0 * pi / lz;
        c->params.twopi_over_3v = 2.0 * pi / 3.0 / boxv;
    }
}

void npt_record(double *row, const NptScalars &q, const mg_energies &el, const mg_energies &es, double lx,
                double boxv) {
    if (!row) return;
    const double r[MG_NPT_LOG] = {q.ukin,  el.uinter + es.uinter, es.uintra, el.ushift + es.ushift,
                                  q.vts,   q.vbs,                 q.rts,     q.utsbs,
                                  q.tinst, q.pinst,               lx,        boxv};
    for (int k = 0; k < MG_NPT_LOG; k++) row[k] = r[k];
}

}  // namespace

extern "C" mg_status mg_npt_run(mg_ctx *c, const mg_npt_params *mp, int nsteps, double *x, double *y, double *z,
                                double *vx, double *vy, double *vz, double *box, mg_npt_state *state, double *log) {
    if (!c || !mp || !state || !box || nsteps < 0 || !x || !y || !z || !vx || !vy || !vz) return MG_ERR_INVALID;
    if (mp->nstep_inner < 1 || !(mp->delt > 0) || !(mp->nfree > 0) || !(mp->qts > 0 && mp->qbs > 0))
        return mg_fail(c, MG_ERR_INVALID, "nstep_inner, delt, nfree and the masses must be positive");
    if (!(box[0] > 0 && box[1] > 0 && box[2] > 0)) return mg_fail(c, MG_ERR_INVALID, "box lengths must be positive");
    if (!c->have_topology || !c->have_params)
        return mg_fail(c, MG_ERR_STATE, "set topology and params before integrating");
    cudaSetDevice(c->device);
    const int n = c->natom;
    MdRun R;
    mg_status st = md_prepare(c, 1, R);
    if (st) return st;
    cudaStream_t s = R.s;
    const size_t nb1 = sizeof(double) * n;
    MG_CUDA(cudaMemcpyAsync(R.A.x, x, nb1, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(R.A.y, y, nb1, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(R.A.z, z, nb1, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(R.A.v, vx, nb1, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(R.A.v + n, vy, nb1, cudaMemcpyHostToDevice, s));
    MG_CUDA(cudaMemcpyAsync(R.A.v + 2 * n, vz, nb1, cudaMemcpyHostToDevice, s));
    npt_set_box(c, box[0], box[1], box[2]);
    c->have_box = true;
    double *fl = (double *)c->d_fl.p, *fs = (double *)c->d_fs.p;
    const double h = mp->delt / 2.0, dts = mp->delt / mp->nstep_inner, hs = dts / 2.0;
    double boxv = c->lx * c->ly * c->lz;
    NptScalars q = {};
    q.vts = state->vts;
    q.vbs = state->vbs;
    q.rts = state->rts;
    q.pljlrc = npt_pljlrc(c, mp->lj_lrc, boxv);
    mg_energies el, es;
    if ((st = mg_compute_forces(c, R.A.x, R.A.y, R.A.z, MG_TERMS_ALL, fl, fs, &el))) return st;
    es = el;
    el.uintra = 0.0;
    es.uinter = es.ushift = es.virial_inter = 0.0;
    {  // start record: kinetic energy of the given velocities, pressure of the start forces
        k_npt_mvsq<<<R.nb, MD_TPB, 0, s>>>(R.A);
        k_npt_mvsq_scalar<<<1, MD_TPB, 0, s>>>(R.A, R.nb);
        double mvsq = 0.0;
        MG_CUDA(cudaMemcpyAsync(&mvsq, &R.A.s->sumv2, sizeof(double), cudaMemcpyDeviceToHost, s));
        MG_CUDA(cudaStreamSynchronize(s));
        q.ukin = mvsq / 2.0;
        q.tinst = 2.0 * q.ukin / mp->nfree;
        q.utsbs = 0.5 * mp->qbs * q.vbs * q.vbs + 0.5 * mp->qts * q.vts * q.vts +
                  (mp->nfree + 1) * mp->treq * q.rts + mp->preq * boxv;
        q.pinst = n / boxv * q.tinst + (el.virial_inter + es.virial_intra) / 3.0 / boxv + q.pljlrc;
        npt_record(log, q, el, es, c->lx, boxv);
    }
    if ((st = mg_traj_start(c, R.A.x))) return st;
    for (int step = 1; step <= nsteps; step++) {
        if ((st = npt_operator(R, mp, el.virial_inter + es.virial_inter + es.virial_intra, boxv, q))) return st;
        k_md_kick<<<R.nb, MD_TPB, 0, s>>>(R.A, fl, h, 0, 0);
        for (int ll = 0; ll < mp->nstep_inner; ll++) {
            const double AA = exp(hs * q.vbs);
            k_npt_inner<<<R.nb, MD_TPB, 0, s>>>(R.A, hs, dts, AA);
            MG_CUDA(cudaGetLastError());
            c->launches += 1;
            const double ef = exp(dts * q.vbs);
            npt_set_box(c, c->lx * ef, c->ly * ef, c->lz * ef);
            boxv = c->lx * c->ly * c->lz;
            q.pljlrc = npt_pljlrc(c, mp->lj_lrc, boxv);
            if ((st = mg_compute_forces(c, R.A.x, R.A.y, R.A.z, MG_TERMS_SHORT, fl, fs, &es))) return st;
            k_md_kick<<<R.nb, MD_TPB, 0, s>>>(R.A, fs, hs, 0, 0);
        }
        if ((st = mg_compute_forces(c, R.A.x, R.A.y, R.A.z, MG_TERMS_LONG, fl, fs, &el))) return st;
        k_md_kick<<<R.nb, MD_TPB, 0, s>>>(R.A, fl, h, 0, 0);
        MG_CUDA(cudaGetLastError());
        if ((st = npt_operator(R, mp, el.virial_inter + es.virial_inter + es.virial_intra, boxv, q))) return st;
        npt_record(log ? log + (size_t)step * MG_NPT_LOG : nullptr, q, el, es, c->lx, boxv);
        if ((st = mg_traj_tick(c, R.A.x))) return st;
    }
    MG_CUDA(cudaMemcpyAsync(x, R.A.x, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(y, R.A.y, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(z, R.A.z, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(vx, R.A.v, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(vy, R.A.v + n, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaMemcpyAsync(vz, R.A.v + 2 * n, nb1, cudaMemcpyDeviceToHost, s));
    MG_CUDA(cudaStreamSynchronize(s));
    MG_CUDA(cudaGetLastError());
    box[0] = c->lx;
    box[1] = c->ly;
    box[2] = c->lz;
    state->vts = q.vts;
    state->vbs = q.vbs;
    state->rts = q.rts;
    state->utsbs = q.utsbs;
    state->ukin = q.ukin;
    state->tinst = q.tinst;
    state->pinst = q.pinst;
    return MG_OK;
}
