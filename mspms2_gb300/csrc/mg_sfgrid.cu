// mg_sfgrid.cu - solid-fluid potential grids on the GPU: the tables that the my-interp
// and Tasos solid-fluid models interpolate (src/sffrc.c:149-222, :228-748).
//
// The reference builds them on the CPU with tools/sfgridgen.c:71-354 (energy, gradient
// and second derivatives of the Lennard-Jones solid-fluid energy on a regular grid over
// one unit cell, the cell periodic in z only); the generator of the Tasos tables (F,
// Dx, Dy, Dz, Dxy, Dxz, Dyz, Dxyz per node, mylibtasos/grid.f90:81-93) is not part of the
// reference. One thread evaluates one node: it sums over the cell's solid atoms (staged
// in shared memory) and their z images, in the reference's order (images outer, atoms
// inner), with the pair energy written as g(s), s = r^2:
//   g(s) = 4 eps_sf ((sig_sf^2/s)^6 - (sig_sf^2/s)^3) S(s),
// S the reference's energy switch (1 inside rcuton), so that
//   dU/dx_a = 2 d_a g'(s),  d2U/dx_a dx_b = 4 d_a d_b g''(s) + 2 delta_ab g'(s),
//   d3U/dx dy dz = 8 d_x d_y d_z g'''(s)  (d = fluid - solid position).
// Sums are FP64, or FP32 pair terms carried in exact FP32 hi+lo pairs (MG_PREC_MIXED).
//
// Deviation: with the switch on, tools/sfgridgen.c:268-270 leaves the second
// derivatives of pairs between rcuton and rcutoff unassigned (the previous pair's, or
// uninitialised, values are added); here they are the derivatives of the switched
// energy.
#include <math.h>

#include "mg_internal.cuh"

#define SG_TPB 128
#define SG_MAX_SOLID 2048  // solid atoms per cell held in shared memory

namespace {

struct SgArgs {
    int nsolid;
    const double *solid;  // [3][nsolid]
    double uclz;
    int nimg;             // images -nimg..nimg in z
    double sig2, eps4;    // sig_sf^2 and 4 eps_sf (output energy unit)
    double ron2, roff2, swd;
    int lj_switch;
    int tasos;            // 0: sfgridgen layout and fields, 1: Tasos layout and fields
    int nx, ny, nz;
    double x0, y0, z0, hx, hy, hz;
    double *out;          // sfgridgen: [13][nx*ny*nz]; Tasos: [nz][ny][nx][8]
    float *out_f32;       // Tasos table written in FP32 instead (the mixed path's layout)
    double *blockmin;     // per-block minimum of F (Tasos), or null
};

// g, g', g'', g''' of the switched LJ term at s = r^2 (derivatives with respect to s)
template <typename R>
__device__ __forceinline__ void lj_s_derivs(R s, R sig2, R eps4, R ron2, R roff2, R swd, int sw, R (&g)[4]) {
    const R is = (R)1 / s, a3 = sig2 * sig2 * sig2 * is * is * is, a6 = a3 * a3;
    // u = eps4 (a6 - a3); d/ds of a6 = -6 a6/s, of a3 = -3 a3/s
    R u0 = eps4 * (a6 - a3);
    R u1 = eps4 * (-6 * a6 + 3 * a3) * is;
    R u2 = eps4 * (42 * a6 - 12 * a3) * is * is;
    R u3 = eps4 * (-336 * a6 + 60 * a3) * is * is * is;
    if (sw && !(s < ron2)) {
        // S = (c - s)^2 (c + 2 s - 3 b) / D, a cubic in s
        const R c = roff2, b = ron2, t = c - s, w = c + 2 * s - 3 * b;
        const R S0 = t * t * w / swd;
        const R S1 = (-2 * t * w + 2 * t * t) / swd;
        const R S2 = (2 * w - 8 * t) / swd;
        const R S3 = (R)12 / swd;
        g[0] = u0 * S0;
        g[1] = u1 * S0 + u0 * S1;
        g[2] = u2 * S0 + 2 * u1 * S1 + u0 * S2;
        g[3] = u3 * S0 + 3 * u2 * S1 + 3 * u1 * S2 + u0 * S3;
    } else {
        g[0] = u0;
        g[1] = u1;
        g[2] = u2;
        g[3] = u3;
    }
}

template <typename R>
__device__ double sfgrid_node(const SgArgs &A, const double (*ss)[SG_MAX_SOLID], long long t);

template <typename R>
__global__ void __launch_bounds__(SG_TPB) k_sfgrid(SgArgs A) {
    __shared__ double ss[3][SG_MAX_SOLID];
    for (int i = threadIdx.x; i < A.nsolid; i += SG_TPB) {
        ss[0][i] = A.solid[i];
        ss[1][i] = A.solid[A.nsolid + i];
        ss[2][i] = A.solid[2 * A.nsolid + i];
    }
    __syncthreads();
    const long long nn = (long long)A.nx * A.ny * A.nz;
    const long long t = (long long)blockIdx.x * SG_TPB + threadIdx.x;
    if (A.blockmin) {  // every thread takes part in the block minimum below
        double f0 = 10e10;  // the initial minPE of mylibtasos/grid.f90:75-97
        if (t < nn) f0 = sfgrid_node<R>(A, ss, t);
        __syncthreads();            // the solid atoms are no longer read:
        double *smin = &ss[0][0];   // their first SG_TPB entries hold the block's minima
        smin[threadIdx.x] = f0;
        __syncthreads();
        for (int o = SG_TPB / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
            __syncthreads();
        }
        if (threadIdx.x == 0) A.blockmin[blockIdx.x] = smin[0];
        return;
    }
    if (t >= nn) return;
    sfgrid_node<R>(A, ss, t);
}

// one node: sums over the solid atoms and their z images, writes the node's values and
// returns F
template <typename R>
__device__ double sfgrid_node(const SgArgs &A, const double (*ss)[SG_MAX_SOLID], long long t) {
    const long long nn = (long long)A.nx * A.ny * A.nz;
    int ix, iy, iz;
    if (A.tasos) {  // I fastest
        ix = (int)(t % A.nx);
        iy = (int)((t / A.nx) % A.ny);
        iz = (int)(t / ((long long)A.nx * A.ny));
    } else {        // ii*ny*nz + jj*nz + kk
        iz = (int)(t % A.nz);
        iy = (int)((t / A.nz) % A.ny);
        ix = (int)(t / ((long long)A.ny * A.nz));
    }
    const double fx = A.x0 + A.hx * ix, fy = A.y0 + A.hy * iy, fz = A.z0 + A.hz * iz;
    const R sig2 = (R)A.sig2, eps4 = (R)A.eps4, ron2 = (R)A.ron2, roff2 = (R)A.roff2, swd = (R)A.swd;
    // accumulators (hi + lo): energy, gradient [3], second derivatives [6: xx yy zz xy xz yz], xyz
    R hi[11], lo[11];
#pragma unroll
    for (int k = 0; k < 11; k++) hi[k] = lo[k] = (R)0;
    for (int p = -A.nimg; p <= A.nimg; p++) {
        const double zs = p * A.uclz;
        for (int a = 0; a < A.nsolid; a++) {
            const R dx = (R)(fx - ss[0][a]), dy = (R)(fy - ss[1][a]);
            const R dz = (R)(fz - ss[2][a] + zs);
            const R s = dx * dx + dy * dy + dz * dz;
            if (!(s < roff2)) continue;
            R g[4];
            lj_s_derivs<R>(s, sig2, eps4, ron2, roff2, swd, A.lj_switch, g);
            const R g1x2 = 2 * g[1], g2x4 = 4 * g[2];
            const R v[11] = {g[0],
                             g1x2 * dx, g1x2 * dy, g1x2 * dz,
                             g2x4 * dx * dx + g1x2, g2x4 * dy * dy + g1x2, g2x4 * dz * dz + g1x2,
                             g2x4 * dx * dy, g2x4 * dx * dz, g2x4 * dy * dz,
                             8 * g[3] * dx * dy * dz};
#pragma unroll
            for (int k = 0; k < 11; k++) mg_acc2(hi[k], lo[k], v[k]);
        }
    }
    double r[11];
#pragma unroll
    for (int k = 0; k < 11; k++) r[k] = (double)hi[k] + (double)lo[k];
    if (A.tasos) {  // F, Dx, Dy, Dz, Dxy, Dxz, Dyz, Dxyz
        const double v[8] = {r[0], r[1], r[2], r[3], r[7], r[8], r[9], r[10]};
        if (A.out_f32) {
            float *o = A.out_f32 + 8 * t;
            for (int k = 0; k < 8; k++) o[k] = (float)v[k];
        } else {
            double *o = A.out + 8 * t;
            for (int k = 0; k < 8; k++) o[k] = v[k];
        }
    } else {  // Ene, dEx, dEy, dEz, dF = -Hessian: xx xy xz yx yy yz zx zy zz
        const double v[13] = {r[0], r[1], r[2], r[3], -r[4], -r[7], -r[8], -r[7], -r[5], -r[9], -r[8], -r[9], -r[6]};
        for (int k = 0; k < 13; k++) A.out[(size_t)k * nn + t] = v[k];
    }
    return r[0];
}

mg_status run_grid(int device, const mg_sfgrid_spec *sp, SgArgs A, int precision, double *host_out, size_t out_doubles) {
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return MG_ERR_NO_DEVICE;
    }
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device);
    if (major != 10 || minor != 3) return MG_ERR_NO_DEVICE;
    int prev = 0;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return MG_ERR_CUDA;
    }
    mg_status st = MG_OK;
    double *d_solid = nullptr, *d_out = nullptr;
    const size_t ns = (size_t)sp->nsolid;
    std::vector<double> solid(3 * ns);
    for (size_t i = 0; i < ns; i++) {
        solid[i] = sp->sx[i];
        solid[ns + i] = sp->sy[i];
        solid[2 * ns + i] = sp->sz[i];
    }
    cudaStream_t s = nullptr;
    const long long nn = (long long)A.nx * A.ny * A.nz;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&d_solid, sizeof(double) * 3 * (ns ? ns : 1)) != cudaSuccess ||
        cudaMalloc(&d_out, sizeof(double) * out_doubles) != cudaSuccess) {
        st = MG_ERR_ALLOC;
    } else {
        cudaMemcpyAsync(d_solid, solid.data(), sizeof(double) * 3 * ns, cudaMemcpyHostToDevice, s);
        A.solid = d_solid;
        A.out = d_out;
        const unsigned blocks = (unsigned)((nn + SG_TPB - 1) / SG_TPB);
        if (precision == MG_PREC_FP64)
            k_sfgrid<double><<<blocks, SG_TPB, 0, s>>>(A);
        else
            k_sfgrid<float><<<blocks, SG_TPB, 0, s>>>(A);
        cudaMemcpyAsync(host_out, d_out, sizeof(double) * out_doubles, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) st = MG_ERR_CUDA;
    }
    cudaGetLastError();
    if (d_solid) cudaFree(d_solid);
    if (d_out) cudaFree(d_out);
    if (s) cudaStreamDestroy(s);
    cudaSetDevice(prev);
    return st;
}

SgArgs base_args(const mg_sfgrid_spec *sp, double eps_unit) {
    SgArgs A = {};
    A.nsolid = sp->nsolid;
    A.uclz = sp->uclz;
    int nimg = 1;  // tools/sfgridgen.c:137-140
    while (nimg * sp->uclz < sp->rcutoff) nimg++;
    A.nimg = nimg;
    const double sig = (sp->f_sigma + sp->s_sigma) / 2.0;
    A.sig2 = sig * sig;
    A.eps4 = 4.0 * sqrt(sp->f_epsilon * sp->s_epsilon) * eps_unit;
    A.ron2 = sp->rcuton * sp->rcuton;
    A.roff2 = sp->rcutoff * sp->rcutoff;
    const double d = A.roff2 - A.ron2;
    A.swd = d * d * d;
    A.lj_switch = sp->lj_switch;
    return A;
}

bool spec_ok(const mg_sfgrid_spec *sp) {
    return sp && sp->nsolid >= 0 && sp->nsolid <= SG_MAX_SOLID && (sp->nsolid == 0 || (sp->sx && sp->sy && sp->sz)) &&
           sp->uclx > 0 && sp->ucly > 0 && sp->uclz > 0 && sp->rcutoff > 0 &&
           (!sp->lj_switch || (sp->rcuton >= 0 && sp->rcuton < sp->rcutoff));
}

}  // namespace

extern "C" mg_status mg_sfgrid_sfgridgen(int device, const mg_sfgrid_spec *sp, double itvl, int precision, int *dims,
                                        double *out) {
    if (!spec_ok(sp) || !(itvl > 0) || !dims) return MG_ERR_INVALID;
    // tools/sfgridgen.c:129-131 and :143-153
    dims[0] = (int)floor(sp->uclx / itvl) + 2;
    dims[1] = (int)floor(sp->ucly / itvl) + 2;
    dims[2] = (int)floor(sp->uclz / itvl) + 2;
    if (!out) return MG_OK;
    SgArgs A = base_args(sp, 8.314472);  // J/mol (Rgas, tools/sfgridgen.c:126)
    A.tasos = 0;
    A.nx = dims[0];
    A.ny = dims[1];
    A.nz = dims[2];
    A.x0 = sp->uclx / 2.0 - sp->uclx / 2.0;
    A.y0 = sp->ucly / 2.0 - sp->ucly / 2.0;
    A.z0 = 0.0;
    A.hx = A.hy = A.hz = itvl;
    return run_grid(device, sp, A, precision, out, 13 * (size_t)dims[0] * dims[1] * dims[2]);
}

extern "C" mg_status mg_sfgrid_tasos(int device, const mg_sfgrid_spec *sp, int nx, int ny, int nz, double hx,
                                    double hy, double hz, int precision, double *values) {
    if (!spec_ok(sp) || nx < 2 || ny < 2 || nz < 2 || !(hx > 0 && hy > 0 && hz > 0) || !values)
        return MG_ERR_INVALID;
    SgArgs A = base_args(sp, 1.0);  // K
    A.tasos = 1;
    A.nx = nx;
    A.ny = ny;
    A.nz = nz;
    A.x0 = A.y0 = A.z0 = 0.0;
    A.hx = hx;
    A.hy = hy;
    A.hz = hz;
    return run_grid(device, sp, A, precision, values, 8 * (size_t)nx * ny * nz);
}

namespace {
__global__ void k_min_reduce(const double *__restrict__ in, int n, double *__restrict__ out) {
    __shared__ double smin[256];
    double m = 10e10;
    for (int i = threadIdx.x; i < n; i += 256) m = fmin(m, in[i]);
    smin[threadIdx.x] = m;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) smin[threadIdx.x] = fmin(smin[threadIdx.x], smin[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = smin[0];
}
}  // namespace

// A Tasos table evaluated on the device straight into the context's table `type`: the
// same values as mg_sfgrid_tasos followed by mg_sf_tasos_set_grid, without the round
// trip through host memory (1.3 GB per FP32 table for a 0.1 A grid over a 127 A bundle
// cell). The table's minimum F (the PE flip threshold) is reduced on the device.
extern "C" mg_status mg_sf_tasos_generate(mg_ctx *c, int type, const mg_sfgrid_spec *sp, int nx, int ny, int nz,
                                         double hx, double hy, double hz, double cuc) {
    if (!c || type < 1 || type > 64 || !spec_ok(sp) || nx < 3 || ny < 3 || nz < 3 || !(hx > 0 && hy > 0 && hz > 0) ||
        !(cuc > 0))
        return c ? mg_fail(c, MG_ERR_INVALID, "invalid Tasos grid") : MG_ERR_INVALID;
    cudaSetDevice(c->device);
    if ((int)c->tasos.size() < type) {
        c->tasos.resize(type);
        c->tasos_buf.resize(type);
    }
    const bool fp64 = c->opt.precision == MG_PREC_FP64;
    const size_t nn = (size_t)nx * ny * nz;
    DevBuf &buf = mg_tasos_storage(c, type);
    if (!mg_ensure(c, buf, (fp64 ? sizeof(double) : sizeof(float)) * 8 * nn)) return MG_ERR_ALLOC;
    SgArgs A = base_args(sp, 1.0);  // K
    A.tasos = 1;
    A.nx = nx;
    A.ny = ny;
    A.nz = nz;
    A.x0 = A.y0 = A.z0 = 0.0;
    A.hx = hx;
    A.hy = hy;
    A.hz = hz;
    if (fp64) A.out = (double *)buf.p;
    else A.out_f32 = (float *)buf.p;
    const size_t ns = (size_t)sp->nsolid;
    std::vector<double> solid(3 * (ns ? ns : 1));
    for (size_t i = 0; i < ns; i++) {
        solid[i] = sp->sx[i];
        solid[ns + i] = sp->sy[i];
        solid[2 * ns + i] = sp->sz[i];
    }
    const unsigned blocks = (unsigned)((nn + SG_TPB - 1) / SG_TPB);
    double *d_solid = nullptr, *d_min = nullptr;
    cudaStream_t s = c->stream;
    mg_status st = MG_OK;
    if (cudaMalloc(&d_solid, sizeof(double) * solid.size()) != cudaSuccess ||
        cudaMalloc(&d_min, sizeof(double) * ((size_t)blocks + 1)) != cudaSuccess) {
        st = MG_ERR_ALLOC;
    } else {
        double mn = 0.0;
        cudaMemcpyAsync(d_solid, solid.data(), sizeof(double) * solid.size(), cudaMemcpyHostToDevice, s);
        A.solid = d_solid;
        A.blockmin = d_min;
        // the same arithmetic precision as mg_sfgrid_tasos with the context's precision
        if (fp64) k_sfgrid<double><<<blocks, SG_TPB, 0, s>>>(A);
        else k_sfgrid<float><<<blocks, SG_TPB, 0, s>>>(A);
        k_min_reduce<<<1, 256, 0, s>>>(d_min, (int)blocks, d_min + blocks);
        cudaMemcpyAsync(&mn, d_min + blocks, sizeof(double), cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
            st = MG_ERR_CUDA;
        } else {
            TasosDev &t = c->tasos[type - 1];
            t.nx = nx;
            t.ny = ny;
            t.nz = nz;
            t.hx = hx;
            t.hy = hy;
            t.hz = hz;
            t.cuc = cuc;
            t.min_pe = mn;
            t.values = buf.p;
        }
    }
    if (d_solid) cudaFree(d_solid);
    if (d_min) cudaFree(d_min);
    if (st) return mg_fail(c, st, "Tasos grid generation failed");
    if (!mg_ensure(c, c->d_tasos, sizeof(TasosDev) * c->tasos.size())) return MG_ERR_ALLOC;
    MG_CUDA(cudaMemcpy(c->d_tasos.p, c->tasos.data(), sizeof(TasosDev) * c->tasos.size(), cudaMemcpyHostToDevice));
    return MG_OK;
}
