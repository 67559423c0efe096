// mg_ewald.cu - Ewald reciprocal space (src/frclong.c:988-1048).
//
// The reference sums, for every k = (kx*TWOPI_LX, ky*TWOPI_LY, kz*TWOPI_LZ) with
// 0 < kx^2+ky^2+kz^2 <= KSQMAX and |k_d| <= KMAX_d, S(k) = sum_j q_j e^{i k.r_j} and then
// U = Vfactor*C * sum_k exp(-B k^2)/k^2 |S(k)|^2 and
// F_i = sum_k 2 q_i Im(conj(S) e^{i k.r_i}) Vfactor*C*exp(-B k^2)/k^2 * k.
// Here only the half space (kx > 0, or kx = 0 and ky > 0, or kx = ky = 0 and kz > 0)
// is evaluated; S(-k) = conj S(k) gives the other half, so energy and forces carry a
// factor 2.
//
// Phases: u_d = frac(x_d * TWOPI_L_d / 2pi) is turned once per site into a 32-bit (mixed)
// or 64-bit (FP64 path) fixed-point fraction U; n*U modulo 2^32 (2^64) is then the exact
// phase of harmonic n, so e^{2 pi i n u} = sincospi(2 n U / 2^32) needs no range reduction
// and no recurrence. Tables per site: X[0..KMAXX], Y[0..KMAXY], Z[0..KMAXZ].
//
// k-vectors are grouped in rows (kx, ky) holding |kz| = 0..kzmax(kx,ky) with both signs
// of kz. Structure factors, mixed path: k_sk_mma runs the sum over sites as FP16 MMAs on
// the tensor cores ((row, Re/Im of q X Y) x site against site x (|kz|, Re/Im of Z), 3-term
// split products, accumulators in tensor memory); k_sk2 is the CUDA-core form (KMAXZ > 30,
// or the tensor pass off): a thread owns (row, up to 8 consecutive |kz|) = up to 16
// k-vectors, chunks balanced per row; tasks are sorted by length and each length group
// padded to whole warps, so a warp runs one unrolled loop; the block stages tiles of
// site tables in shared memory and sums its EW_SITES sites in R. Either way a fixed-order
// FP64 reduction over site blocks gives S(k) (deterministic).
// Forces: for one site and one row the kz sums are two complex polynomials in Z = e^{i
// theta_z}, P(Z) = sum_a conj(c S+_a) Z^a and Q(Z) = sum_a c S-_a Z^a, and the z force
// needs their derivatives; all four are evaluated by Horner's rule (16 FMA per |kz|, no
// power recurrence). Four thread groups share the rows of a site; their partial forces
// are combined in shared memory in a fixed order.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <numeric>
#include <type_traits>

#include <cuda_fp16.h>

#include "mg_internal.cuh"

#define EW_TILE 32      // sites per shared-memory tile in the S(k) pass
#ifndef EW_CH
#define EW_CH 8         // |kz| values per thread in the S(k) pass (at most; even)
#endif
#define EW_TPB 128      // threads per block in the S(k) pass
#define EW_SITES 512    // sites per block in the S(k) pass (summed in R)
#define EW_FROWS 32     // rows staged per step in the force pass
#define EW_FG 4         // thread groups sharing the rows of a site in the force pass
#define EW_FSITES 64    // sites per force block (EW_FG * EW_FSITES threads)
#ifndef EW_FCHUNK
#define EW_FCHUNK 8     // rows per chunk of the FP32 table force pass (accumulators per site)
#endif
#ifndef EW_SK2_MINB
#define EW_SK2_MINB 3   // resident blocks per SM the FP32 S(k) pass is compiled for
#endif
#ifndef EW_FMM_NS
#define EW_FMM_NS 2     // sites per thread of the table force pass
#endif
#ifndef EW_FMM_MINB
#define EW_FMM_MINB 4   // resident blocks per SM the table force pass is compiled for
#endif
#define EW_FMM_TPB 128  // sites (threads) per block of the FP32 table force pass
#define EW_FMM_MAXA 64  // largest kzmax + 1 the table force pass stages on chip
#define EW_MAXSPLIT 16  // row-chunk ranges of the FP32 table force pass

namespace {

template <typename R>
struct C2;
template <>
struct C2<float> {
    typedef float2 T;
    typedef float4 T4;
};
template <>
struct C2<double> {
    typedef double2 T;
    typedef double4 T4;
};

template <typename T>
__device__ __forceinline__ T cmul(T a, T b) {
    T r;
    r.x = a.x * b.x - a.y * b.y;
    r.y = a.x * b.y + a.y * b.x;
    return r;
}

// x <- x*z + c
template <typename T>
__device__ __forceinline__ T cfma(T x, T z, T c) {
    T r;
    r.x = fma(x.x, z.x, fma(-x.y, z.y, c.x));
    r.y = fma(x.x, z.y, fma(x.y, z.x, c.y));
    return r;
}

// Two FP32 lanes in one 64-bit register for the packed f32x2 arithmetic of sm_100 and
// later (one instruction, two independent IEEE round-to-nearest results).
typedef unsigned long long f32x2;

__device__ __forceinline__ f32x2 pk2(float lo, float hi) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}

__device__ __forceinline__ void up2(f32x2 v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}

// a*b + c per lane
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// f += q t (2 pi / L) with each operation rounded on its own (no contraction into an
// FMA), so that adding the same increment later, from a separate buffer, gives the same
// bits as adding it here
__device__ __forceinline__ void ew_addf(double *f, double q, double t, double tw) {
    *f = __dadd_rn(*f, __dmul_rn(__dmul_rn(q, t), tw));
}

// FP32 phase tables: X [KMAXX + 1][n] and Y [KMAXY + 1][n] as float2 e^{2 pi i k u}, then,
// from the first 16-byte boundary, Z as |kz| pairs [(KMAXZ + 2) / 2][n] of
// {zr_2p, zr_2p+1, zi_2p, zi_2p+1} (zero past KMAXZ), so that one 16-byte load gives a
// site's two |kz| in the lanes of the packed f32x2 sums.
__host__ __device__ inline int ew_zpairs(int KZ) { return (KZ + 2) / 2; }
__host__ __device__ inline size_t ew_zoff(int KX, int KY, int n) { return ((size_t)(KX + 1 + KY + 1) * n + 1) & ~(size_t)1; }
__host__ __device__ inline size_t ew_tabf_entries(int KX, int KY, int KZ, int n) {
    return ew_zoff(KX, KY, n) + (size_t)2 * ew_zpairs(KZ) * n;  // float2 units
}

__device__ __forceinline__ float2 ew_phase_f(unsigned U, int k) {
    const unsigned V = U * (unsigned)k;
    const float v = (float)(int)V * 4.656612873077393e-10f;  // 2^-31
    float s, c;
    sincospif(v, &s, &c);
    return make_float2(c, s);
}

// one thread per (site, axis), the axis blockIdx.y (0: X, 1: Y, 2: the Z pairs): three
// times the threads of one thread per site, each with a third of the serial work
__global__ void k_phase_f(int n, const double *__restrict__ x, const double *__restrict__ y,
                          const double *__restrict__ z, double sx, double sy, double sz, int kx, int ky, int kz,
                          float2 *__restrict__ tab) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x, d = blockIdx.y;
    if (a >= n) return;
    double t = d == 0 ? x[a] * sx : d == 1 ? y[a] * sy : z[a] * sz;
    t = t - floor(t);
    const double tu = t * 4294967296.0;
    const unsigned U = tu >= 4294967295.0 ? 0xffffffffu : (unsigned)tu;
    if (d == 0) {
        for (int k = 0; k <= kx; k++) tab[(size_t)k * n + a] = ew_phase_f(U, k);
    } else if (d == 1) {
        for (int k = 0; k <= ky; k++) tab[(size_t)(kx + 1 + k) * n + a] = ew_phase_f(U, k);
    } else {
        float4 *zp = (float4 *)(tab + ew_zoff(kx, ky, n));
        for (int p = 0; p < ew_zpairs(kz); p++) {
            const float2 z0 = ew_phase_f(U, 2 * p);
            const float2 z1 = 2 * p + 1 <= kz ? ew_phase_f(U, 2 * p + 1) : make_float2(0.f, 0.f);
            zp[(size_t)p * n + a] = make_float4(z0.x, z1.x, z0.y, z1.y);
        }
    }
}

// Z^1 of site a from either precision's tables
template <typename R>
__device__ inline typename C2<R>::T ew_z1(const void *tab, int kx, int ky, int n, int a);
template <>
__device__ inline float2 ew_z1<float>(const void *tab, int kx, int ky, int n, int a) {
    const float4 v = ((const float4 *)((const float2 *)tab + ew_zoff(kx, ky, n)))[a];
    return make_float2(v.y, v.w);
}
template <>
__device__ inline double2 ew_z1<double>(const void *tab, int kx, int ky, int n, int a) {
    return ((const double2 *)tab)[(size_t)(kx + 1 + ky + 1 + 1) * n + a];
}

__global__ void k_phase_d(int n, const double *__restrict__ x, const double *__restrict__ y,
                          const double *__restrict__ z, double sx, double sy, double sz, int kx, int ky, int kz,
                          double2 *__restrict__ tab) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const double pos[3] = {x[a], y[a], z[a]};
    const double sc[3] = {sx, sy, sz};
    const int km[3] = {kx, ky, kz};
    size_t off = 0;
    for (int d = 0; d < 3; d++) {
        double t = pos[d] * sc[d];
        t = t - floor(t);
        unsigned long long U = __double2ull_rz(t * 18446744073709551616.0);
        for (int k = 0; k <= km[d]; k++) {
            unsigned long long V = U * (unsigned long long)k;
            double v = (double)(long long)V * 1.0842021724855044e-19;  // 2^-63
            double s, c;
            sincospi(v, &s, &c);
            tab[off + (size_t)k * n + a] = make_double2(c, s);
        }
        off += (size_t)(km[d] + 1) * n;
    }
}

// largest |kz| of row (kx, ky): min(KZ, floor(sqrt(rem))), rem = KSQMAX - kx^2 - ky^2 >= 0
__host__ __device__ inline int ew_kzmax(int KZ, int rem) {
    int k = 0;
    while (k + 1 <= KZ && (k + 1) * (k + 1) <= rem) k++;
    return k;
}

// Visits the half-space rows, f(kx, ky, kzmax, half), in the order every table uses:
// (kx, -ky), (kx, ky) for kx, ky >= 1; then (j, 0), (0, j) for j >= 1; then (0, 0). Both
// rows of each of the first pairs have the same KSQMAX - kx^2 - ky^2, hence the same
// kzmax, and so do (j, 0) and (0, j): rows 2u and 2u+1 form the units of the packed
// force pass, of equal length unless KMAXX != KMAXY leaves one of (j, 0), (0, j) out.
// (host and device callers each pass their own callables)
#pragma nv_exec_check_disable
template <typename F>
__host__ __device__ inline void ew_visit_row(int KZ, int KS, int kx, int ky, F &f) {
    const int rem = KS - kx * kx - ky * ky;
    if (rem < 0) return;
    const int half = (kx == 0 && ky == 0) ? 1 : 0;
    const int kzmax = ew_kzmax(KZ, rem);
    if (half && kzmax < 1) return;
    f(kx, ky, kzmax, half);
}

#pragma nv_exec_check_disable
template <typename F>
__host__ __device__ inline void ew_for_rows(int KX, int KY, int KZ, int KS, F f) {
    for (int kx = 1; kx <= KX; kx++)
        for (int ky = 1; ky <= KY; ky++) {
            ew_visit_row(KZ, KS, kx, -ky, f);
            ew_visit_row(KZ, KS, kx, ky, f);
        }
    const int J = KX > KY ? KX : KY;
    for (int j = 1; j <= J; j++) {
        if (j <= KX) ew_visit_row(KZ, KS, j, 0, f);
        if (j <= KY) ew_visit_row(KZ, KS, 0, j, f);
    }
    ew_visit_row(KZ, KS, 0, 0, f);
}

// Chunks of the S(k) pass for a row with nv |kz| values: the pairs (0, 1), (2, 3), ...
// split into ceil(pairs / (EW_CH / 2)) balanced runs, so that chunk h starts at an even
// |kz| and holds at most EW_CH |kz| values (k0, len).
__host__ __device__ inline int ew_nchunk(int nv) { return ((nv + 1) / 2 + EW_CH / 2 - 1) / (EW_CH / 2); }
__host__ __device__ inline void ew_chunk(int nv, int h, int &k0, int &len) {
    const int np = (nv + 1) / 2, nch = (np + EW_CH / 2 - 1) / (EW_CH / 2);
    const int p0 = h * (np / nch) + (h < np % nch ? h : np % nch);
    const int pl = np / nch + (h < np % nch ? 1 : 0);
    k0 = 2 * p0;
    len = 2 * pl < nv - k0 ? 2 * pl : nv - k0;
}

struct EwArgs {
    int n, nrows, nslots, ntasks;
    int kx, ky, kz;  // KMAX per axis (table extents)
    const int4 *rows;       // kx, ky, kzmax, half_only
    const int *row_slot;    // first slot of each row (two slots per |kz|: +kz, -kz)
    const int4 *tasks;      // row, first |kz|, count, -
    const void *tab;
    const double *q;
    float *qf;              // [n] FP32 copy of q for the FP32 S(k) pass
    void *spart;            // [site blocks][nslots][2] R
    void *scoef;            // [nslots] R2: plus slots conj(c S), minus slots c S
    double twopi[3];
    double bfac, vfac, coul;
    double *rows_e;
    int row0;
    double *f;
    // FP32 table force pass: rows by kzmax (longest first) in chunks of EW_FCHUNK; the
    // chunk coefficients start at coff[chunk] * EW_FCHUNK in fcoef; block row y of the
    // grid takes chunks [csplit[y], csplit[y + 1]) and, if fsplit > 1, writes its partial
    // forces to fpart[y][3][n]
    const int *forder;  // [nrows] row at each force-order position
    const int *rpos;    // [nrows] force-order position of each row
    const int *coff;    // [nchunk + 1]
    int nchunk, fsplit;
    int csplit[EW_MAXSPLIT + 1];
    float4 *fcoef;
    double *fpart;
    // status word of the call (MG_FLAG_*): the tensor-core S(k) pass sets its bits, the
    // S(k) reduction reads them (coefficients and energy turn NaN after a give-up)
    const unsigned *flags;
    long long mma_wait;  // polls of each pipeline wait of the tensor-core S(k) pass
};

// One tile of sites for a thread owning CH consecutive |kz| of one row (FP64 path):
// straight-line code, A*Z and A*conj(Z) sharing four products, Z advanced by the site's Z1.
template <typename R, int CH, typename T2>
__device__ __forceinline__ void sk_tile(const T2 *sX, const T2 *sY, const T2 *sZ, const R *sQ, int P, int tn,
                                        int kx, int aky, R ysign, int kz0, R (&pP)[EW_CH][2], R (&pM)[EW_CH][2]) {
    {
        for (int s = 0; s < tn; s++) {
            T2 X = sX[kx * P + s];
            T2 Y = sY[aky * P + s];
            Y.y *= ysign;
            const R q = sQ[s];
            T2 Aq = cmul(X, Y);
            Aq.x *= q;
            Aq.y *= q;
            T2 Z = sZ[kz0 * P + s];
            const T2 Z1 = sZ[1 * P + s];
#pragma unroll
            for (int j = 0; j < CH; j++) {
                const R p1 = Aq.x * Z.x, p2 = Aq.y * Z.y, p3 = Aq.x * Z.y, p4 = Aq.y * Z.x;
                pP[j][0] += p1 - p2;
                pP[j][1] += p3 + p4;
                pM[j][0] += p1 + p2;
                pM[j][1] += p4 - p3;
                if (j + 1 < CH) Z = cmul(Z, Z1);
            }
        }
    }
}

// Structure-factor partials of one block of EW_SITES sites, summed in R (the block sum
// of this stage); the cross-block sum is done in FP64 by k_sk_reduce. Task counts are
// uniform within a warp (tasks sorted by count and padded per count to whole warps),
// so the switch below does not diverge.
template <typename R>
__global__ void __launch_bounds__(EW_TPB) k_sk(EwArgs A) {
    typedef typename C2<R>::T T2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T2 *sX = (T2 *)smem_raw;
    const int P = EW_TILE + 1;  // padded tile pitch
    T2 *sY = sX + (size_t)(A.kx + 1) * P;
    T2 *sZ = sY + (size_t)(A.ky + 1) * P;
    R *sQ = (R *)(sZ + (size_t)(A.kz + 1) * P);
    const T2 *tab = (const T2 *)A.tab;
    const T2 *tX = tab, *tY = tab + (size_t)(A.kx + 1) * A.n, *tZ = tY + (size_t)(A.ky + 1) * A.n;
    const int task = blockIdx.x * EW_TPB + threadIdx.x;
    int kx = 0, ky = 0, half = 0, kz0 = 0, cnt = 0, slot0 = 0;
    if (task < A.ntasks) {
        int4 t = A.tasks[task];
        int4 r = A.rows[t.x];
        kx = r.x;
        ky = r.y;
        half = r.w;
        kz0 = t.y;
        cnt = t.z;
        slot0 = A.row_slot[t.x];
    }
    const int aky = ky < 0 ? -ky : ky;
    const R ysign = ky < 0 ? (R)-1 : (R)1;
    R pP[EW_CH][2], pM[EW_CH][2];
#pragma unroll
    for (int j = 0; j < EW_CH; j++) pP[j][0] = pP[j][1] = pM[j][0] = pM[j][1] = (R)0;
    const int a_begin = blockIdx.y * EW_SITES, a_end = min(A.n, a_begin + EW_SITES);
    for (int t0 = a_begin; t0 < a_end; t0 += EW_TILE) {
        const int tn = min(EW_TILE, a_end - t0);
        __syncthreads();
        for (int i = threadIdx.x; i < (A.kx + 1) * EW_TILE; i += EW_TPB) {
            int k = i / EW_TILE, s = i % EW_TILE;
            if (s < tn) sX[k * P + s] = tX[(size_t)k * A.n + t0 + s];
        }
        for (int i = threadIdx.x; i < (A.ky + 1) * EW_TILE; i += EW_TPB) {
            int k = i / EW_TILE, s = i % EW_TILE;
            if (s < tn) sY[k * P + s] = tY[(size_t)k * A.n + t0 + s];
        }
        for (int i = threadIdx.x; i < (A.kz + 1) * EW_TILE; i += EW_TPB) {
            int k = i / EW_TILE, s = i % EW_TILE;
            if (s < tn) sZ[k * P + s] = tZ[(size_t)k * A.n + t0 + s];
        }
        for (int s = threadIdx.x; s < tn; s += EW_TPB) sQ[s] = (R)A.q[t0 + s];
        __syncthreads();
        switch (cnt) {
#if EW_CH >= 12
        case 12: sk_tile<R, 12>(sX, sY, sZ, sQ, P, tn, kx, aky, ysign, kz0, pP, pM); break;
        case 11: sk_tile<R, 11>(sX, sY, sZ, sQ, P, tn, kx, aky, ysign, kz0, pP, pM); break;
#endif
#if EW_CH >= 10
        case 10: sk_tile<R, 10>(sX, sY, sZ, sQ, P, tn, kx, aky, ysign, kz0, pP, pM); break;
        case 9: sk_tile<R, 9>(sX, sY, sZ, sQ, P, tn, kx, aky, ysign, kz0, pP, pM); break;
#endif
        case 8: sk_tile<R, 8>(sX, sY, sZ, sQ, P, tn, kx, aky, ysign, kz0, pP, pM); break;
        case 7: sk_tile<R, 7>(sX, sY, sZ, sQ, P, tn, kx, aky, ysign, kz0, pP, pM); break;
        case 6: sk_tile<R, 6>(sX, sY, sZ, sQ, P, tn, kx, aky, ysign, kz0, pP, pM); break;
        case 5: sk_tile<R, 5>(sX, sY, sZ, sQ, P, tn, kx, aky, ysign, kz0, pP, pM); break;
        case 4: sk_tile<R, 4>(sX, sY, sZ, sQ, P, tn, kx, aky, ysign, kz0, pP, pM); break;
        case 3: sk_tile<R, 3>(sX, sY, sZ, sQ, P, tn, kx, aky, ysign, kz0, pP, pM); break;
        case 2: sk_tile<R, 2>(sX, sY, sZ, sQ, P, tn, kx, aky, ysign, kz0, pP, pM); break;
        case 1: sk_tile<R, 1>(sX, sY, sZ, sQ, P, tn, kx, aky, ysign, kz0, pP, pM); break;
        default: break;
        }
    }
    if (task >= A.ntasks || cnt == 0) return;
    R *out = (R *)A.spart + (size_t)blockIdx.y * A.nslots * 2;
#pragma unroll
    for (int j = 0; j < EW_CH; j++) {
        if (j >= cnt) break;
        int a = kz0 + j;
        int sp = slot0 + 2 * a, sm = sp + 1;
        out[2 * sp] = pP[j][0];
        out[2 * sp + 1] = pP[j][1];
        bool has_minus = (a > 0) && !half;
        out[2 * sm] = has_minus ? pM[j][0] : (R)0;
        out[2 * sm + 1] = has_minus ? pM[j][1] : (R)0;
    }
}

// FP32 structure factors from the phase tables. A thread owns one task (row, |kz| from
// an even k0, at most EW_CH values): per site, with Aq = q X^kx Y^ky and z = Z^|kz| from
// the table, the four real sums RR = sum Ar zr, II = sum Ai zi, RI = sum Ar zi and
// IR = sum Ai zr give S(+kz) = (RR - II, RI + IR) and S(-kz) = (RR + II, IR - RI): 4 FMAs
// per site and |kz| for both signs. The lanes of the packed f32x2 sums are |kz| = k,
// k + 1; the tile stages Z as [site][pair]{zr_k, zr_k+1, zi_k, zi_k+1} (zero past KMAXZ).
template <int NP>
__device__ __forceinline__ void sk2_tile(const ulonglong2 *sZ, const float2 *sX, const float2 *sY, const float *sQ,
                                         int NPP, int P, int tn, int kx, int aky, float ysign, int p0,
                                         f32x2 (&RR)[EW_CH / 2], f32x2 (&II)[EW_CH / 2], f32x2 (&RI)[EW_CH / 2],
                                         f32x2 (&IR)[EW_CH / 2]) {
    for (int s = 0; s < tn; s++) {
        const float2 X = sX[kx * P + s];
        float2 Y = sY[aky * P + s];
        Y.y *= ysign;
        const float q = sQ[s];
        float2 Aq = cmul(X, Y);
        Aq.x *= q;
        Aq.y *= q;
        const f32x2 AR = pk2(Aq.x, Aq.x), AI = pk2(Aq.y, Aq.y);
        const ulonglong2 *z = sZ + s * NPP + p0;
#pragma unroll
        for (int h = 0; h < NP; h++) {
            const ulonglong2 zz = z[h];  // (zr_k, zr_k+1), (zi_k, zi_k+1)
            RR[h] = fma2(AR, zz.x, RR[h]);
            II[h] = fma2(AI, zz.y, II[h]);
            RI[h] = fma2(AR, zz.y, RI[h]);
            IR[h] = fma2(AI, zz.x, IR[h]);
        }
    }
}

__device__ __forceinline__ void cp_async(void *dst, const void *src, int bytes) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if (bytes == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
    else if (bytes == 8)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

#define EW_SK_TPB 256  // tasks (threads) per block of the FP32 S(k) pass

// bytes of one staged tile of the FP32 S(k) pass (Z pairs, X, Y, q), a multiple of 16
__host__ __device__ inline size_t ew_sk2_stage(int KX, int KY, int KZ) {
    const size_t b = 16 * (size_t)EW_TILE * ew_zpairs(KZ) + 8 * (size_t)(KX + 1 + KY + 1) * (EW_TILE + 1) + 4 * EW_TILE;
    return (b + 15) & ~(size_t)15;
}

__global__ void k_qcast(int n, const double *__restrict__ q, float *__restrict__ qf) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < n) qf[a] = (float)q[a];
}

// The tiles of EW_TILE sites are copied into shared memory with cp.async, two stages:
// the copy of tile t + 1 runs while tile t is summed.
__global__ void __launch_bounds__(EW_SK_TPB, EW_SK2_MINB) k_sk2(EwArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int P = EW_TILE + 1;            // padded tile pitch of X and Y
    const int NPP = ew_zpairs(A.kz);      // |kz| pairs per site
    const size_t stage = ew_sk2_stage(A.kx, A.ky, A.kz);
    const float2 *tab = (const float2 *)A.tab;
    const float2 *tX = tab, *tY = tab + (size_t)(A.kx + 1) * A.n;
    const ulonglong2 *tZP = (const ulonglong2 *)(tab + ew_zoff(A.kx, A.ky, A.n));
    const int task = blockIdx.x * EW_SK_TPB + threadIdx.x;
    int kx = 0, ky = 0, half = 0, kz0 = 0, cnt = 0, slot0 = 0;
    if (task < A.ntasks) {
        const int4 t = A.tasks[task];
        const int4 r = A.rows[t.x];
        kx = r.x;
        ky = r.y;
        half = r.w;
        kz0 = t.y;
        cnt = t.z;
        slot0 = A.row_slot[t.x];
    }
    const int aky = ky < 0 ? -ky : ky;
    const float ysign = ky < 0 ? -1.f : 1.f;
    const int np = (cnt + 1) / 2, p0 = kz0 / 2;
    f32x2 RR[EW_CH / 2], II[EW_CH / 2], RI[EW_CH / 2], IR[EW_CH / 2];
#pragma unroll
    for (int h = 0; h < EW_CH / 2; h++) RR[h] = II[h] = RI[h] = IR[h] = 0;
    const int a_begin = blockIdx.y * EW_SITES, a_end = min(A.n, a_begin + EW_SITES);
    const int ntile = (a_end - a_begin + EW_TILE - 1) / EW_TILE;
    auto copy_tile = [&](int b, int t0) {
        unsigned char *base = smem_raw + b * stage;
        ulonglong2 *sZ = (ulonglong2 *)base;
        float2 *sX = (float2 *)(sZ + (size_t)EW_TILE * NPP);
        float2 *sY = sX + (size_t)(A.kx + 1) * P;
        float *sQ = (float *)(sY + (size_t)(A.ky + 1) * P);
        const int tn = min(EW_TILE, a_end - t0);
        for (int i = threadIdx.x; i < NPP * EW_TILE; i += EW_SK_TPB) {
            const int pp = i / EW_TILE, s = i % EW_TILE;
            if (s < tn) cp_async(&sZ[s * NPP + pp], &tZP[(size_t)pp * A.n + t0 + s], 16);
        }
        for (int i = threadIdx.x; i < (A.kx + 1) * EW_TILE; i += EW_SK_TPB) {
            const int k = i / EW_TILE, s = i % EW_TILE;
            if (s < tn) cp_async(&sX[k * P + s], &tX[(size_t)k * A.n + t0 + s], 8);
        }
        for (int i = threadIdx.x; i < (A.ky + 1) * EW_TILE; i += EW_SK_TPB) {
            const int k = i / EW_TILE, s = i % EW_TILE;
            if (s < tn) cp_async(&sY[k * P + s], &tY[(size_t)k * A.n + t0 + s], 8);
        }
        if (threadIdx.x < tn) cp_async(&sQ[threadIdx.x], &A.qf[t0 + threadIdx.x], 4);
        cp_async_commit();
    };
    if (ntile > 0) copy_tile(0, a_begin);
    for (int t = 0; t < ntile; t++) {
        const int t0 = a_begin + t * EW_TILE, tn = min(EW_TILE, a_end - t0);
        if (t + 1 < ntile) {
            copy_tile((t + 1) & 1, t0 + EW_TILE);  // its buffer was last read before the barrier below
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const unsigned char *base = smem_raw + (t & 1) * stage;
        const ulonglong2 *sZ = (const ulonglong2 *)base;
        const float2 *sX = (const float2 *)(sZ + (size_t)EW_TILE * NPP);
        const float2 *sY = sX + (size_t)(A.kx + 1) * P;
        const float *sQ = (const float *)(sY + (size_t)(A.ky + 1) * P);
        switch (np) {
#if EW_CH >= 12
        case 6: sk2_tile<6>(sZ, sX, sY, sQ, NPP, P, tn, kx, aky, ysign, p0, RR, II, RI, IR); break;
#endif
#if EW_CH >= 10
        case 5: sk2_tile<5>(sZ, sX, sY, sQ, NPP, P, tn, kx, aky, ysign, p0, RR, II, RI, IR); break;
#endif
        case 4: sk2_tile<4>(sZ, sX, sY, sQ, NPP, P, tn, kx, aky, ysign, p0, RR, II, RI, IR); break;
        case 3: sk2_tile<3>(sZ, sX, sY, sQ, NPP, P, tn, kx, aky, ysign, p0, RR, II, RI, IR); break;
        case 2: sk2_tile<2>(sZ, sX, sY, sQ, NPP, P, tn, kx, aky, ysign, p0, RR, II, RI, IR); break;
        case 1: sk2_tile<1>(sZ, sX, sY, sQ, NPP, P, tn, kx, aky, ysign, p0, RR, II, RI, IR); break;
        default: break;
        }
        __syncthreads();
    }
    if (task >= A.ntasks || cnt == 0) return;
    float *out = (float *)A.spart + (size_t)blockIdx.y * A.nslots * 2;
#pragma unroll
    for (int h = 0; h < EW_CH / 2; h++) {
        if (h >= np) break;
        float rr[2], ii[2], ri[2], ir[2];
        up2(RR[h], rr[0], rr[1]);
        up2(II[h], ii[0], ii[1]);
        up2(RI[h], ri[0], ri[1]);
        up2(IR[h], ir[0], ir[1]);
#pragma unroll
        for (int l = 0; l < 2; l++) {
            const int j = 2 * h + l;
            if (j >= cnt) break;
            const int a = kz0 + j;
            const int sp = slot0 + 2 * a, sm = sp + 1;
            out[2 * sp] = rr[l] - ii[l];
            out[2 * sp + 1] = ri[l] + ir[l];
            const bool has_minus = (a > 0) && !half;
            out[2 * sm] = has_minus ? rr[l] + ii[l] : 0.f;
            out[2 * sm + 1] = has_minus ? ir[l] - ri[l] : 0.f;
        }
    }
}

// the S(k) pass of one precision over nblk site blocks
template <typename R>
cudaError_t launch_sk(const EwArgs &A, int nblk, cudaStream_t s) {
    cudaError_t e;
    if constexpr (std::is_same<R, float>::value) {
        if (A.n == 0) return cudaSuccess;
        k_qcast<<<(A.n + 255) / 256, 256, 0, s>>>(A.n, A.q, A.qf);
        const dim3 grid((unsigned)((A.ntasks + EW_SK_TPB - 1) / EW_SK_TPB), (unsigned)nblk);
        const size_t smem = 2 * ew_sk2_stage(A.kx, A.ky, A.kz);
        e = cudaFuncSetAttribute(k_sk2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) k_sk2<<<grid, EW_SK_TPB, smem, s>>>(A);
    } else {
        const dim3 grid((unsigned)((A.ntasks + EW_TPB - 1) / EW_TPB), (unsigned)nblk);
        const int P = EW_TILE + 1;
        const size_t smem = sizeof(double2) * (size_t)(A.kx + 1 + A.ky + 1 + A.kz + 1) * P + sizeof(double) * EW_TILE;
        e = cudaFuncSetAttribute(k_sk<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) k_sk<double><<<grid, EW_TPB, smem, s>>>(A);
    }
    return e == cudaSuccess ? cudaGetLastError() : e;
}

// ---------------------------------------------------------------------------------
// Tensor-core structure factors (FP32 path): the site sum as a GEMM on tcgen05
// ---------------------------------------------------------------------------------
// For a tile of 64 rows (taken in force order, longest kzmax first) and a block of
// EW_MMA_SITES sites, D[m][n] = sum_s A[m][s] B[n][s] with
//   A[r][s] = Re(q_s X^kx_s Y^ky_s), A[64 + r][s] = Im(...)        (M = 128)
//   B[kz][s] = Re Z^kz_s, B[H + kz][s] = Im Z^kz_s, H = 16 or 32     (N = 2H)
// so that lane r of D holds RR (columns kz) and RI (H + kz) and lane 64 + r holds IR and
// II, and S(+kz) = (RR - II, RI + IR), S(-kz) = (RR + II, IR - RI) as in k_sk2. A is made
// per chunk of 32 sites by the CUDA cores from the phase tables (the charges scaled by the
// power of two that brings the CTA's largest |q| into [1/2, 1), undone on the partials), B
// from the Z pairs (|Z| = 1); both go to shared memory as FP16 hi + lo pairs (round to
// nearest, then the exact remainder rounded again: 22 significant bits) in the canonical
// K-major 128-byte-swizzled layout, and one thread issues kind::f16 MMAs (K = 16) for
// hi*hi + hi*lo + lo*hi (the 3-term split product keeps the FP32 operands' accuracy; the
// dropped lo*lo term is below 2^-22 relative). The tensor core's
// FP32 accumulation does not round to nearest (over a 1024-site block it shrank |S| by a
// few 1e-6, the Fourier energy by 1e-5), so each group of EW_MMA_GROUP chunks accumulates
// in one of two tensor-memory accumulators and is then added, by the CUDA cores in
// round-to-nearest FP32, to a running total kept in tensor memory: the truncation then
// acts on 128-site partials of either sign and averages out. Partials per site block go to
// k_sk_reduce, which sums them in fixed order. Two chunk stages: the CUDA cores fill stage c & 1 while
// the tensor core works on the other; a tcgen05.commit per chunk signals an mbarrier that
// guards the stage's reuse. Every wait is bounded (A.mma_wait polls). When one runs out the
// CTA stops issuing, records MG_FLAG_WAIT_TIMEOUT, waits with the full default bound for the
// commits of the last two chunks it issued (one per barrier; a commit covers every earlier
// MMA of the issuing thread), so that no MMA still reads its shared memory or writes its
// tensor memory, then frees the tensor memory and returns without writing partials. If that
// wait runs out too it also records MG_FLAG_MMA_UNDRAINED: tensor memory of the SM may then be
// overwritten by MMAs still in flight for the rest of the launch, and the call's results are
// invalid as a whole (the host fails the call; the S(k) reduction turns every coefficient
// and the energy into NaN).
#define EW_MMA_ROWS 64     // rows per CTA (two accumulator lanes each)
#ifndef EW_MMA_SITES
#define EW_MMA_SITES 1024  // sites per CTA (a multiple of EW_SITES)
#endif
#define EW_MMA_TPB 256
#define EW_MMA_KC 32       // sites per chunk: 32 FP16 values of each 128-byte row of the swizzled layout
#define EW_MMA_MAXKZ 30    // largest KMAXZ the pass takes (Z pairs within 32 columns)
#define EW_MMA_STAGE 49152 // A hi, A lo (16 KB each), B hi, B lo (8 KB each)
#define EW_MMA_SMEM (2 * EW_MMA_STAGE + 64 + 1024)
#define EW_MMA_WAIT (1ll << 20)  // default polls of each pipeline wait (mg_set_wait_limit)
#ifndef EW_MMA_GROUP
#define EW_MMA_GROUP 2     // chunks summed in one tensor-memory accumulator before each drain
#endif
#define EW_MMA_TCOLS 256   // tensor-memory columns per CTA: two group accumulators and the total

// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 bytes apart
__device__ __forceinline__ unsigned long long umma_desc(unsigned saddr) {
    return (unsigned long long)((saddr >> 4) & 0x3FFFu) | (1ull << 16) | ((unsigned long long)(1024 >> 4) << 32) |
           (1ull << 46) | (2ull << 61);
}

__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, long long limit) {
    for (long long i = 0; i < limit; i++) {
        unsigned ok;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(bar), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}

// instruction descriptor of kind::f16: D F32, A and B F16, both K-major, M = 128, N = n
__host__ __device__ constexpr unsigned umma_idesc_f16(int n) {
    return (1u << 4) | ((unsigned)(n >> 3) << 17) | ((unsigned)(128 >> 4) << 24);
}

__device__ __forceinline__ void umma_f16(unsigned d, unsigned long long a, unsigned long long b, unsigned idesc,
                                         unsigned acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

// FP16 hi + lo of two FP32 values a, b, each pair packed (a in the low 16 bits): hi rounded
// to nearest, lo the exact remainder rounded to nearest. One packed conversion converts both
// values (conversions to narrower types issue at a fraction of the FP32 rate); the bits are
// those of two scalar round-to-nearest conversions.
__device__ __forceinline__ void f16x2_split(float a, float b, unsigned &hi, unsigned &lo) {
    const __half2 h = __floats2half2_rn(a, b);
    const float2 hf = __half22float2(h);
    const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const unsigned *>(&h);
    lo = *reinterpret_cast<const unsigned *>(&l);
}

// FP16 hi + lo of four FP32 values, as two 8-byte pieces
__device__ __forceinline__ void f16_split4(const float (&x)[4], uint2 &hi, uint2 &lo) {
    f16x2_split(x[0], x[1], hi.x, lo.x);
    f16x2_split(x[2], x[3], hi.y, lo.y);
}

__device__ __forceinline__ void sts64(unsigned a, uint2 v) {
    asm volatile("st.shared.v2.b32 [%0], {%1, %2};" ::"r"(a), "r"(v.x), "r"(v.y) : "memory");
}

__device__ __forceinline__ void tmem_ld16(unsigned addr, float (&v)[16]) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(addr)
        : "memory");
#pragma unroll
    for (int j = 0; j < 16; j++) v[j] = __uint_as_float(r[j]);
}

__device__ __forceinline__ void tmem_st16(unsigned addr, const float (&v)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16};" ::"r"(addr),
        "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]), "f"(v[9]),
        "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
        : "memory");
}

__global__ void __launch_bounds__(EW_MMA_TPB, 2) k_sk_mma(EwArgs A, unsigned *flags) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned raw = (unsigned)__cvta_generic_to_shared(smem_raw);
    const unsigned base = (raw + 1023u) & ~1023u;  // the swizzled tiles need 1024-byte alignment
    unsigned char *gbase = smem_raw + (base - raw);
    const unsigned bar0 = base + 2 * EW_MMA_STAGE, tslot = bar0 + 16;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int pos0 = blockIdx.x * EW_MMA_ROWS;
    const int H = A.rows[A.forder[pos0]].z + 1 <= 16 ? 16 : 32;  // rows sorted by kzmax, longest first
    const int NPP = min(ew_zpairs(A.kz), (A.rows[A.forder[pos0]].z + 2) / 2);
    const unsigned idesc = umma_idesc_f16(2 * H);

    // zero both stages (rows no chunk writes stay zero), barriers, tensor memory
    for (int i = threadIdx.x; i < 2 * EW_MMA_STAGE / 16; i += EW_MMA_TPB)
        ((uint4 *)gbase)[i] = make_uint4(0u, 0u, 0u, 0u);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar0), "r"(1) : "memory");
        asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar0 + 8), "r"(1) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tslot),
                     "r"(EW_MMA_TCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = *(volatile unsigned *)(gbase + (tslot - base));
    // the power of two that brings the largest |q| of the CTA's sites into [1/2, 1): the A
    // operand (|q X Y| <= |q|) then stays within FP16's range; the partials are scaled back
    float qs, qus;
    {
        float *s_qmax = (float *)(gbase + (tslot - base) + 16);  // eight words after the barriers
        const int a0 = blockIdx.y * EW_MMA_SITES, a1 = min(A.n, a0 + EW_MMA_SITES);
        float m = 0.f;
        for (int a = a0 + (int)threadIdx.x; a < a1; a += EW_MMA_TPB) m = fmaxf(m, fabsf(A.qf[a]));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) s_qmax[warp] = m;
        __syncthreads();
        m = 0.f;
#pragma unroll
        for (int k = 0; k < EW_MMA_TPB / 32; k++) m = fmaxf(m, s_qmax[k]);
        int e2 = 0;
        frexpf(m, &e2);
        qs = ldexpf(1.f, -e2);
        qus = ldexpf(1.f, e2);
    }
    // group accumulator g & 1 at columns 64 (g & 1); the running total at columns 128..
    // (lane quarter warp & 3; warps w and w + 4 drain the two column halves)
    const unsigned tlane = tmem + ((unsigned)((warp & 3) * 32) << 16);
    int ndrained = 0;
    auto drain = [&](int g) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (int piece = 0; piece < H / 16; piece++) {
            const unsigned col = (unsigned)((warp >> 2) * H + piece * 16);
            float v[16], t[16];
            tmem_ld16(tlane + 64u * (unsigned)(g & 1) + col, v);
            if (ndrained > 0) tmem_ld16(tlane + 128u + col, t);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 16; j++) t[j] = ndrained > 0 ? t[j] + v[j] : v[j];
            tmem_st16(tlane + 128u + col, t);
            asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
        }
        ndrained++;
    };

    // A: lane (g = lane & 7, i0 = lane >> 3) makes sites 4g..4g+3 of the warp's rows i0 and
    // i0 + 4, one 16-byte swizzle chunk per row and operand; B: thread t, renumbered
    // t' = (t + 128) mod 256, makes Z pair t' >> 3 for sites 4 (t & 7)..+3 when t' < 8 NPP.
    // The loads of chunk c + 1 are issued before the
    // barrier of chunk c (registers), so their latency overlaps the barrier and the wait.
    const int g = lane & 7, i0 = lane >> 3;
    int rkx[2], raky[2];
    float rys[2];
    bool rok[2];
    unsigned aoff[2];
#pragma unroll
    for (int j = 0; j < 2; j++) {
        const int i = i0 + 4 * j, pos = pos0 + warp * 8 + i;
        rok[j] = pos < A.nrows;
        const int4 r = rok[j] ? A.rows[A.forder[pos]] : make_int4(0, 0, 0, 0);
        rkx[j] = r.x;
        raky[j] = r.y < 0 ? -r.y : r.y;
        rys[j] = r.y < 0 ? -1.f : 1.f;
        aoff[j] = (unsigned)(warp * 1024 + i * 128 + ((((g >> 1) ^ i) & 7) << 4) + (g & 1) * 8);
    }
    // the B (Z) chunks go to the upper warps first: warp 0 also issues the MMAs (C2: S(k)
    // 0.336 -> 0.322 ms against giving them to warps 0..3)
    const int tb = (int)((threadIdx.x + EW_MMA_TPB / 2) % EW_MMA_TPB);
    const bool bwork = tb < 8 * NPP;
    const int bp = tb >> 3;
    unsigned boff[4];
    {
        const int nrow[4] = {2 * bp, 2 * bp + 1, H + 2 * bp, H + 2 * bp + 1};
#pragma unroll
        for (int j = 0; j < 4; j++)
            boff[j] = (unsigned)((nrow[j] >> 3) * 1024 + (nrow[j] & 7) * 128 + ((((g >> 1) ^ nrow[j]) & 7) << 4) + (g & 1) * 8);
    }
    const float2 *tab = (const float2 *)A.tab;
    const float2 *tX = tab, *tY = tab + (size_t)(A.kx + 1) * A.n;
    const float4 *tZP = (const float4 *)(tab + ew_zoff(A.kx, A.ky, A.n));
    const int a_begin = blockIdx.y * EW_MMA_SITES, a_end = min(A.n, a_begin + EW_MMA_SITES);
    const int nch = (a_end - a_begin + EW_MMA_KC - 1) / EW_MMA_KC;
    const bool even = (A.n & 1) == 0;  // 16-byte loads of two float2 table entries
    float2 X[2][4], Y[2][4];
    float Q[4];
    float4 Z[4];
    auto load = [&](int c) {
        const int s0 = a_begin + c * EW_MMA_KC + 4 * g;
        const bool full = s0 + 3 < a_end;
        if (full) {
            const float4 t = *(const float4 *)(A.qf + s0);
            Q[0] = t.x, Q[1] = t.y, Q[2] = t.z, Q[3] = t.w;
        } else {
#pragma unroll
            for (int j = 0; j < 4; j++) Q[j] = s0 + j < a_end ? A.qf[s0 + j] : 0.f;
        }
#pragma unroll
        for (int jr = 0; jr < 2; jr++) {
            if (!rok[jr]) continue;
            const float2 *px = tX + (size_t)rkx[jr] * A.n + s0, *py = tY + (size_t)raky[jr] * A.n + s0;
            if (full && even) {
                const float4 x0 = *(const float4 *)px, x1 = *(const float4 *)(px + 2);
                const float4 y0 = *(const float4 *)py, y1 = *(const float4 *)(py + 2);
                X[jr][0] = make_float2(x0.x, x0.y), X[jr][1] = make_float2(x0.z, x0.w);
                X[jr][2] = make_float2(x1.x, x1.y), X[jr][3] = make_float2(x1.z, x1.w);
                Y[jr][0] = make_float2(y0.x, y0.y), Y[jr][1] = make_float2(y0.z, y0.w);
                Y[jr][2] = make_float2(y1.x, y1.y), Y[jr][3] = make_float2(y1.z, y1.w);
            } else {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const bool in = s0 + j < a_end;
                    X[jr][j] = in ? px[j] : make_float2(0.f, 0.f);
                    Y[jr][j] = in ? py[j] : make_float2(0.f, 0.f);
                }
            }
        }
        if (bwork) {
#pragma unroll
            for (int j = 0; j < 4; j++)
                Z[j] = s0 + j < a_end ? tZP[(size_t)bp * A.n + s0 + j] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    };
    if (nch > 0) load(0);
    bool timeout = false;
    int issued = 0;  // chunks whose MMAs were issued and committed
    for (int c = 0; c < nch; c++) {
        const int b = c & 1;
        const unsigned st = base + b * EW_MMA_STAGE;
        bool to = false;
        if (c >= 2) to = !mbar_wait(bar0 + 8 * b, ((c - 2) >> 1) & 1, A.mma_wait);
        // one decision per warp: drain() runs warp-wide tcgen05 loads and stores
        to = __any_sync(0xffffffffu, to);
        if (!to) {
            // chunk c - 2 is complete: if it closed a group, fold that group into the total
            // before the group two ahead reuses its accumulator
            if (c >= 2 && (c - 2) % EW_MMA_GROUP == EW_MMA_GROUP - 1) drain((c - 2) / EW_MMA_GROUP);
#pragma unroll
            for (int jr = 0; jr < 2; jr++) {
                if (!rok[jr]) continue;
                float re[4], im[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    float2 y = Y[jr][j];
                    y.y *= rys[jr];
                    const float2 aq = cmul(X[jr][j], y);
                    const float qj = Q[j] * qs;
                    re[j] = aq.x * qj;
                    im[j] = aq.y * qj;
                }
                uint2 hr, lr, hi, li;
                f16_split4(re, hr, lr);
                f16_split4(im, hi, li);
                sts64(st + aoff[jr], hr);
                sts64(st + 16384 + aoff[jr], lr);
                sts64(st + 8192 + aoff[jr], hi);
                sts64(st + 16384 + 8192 + aoff[jr], li);
            }
            if (bwork) {
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    float v[4];
                    v[0] = j == 0 ? Z[0].x : j == 1 ? Z[0].y : j == 2 ? Z[0].z : Z[0].w;
                    v[1] = j == 0 ? Z[1].x : j == 1 ? Z[1].y : j == 2 ? Z[1].z : Z[1].w;
                    v[2] = j == 0 ? Z[2].x : j == 1 ? Z[2].y : j == 2 ? Z[2].z : Z[2].w;
                    v[3] = j == 0 ? Z[3].x : j == 1 ? Z[3].y : j == 2 ? Z[3].z : Z[3].w;
                    uint2 h, l;
                    f16_split4(v, h, l);
                    sts64(st + 32768 + boff[j], h);
                    sts64(st + 40960 + boff[j], l);
                }
            }
            if (c + 1 < nch) load(c + 1);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        if (__syncthreads_or(to)) {
            timeout = true;
            break;
        }
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const unsigned acc = tmem + 64u * (unsigned)((c / EW_MMA_GROUP) & 1);
            const bool fresh = c % EW_MMA_GROUP == 0;
#pragma unroll
            for (int k = 0; k < EW_MMA_KC / 16; k++) {  // K = 16 FP16 values (32 bytes) per MMA
                const unsigned long long ah = umma_desc(st + 32 * k), al = umma_desc(st + 16384 + 32 * k);
                const unsigned long long bh = umma_desc(st + 32768 + 32 * k), bl = umma_desc(st + 40960 + 32 * k);
                umma_f16(acc, ah, bh, idesc, (fresh && k == 0) ? 0u : 1u);
                umma_f16(acc, ah, bl, idesc, 1u);
                umma_f16(acc, al, bh, idesc, 1u);
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar0 + 8 * b)
                         : "memory");
        }
        issued = c + 1;
    }
    if (!timeout && nch > 0) {
        const bool to = !mbar_wait(bar0 + 8 * ((nch - 1) & 1), ((nch - 1) >> 1) & 1, A.mma_wait);
        timeout = __syncthreads_or(to);
    }
    if (timeout) {
        // the MMAs of the issued chunks may still run: wait, with the full default bound, for
        // the commits of the last two issued chunks before the tensor memory is released
        bool done = true;
        for (int c = max(0, issued - 2); c < issued; c++) done &= mbar_wait(bar0 + 8 * (c & 1), (c >> 1) & 1, EW_MMA_WAIT);
        done = __syncthreads_and(done);
        if (threadIdx.x == 0 && flags) atomicOr(flags, done ? MG_FLAG_WAIT_TIMEOUT : MG_FLAG_WAIT_TIMEOUT | MG_FLAG_MMA_UNDRAINED);
    } else {
        const int ngroup = (nch + EW_MMA_GROUP - 1) / EW_MMA_GROUP;
        while (ndrained < ngroup) drain(ndrained);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    float *D = (float *)gbase;  // 128 x 65 floats over stage 0 (all MMAs have completed)
    if (!timeout && warp < 4 && nch > 0) {
        for (int cc = 0; cc < 2 * H / 16; cc++) {
            float v[16];
            tmem_ld16(tlane + 128u + (unsigned)(cc * 16), v);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 16; j++) D[(warp * 32 + lane) * 65 + cc * 16 + j] = v[j];
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(EW_MMA_TCOLS) : "memory");
    if (timeout) return;
    float *out = (float *)A.spart + (size_t)blockIdx.y * A.nslots * 2;
    for (int idx = threadIdx.x; idx < EW_MMA_ROWS * 32; idx += EW_MMA_TPB) {
        const int r = idx >> 5, a = idx & 31, pos = pos0 + r;
        if (pos >= A.nrows) break;
        const int row = A.forder[pos];
        const int4 rw = A.rows[row];
        if (a > rw.z) continue;
        float RR = 0.f, RI = 0.f, IR = 0.f, II = 0.f;
        if (nch > 0) {  // back from the charge scale (exact)
            RR = D[r * 65 + a] * qus;
            RI = D[r * 65 + H + a] * qus;
            IR = D[(64 + r) * 65 + a] * qus;
            II = D[(64 + r) * 65 + H + a] * qus;
        }
        const int sp = A.row_slot[row] + 2 * a, sm = sp + 1;
        out[2 * sp] = RR - II;
        out[2 * sp + 1] = RI + IR;
        const bool has_minus = (a > 0) && !rw.w;
        out[2 * sm] = has_minus ? RR + II : 0.f;
        out[2 * sm + 1] = has_minus ? IR - RI : 0.f;
    }
}

// the tensor-core S(k) pass (A.forder must be set); returns the number of site blocks of partials
cudaError_t launch_sk_mma(const EwArgs &A, unsigned *flags, cudaStream_t s, int *nblk) {
    *nblk = (A.n + EW_MMA_SITES - 1) / EW_MMA_SITES;
    if (A.n == 0 || A.nrows == 0) return cudaSuccess;
    if (!A.forder || !A.rows || !A.row_slot || !A.qf) return cudaErrorInvalidValue;
    k_qcast<<<(A.n + 255) / 256, 256, 0, s>>>(A.n, A.q, A.qf);
    cudaError_t e = cudaFuncSetAttribute(k_sk_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, EW_MMA_SMEM);
    if (e != cudaSuccess) return e;
    const dim3 grid((unsigned)((A.nrows + EW_MMA_ROWS - 1) / EW_MMA_ROWS), (unsigned)*nblk);
    k_sk_mma<<<grid, EW_MMA_TPB, EW_MMA_SMEM, s>>>(A, flags);
    return cudaGetLastError();
}

// S(k) from the partials: a block of EW_RED_PARTS * 256 threads takes 256 slots; part p
// sums site blocks [p nblk / PARTS, (p + 1) nblk / PARTS) in order (FP32 hi + lo on the
// FP32 path, FP64 on the FP64 path) and the parts are added in order in FP64 (fixed order
// throughout); then energy rows and force coefficients
#define EW_RED_PARTS 4
template <typename R>
__global__ void __launch_bounds__(EW_RED_PARTS * 256) k_sk_reduce(EwArgs A, int nblk, const int *__restrict__ slot_row) {
    typedef typename C2<R>::T T2;
    __shared__ double2 sp[EW_RED_PARTS][256];
    double e[1] = {0.0};
    const int part = threadIdx.x / 256, sl = threadIdx.x % 256;
    int slot = blockIdx.x * 256 + sl;
    if (slot < A.nslots) {
        // FP32 partials summed as exact hi + lo pairs (no FP64 instruction in the loop;
        // FP64 arithmetic runs at a small fraction of the FP32 rate on this part)
        R hr = 0, lr = 0, hi = 0, li = 0;
        const int b0 = (int)((long long)nblk * part / EW_RED_PARTS), b1 = (int)((long long)nblk * (part + 1) / EW_RED_PARTS);
        for (int b = b0; b < b1; b++) {
            const R *p = (const R *)A.spart + ((size_t)b * A.nslots + slot) * 2;
            mg_acc2(hr, lr, p[0]);
            mg_acc2(hi, li, p[1]);
        }
        sp[part][sl] = make_double2((double)hr + (double)lr, (double)hi + (double)li);
    }
    __syncthreads();
    if (part == 0 && slot < A.nslots) {
        double sr = sp[0][sl].x, si = sp[0][sl].y;
        for (int q = 1; q < EW_RED_PARTS; q++) {
            sr += sp[q][sl].x;
            si += sp[q][sl].y;
        }
        int r = slot_row[slot];
        int4 row = A.rows[r];
        int local = slot - A.row_slot[r];
        int a = local >> 1, minus = local & 1;
        bool valid = a <= row.z && !(minus && (a == 0 || row.w)) && !(row.w && a == 0);
        T2 c;
        c.x = c.y = (R)0;
        if (A.flags && (*A.flags & MG_FLAG_WAIT_TIMEOUT)) {
            // the tensor-core pass gave up: its partials are incomplete, so the coefficients
            // (and with them every force of the pass) and the energy become NaN
            c.x = c.y = (R)NAN;
            e[0] = NAN;
        } else if (valid) {
            double kz = minus ? -a : a;
            double rkx = A.twopi[0] * row.x, rky = A.twopi[1] * row.y, rkz = A.twopi[2] * kz;
            double rksq = rkx * rkx + rky * rky + rkz * rkz;
            double kvec = exp(-A.bfac * rksq) / rksq;
            e[0] = 2.0 * kvec * (sr * sr + si * si) * A.vfac * A.coul;
            double cf = 4.0 * A.vfac * A.coul * kvec;
            c.x = (R)(cf * sr);
            c.y = (R)(minus ? cf * si : -cf * si);  // plus slots hold conj(c S)
        }
        ((T2 *)A.scoef)[slot] = c;
    }
    const int ids[1] = {E_UFOURIER};
    mg_block_row<1>(e, ids, A.rows_e, A.row0 + blockIdx.x);
}

// FG thread groups share the rows of a site (the threads per site; tuned per context)
template <typename R, int FG = EW_FG>
__global__ void __launch_bounds__(FG * EW_FSITES) k_kforce(EwArgs A, int maxa) {
    typedef typename C2<R>::T T2;
    typedef typename C2<R>::T4 T4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T4 *sC = (T4 *)smem_raw;  // [EW_FROWS][maxa]: conj(c S+_a), c S-_a
    __shared__ int4 sRow[EW_FROWS];
    __shared__ double sF[FG][3][EW_FSITES];
    const int g = threadIdx.x / EW_FSITES, l = threadIdx.x % EW_FSITES;
    const int a = blockIdx.x * EW_FSITES + l;
    const bool act = a < A.n;
    const T2 *tab = (const T2 *)A.tab;
    const T2 *tX = tab, *tY = tab + (size_t)(A.kx + 1) * A.n;
    T2 Z;
    if (act) {
        Z = ew_z1<R>(A.tab, A.kx, A.ky, A.n, a);
    } else {
        Z.x = (R)1;
        Z.y = (R)0;
    }
    R Fh[3] = {0, 0, 0}, Fl[3] = {0, 0, 0};  // per-chunk sums accumulated as hi + lo
    const T4 *coef = (const T4 *)A.scoef;
    for (int r0 = 0; r0 < A.nrows; r0 += EW_FROWS) {
        const int nr = min(EW_FROWS, A.nrows - r0);
        __syncthreads();
        for (int i = threadIdx.x; i < nr * maxa; i += blockDim.x) {
            int rr = i / maxa, s = i % maxa;
            int4 row = A.rows[r0 + rr];
            T4 v;
            v.x = v.y = v.z = v.w = (R)0;
            if (s <= row.z) v = coef[A.row_slot[r0 + rr] / 2 + s];
            sC[rr * maxa + s] = v;
        }
        if (threadIdx.x < nr) sRow[threadIdx.x] = A.rows[r0 + threadIdx.x];
        __syncthreads();
        if (!act) continue;
        R fx = 0, fy = 0, fz = 0;
        for (int rr = g; rr < nr; rr += FG) {
            const int4 row = sRow[rr];
            T2 X = tX[(size_t)row.x * A.n + a];
            T2 Y = tY[(size_t)(row.y < 0 ? -row.y : row.y) * A.n + a];
            if (row.y < 0) Y.y = -Y.y;
            const T2 Aa = cmul(X, Y);
            const T4 *cs = sC + rr * maxa;
            // Horner: p = P(Z), dp = P'(Z), q = Q(Z), dq = Q'(Z)
            T4 top = cs[row.z];
            T2 p, q, dp, dq;
            p.x = top.x; p.y = top.y;
            q.x = top.z; q.y = top.w;
            dp.x = dp.y = dq.x = dq.y = (R)0;
            for (int k = row.z - 1; k >= 0; k--) {
                const T4 c = cs[k];
                T2 cu, cv;
                cu.x = c.x; cu.y = c.y;
                cv.x = c.z; cv.y = c.w;
                dp = cfma(dp, Z, p);
                p = cfma(p, Z, cu);
                dq = cfma(dq, Z, q);
                q = cfma(q, Z, cv);
            }
            // sum_a g+ + g- = Im(A p) + Im(A conj(q)); sum_a a (g+ - g-) = Im(A Z dp) - Im(A conj(Z dq))
            const R gsum = (Aa.x * p.y + Aa.y * p.x) + (Aa.y * q.x - Aa.x * q.y);
            const T2 zdp = cmul(Z, dp), zdq = cmul(Z, dq);
            const R gz = (Aa.x * zdp.y + Aa.y * zdp.x) - (Aa.y * zdq.x - Aa.x * zdq.y);
            fx += gsum * (R)row.x;
            fy += gsum * (R)row.y;
            fz += gz;
        }
        mg_acc2(Fh[0], Fl[0], fx);
        mg_acc2(Fh[1], Fl[1], fy);
        mg_acc2(Fh[2], Fl[2], fz);
    }
    for (int d = 0; d < 3; d++) sF[g][d][l] = (double)Fh[d] + (double)Fl[d];
    __syncthreads();
    if (g != 0 || !act) return;
    double fxs = 0, fys = 0, fzs = 0;
    for (int k = 0; k < FG; k++) {
        fxs += sF[k][0][l];
        fys += sF[k][1][l];
        fzs += sF[k][2][l];
    }
    const double q = A.q[a];
    ew_addf(&A.f[a], q, fxs, A.twopi[0]);
    ew_addf(&A.f[A.n + a], q, fys, A.twopi[1]);
    ew_addf(&A.f[2 * A.n + a], q, fzs, A.twopi[2]);
}

// FP32 force pass on units of two rows (rows 2u and 2u+1 of the table order), one row
// per lane of the packed f32x2 arithmetic: the site's Z is the same in both lanes, so
// one Horner step of the unit is 16 packed FMAs where two rows took 32 scalar ones. Each
// lane runs the nesting of k_kforce's cfma, and a row shorter than its partner reads
// zero coefficients above its own top, which leave p, q, p', q' exactly as they were
// (zero) until its top is reached: per row the lane gives k_kforce's bits. Units are
// staged EW_FUNITS at a time as [unit][|kz|]{P coefficients, Q coefficients}, each a
// (re of both rows, im of both rows) pair of f32x2.
#define EW_FUNITS (EW_FROWS / 2)

template <int FG>
__global__ void __launch_bounds__(FG * EW_FSITES, 16 / FG) k_kforce_f2(EwArgs A, int maxa) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ulonglong2 *sC = (ulonglong2 *)smem_raw;  // [EW_FUNITS][maxa][2]
    __shared__ int4 sRow[EW_FROWS];
    __shared__ double sF[FG][3][EW_FSITES];
    const int g = threadIdx.x / EW_FSITES, l = threadIdx.x % EW_FSITES;
    const int a = blockIdx.x * EW_FSITES + l;
    const bool act = a < A.n;
    const float2 *tab = (const float2 *)A.tab;
    const float2 *tX = tab, *tY = tab + (size_t)(A.kx + 1) * A.n;
    const float2 Z = act ? ew_z1<float>(A.tab, A.kx, A.ky, A.n, a) : make_float2(1.f, 0.f);
    const f32x2 ZX = pk2(Z.x, Z.x), ZY = pk2(Z.y, Z.y), NZY = pk2(-Z.y, -Z.y);
    float Fh[3] = {0, 0, 0}, Fl[3] = {0, 0, 0};  // per-chunk sums accumulated as hi + lo
    const float4 *coef = (const float4 *)A.scoef;
    for (int r0 = 0; r0 < A.nrows; r0 += EW_FROWS) {
        const int nr = min(EW_FROWS, A.nrows - r0);
        const int nu = (nr + 1) / 2;
        __syncthreads();
        for (int i = threadIdx.x; i < nu * maxa; i += blockDim.x) {
            const int uu = i / maxa, s = i % maxa;
            const int ra = r0 + 2 * uu, rb = ra + 1;
            float4 c0 = make_float4(0.f, 0.f, 0.f, 0.f), c1 = c0;
            if (s <= A.rows[ra].z) c0 = coef[A.row_slot[ra] / 2 + s];
            if (2 * uu + 1 < nr && s <= A.rows[rb].z) c1 = coef[A.row_slot[rb] / 2 + s];
            sC[2 * (uu * maxa + s)] = make_ulonglong2(pk2(c0.x, c1.x), pk2(c0.y, c1.y));
            sC[2 * (uu * maxa + s) + 1] = make_ulonglong2(pk2(c0.z, c1.z), pk2(c0.w, c1.w));
        }
        if (threadIdx.x < 2 * nu)  // an absent second row of the last unit: (0, 0), no |kz|
            sRow[threadIdx.x] = threadIdx.x < nr ? A.rows[r0 + threadIdx.x] : make_int4(0, 0, -1, 0);
        __syncthreads();
        if (!act) continue;
        float fx = 0, fy = 0, fz = 0;
        for (int uu = g; uu < nu; uu += FG) {
            const int4 ra = sRow[2 * uu], rb = sRow[2 * uu + 1];
            float2 X0 = tX[(size_t)ra.x * A.n + a], Y0 = tY[(size_t)(ra.y < 0 ? -ra.y : ra.y) * A.n + a];
            float2 X1 = tX[(size_t)rb.x * A.n + a], Y1 = tY[(size_t)(rb.y < 0 ? -rb.y : rb.y) * A.n + a];
            if (ra.y < 0) Y0.y = -Y0.y;
            if (rb.y < 0) Y1.y = -Y1.y;
            const float2 A0 = cmul(X0, Y0), A1 = cmul(X1, Y1);
            const ulonglong2 *cs = sC + 2 * uu * maxa;
            const int m = max(ra.z, rb.z);
            const ulonglong2 tu = cs[2 * m], tv = cs[2 * m + 1];
            f32x2 pr = tu.x, pi = tu.y, qr = tv.x, qi = tv.y;
            f32x2 dpr = 0, dpi = 0, dqr = 0, dqi = 0;
#pragma unroll 2
            for (int k = m - 1; k >= 0; k--) {
                const ulonglong2 cu = cs[2 * k], cv = cs[2 * k + 1];
                // dp <- dp Z + p, p <- p Z + cu, dq <- dq Z + q, q <- q Z + cv
                const f32x2 ndpr = fma2(dpr, ZX, fma2(dpi, NZY, pr));
                const f32x2 ndpi = fma2(dpr, ZY, fma2(dpi, ZX, pi));
                const f32x2 npr = fma2(pr, ZX, fma2(pi, NZY, cu.x));
                const f32x2 npi = fma2(pr, ZY, fma2(pi, ZX, cu.y));
                const f32x2 ndqr = fma2(dqr, ZX, fma2(dqi, NZY, qr));
                const f32x2 ndqi = fma2(dqr, ZY, fma2(dqi, ZX, qi));
                const f32x2 nqr = fma2(qr, ZX, fma2(qi, NZY, cv.x));
                const f32x2 nqi = fma2(qr, ZY, fma2(qi, ZX, cv.y));
                dpr = ndpr;
                dpi = ndpi;
                pr = npr;
                pi = npi;
                dqr = ndqr;
                dqi = ndqi;
                qr = nqr;
                qi = nqi;
            }
            float2 p[2], q[2], dp[2], dq[2];
            up2(pr, p[0].x, p[1].x);
            up2(pi, p[0].y, p[1].y);
            up2(qr, q[0].x, q[1].x);
            up2(qi, q[0].y, q[1].y);
            up2(dpr, dp[0].x, dp[1].x);
            up2(dpi, dp[0].y, dp[1].y);
            up2(dqr, dq[0].x, dq[1].x);
            up2(dqi, dq[0].y, dq[1].y);
            const float2 Aa[2] = {A0, A1};
            const int4 rw[2] = {ra, rb};
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const float gsum = (Aa[h].x * p[h].y + Aa[h].y * p[h].x) + (Aa[h].y * q[h].x - Aa[h].x * q[h].y);
                const float2 zdp = cmul(Z, dp[h]), zdq = cmul(Z, dq[h]);
                const float gz = (Aa[h].x * zdp.y + Aa[h].y * zdp.x) - (Aa[h].y * zdq.x - Aa[h].x * zdq.y);
                fx += gsum * (float)rw[h].x;
                fy += gsum * (float)rw[h].y;
                fz += gz;
            }
        }
        mg_acc2(Fh[0], Fl[0], fx);
        mg_acc2(Fh[1], Fl[1], fy);
        mg_acc2(Fh[2], Fl[2], fz);
    }
    for (int d = 0; d < 3; d++) sF[g][d][l] = (double)Fh[d] + (double)Fl[d];
    __syncthreads();
    if (g != 0 || !act) return;
    double fxs = 0, fys = 0, fzs = 0;
    for (int k = 0; k < FG; k++) {
        fxs += sF[k][0][l];
        fys += sF[k][1][l];
        fzs += sF[k][2][l];
    }
    const double q = A.q[a];
    ew_addf(&A.f[a], q, fxs, A.twopi[0]);
    ew_addf(&A.f[A.n + a], q, fys, A.twopi[1]);
    ew_addf(&A.f[2 * A.n + a], q, fzs, A.twopi[2]);
}

// FP32 force pass from the phase tables. For one site and one row, with z_a = Z^a from
// the table and z^-a = conj(z^a), the row's kz sums are
//   gsum = Im(A W),  W  = sum_a [ u_a z^a + conj(v_a) conj(z^a) ]
//   gz   = Im(A W'), W' = sum_a a [ u_a z^a - conj(v_a) conj(z^a) ]
// (u_a = conj(c S+_a), v_a = c S-_a, the same values k_kforce's Horner sums use). With
// s = u + v, d = u - v per |kz|: W_r = sum zr s_r - zi s_i, W_i = sum zr d_i + zi d_r,
// W'_r = sum a (zr d_r - zi d_i), W'_i = sum a (zi s_r + zr s_i): 8 FMAs per site, row
// and |kz| against Horner's 16. k_fcoef stores (k0, k2, k1, k3) = (s_r, d_i, -s_i, d_r)
// per [chunk][|kz|][row of the chunk]; a thread owns one site and the 16 rows of a chunk
// (W in packed f32x2 as (W_r, W_i), W' in scalar FMAs, so both FP32 pipe halves work
// from one broadcast 16-byte shared load per row and |kz|).
__global__ void k_fcoef(EwArgs A) {
    const int c = blockIdx.x;
    const int m = A.rows[A.forder[c * EW_FCHUNK]].z;
    const float4 *coef = (const float4 *)A.scoef;
    float4 *out = A.fcoef + (size_t)A.coff[c] * EW_FCHUNK;
    for (int i = threadIdx.x; i < (m + 1) * EW_FCHUNK; i += blockDim.x) {
        const int a = i / EW_FCHUNK, p = c * EW_FCHUNK + i % EW_FCHUNK;
        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
        if (p < A.nrows) {
            const int r = A.forder[p];
            if (a <= A.rows[r].z) {
                const float4 uv = coef[A.row_slot[r] / 2 + a];  // u_r, u_i, v_r, v_i
                const float sr = uv.x + uv.z, si = uv.y + uv.w, dr = uv.x - uv.z, di = uv.y - uv.w;
                v = make_float4(sr, di, -si, dr);
            }
        }
        out[i] = v;
    }
}

__global__ void __launch_bounds__(EW_FMM_TPB, EW_FMM_MINB) k_kforce_mm(EwArgs A, int maxa) {
    constexpr int NS = EW_FMM_NS, NB = EW_FMM_TPB * EW_FMM_NS;  // sites per thread, per block
    extern __shared__ __align__(16) unsigned char smem_raw[];
    ulonglong2 *sK = (ulonglong2 *)smem_raw;                      // [maxa][EW_FCHUNK]
    float2 *sZ = (float2 *)(sK + (size_t)maxa * EW_FCHUNK);       // [maxa][NB]
    __shared__ int2 sR[EW_FCHUNK];                                // (kx, ky); (0, 0) pads
    const float2 *tab = (const float2 *)A.tab;
    const float2 *tX = tab, *tY = tab + (size_t)(A.kx + 1) * A.n;
    const float4 *tZP = (const float4 *)(tab + ew_zoff(A.kx, A.ky, A.n));
    int site[NS];  // idle threads read a valid site and store nothing
#pragma unroll
    for (int k = 0; k < NS; k++) {
        const int a_site = blockIdx.x * NB + k * EW_FMM_TPB + threadIdx.x;
        site[k] = a_site < A.n ? a_site : A.n - 1;
        for (int pp = 0; 2 * pp < maxa; pp++) {
            const float4 v = tZP[(size_t)pp * A.n + site[k]];
            sZ[2 * pp * NB + k * EW_FMM_TPB + threadIdx.x] = make_float2(v.x, v.z);
            if (2 * pp + 1 < maxa) sZ[(2 * pp + 1) * NB + k * EW_FMM_TPB + threadIdx.x] = make_float2(v.y, v.w);
        }
    }
    float Fh[NS][3], Fl[NS][3];  // per-chunk sums accumulated as hi + lo
#pragma unroll
    for (int k = 0; k < NS; k++)
        for (int d = 0; d < 3; d++) Fh[k][d] = Fl[k][d] = 0.f;
    const int c_lo = A.csplit[blockIdx.y], c_hi = A.csplit[blockIdx.y + 1];
    for (int c = c_lo; c < c_hi; c++) {
        const int m = A.rows[A.forder[c * EW_FCHUNK]].z;
        __syncthreads();
        const ulonglong2 *src = (const ulonglong2 *)(A.fcoef + (size_t)A.coff[c] * EW_FCHUNK);
        for (int i = threadIdx.x; i < (m + 1) * EW_FCHUNK; i += EW_FMM_TPB) sK[i] = src[i];
        if (threadIdx.x < EW_FCHUNK) {
            const int p = c * EW_FCHUNK + threadIdx.x;
            int2 kk = make_int2(0, 0);
            if (p < A.nrows) {
                const int4 r = A.rows[A.forder[p]];
                kk = make_int2(r.x, r.y);
            }
            sR[threadIdx.x] = kk;
        }
        __syncthreads();
        f32x2 W[NS][EW_FCHUNK];
        float Pr[NS][EW_FCHUNK], Pi[NS][EW_FCHUNK];
#pragma unroll
        for (int k = 0; k < NS; k++)
#pragma unroll
            for (int j = 0; j < EW_FCHUNK; j++) {
                W[k][j] = 0;
                Pr[k][j] = Pi[k][j] = 0.f;
            }
        for (int a = 0; a <= m; a++) {
            f32x2 ZR[NS], ZI[NS];
            float azr[NS], azi[NS];
#pragma unroll
            for (int k = 0; k < NS; k++) {
                const float2 z = sZ[a * NB + k * EW_FMM_TPB + threadIdx.x];
                azr[k] = (float)a * z.x;
                azi[k] = (float)a * z.y;
                ZR[k] = pk2(z.x, z.x);
                ZI[k] = pk2(z.y, z.y);
            }
            const ulonglong2 *kr = sK + a * EW_FCHUNK;
#pragma unroll
            for (int j = 0; j < EW_FCHUNK; j++) {
                const ulonglong2 kk = kr[j];  // (k0, k2), (k1, k3)
                float k0, k1, k2, k3;
                up2(kk.x, k0, k2);
                up2(kk.y, k1, k3);
#pragma unroll
                for (int k = 0; k < NS; k++) {
                    W[k][j] = fma2(ZI[k], kk.y, fma2(ZR[k], kk.x, W[k][j]));
                    Pr[k][j] = fmaf(azr[k], k3, fmaf(-azi[k], k2, Pr[k][j]));
                    Pi[k][j] = fmaf(azi[k], k0, fmaf(-azr[k], k1, Pi[k][j]));
                }
            }
        }
#pragma unroll
        for (int k = 0; k < NS; k++) {
            float fx = 0, fy = 0, fz = 0;
#pragma unroll
            for (int j = 0; j < EW_FCHUNK; j++) {
                const int2 kk = sR[j];
                const float2 X = tX[(size_t)kk.x * A.n + site[k]];
                float2 Y = tY[(size_t)(kk.y < 0 ? -kk.y : kk.y) * A.n + site[k]];
                if (kk.y < 0) Y.y = -Y.y;
                const float2 Aa = cmul(X, Y);
                float wr, wi;
                up2(W[k][j], wr, wi);
                const float gsum = Aa.x * wi + Aa.y * wr;
                fx += gsum * (float)kk.x;
                fy += gsum * (float)kk.y;
                fz += Aa.x * Pi[k][j] + Aa.y * Pr[k][j];
            }
            mg_acc2(Fh[k][0], Fl[k][0], fx);
            mg_acc2(Fh[k][1], Fl[k][1], fy);
            mg_acc2(Fh[k][2], Fl[k][2], fz);
        }
    }
#pragma unroll
    for (int k = 0; k < NS; k++) {
        const int a_site = blockIdx.x * NB + k * EW_FMM_TPB + threadIdx.x;
        if (a_site >= A.n) continue;
        if (A.fsplit == 1) {
            const double q = A.q[a_site];
            for (int d = 0; d < 3; d++)
                ew_addf(&A.f[(size_t)d * A.n + a_site], q, (double)Fh[k][d] + (double)Fl[k][d], A.twopi[d]);
        } else {
            for (int d = 0; d < 3; d++)
                A.fpart[((size_t)blockIdx.y * 3 + d) * A.n + a_site] = (double)Fh[k][d] + (double)Fl[k][d];
        }
    }
}

// forces from the partials of the row-chunk ranges, summed in range order
__global__ void k_kforce_sum(EwArgs A) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= A.n) return;
    const double q = A.q[a];
    for (int d = 0; d < 3; d++) {
        double t = 0.0;
        for (int y = 0; y < A.fsplit; y++) t += A.fpart[((size_t)y * 3 + d) * A.n + a];
        ew_addf(&A.f[(size_t)d * A.n + a], q, t, A.twopi[d]);
    }
}

inline size_t fmm_smem(int maxa) {
    return (size_t)maxa * (EW_FCHUNK * sizeof(ulonglong2) + EW_FMM_NS * EW_FMM_TPB * sizeof(float2));
}

// ---------------------------------------------------------------------------------
// Tensor-core k-space forces (FP32 path, KMAXZ <= 30). The four kz sums of one site and
// one row that k_kforce_mm forms with FMAs,
//   W_r = sum_a zr s_r - zi s_i         W_i = sum_a zr d_i + zi d_r
//   W'_r = sum_a a (zr d_r - zi d_i)     W'_i = sum_a a (zr s_i + zi s_r)
// (z = Z^a of the site, s = u + v and d = u - v from the row's S(k) coefficients at |kz| a),
// are, for a tile of KF_SITES sites and KF_ROWS rows, one product
//   D[site][4 row + c] = sum_k A[site][k] B[k][4 row + c],  k = 2a (real part), 2a + 1 (imaginary)
// with A the sites' Z table and B the rows' coefficients, K = 2 (kzmax + 1) <= 64.
// Operands are FP16 hi + lo pairs (hi = x rounded to FP16, lo = the remainder rounded again;
// 22 significant bits, as a TF32 pair) and the MMAs kind::f16 with FP32 accumulation: hi*hi +
// hi*lo + lo*hi, the dropped lo*lo term below 2^-22 relative. |z| <= 1; each row's B is
// scaled by a power of two that brings its largest value into [1/2, 1) (exact, undone in the
// epilogue), so every coefficient of the row is within FP16's range.
// k_fcoef_mma writes every row tile once per call as the shared-memory image the MMAs read
// (K-major, 128-byte swizzle: one 64-wide K atom), and per row its table offsets, wave
// numbers and scale. k_kforce_mma takes KF_SITES sites per CTA: A, the sites' X and Y tables
// and the rows of its range go to shared memory once, then the row tiles stream through,
// warp-specialised:
//   - one thread of the last warp brings each tile's B in by one bulk copy into one of
//     KF_NST stages, KF_NST - 1 tiles ahead, and issues the MMAs into one of two
//     tensor-memory accumulators (128 lanes x KF_N columns), a tcgen05.commit per tile;
//   - eight epilogue warps (warp w: sites 32 (w & 3).., rows 32 (w >> 2)..) wait for a
//     tile's commit, read its accumulator (two passes of 16 rows), release it (an mbarrier
//     the MMA thread waits on before it reuses it), and finish the rows on the CUDA cores:
//     A_k = X^kx Y^ky,
//     gsum = Im(A_k W), Fx += kx gsum, Fy += ky gsum, Fz += Im(A_k W').
// So the tensor core has the next tile queued while the CUDA cores finish the last one.
// A CTA takes its range's tiles in a rotated order (from tile blockIdx.x mod range). Per-tile
// FP32 sums go into hi + lo pairs; the two row halves of a site are added in fixed order at
// the end. Every wait is bounded; a wait that runs out (or sees another role give up) sets a shared abort word that the other waits also poll, so every role stops; then
// the CTA waits (default bound) for its last commit and any copy in flight, records
// MG_FLAG_WAIT_TIMEOUT (and MG_FLAG_MMA_UNDRAINED if that wait ran out too), frees its
// tensor memory and writes NaN forces for its sites.
#define KF_SITES 128
#define KF_ROWS 64
#define KF_N (4 * KF_ROWS)      // MMA N: four sums per row
#define KF_EPI_WARPS 8          // epilogue warps; one more warp issues the copies and MMAs
#define KF_TPB (32 * (KF_EPI_WARPS + 1))
#define KF_MAXKZ 30             // K = 2 (kzmax + 1) <= 64: one 64-wide FP16 atom
#define KF_A_BYTES 16384        // A: 128 sites x 128 bytes (hi or lo)
#define KF_B_BYTES 32768        // B: 256 (row, sum) x 128 bytes (hi or lo)
#define KF_BTILE (2 * KF_B_BYTES) // a row tile's B: hi then lo
#define KF_NST 2                // B stages (freed when the tile's MMAs complete)
#define KF_OFF_B (2 * KF_A_BYTES) // the B stages after A (hi, lo)
#define KF_OFF_XY (KF_OFF_B + KF_NST * KF_BTILE)
#define KF_TCOLS 512            // two accumulators of KF_N columns (all of an SM's tensor memory)
#define KF_MAXSPLIT 2           // row-tile ranges (each CTA stages its sites' tables once per range)

inline size_t kf_smem(int KX, int KY, int ntiles_range) {
    return 1024 + KF_OFF_XY + (size_t)(KX + 1 + KY + 1) * KF_SITES * sizeof(float2) +
           (size_t)ntiles_range * KF_ROWS * sizeof(uint4) + (((size_t)4 * ntiles_range + 15) & ~(size_t)15) + 128;
}

// device layout of the force pass's tiles: B of each row tile, the tiles' kzmax, then per row
// (X offset | Y offset << 16, kx scale, ky scale, scale; the last three as FP32 bits), the
// offsets in float2 units of the staged tables
inline size_t kf_off_tkz(int ntiles) { return (size_t)KF_BTILE * ntiles; }
inline size_t kf_off_rinfo(int ntiles) { return (kf_off_tkz(ntiles) + sizeof(int) * (size_t)ntiles + 15) & ~(size_t)15; }
inline size_t kf_bytes(int ntiles) { return kf_off_rinfo(ntiles) + sizeof(uint4) * (size_t)ntiles * KF_ROWS; }

// byte offset of 16-byte chunk c (elements 8c..8c+7 of a 64-wide FP16 row) of row m in a
// K-major tile with 128-byte rows and the 128-byte swizzle
__device__ __forceinline__ unsigned kf_chunk(int m, int c) {
    return (unsigned)((m >> 3) * 1024 + (m & 7) * 128 + (((c ^ m) & 7) << 4));
}

// FP16 hi + lo of eight FP32 values, as two 16-byte chunks
__device__ __forceinline__ void kf_split8(const float (&x)[8], uint4 &hi, uint4 &lo) {
    f16x2_split(x[0], x[1], hi.x, lo.x);
    f16x2_split(x[2], x[3], hi.y, lo.y);
    f16x2_split(x[4], x[5], hi.z, lo.z);
    f16x2_split(x[6], x[7], hi.w, lo.w);
}

// one warp per row of a tile (grid: tiles x KF_ROWS / 8, eight warps a block): lane (c, ch)
// takes the row's sum c = lane >> 3 and 16-byte chunk ch = lane & 7 (k = 8 ch..8 ch + 7); the
// row's scale (the power of two taking its largest |B| into [1/2, 1)) is the warp's maximum;
// then B as FP16 hi + lo chunks, and the row's table data
__global__ void __launch_bounds__(256) k_fcoef_mma(EwArgs A, unsigned char *__restrict__ fb, int *__restrict__ tkz,
                                                   uint4 *__restrict__ rinfo) {
    const int T = blockIdx.x, lane = threadIdx.x & 31, j = blockIdx.y * 8 + (threadIdx.x >> 5);
    const int p = T * KF_ROWS + j, comp = lane >> 3, ch = lane & 7, n = 4 * j + comp;
    if (blockIdx.y == 0 && threadIdx.x == 0) tkz[T] = A.rows[A.forder[T * KF_ROWS]].z;  // rows run by kzmax
    const float4 *coef = (const float4 *)A.scoef;
    float x[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int4 row = make_int4(0, 0, -1, 0);
    if (p < A.nrows) {
        const int r = A.forder[p];
        row = A.rows[r];
        const int slot = A.row_slot[r] / 2;
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
            const int a = 4 * ch + e / 2;  // k = 8 ch + e (real part), + 1 (imaginary part)
            if (a > row.z) continue;
            const float4 uv = coef[slot + a];  // u_r, u_i, v_r, v_i
            const float sr = uv.x + uv.z, si = uv.y + uv.w, dr = uv.x - uv.z, di = uv.y - uv.w;
            const float fa = (float)a;
            x[e] = comp == 0 ? sr : comp == 1 ? di : comp == 2 ? fa * dr : fa * si;
            x[e + 1] = comp == 0 ? -si : comp == 1 ? dr : comp == 2 ? -fa * di : fa * sr;
        }
    }
    float m = 0.f;
#pragma unroll
    for (int e = 0; e < 8; e++) m = fmaxf(m, fabsf(x[e]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    int e2 = 0;
    frexpf(m, &e2);
    const float inv = ldexpf(1.f, -e2), sc = ldexpf(1.f, e2);  // exact powers of two
#pragma unroll
    for (int e = 0; e < 8; e++) x[e] *= inv;
    uint4 hi, lo;
    kf_split8(x, hi, lo);
    unsigned char *out = fb + (size_t)T * KF_BTILE;
    const unsigned off = kf_chunk(n, ch);
    *(uint4 *)(out + off) = hi;
    *(uint4 *)(out + KF_B_BYTES + off) = lo;
    if (lane == 0) {
        uint4 info = make_uint4(0u, 0u, 0u, 0u);  // padding rows: X^0 Y^0 against zero sums
        if (p < A.nrows)  // the products with the power of two are exact
            info = make_uint4((unsigned)(row.x * KF_SITES) | ((unsigned)((row.y < 0 ? -row.y : row.y) * KF_SITES) << 16),
                              __float_as_uint((float)row.x * sc), __float_as_uint((float)row.y * sc), __float_as_uint(sc));
        rinfo[p] = info;
    }
}

// a bounded mbarrier wait that also gives up when another role of the CTA has given up:
// the non-blocking test (the MMA thread, whose phases are mostly complete already), or the
// potentially blocking try (the epilogue's pollers, which mostly wait and should not flood
// the shared-memory pipe with tests)
template <bool BLOCKING>
__device__ __forceinline__ bool kf_wait(unsigned bar, unsigned parity, long long limit, const volatile int *abort_word) {
    for (long long i = 0; i < limit; i++) {
        unsigned ok;
        if (BLOCKING)
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(ok)
                : "r"(bar), "r"(parity)
                : "memory");
        else
            asm volatile(
                "{\n.reg .pred p;\nmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
                : "=r"(ok)
                : "r"(bar), "r"(parity)
                : "memory");
        if (ok) return true;
        if ((i & 63) == 63 && *abort_word) return false;
    }
    return false;
}

__global__ void __launch_bounds__(KF_TPB, 1)
    k_kforce_mma(EwArgs A, const unsigned char *__restrict__ fb, const int *__restrict__ tkz,
                 const uint4 *__restrict__ rinfo, unsigned *flags) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const unsigned raw = (unsigned)__cvta_generic_to_shared(smem_raw);
    const unsigned base = (raw + 1023u) & ~1023u;  // the swizzled tiles need 1024-byte alignment
    unsigned char *gbase = smem_raw + (base - raw);
    const int KXn = A.kx + 1, KYn = A.ky + 1;
    const int T0 = A.csplit[blockIdx.y], nt = A.csplit[blockIdx.y + 1] - T0;
    // CTAs take the range's tiles starting at different tiles (by site tile), so that at any
    // moment they read different coefficient tiles from L2
    const int rot = nt > 0 ? (int)(blockIdx.x % (unsigned)nt) : 0;
    const unsigned o_rs = KF_OFF_XY + (unsigned)(KXn + KYn) * KF_SITES * 8u;  // the range's rows
    const unsigned o_tkz = o_rs + (unsigned)(nt * KF_ROWS) * 16u;
    const unsigned o_bar = (o_tkz + 4u * (unsigned)nt + 15u) & ~15u;
    // barriers: bfull[KF_NST] (copy landed), mdone[2] (tile's MMAs done), afree[2] (tile's
    // accumulator read); then the tensor-memory address and the abort word
    const unsigned bfull = base + o_bar, mdone = bfull + 8 * KF_NST, afree = mdone + 16, tslot = afree + 16;
    volatile int *abort_word = (volatile int *)(gbase + (tslot - base) + 8);
    float2 *sX = (float2 *)(gbase + KF_OFF_XY), *sY = sX + KXn * KF_SITES;
    uint4 *sRow = (uint4 *)(gbase + o_rs);
    int *sT = (int *)(gbase + o_tkz);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int site0 = blockIdx.x * KF_SITES;
    const unsigned idesc = umma_idesc_f16(KF_N);

    if (threadIdx.x == 0) {
        for (int b = 0; b < KF_NST + 2; b++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bfull + 8 * b), "r"(1) : "memory");
        for (int b = 0; b < 2; b++)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(afree + 8 * b), "r"(KF_EPI_WARPS) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *abort_word = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(tslot), "r"(KF_TCOLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // the sites' X and Y tables and the range's rows by cp.async (all in flight at once), then
    // A: Z^a of the tile's sites as (zr, zi) pairs along k, FP16 hi + lo (zero past the table
    // and past the last site), each thread's loads issued before their stores
    {
        const float2 *tab = (const float2 *)A.tab;
        const float4 *tZP = (const float4 *)(tab + ew_zoff(A.kx, A.ky, A.n));
        const float2 *tX = tab, *tY = tab + (size_t)KXn * A.n;
        for (int it = threadIdx.x; it < (KXn + KYn) * KF_SITES; it += KF_TPB) {
            const int k = it / KF_SITES, sl = it % KF_SITES;
            if (site0 + sl < A.n)
                cp_async(sX + it, k < KXn ? tX + (size_t)k * A.n + site0 + sl : tY + (size_t)(k - KXn) * A.n + site0 + sl,
                         8);
            else
                sX[it] = make_float2(0.f, 0.f);
        }
        for (int i = threadIdx.x; i < nt * KF_ROWS; i += KF_TPB) {  // in the CTA's tile order
            const int li = i / KF_ROWS, T = T0 + (li + rot) % nt;
            cp_async(sRow + i, rinfo + (size_t)T * KF_ROWS + i % KF_ROWS, 16);
        }
        cp_async_commit();
        const int NPP = ew_zpairs(A.kz);
        constexpr int NI = KF_SITES * 8, NJ = (NI + KF_TPB - 1) / KF_TPB;  // (site, chunk of four |kz|)
        float4 z[NJ][2];
#pragma unroll
        for (int j = 0; j < NJ; j++) {
            const int it = threadIdx.x + j * KF_TPB, sl = it % KF_SITES, c = it / KF_SITES;
            const bool in = it < NI && site0 + sl < A.n;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int pp = 2 * c + h;
                z[j][h] = (in && pp < NPP) ? tZP[(size_t)pp * A.n + site0 + sl] : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
#pragma unroll
        for (int j = 0; j < NJ; j++) {
            const int it = threadIdx.x + j * KF_TPB, sl = it % KF_SITES, c = it / KF_SITES;
            if (it >= NI) continue;
            // k = 8c..8c+7: (zr, zi) of |kz| 4c, 4c+1 (pair 2c), 4c+2, 4c+3 (pair 2c + 1)
            const float x[8] = {z[j][0].x, z[j][0].z, z[j][0].y, z[j][0].w, z[j][1].x, z[j][1].z, z[j][1].y, z[j][1].w};
            uint4 hi, lo;
            kf_split8(x, hi, lo);
            const unsigned off = kf_chunk(sl, c);
            *(uint4 *)(gbase + off) = hi;
            *(uint4 *)(gbase + KF_A_BYTES + off) = lo;
        }
        for (int i = threadIdx.x; i < nt; i += KF_TPB) sT[i] = tkz[T0 + (i + rot) % nt];
        cp_async_wait<0>();
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const unsigned tmem = *(volatile unsigned *)(gbase + (tslot - base));

    float Fh[3] = {0.f, 0.f, 0.f}, Fl[3] = {0.f, 0.f, 0.f};
    int copied = 0, issued = 0;  // tiles whose copies / MMAs were issued (MMA thread)
    if (warp == KF_EPI_WARPS) {
        if (lane == 0) {
            // row tile li: its B (hi, lo) into stage li % KF_NST
            auto copy_tile = [&](int li) {
                const unsigned bar = bfull + 8 * (li % KF_NST);
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(KF_BTILE) : "memory");
                asm volatile(
                    "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                        base + KF_OFF_B + (unsigned)(li % KF_NST) * KF_BTILE),
                    "l"(fb + (size_t)(T0 + (li + rot) % nt) * KF_BTILE), "r"(KF_BTILE), "r"(bar)
                    : "memory");
            };
            for (; copied < min(nt, KF_NST - 1); copied++) copy_tile(copied);
            // descriptors differ from the first one by the byte offset / 16 (all shared
            // addresses here are below 2^18, so the 14-bit address field never carries)
            const unsigned long long dA0 = umma_desc(base), dB0 = umma_desc(base + KF_OFF_B);
            for (int li = 0; li < nt; li++) {
                bool ok = kf_wait<false>(bfull + 8 * (li % KF_NST), (li / KF_NST) & 1, A.mma_wait, abort_word);
                // accumulator li & 1 was read by tile li - 2's epilogue
                if (ok && li >= 2) ok = kf_wait<false>(afree + 8 * (li & 1), ((li - 2) >> 1) & 1, A.mma_wait, abort_word);
                if (!ok) {
                    *abort_word = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const int nks = (2 * (sT[li] + 1) + 15) / 16;
                const unsigned acc = tmem + (unsigned)(li & 1) * KF_N;
                const unsigned long long dB = dB0 + (unsigned)(li % KF_NST) * (KF_BTILE >> 4);
#pragma unroll
                for (int ks = 0; ks < 4; ks++) {
                    if (ks < nks) {
                        const unsigned long long ah = dA0 + 2 * ks, al = ah + (KF_A_BYTES >> 4);
                        const unsigned long long bh = dB + 2 * ks, bl = bh + (KF_B_BYTES >> 4);
                        umma_f16(acc, ah, bh, idesc, ks > 0 ? 1u : 0u);
                        umma_f16(acc, ah, bl, idesc, 1u);
                        umma_f16(acc, al, bh, idesc, 1u);
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 mdone + 8 * (li & 1))
                             : "memory");
                issued = li + 1;
                if (li + KF_NST - 1 < nt) {
                    // stage (li + KF_NST - 1) % KF_NST was read by tile li - 1's MMAs
                    if (li >= 1 && !kf_wait<false>(mdone + 8 * ((li - 1) & 1), ((li - 1) >> 1) & 1, A.mma_wait, abort_word)) {
                        *abort_word = 1;
                        break;
                    }
                    copy_tile(li + KF_NST - 1);
                    copied = li + KF_NST;
                }
            }
        }
        __syncwarp();
    } else {
        const int qd = warp & 3, hh = warp >> 2, s = 32 * qd + lane;
        const unsigned tl = tmem + ((unsigned)(32 * qd) << 16) + (unsigned)(KF_N / 2) * (unsigned)hh;
        for (int li = 0; li < nt; li++) {
            const uint4 *rr = sRow + li * KF_ROWS + (KF_ROWS / 2) * hh;
            float fx = 0.f, fy = 0.f, fz = 0.f;
            // lane 0 polls; its answer is the warp's one decision before the warp-wide loads
            int ok = 0;
            if (lane == 0) ok = kf_wait<true>(mdone + 8 * (li & 1), (li >> 1) & 1, A.mma_wait, abort_word);
            ok = __shfl_sync(0xffffffffu, ok, 0);
            if (!ok) {
                if (lane == 0) *abort_word = 1;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            // the warp's 32 rows in two passes of 16 (64 accumulator columns each); the
            // accumulator is released once the second pass has been read
#pragma unroll 1
            for (int pass = 0; pass < 2; pass++) {
            float v[4][16];
            const unsigned col = tl + (unsigned)(li & 1) * KF_N + 64u * (unsigned)pass;
#pragma unroll
            for (int q = 0; q < 4; q++) tmem_ld16(col + 16u * q, v[q]);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (pass == 1) {
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(afree + 8 * (li & 1)) : "memory");
            }
#pragma unroll
            for (int jj = 0; jj < 16; jj++) {
                const uint4 info = rr[16 * pass + jj];
                const float kxs = __uint_as_float(info.y), kys = __uint_as_float(info.z), sc = __uint_as_float(info.w);
                const float2 X = sX[(info.x & 0xffffu) + s];
                float2 Y = sY[(info.x >> 16) + s];
                Y.y = kys < 0.f ? -Y.y : Y.y;
                const float2 Ak = cmul(X, Y);
                const float *w = v[jj >> 2] + 4 * (jj & 3);
                const float g = Ak.x * w[1] + Ak.y * w[0];
                fx += g * kxs;
                fy += g * kys;
                fz += (Ak.x * w[3] + Ak.y * w[2]) * sc;
            }
            }
            mg_acc2(Fh[0], Fl[0], fx);
            mg_acc2(Fh[1], Fl[1], fy);
            mg_acc2(Fh[2], Fl[2], fz);
        }
    }
    __syncthreads();
    const bool timeout = *abort_word != 0;
    if (timeout) {
        // MMAs and copies may still run: wait, with the full default bound, for the commit of
        // the last issued tile (it covers every earlier MMA) and for copies not yet waited on
        bool done = true;
        if (warp == KF_EPI_WARPS && lane == 0) {
            if (issued > 0) done &= mbar_wait(mdone + 8 * ((issued - 1) & 1), ((issued - 1) >> 1) & 1, EW_MMA_WAIT);
            for (int li = issued; li < copied; li++)
                done &= mbar_wait(bfull + 8 * (li % KF_NST), (li / KF_NST) & 1, EW_MMA_WAIT);
        }
        done = __syncthreads_and(done);
        if (threadIdx.x == 0 && flags)
            atomicOr(flags, done ? MG_FLAG_WAIT_TIMEOUT : MG_FLAG_WAIT_TIMEOUT | MG_FLAG_MMA_UNDRAINED);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(KF_TCOLS) : "memory");
    if (warp >= KF_EPI_WARPS) return;
    const int hh = warp >> 2, s = 32 * (warp & 3) + lane, a_site = site0 + s;
    if (timeout) {  // the sites' forces carry the failure
        if (hh == 0 && a_site < A.n) {
            const double nan = __longlong_as_double(0x7ff8000000000000ll);
            for (int d = 0; d < 3; d++) {
                if (A.fsplit == 1) A.f[(size_t)d * A.n + a_site] = nan;
                else A.fpart[((size_t)blockIdx.y * 3 + d) * A.n + a_site] = nan;
            }
        }
        return;
    }
    // the second row half of each site (warps 4..7) joins the first, over A (no MMA reads it now)
    float *cmb = (float *)gbase;
    if (hh == 1)
#pragma unroll
        for (int d = 0; d < 3; d++) {
            cmb[(2 * d) * KF_SITES + s] = Fh[d];
            cmb[(2 * d + 1) * KF_SITES + s] = Fl[d];
        }
    asm volatile("bar.sync 1, %0;" ::"n"(32 * KF_EPI_WARPS) : "memory");  // the epilogue warps only
    if (hh == 0 && a_site < A.n) {
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const double F = ((double)Fh[d] + (double)Fl[d]) +
                             ((double)cmb[(2 * d) * KF_SITES + s] + (double)cmb[(2 * d + 1) * KF_SITES + s]);
            if (A.fsplit == 1) ew_addf(&A.f[(size_t)d * A.n + a_site], A.q[a_site], F, A.twopi[d]);
            else A.fpart[((size_t)blockIdx.y * 3 + d) * A.n + a_site] = F;
        }
    }
}

// Row-tile ranges for k_kforce_mma: S ranges of about equal work (K steps of a tile plus a
// fixed share for its CUDA-core pass), S in [1, smax] chosen so that site tiles x S fill the
// SMs (one CTA each) in whole waves; fills csplit[0..S] in tiles and returns S.
int kf_split(const std::vector<int> &tile_kz, int n, int nsm, int smax, int *csplit) {
    const int nt = (int)tile_kz.size();
    const long long nb = (n + KF_SITES - 1) / KF_SITES;
    smax = std::max(1, std::min(std::min(smax, EW_MAXSPLIT), nt));
    int best = 1;
    double best_eff = 0.0;
    for (int S = 1; S <= smax; S++) {
        const long long items = nb * S, rounds = (items + nsm - 1) / nsm;
        const double eff = (double)items / (double)(rounds * nsm);
        if (eff > best_eff + 0.02) {
            best_eff = eff;
            best = S;
        }
    }
    auto work = [](int kz) { return (long long)((2 * (kz + 1) + 15) / 16) + 4; };
    long long total = 0;
    for (int k : tile_kz) total += work(k);
    csplit[0] = 0;
    long long acc = 0;
    int c = 0;
    for (int y = 1; y < best; y++) {
        const long long target = total * y / best;
        while (c < nt && acc + work(tile_kz[c]) <= target) acc += work(tile_kz[c++]);
        csplit[y] = std::max(c, csplit[y - 1]);
    }
    csplit[best] = nt;
    return best;
}

int device_sms() {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    return std::max(1, nsm);
}

// whether the tensor-core force pass takes these tables (KMAXZ and the shared-memory budget)
bool kf_fits(int KX, int KY, int KZ, int nrows) {
    return nrows > 0 && std::max(KZ, 1) <= KF_MAXKZ &&
           kf_smem(KX, KY, (nrows + KF_ROWS - 1) / KF_ROWS) <= (size_t)227 * 1024;
}

// kzmax of each row tile (its first row) from the kzmax of each EW_FCHUNK-row chunk
std::vector<int> kf_tile_kz(const std::vector<int> &chunk_kz, int nrows) {
    std::vector<int> t((nrows + KF_ROWS - 1) / KF_ROWS);
    for (size_t T = 0; T < t.size(); T++) t[T] = chunk_kz[T * KF_ROWS / EW_FCHUNK];
    return t;
}

// launches of the tensor-core force pass for A (A.csplit / A.fsplit in row tiles; fb holds
// the B tiles, then their kzmax): B tiles, forces and, for a split, the sum
cudaError_t kf_launch(const EwArgs &A, unsigned char *fb, int ntiles, unsigned *flags, cudaStream_t s) {
    int *tkz = (int *)(fb + kf_off_tkz(ntiles));
    uint4 *rinfo = (uint4 *)(fb + kf_off_rinfo(ntiles));
    int range = 0;
    for (int y = 0; y < A.fsplit; y++) range = std::max(range, A.csplit[y + 1] - A.csplit[y]);
    const size_t smem = kf_smem(A.kx, A.ky, range);
    k_fcoef_mma<<<dim3((unsigned)ntiles, KF_ROWS / 8), 256, 0, s>>>(A, fb, tkz, rinfo);
    cudaError_t e = cudaFuncSetAttribute(k_kforce_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const dim3 grid((unsigned)((A.n + KF_SITES - 1) / KF_SITES), (unsigned)A.fsplit);
    k_kforce_mma<<<grid, KF_TPB, smem, s>>>(A, fb, tkz, rinfo, flags);
    if (A.fsplit > 1) k_kforce_sum<<<(A.n + 255) / 256, 256, 0, s>>>(A);
    return cudaGetLastError();
}

// resident blocks of k_kforce_mm per SM x SMs, per device and dynamic shared memory size
int fmm_slots(int maxa) {
    static std::mutex mu;
    static int cache_dev = -1, cache_maxa = -1, cache_slots = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lock(mu);
    if (dev == cache_dev && maxa == cache_maxa) return cache_slots;
    const size_t smem = fmm_smem(maxa);
    int per_sm = 0, nsm = 0;
    cudaFuncSetAttribute(k_kforce_mm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_kforce_mm, EW_FMM_TPB, smem);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaGetLastError();
    cache_dev = dev;
    cache_maxa = maxa;
    cache_slots = std::max(1, per_sm) * std::max(1, nsm);
    return cache_slots;
}

// Splits the chunks into S ranges of about equal work (sum of kzmax + 1) and picks S in
// [1, smax] so that site blocks x S fill the device's resident-block slots in whole
// waves; returns S and fills csplit[0..S].
int fmm_split(const std::vector<int> &chunk_kz, int n, int slots, int smax, int *csplit) {
    const int nc = (int)chunk_kz.size();
    const long long nb = (n + EW_FMM_NS * EW_FMM_TPB - 1) / (EW_FMM_NS * EW_FMM_TPB);
    smax = std::max(1, std::min(std::min(smax, EW_MAXSPLIT), nc));
    int best = 1;
    double best_eff = 0.0;
    for (int S = 1; S <= smax; S++) {
        const long long items = nb * S;
        const long long rounds = (items + slots - 1) / slots;
        const double eff = (double)items / (double)(rounds * slots);
        if (eff > best_eff + 0.02) {
            best_eff = eff;
            best = S;
        }
    }
    long long total = 0;
    for (int k : chunk_kz) total += k + 1;
    csplit[0] = 0;
    long long acc = 0;
    int c = 0;
    for (int y = 1; y < best; y++) {
        const long long target = total * y / best;
        while (c < nc && acc + chunk_kz[c] + 1 <= target) {
            acc += chunk_kz[c] + 1;
            c++;
        }
        csplit[y] = std::max(c, csplit[y - 1]);
    }
    csplit[best] = nc;
    return best;
}

// chunk kzmax (first row of each chunk) from a kzmax histogram of the rows
std::vector<int> fmm_chunk_kz(const int *hist, int nrows) {
    std::vector<int> out((nrows + EW_FCHUNK - 1) / EW_FCHUNK);
    int pos = 0;
    for (int k = 255; k >= 0; k--)
        for (int i = 0; i < hist[k]; i++, pos++)
            if (pos % EW_FCHUNK == 0) out[pos / EW_FCHUNK] = k;
    return out;
}

// launches of the FP32 force pass for A (with the table pass: coefficients, forces and,
// for a split, the sum)
int fmm_launches(const EwArgs &A, int maxa) {
    if (!A.fcoef || maxa > EW_FMM_MAXA) return 1;
    return A.fsplit > 1 ? 3 : 2;
}

// The FP32 table force pass's tables and buffers of a context (none for the FP64 path
// or rows longer than EW_FMM_MAXA, which take k_kforce); false if a buffer could not
// be allocated.
bool ew_force_fields(mg_ctx *c, EwArgs &A, int maxa) {
    A.fcoef = nullptr;
    A.fpart = nullptr;
    A.fsplit = 1;
    const int nr = c->nrows;
    A.forder = (const int *)c->d_row_slot.p + nr + c->nslots;
    A.rpos = A.forder + nr;
    A.coff = A.rpos + nr;
    A.nchunk = (int)c->h_chunk_kz.size();
    A.csplit[0] = 0;
    A.csplit[1] = A.nchunk;
    if (c->opt.precision == MG_PREC_FP64 || maxa > EW_FMM_MAXA || A.nchunk == 0) return true;
    size_t ncoef = 0;
    for (int k : c->h_chunk_kz) ncoef += (size_t)(k + 1) * EW_FCHUNK;
    if (!mg_ensure(c, c->d_fcoef, sizeof(float4) * ncoef)) return false;
    A.fcoef = (float4 *)c->d_fcoef.p;
    A.fsplit = fmm_split(c->h_chunk_kz, A.n, fmm_slots(maxa), EW_MAXSPLIT, A.csplit);
    if (A.fsplit > 1) {
        if (!mg_ensure(c, c->d_fpart, sizeof(double) * 3 * (size_t)A.fsplit * A.n)) return false;
        A.fpart = (double *)c->d_fpart.p;
    }
    return true;
}

// k_kforce with fg threads per site (2, 4 or 8) and its dynamic shared memory
template <typename R>
cudaError_t launch_kforce(int fg, unsigned blocks, size_t smem, cudaStream_t s, const EwArgs &A, int maxa) {
    cudaError_t e;
    if constexpr (std::is_same<R, float>::value) {
        if (A.fcoef && maxa <= EW_FMM_MAXA) {
            if (A.n == 0 || A.nchunk == 0) return cudaSuccess;
            k_fcoef<<<A.nchunk, 256, 0, s>>>(A);
            const size_t msmem = fmm_smem(maxa);
            e = cudaFuncSetAttribute(k_kforce_mm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)msmem);
            if (e != cudaSuccess) return e;
            const dim3 grid((unsigned)((A.n + EW_FMM_NS * EW_FMM_TPB - 1) / (EW_FMM_NS * EW_FMM_TPB)), (unsigned)A.fsplit);
            k_kforce_mm<<<grid, EW_FMM_TPB, msmem, s>>>(A, maxa);
            if (A.fsplit > 1) k_kforce_sum<<<(A.n + 255) / 256, 256, 0, s>>>(A);
            return cudaGetLastError();
        }
        switch (fg) {
        case 2:
            e = cudaFuncSetAttribute(k_kforce_f2<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_kforce_f2<2><<<blocks, 2 * EW_FSITES, smem, s>>>(A, maxa);
            break;
        case 8:
            e = cudaFuncSetAttribute(k_kforce_f2<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_kforce_f2<8><<<blocks, 8 * EW_FSITES, smem, s>>>(A, maxa);
            break;
        default:
            e = cudaFuncSetAttribute(k_kforce_f2<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_kforce_f2<4><<<blocks, 4 * EW_FSITES, smem, s>>>(A, maxa);
        }
    } else {
        switch (fg) {
        case 2:
            e = cudaFuncSetAttribute(k_kforce<R, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_kforce<R, 2><<<blocks, 2 * EW_FSITES, smem, s>>>(A, maxa);
            break;
        case 8:
            e = cudaFuncSetAttribute(k_kforce<R, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_kforce<R, 8><<<blocks, 8 * EW_FSITES, smem, s>>>(A, maxa);
            break;
        default:
            e = cudaFuncSetAttribute(k_kforce<R, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) k_kforce<R, 4><<<blocks, 4 * EW_FSITES, smem, s>>>(A, maxa);
        }
    }
    return e == cudaSuccess ? cudaGetLastError() : e;
}

}  // namespace

// k-vector rows for the half space and the S(k)-pass tasks
mg_status mg_ewald_setup(mg_ctx *c) {
    const mg_params &p = c->params;
    int KX = p.kmax[0], KY = p.kmax[1], KZ = p.kmax[2], KS = p.ksqmax;
    std::vector<int> rows, slot_start, slot_row;
    std::vector<int4> tasks;
    int nslots = 0;
    long long kvec = 0;
    ew_for_rows(KX, KY, KZ, KS, [&](int kx, int ky, int kzmax, int half) {
        int r = (int)(rows.size() / 4);
        rows.push_back(kx);
        rows.push_back(ky);
        rows.push_back(kzmax);
        rows.push_back(half);
        slot_start.push_back(nslots);
        int ns = 2 * (kzmax + 1);
        for (int s = 0; s < ns; s++) slot_row.push_back(r);
        nslots += ns;
        kvec += half ? kzmax : 2 * kzmax + 1;
        const int nv = kzmax + 1;
        for (int h = 0; h < ew_nchunk(nv); h++) {
            int k0, len;
            ew_chunk(nv, h, k0, len);
            tasks.push_back(make_int4(r, k0, len, 0));
        }
    });
    // longest first; within a length by first |kz|, so that a warp's tasks mostly share their
    // Z loads (broadcast shared-memory reads)
    std::stable_sort(tasks.begin(), tasks.end(),
                     [](const int4 &a, const int4 &b) { return a.z != b.z ? a.z > b.z : a.y < b.y; });
    {  // pad each length group to whole warps with empty tasks (row 0, count 0)
        std::vector<int4> padded;
        padded.reserve(tasks.size() + 32 * EW_CH);
        for (size_t i = 0; i < tasks.size(); i++) {
            padded.push_back(tasks[i]);
            if (i + 1 == tasks.size() || tasks[i + 1].z != tasks[i].z)
                while (padded.size() % 32) padded.push_back(make_int4(0, 0, 0, 0));
        }
        tasks.swap(padded);
    }
    c->nrows = (int)(rows.size() / 4);
    c->nslots = nslots;
    c->kvectors = kvec;
    c->ntasks = (int)tasks.size();
    c->kmaxx = KX;
    c->kmaxy = KY;
    c->kmaxz = KZ;
    c->h_rows = rows;
    c->ewald_box[0] = c->lx;
    c->ewald_box[1] = c->ly;
    c->ewald_box[2] = c->lz;
    c->h_chunk_kz.clear();
    if (c->nrows == 0) return MG_OK;
    // force order of the FP32 table pass: rows by kzmax, longest first (ties in row order),
    // then the chunks' coefficient offsets
    const int nr = c->nrows;
    std::vector<int> forder(nr), rpos(nr);
    std::iota(forder.begin(), forder.end(), 0);
    std::stable_sort(forder.begin(), forder.end(), [&](int a, int b) { return rows[4 * a + 2] > rows[4 * b + 2]; });
    for (int q = 0; q < nr; q++) rpos[forder[q]] = q;
    const int nchunk = (nr + EW_FCHUNK - 1) / EW_FCHUNK;
    std::vector<int> coff(nchunk + 1, 0);
    c->h_chunk_kz.resize(nchunk);
    for (int k = 0; k < nchunk; k++) {
        c->h_chunk_kz[k] = rows[4 * forder[k * EW_FCHUNK] + 2];
        coff[k + 1] = coff[k] + c->h_chunk_kz[k] + 1;
    }
    std::vector<int> packed;
    packed.reserve(slot_start.size() + slot_row.size() + 2 * nr + nchunk + 1);
    packed.insert(packed.end(), slot_start.begin(), slot_start.end());
    packed.insert(packed.end(), slot_row.begin(), slot_row.end());
    packed.insert(packed.end(), forder.begin(), forder.end());
    packed.insert(packed.end(), rpos.begin(), rpos.end());
    packed.insert(packed.end(), coff.begin(), coff.end());
    if (!mg_ensure(c, c->d_rows, sizeof(int) * rows.size()) || !mg_ensure(c, c->d_row_slot, sizeof(int) * packed.size()) ||
        !mg_ensure(c, c->d_tasks, sizeof(int4) * tasks.size()))
        return MG_ERR_ALLOC;
    MG_CUDA(cudaMemcpy(c->d_rows.p, rows.data(), sizeof(int) * rows.size(), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(c->d_row_slot.p, packed.data(), sizeof(int) * packed.size(), cudaMemcpyHostToDevice));
    MG_CUDA(cudaMemcpy(c->d_tasks.p, tasks.data(), sizeof(int4) * tasks.size(), cudaMemcpyHostToDevice));
    return MG_OK;
}

namespace {
__global__ void k_add_forces(size_t m, double *__restrict__ f, const double *__restrict__ g) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < m) f[i] += g[i];
}
}  // namespace

#ifndef MG_KSTREAM_HIGH
#define MG_KSTREAM_HIGH 0  // the chain's stream at the highest priority (else the lowest)
#endif

// Starts the reciprocal-space chain on the context's second stream (created on first
// use): it waits for what the context's stream has enqueued so
// far, writes its forces into d_fk (zeroed first) and its energy rows into d_erows_k.
mg_status mg_ewald_fork(mg_ctx *c, const double *dx, const double *dy, const double *dz) {
    c->forked = false;
    if (!c->kstream) {
        int least = 0, greatest = 0;
        MG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
        MG_CUDA(cudaStreamCreateWithPriority(&c->kstream, cudaStreamNonBlocking, MG_KSTREAM_HIGH ? greatest : least));
        MG_CUDA(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
        MG_CUDA(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
    }
    const unsigned rblocks = (unsigned)((c->nslots + 255) / 256);
    if (!mg_ensure(c, c->d_fk, sizeof(double) * 3 * (size_t)c->natom) ||
        !mg_ensure(c, c->d_erows_k, sizeof(double) * E_NCOMP * (size_t)rblocks))
        return mg_fail(c, MG_ERR_ALLOC, "k-space chain buffers");
    cudaStream_t s = c->stream;
    MG_CUDA(cudaEventRecord(c->ev_fork, s));
    MG_CUDA(cudaStreamWaitEvent(c->kstream, c->ev_fork, 0));
    c->stream = c->kstream;
    if (c->timing) cudaEventRecord(c->ev[3], c->kstream);
    mg_status st = MG_OK;
    if (cudaMemsetAsync(c->d_fk.p, 0, sizeof(double) * 3 * (size_t)c->natom, c->kstream) != cudaSuccess)
        st = mg_fail(c, MG_ERR_CUDA, "cudaMemsetAsync");
    c->ew_rows = (double *)c->d_erows_k.p;
    if (!st) st = mg_launch_ewald(c, dx, dy, dz, (double *)c->d_fk.p);
    c->ew_rows = nullptr;
    if (c->timing) cudaEventRecord(c->ev[5], c->kstream);
    cudaEventRecord(c->ev_join, c->kstream);
    c->stream = s;
    if (!st) c->forked = true;
    return st;
}

// Waits on the context's stream for the chain, adds its forces into fl and copies its
// energy rows into rows reserved now (where the serial order reserves them).
mg_status mg_ewald_join(mg_ctx *c, double *fl) {
    cudaStream_t s = c->stream;
    MG_CUDA(cudaStreamWaitEvent(s, c->ev_join, 0));
    const size_t m = 3 * (size_t)c->natom;
    k_add_forces<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(m, fl, (const double *)c->d_fk.p);
    MG_CUDA(cudaGetLastError());
    const unsigned rblocks = (unsigned)((c->nslots + 255) / 256);
    const int r0 = mg_reserve_rows(c, rblocks);
    if (r0 < 0) return mg_fail(c, MG_ERR_ALLOC, "energy partial rows exhausted");
    MG_CUDA(cudaMemcpyAsync((double *)c->d_epart.p + (size_t)r0 * E_NCOMP, c->d_erows_k.p,
                            sizeof(double) * E_NCOMP * rblocks, cudaMemcpyDeviceToDevice, s));
    c->launches += 1;
    return MG_OK;
}

bool mg_ewald_sk_tensor(const mg_ctx *c) {
    static_assert(EW_MMA_SITES % EW_SITES == 0, "tensor-core site blocks must cover whole S(k) partial blocks");
    return c->opt.precision != MG_PREC_FP64 && c->kspace_tensor && std::max(c->kmaxz, 1) <= EW_MMA_MAXKZ;
}

// the k-space forces on the tensor cores (k_kforce_mma): FP32 path, tensor passes on,
// KMAXZ <= 30, and the sites' X and Y tables fit in shared memory beside the operands
bool mg_ewald_kf_tensor(const mg_ctx *c) {
    return c->opt.precision != MG_PREC_FP64 && c->kspace_tensor && kf_fits(c->kmaxx, c->kmaxy, c->kmaxz, c->nrows);
}

// the tensor-core force pass of a context: B tiles, row-tile ranges, launches
static mg_status launch_kforce_mma(mg_ctx *c, EwArgs &A, cudaStream_t s, int *launches) {
    const std::vector<int> tile_kz = kf_tile_kz(c->h_chunk_kz, c->nrows);
    const int ntiles = (int)tile_kz.size();
    if (!mg_ensure(c, c->d_kfb, kf_bytes(ntiles)))
        return mg_fail(c, MG_ERR_ALLOC, "k-space force tiles");
    A.forder = (const int *)c->d_row_slot.p + c->nrows + c->nslots;
    A.fcoef = nullptr;
    A.fpart = nullptr;
    A.fsplit = kf_split(tile_kz, A.n, device_sms(), KF_MAXSPLIT, A.csplit);
    if (A.fsplit > 1) {
        if (!mg_ensure(c, c->d_fpart, sizeof(double) * 3 * (size_t)A.fsplit * A.n))
            return mg_fail(c, MG_ERR_ALLOC, "k-space partial forces");
        A.fpart = (double *)c->d_fpart.p;
    }
    MG_CUDA(kf_launch(A, (unsigned char *)c->d_kfb.p, ntiles, (unsigned *)c->d_flags.p, s));
    *launches = A.fsplit > 1 ? 3 : 2;
    return MG_OK;
}

bool mg_ewald_horner_force(const mg_ctx *c) {
    const int maxa = c->h_chunk_kz.empty() ? 1 : c->h_chunk_kz[0] + 1;
    return c->opt.precision == MG_PREC_FP64 || maxa > EW_FMM_MAXA;
}

mg_status mg_launch_ewald(mg_ctx *c, const double *dx, const double *dy, const double *dz, double *fl) {
    if (c->nrows == 0) return MG_OK;
    const mg_params &p = c->params;
    const int n = c->natom;
    const bool fp64 = c->opt.precision == MG_PREC_FP64;
    const size_t esz = fp64 ? sizeof(double2) : sizeof(float2);
    const int KX = c->kmaxx, KY = c->kmaxy, KZ = std::max(c->kmaxz, 1);
    const size_t tab_entries = fp64 ? (size_t)(KX + 1 + KY + 1 + KZ + 1) * n : ew_tabf_entries(KX, KY, KZ, n);
    const int nblk = (n + EW_SITES - 1) / EW_SITES;
    if ((!fp64 && !mg_ensure(c, c->d_qf, sizeof(float) * (size_t)n)) || !mg_ensure(c, c->d_phase, esz * tab_entries) ||
        !mg_ensure(c, c->d_spart, (esz / 2) * 2 * (size_t)c->nslots * nblk) ||
        !mg_ensure(c, c->d_scoef, esz * (size_t)c->nslots))
        return MG_ERR_ALLOC;
    const double twopi = 6.283185307179586;
    double sc[3] = {p.twopi_lx / twopi, p.twopi_ly / twopi, p.twopi_lz / twopi};
    cudaStream_t s = c->stream;
    if (fp64)
        k_phase_d<<<(n + 127) / 128, 128, 0, s>>>(n, dx, dy, dz, sc[0], sc[1], sc[2], KX, KY, KZ, (double2 *)c->d_phase.p);
    else
        k_phase_f<<<dim3((n + 127) / 128, 3), 128, 0, s>>>(n, dx, dy, dz, sc[0], sc[1], sc[2], KX, KY, KZ, (float2 *)c->d_phase.p);
    EwArgs A = {};
    A.n = n;
    A.nrows = c->nrows;
    A.nslots = c->nslots;
    A.ntasks = c->ntasks;
    A.kx = KX;
    A.ky = KY;
    A.kz = KZ;
    A.rows = (const int4 *)c->d_rows.p;
    A.row_slot = (const int *)c->d_row_slot.p;
    A.tasks = (const int4 *)c->d_tasks.p;
    A.tab = c->d_phase.p;
    A.q = (const double *)c->d_site_q.p;
    A.qf = (float *)c->d_qf.p;
    A.spart = c->d_spart.p;
    A.scoef = c->d_scoef.p;
    A.twopi[0] = p.twopi_lx;
    A.twopi[1] = p.twopi_ly;
    A.twopi[2] = p.twopi_lz;
    A.bfac = p.bfactor_ewald;
    A.vfac = p.vfactor_ewald;
    A.coul = p.coulomb_prefactor;
    A.rows_e = (double *)c->d_epart.p;
    A.f = fl;
    A.flags = (const unsigned *)c->d_flags.p;
    A.mma_wait = mg_wait_limit();
    int nblk_red = nblk;
    if (fp64) {
        MG_CUDA(launch_sk<double>(A, nblk, s));
    } else if (mg_ewald_sk_tensor(c)) {
        A.forder = (const int *)c->d_row_slot.p + c->nrows + c->nslots;
        MG_CUDA(launch_sk_mma(A, (unsigned *)c->d_flags.p, s, &nblk_red));
    } else {
        MG_CUDA(launch_sk<float>(A, nblk, s));
    }
    const int *slot_row = (const int *)c->d_row_slot.p + c->nrows;
    unsigned rblocks = (unsigned)((c->nslots + 255) / 256);
    if (c->ew_rows) {  // enqueued on its own stream: rows of its own, copied in at the join
        A.rows_e = c->ew_rows;
        A.row0 = 0;
    } else {
        A.row0 = mg_reserve_rows(c, rblocks);
        if (A.row0 < 0) return mg_fail(c, MG_ERR_ALLOC, "energy partial rows exhausted");
    }
    if (fp64)
        k_sk_reduce<double><<<rblocks, EW_RED_PARTS * 256, 0, s>>>(A, nblk, slot_row);
    else
        k_sk_reduce<float><<<rblocks, EW_RED_PARTS * 256, 0, s>>>(A, nblk_red, slot_row);
    if (c->timing) cudaEventRecord(c->ev[4], s);
    int maxa = 1;
    for (int r = 0; r < c->nrows; r++) maxa = std::max(maxa, c->h_rows[4 * r + 2] + 1);
    size_t fsmem = 2 * esz * (size_t)EW_FROWS * maxa;
    unsigned fblocks = (unsigned)((n + EW_FSITES - 1) / EW_FSITES);
    if (fp64) {
        MG_CUDA(launch_kforce<double>(c->tune.kforce_threads, fblocks, fsmem, s, A, maxa));
        c->launches += 4;
    } else if (mg_ewald_kf_tensor(c)) {
        int nl = 0;
        const mg_status st = launch_kforce_mma(c, A, s, &nl);
        if (st) return st;
        c->launches += 3 + nl;
    } else {
        if (!ew_force_fields(c, A, maxa)) return mg_fail(c, MG_ERR_ALLOC, "k-space force buffers");
        MG_CUDA(launch_kforce<float>(c->tune.kforce_threads, fblocks, fsmem, s, A, maxa));
        c->launches += 3 + fmm_launches(A, maxa);
    }
    return MG_OK;
}

// ---------------------------------------------------------------------------------
// mg_ewald_recip_static: the same reciprocal-space pass with no device allocation
// ---------------------------------------------------------------------------------
// Every piece of scratch (k-vector row and task tables, phase tables, S(k) partials and
// coefficients, energy rows, the status word) is carved out of g_ew_scratch. Its device
// address is looked up once per device, with that device current, and handed to the
// kernels as a plain pointer. The row and task tables depend on KMAX/KSQMAX only; the key
// they were built for is kept in the first words of the scratch, and the table kernel,
// launched by every call, compares it on the device and rebuilds only on a change, so the
// check holds in stream order and inside a captured graph alike. Every other byte a kernel
// reads was written before in the same call (the status word is cleared per call). Calls on
// one device share the array; calls that are not ordered on the device race on it.
namespace {

static __device__ __align__(256) unsigned char g_ew_scratch[MG_EWALD_STATIC_SCRATCH_BYTES];

constexpr int EW_STATIC_MAX_DEVICES = 64;

struct EwStaticDevice {
    unsigned char *base = nullptr;  // device address of g_ew_scratch on this device
};
constexpr int EW_STATIC_KEY_MAGIC = 0x6d677374;  // marks a key word block the table kernel wrote
EwStaticDevice g_ew_static[EW_STATIC_MAX_DEVICES];
std::mutex g_ew_static_mutex;
std::atomic<int> g_ew_static_split{0};  // row split of the last call's force pass

struct EwCounts {
    int nrows = 0, nslots = 0, ntasks = 0, maxa = 1;
    std::vector<int> chunk_kz;  // kzmax of each chunk of the FP32 table force pass
};

EwCounts ew_count(int KX, int KY, int KZ, int KS) {
    EwCounts c;
    int by_len[EW_CH + 1] = {0};
    int hist[256] = {0};
    ew_for_rows(KX, KY, KZ, KS, [&](int, int, int kzmax, int) {
        int nv = kzmax + 1;
        hist[kzmax]++;
        c.nrows++;
        c.nslots += 2 * nv;
        c.maxa = std::max(c.maxa, nv);
        for (int h = 0; h < ew_nchunk(nv); h++) {
            int k0, len;
            ew_chunk(nv, h, k0, len);
            by_len[len]++;
        }
    });
    for (int L = 1; L <= EW_CH; L++) c.ntasks += (by_len[L] + 31) / 32 * 32;
    c.chunk_kz = fmm_chunk_kz(hist, c.nrows);
    return c;
}

// Row table, packed slot table (first slot of each row, then the row of each slot) and
// the task list sorted by length (longest first), then first |kz|, then row, with each
// length group padded to whole warps: the same tables mg_ewald_setup builds on the host.
// With key != null (the allocation-free pass) the kernel first compares key[0..4] with
// (magic, KX, KY, KZ, KS) and returns when the tables in place were built for them.
__global__ void k_ew_tables(int KX, int KY, int KZ, int KS, int nrows, int nslots, int4 *__restrict__ rows,
                            int *__restrict__ row_slot, int4 *__restrict__ tasks, int *__restrict__ key) {
    if (key) {
        const bool same = key[0] == EW_STATIC_KEY_MAGIC && key[1] == KX && key[2] == KY && key[3] == KZ && key[4] == KS;
        if (same) return;  // uniform over the block: every thread reads the same words
        __syncthreads();   // all threads have read the old key before thread 0 rewrites it
        if (threadIdx.x == 0) {
            key[0] = EW_STATIC_KEY_MAGIC;
            key[1] = KX;
            key[2] = KY;
            key[3] = KZ;
            key[4] = KS;
        }
    }
    if (threadIdx.x == 0) {
        int r = 0, slot = 0;
        ew_for_rows(KX, KY, KZ, KS, [&](int kx, int ky, int kzmax, int half) {
            rows[r] = make_int4(kx, ky, kzmax, half);
            row_slot[r] = slot;
            slot += 2 * (kzmax + 1);
            r++;
        });
        // counting sort by (length descending, first |kz| ascending), ties in row order;
        // each length group padded to whole warps
        int pos[EW_CH + 1][128];
        for (int L = 0; L <= EW_CH; L++)
            for (int k = 0; k < 128; k++) pos[L][k] = 0;
        for (int q = 0; q < nrows; q++) {
            const int nv = rows[q].z + 1;
            for (int h = 0; h < ew_nchunk(nv); h++) {
                int k0, len;
                ew_chunk(nv, h, k0, len);
                pos[len][k0 / 2]++;
            }
        }
        int t = 0;
        for (int L = EW_CH; L >= 1; L--) {
            const int start = t;
            for (int k = 0; k < 128; k++) {
                const int c = pos[L][k];
                pos[L][k] = t;
                t += c;
            }
            if (t > start)
                while (t % 32) tasks[t++] = make_int4(0, 0, 0, 0);
        }
        for (int q = 0; q < nrows; q++) {
            const int nv = rows[q].z + 1;
            for (int h = 0; h < ew_nchunk(nv); h++) {
                int k0, len;
                ew_chunk(nv, h, k0, len);
                tasks[pos[len][k0 / 2]++] = make_int4(q, k0, len, 0);
            }
        }
        // force order (kzmax descending, ties in row order) and chunk offsets, by a
        // counting sort over kzmax <= 255
        int *forder = row_slot + nrows + nslots, *rpos = forder + nrows, *coff = rpos + nrows;
        int start[256];
        for (int k = 0; k < 256; k++) start[k] = 0;
        for (int q = 0; q < nrows; q++) start[rows[q].z]++;
        for (int k = 255, run = 0; k >= 0; k--) {
            const int h = start[k];
            start[k] = run;
            run += h;
        }
        for (int q = 0; q < nrows; q++) {
            const int p = start[rows[q].z]++;
            forder[p] = q;
            rpos[q] = p;
        }
        const int nchunk = (nrows + EW_FCHUNK - 1) / EW_FCHUNK;
        coff[0] = 0;
        for (int k = 0; k < nchunk; k++) coff[k + 1] = coff[k] + rows[forder[k * EW_FCHUNK]].z + 1;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nrows; q += blockDim.x) {
        int s0 = row_slot[q], ns = 2 * (rows[q].z + 1);
        for (int s = 0; s < ns; s++) row_slot[nrows + s0 + s] = q;
    }
}

// fixed-order sum of the reciprocal energy over the S(k) reduction's block rows
// the Fourier energy of the allocation-free pass; NaN when a bounded on-chip wait of the
// tensor-core S(k) pass ran out (flags), so that the failure shows without a host sync
__global__ void k_ew_energy(const double *__restrict__ erows, int nrows, const unsigned *__restrict__ flags,
                            double *__restrict__ out) {
    __shared__ double s[256];
    double t = 0.0;
    for (int r = threadIdx.x; r < nrows; r += blockDim.x) t += erows[(size_t)r * E_NCOMP + E_UFOURIER];
    s[threadIdx.x] = t;
    __syncthreads();
    for (int o = blockDim.x >> 1; o > 0; o >>= 1) {
        if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = (flags && (*flags & MG_FLAG_WAIT_TIMEOUT)) ? __longlong_as_double(0x7ff8000000000000ll) : s[0];
}

mg_status ew_static_fail(char *err, size_t err_len, mg_status code, const char *fmt, ...) {
    if (err && err_len) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, err_len, fmt, ap);
        va_end(ap);
    }
    return code;
}

// selects a device for the duration of a call and restores the caller's on exit
struct EwDeviceGuard {
    int prev = -1;
    bool changed = false;
    cudaError_t select(int dev) {
        cudaError_t e = cudaGetDevice(&prev);
        if (e != cudaSuccess) return e;
        if (prev == dev) return cudaSuccess;
        e = cudaSetDevice(dev);
        changed = e == cudaSuccess;
        return e;
    }
    ~EwDeviceGuard() {
        if (changed) cudaSetDevice(prev);
    }
};

inline size_t ew_align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" mg_status mg_ewald_recip_static(int device, void *stream, int precision, int natom,
                                           const double *d_x, const double *d_y, const double *d_z,
                                           const double *d_q, const mg_params *p, double *d_f,
                                           double *d_energy, char *err, size_t err_len) {
#define EWS_CUDA(call, what)                                                                            \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            cudaGetLastError();                                                                         \
            return ew_static_fail(err, err_len, MG_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e_)); \
        }                                                                                               \
    } while (0)
    if (err && err_len) err[0] = 0;
    if (!p || natom < 0 || (precision != MG_PREC_MIXED && precision != MG_PREC_FP64))
        return ew_static_fail(err, err_len, MG_ERR_INVALID, "invalid arguments (params, natom or precision)");
    if (natom > 0 && (!d_x || !d_y || !d_z || !d_q || !d_f))
        return ew_static_fail(err, err_len, MG_ERR_INVALID, "null device pointer");
    const int KX = p->kmax[0], KY = p->kmax[1], KZ0 = p->kmax[2], KS = p->ksqmax;
    if (KX < 0 || KY < 0 || KZ0 < 0 || KX > 255 || KY > 255 || KZ0 > 255 || KS < 0)
        return ew_static_fail(err, err_len, MG_ERR_INVALID, "kmax must lie in [0, 255] and ksqmax be >= 0");
    if (device < 0 || device >= EW_STATIC_MAX_DEVICES)
        return ew_static_fail(err, err_len, MG_ERR_NO_DEVICE, "device %d out of range", device);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device >= ndev) {
        cudaGetLastError();
        return ew_static_fail(err, err_len, MG_ERR_NO_DEVICE, "no CUDA device %d", device);
    }
    EwDeviceGuard guard;
    EWS_CUDA(guard.select(device), "cudaSetDevice");
    cudaStream_t s = (cudaStream_t)stream;
    std::lock_guard<std::mutex> lock(g_ew_static_mutex);
    EwStaticDevice &dev = g_ew_static[device];
    if (!dev.base) {  // set-up, once per device, with the device current
        int major = 0, minor = 0;
        EWS_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, device), "cudaDeviceGetAttribute");
        EWS_CUDA(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, device), "cudaDeviceGetAttribute");
        if (major != 10 || minor != 3)
            return ew_static_fail(err, err_len, MG_ERR_NO_DEVICE, "device %d is sm_%d%d; the kernels are built for sm_103a",
                                  device, major, minor);
        void *ptr = nullptr;
        EWS_CUDA(cudaGetSymbolAddress(&ptr, g_ew_scratch), "cudaGetSymbolAddress");
        dev.base = (unsigned char *)ptr;
    }
    const bool fp64 = precision == MG_PREC_FP64;
    const int n = natom;
    const EwCounts ct = ew_count(KX, KY, KZ0, KS);
    if (n == 0 || ct.nrows == 0) {  // nothing to sum: zero forces and energy
        if (n > 0) EWS_CUDA(cudaMemsetAsync(d_f, 0, sizeof(double) * 3 * (size_t)n, s), "cudaMemsetAsync");
        if (d_energy) EWS_CUDA(cudaMemsetAsync(d_energy, 0, sizeof(double), s), "cudaMemsetAsync");
        return MG_OK;
    }
    // scratch layout: tables first (their offsets depend on KMAX/KSQMAX only), then the
    // per-call arrays
    const size_t esz = fp64 ? sizeof(double2) : sizeof(float2);
    const int KZ = std::max(KZ0, 1);
    const int nblk = (n + EW_SITES - 1) / EW_SITES;
    const unsigned rblocks = (unsigned)((ct.nslots + 255) / 256);
    size_t off = 256;  // words 0..4: the key of the row and task tables (k_ew_tables)
    const size_t o_rows = off;
    off += ew_align256(sizeof(int4) * (size_t)ct.nrows);
    const int nchunk = (int)ct.chunk_kz.size();
    const size_t o_slot = off;  // slot starts, slot rows, force order, its inverse, chunk offsets
    off += ew_align256(sizeof(int) * ((size_t)3 * ct.nrows + ct.nslots + nchunk + 1));
    const size_t o_tasks = off;
    off += ew_align256(sizeof(int4) * (size_t)ct.ntasks);
    const size_t o_tab = off;
    off += ew_align256(fp64 ? esz * (size_t)(KX + 1 + KY + 1 + KZ + 1) * n : esz * ew_tabf_entries(KX, KY, KZ, n));
    const size_t o_qf = off;
    if (!fp64) off += ew_align256(sizeof(float) * (size_t)n);
    const size_t o_spart = off;
    off += ew_align256((esz / 2) * 2 * (size_t)ct.nslots * nblk);
    const size_t o_coef = off;
    off += ew_align256(esz * (size_t)ct.nslots);
    const size_t o_erows = off;
    off += ew_align256(sizeof(double) * E_NCOMP * (size_t)rblocks);
    const size_t o_flags = off;  // status word of the tensor-core S(k) pass
    off += 256;
    // the force pass: on the tensor cores where the context's mixed path takes it there
    // (the same kernels, so both entry points give the same bits), else the FP32 table pass
    const bool kf_tensor = !fp64 && kf_fits(KX, KY, KZ0, ct.nrows);
    const bool table_force = !fp64 && !kf_tensor && ct.maxa <= EW_FMM_MAXA;
    size_t ncoef = 0;
    for (int k : ct.chunk_kz) ncoef += (size_t)(k + 1) * EW_FCHUNK;
    const size_t o_fcoef = off;
    if (table_force) off += ew_align256(sizeof(float4) * ncoef);
    const int kf_ntiles = (ct.nrows + KF_ROWS - 1) / KF_ROWS;
    const size_t o_kfb = off;
    if (kf_tensor) off += ew_align256(kf_bytes(kf_ntiles));
    if (off > (size_t)MG_EWALD_STATIC_SCRATCH_BYTES)
        return ew_static_fail(err, err_len, MG_ERR_CAPACITY,
                              "%d sites with kmax (%d,%d,%d), ksqmax %d need %zu bytes of scratch; the limit is %u",
                              n, KX, KY, KZ0, KS, off, (unsigned)MG_EWALD_STATIC_SCRATCH_BYTES);
    unsigned char *base = dev.base;
    int4 *rows = (int4 *)(base + o_rows);
    int *row_slot = (int *)(base + o_slot);
    int4 *tasks = (int4 *)(base + o_tasks);
    k_ew_tables<<<1, 256, 0, s>>>(KX, KY, KZ0, KS, ct.nrows, ct.nslots, rows, row_slot, tasks, (int *)base);
    EWS_CUDA(cudaGetLastError(), "k_ew_tables launch");
    EWS_CUDA(cudaMemsetAsync(d_f, 0, sizeof(double) * 3 * (size_t)n, s), "cudaMemsetAsync");
    EWS_CUDA(cudaMemsetAsync(base + o_flags, 0, sizeof(unsigned), s), "cudaMemsetAsync");
    const double twopi = 6.283185307179586;
    const double sc[3] = {p->twopi_lx / twopi, p->twopi_ly / twopi, p->twopi_lz / twopi};
    void *tab = base + o_tab;
    if (fp64)
        k_phase_d<<<(n + 127) / 128, 128, 0, s>>>(n, d_x, d_y, d_z, sc[0], sc[1], sc[2], KX, KY, KZ, (double2 *)tab);
    else
        k_phase_f<<<dim3((n + 127) / 128, 3), 128, 0, s>>>(n, d_x, d_y, d_z, sc[0], sc[1], sc[2], KX, KY, KZ, (float2 *)tab);
    EwArgs A = {};
    A.n = n;
    A.nrows = ct.nrows;
    A.nslots = ct.nslots;
    A.ntasks = ct.ntasks;
    A.kx = KX;
    A.ky = KY;
    A.kz = KZ;
    A.rows = rows;
    A.row_slot = row_slot;
    A.tasks = tasks;
    A.tab = tab;
    A.q = d_q;
    A.qf = (float *)(base + o_qf);
    A.spart = base + o_spart;
    A.scoef = base + o_coef;
    A.twopi[0] = p->twopi_lx;
    A.twopi[1] = p->twopi_ly;
    A.twopi[2] = p->twopi_lz;
    A.bfac = p->bfactor_ewald;
    A.vfac = p->vfactor_ewald;
    A.coul = p->coulomb_prefactor;
    A.rows_e = (double *)(base + o_erows);
    A.row0 = 0;
    A.f = d_f;
    A.flags = (const unsigned *)(base + o_flags);
    A.mma_wait = mg_wait_limit();
    A.forder = row_slot + ct.nrows + ct.nslots;
    A.rpos = A.forder + ct.nrows;
    A.coff = A.rpos + ct.nrows;
    A.nchunk = nchunk;
    A.fsplit = 1;
    A.csplit[0] = 0;
    A.csplit[1] = nchunk;
    if (table_force || kf_tensor) {
        if (table_force) A.fcoef = (float4 *)(base + o_fcoef);
        // partial forces of a row split in what scratch is left
        const size_t left = (size_t)MG_EWALD_STATIC_SCRATCH_BYTES - off;
        const size_t per = sizeof(double) * 3 * (size_t)n;
        const int smax = (int)std::min<size_t>(kf_tensor ? KF_MAXSPLIT : EW_MAXSPLIT, per ? left / per : 1);
        if (kf_tensor) {
            A.fsplit = kf_split(kf_tile_kz(ct.chunk_kz, ct.nrows), n, device_sms(), std::max(smax, 1), A.csplit);
            if (A.fsplit > 1) A.fpart = (double *)(base + ew_align256(off));
        } else if (smax >= 2) {
            A.fsplit = fmm_split(ct.chunk_kz, n, fmm_slots(ct.maxa), smax, A.csplit);
            if (A.fsplit > 1) A.fpart = (double *)(base + ew_align256(off));
        }
    }
    const int *slot_row = row_slot + ct.nrows;
    const size_t fsmem = 2 * esz * (size_t)EW_FROWS * ct.maxa;
    const unsigned fblocks = (unsigned)((n + EW_FSITES - 1) / EW_FSITES);
    if (fp64) {
        EWS_CUDA(launch_sk<double>(A, nblk, s), "k_sk launch");
        k_sk_reduce<double><<<rblocks, EW_RED_PARTS * 256, 0, s>>>(A, nblk, slot_row);
        EWS_CUDA(cudaFuncSetAttribute(k_kforce<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem),
                 "cudaFuncSetAttribute");
        k_kforce<double><<<fblocks, EW_FG * EW_FSITES, fsmem, s>>>(A, ct.maxa);
    } else {
        int nblk_red = nblk;
        if (KZ <= EW_MMA_MAXKZ)
            EWS_CUDA(launch_sk_mma(A, (unsigned *)(base + o_flags), s, &nblk_red), "k_sk_mma launch");
        else
            EWS_CUDA(launch_sk<float>(A, nblk, s), "k_sk launch");
        k_sk_reduce<float><<<rblocks, EW_RED_PARTS * 256, 0, s>>>(A, nblk_red, slot_row);
        if (kf_tensor)
            EWS_CUDA(kf_launch(A, base + o_kfb, kf_ntiles, (unsigned *)(base + o_flags), s), "k_kforce_mma launch");
        else
            EWS_CUDA(launch_kforce<float>(EW_FG, fblocks, fsmem, s, A, ct.maxa), "k_kforce launch");
    }
    if (d_energy) k_ew_energy<<<1, 256, 0, s>>>(A.rows_e, (int)rblocks, (const unsigned *)(base + o_flags), d_energy);
    EWS_CUDA(cudaGetLastError(), "kernel launch");
    g_ew_static_split.store(A.fsplit);
    return MG_OK;
#undef EWS_CUDA
}

extern "C" int mg_ewald_recip_static_last_split(void) { return g_ew_static_split.load(); }

// ---------------------------------------------------------------------------------
// adjoint support: structure factors with arbitrary site weights, the k-space field and
// the per-class reciprocal-space charge gradient (used by mg_adjoint.cu)
// ---------------------------------------------------------------------------------
namespace {

// S_w(k) per slot from the block partials, summed in FP64 in block order
template <typename R>
__global__ void k_sk_sum(EwArgs A, int nblk, double2 *__restrict__ out) {
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= A.nslots) return;
    double sr = 0.0, si = 0.0;
    for (int b = 0; b < nblk; b++) {
        const R *p = (const R *)A.spart + ((size_t)b * A.nslots + slot) * 2;
        sr += (double)p[0];
        si += (double)p[1];
    }
    out[slot] = make_double2(sr, si);
}

// sum over slots of cf Im(conj(T^c) (k . A)) per class c, as fixed-order block rows
__global__ void k_kgrad(EwArgs A, const int *__restrict__ slot_row, const double2 *__restrict__ SA,
                        const double2 *__restrict__ ST, int nclass, double *__restrict__ rows) {
    __shared__ double red[256];
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    double cf = 0.0, bx = 0.0, by = 0.0;
    if (slot < A.nslots) {
        const int r = slot_row[slot];
        const int4 row = A.rows[r];
        const int local = slot - A.row_slot[r];
        const int a = local >> 1, minus = local & 1;
        const bool valid = a <= row.z && !(minus && (a == 0 || row.w)) && !(row.w && a == 0);
        if (valid) {
            const double kz = minus ? -a : a;
            const double k0 = A.twopi[0] * row.x, k1 = A.twopi[1] * row.y, k2 = A.twopi[2] * kz;
            const double rksq = k0 * k0 + k1 * k1 + k2 * k2;
            cf = 4.0 * A.vfac * A.coul * exp(-A.bfac * rksq) / rksq;
            const double2 ax = SA[slot], ay = SA[A.nslots + slot], az = SA[2 * A.nslots + slot];
            bx = k0 * ax.x + k1 * ay.x + k2 * az.x;
            by = k0 * ax.y + k1 * ay.y + k2 * az.y;
        }
    }
    for (int c = 0; c < nclass; c++) {
        double v = 0.0;
        if (cf != 0.0) {
            const double2 t = ST[(size_t)c * A.nslots + slot];
            v = cf * (t.x * by - t.y * bx);
        }
        red[threadIdx.x] = v;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) rows[(size_t)blockIdx.x * nclass + c] = red[0];
        __syncthreads();
    }
}

EwArgs ew_args(mg_ctx *c) {
    const mg_params &p = c->params;
    EwArgs A = {};
    A.n = c->natom;
    A.nrows = c->nrows;
    A.nslots = c->nslots;
    A.ntasks = c->ntasks;
    A.kx = c->kmaxx;
    A.ky = c->kmaxy;
    A.kz = std::max(c->kmaxz, 1);
    A.rows = (const int4 *)c->d_rows.p;
    A.row_slot = (const int *)c->d_row_slot.p;
    A.tasks = (const int4 *)c->d_tasks.p;
    A.tab = c->d_phase.p;
    A.q = (const double *)c->d_site_q.p;
    A.qf = (float *)c->d_qf.p;
    A.spart = c->d_spart.p;
    A.scoef = c->d_scoef.p;
    A.twopi[0] = p.twopi_lx;
    A.twopi[1] = p.twopi_ly;
    A.twopi[2] = p.twopi_lz;
    A.bfac = p.bfactor_ewald;
    A.vfac = p.vfactor_ewald;
    A.coul = p.coulomb_prefactor;
    const int maxa = c->h_chunk_kz.empty() ? 1 : c->h_chunk_kz[0] + 1;
    if (!ew_force_fields(c, A, maxa)) {  // the Horner pass needs no extra buffers
        A.fcoef = nullptr;
        A.fsplit = 1;
    }
    return A;
}

}  // namespace

// S_w(k) of every slot for site weights w (device [n]), with the phase tables of the
// last long-range evaluation
mg_status mg_ewald_weighted_sk(mg_ctx *c, const double *w, double2 *out) {
    if (c->nrows == 0) return MG_OK;
    const bool fp64 = c->opt.precision == MG_PREC_FP64;
    EwArgs A = ew_args(c);
    A.q = w;
    const int nblk = (A.n + EW_SITES - 1) / EW_SITES;
    cudaStream_t s = c->stream;
    const unsigned sb = (unsigned)((A.nslots + 255) / 256);
    if (fp64) {
        MG_CUDA(launch_sk<double>(A, nblk, s));
        k_sk_sum<double><<<sb, 256, 0, s>>>(A, nblk, out);
    } else {
        MG_CUDA(launch_sk<float>(A, nblk, s));
        k_sk_sum<float><<<sb, 256, 0, s>>>(A, nblk, out);
    }
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}

// the reciprocal-space force per unit charge (field[3][n], overwritten), from the
// coefficients of the last long-range evaluation
mg_status mg_ewald_field(mg_ctx *c, const double *ones, double *field) {
    cudaStream_t s = c->stream;
    MG_CUDA(cudaMemsetAsync(field, 0, sizeof(double) * 3 * (size_t)c->natom, s));
    if (c->nrows == 0) return MG_OK;
    const bool fp64 = c->opt.precision == MG_PREC_FP64;
    const size_t esz = fp64 ? sizeof(double2) : sizeof(float2);
    EwArgs A = ew_args(c);
    A.q = ones;
    A.f = field;
    int maxa = 1;
    for (int r = 0; r < c->nrows; r++) maxa = std::max(maxa, c->h_rows[4 * r + 2] + 1);
    const size_t fsmem = 2 * esz * (size_t)EW_FROWS * maxa;
    const unsigned fblocks = (unsigned)((A.n + EW_FSITES - 1) / EW_FSITES);
    if (fp64) {
        MG_CUDA(cudaFuncSetAttribute(k_kforce<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem));
        k_kforce<double><<<fblocks, EW_FG * EW_FSITES, fsmem, s>>>(A, maxa);
    } else {
        MG_CUDA(launch_kforce<float>(EW_FG, fblocks, fsmem, s, A, maxa));
    }
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}

// per-class sums over k of cf Im(conj(T^c) (k . A)) as block rows rows[nblocks][nclass]
mg_status mg_ewald_kgrad(mg_ctx *c, const double2 *SA, const double2 *ST, int nclass, double *rows, int *nblocks) {
    *nblocks = 0;
    if (c->nrows == 0) return MG_OK;
    EwArgs A = ew_args(c);
    const unsigned b = (unsigned)((A.nslots + 255) / 256);
    k_kgrad<<<b, 256, 0, c->stream>>>(A, (const int *)c->d_row_slot.p + c->nrows, SA, ST, nclass, rows);
    MG_CUDA(cudaGetLastError());
    *nblocks = (int)b;
    return MG_OK;
}

// ---------------------------------------------------------------------------------
// Hessian-vector product support: the directional derivative of the reciprocal-space
// force F_i = q_i sum_k cf_k Im(conj(S_k) e^{ik.r_i}) k along site displacements v:
//   dF_i = q_i sum_k cf_k k [ (k.v_i) Re(conj(S_k) e^{ik.r_i}) - Re(conj(S^v_k) e^{ik.r_i}) ]
// with S^v_k = sum_j q_j (k.v_j) e^{ik.r_j}. The first term is q_i M_i v_i with the per-site
// matrix M_i = sum_k cf_k Re(conj(S_k) e^{ik.r_i}) k k^T (k_khess, the k-force pass with
// second derivatives of the row polynomials); the second is the k-force pass itself run
// on the coefficients i cf_k S^v_k (k_hvcoef).
// ---------------------------------------------------------------------------------
namespace {

template <typename R>
__global__ void __launch_bounds__(EW_FG * EW_FSITES) k_khess(EwArgs A, int maxa, const double *__restrict__ v,
                                                             double *__restrict__ out) {
    typedef typename C2<R>::T T2;
    typedef typename C2<R>::T4 T4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T4 *sC = (T4 *)smem_raw;
    __shared__ int4 sRow[EW_FROWS];
    __shared__ double sM[EW_FG][6][EW_FSITES];
    const int g = threadIdx.x / EW_FSITES, l = threadIdx.x % EW_FSITES;
    const int a = blockIdx.x * EW_FSITES + l;
    const bool act = a < A.n;
    const T2 *tab = (const T2 *)A.tab;
    const T2 *tX = tab, *tY = tab + (size_t)(A.kx + 1) * A.n;
    T2 Z;
    if (act) {
        Z = ew_z1<R>(A.tab, A.kx, A.ky, A.n, a);
    } else {
        Z.x = (R)1;
        Z.y = (R)0;
    }
    double M[6] = {0, 0, 0, 0, 0, 0};  // xx xy yy xz yz zz in integer k units
    const T4 *coef = (const T4 *)A.scoef;
    for (int r0 = 0; r0 < A.nrows; r0 += EW_FROWS) {
        const int nr = min(EW_FROWS, A.nrows - r0);
        __syncthreads();
        for (int i = threadIdx.x; i < nr * maxa; i += blockDim.x) {
            int rr = i / maxa, s = i % maxa;
            int4 row = A.rows[r0 + rr];
            T4 c4;
            c4.x = c4.y = c4.z = c4.w = (R)0;
            if (s <= row.z) c4 = coef[A.row_slot[r0 + rr] / 2 + s];
            sC[rr * maxa + s] = c4;
        }
        if (threadIdx.x < nr) sRow[threadIdx.x] = A.rows[r0 + threadIdx.x];
        __syncthreads();
        if (!act) continue;
        R m[6] = {0, 0, 0, 0, 0, 0};
        for (int rr = g; rr < nr; rr += EW_FG) {
            const int4 row = sRow[rr];
            T2 X = tX[(size_t)row.x * A.n + a];
            T2 Y = tY[(size_t)(row.y < 0 ? -row.y : row.y) * A.n + a];
            if (row.y < 0) Y.y = -Y.y;
            const T2 Aa = cmul(X, Y);
            const T4 *cs = sC + rr * maxa;
            // Horner with the first and half the second derivative: p = P(Z), dp = P'(Z),
            // hp = P''(Z)/2, and the same for Q
            const T4 top = cs[row.z];
            T2 p, q, dp, dq, hp, hq;
            p.x = top.x; p.y = top.y;
            q.x = top.z; q.y = top.w;
            dp.x = dp.y = dq.x = dq.y = hp.x = hp.y = hq.x = hq.y = (R)0;
            for (int k = row.z - 1; k >= 0; k--) {
                const T4 c = cs[k];
                T2 cu, cv;
                cu.x = c.x; cu.y = c.y;
                cv.x = c.z; cv.y = c.w;
                hp = cfma(hp, Z, dp);
                dp = cfma(dp, Z, p);
                p = cfma(p, Z, cu);
                hq = cfma(hq, Z, dq);
                dq = cfma(dq, Z, q);
                q = cfma(q, Z, cv);
            }
            // sum_a a c_a Z^a = Z P'(Z); sum_a a^2 c_a Z^a = Z P'(Z) + Z^2 P''(Z)
            const T2 zdp = cmul(Z, dp), zdq = cmul(Z, dq);
            const T2 z2 = cmul(Z, Z);
            const T2 hp2 = cmul(z2, hp), hq2 = cmul(z2, hq);
            T2 s2p, s2q;
            s2p.x = zdp.x + (R)2 * hp2.x; s2p.y = zdp.y + (R)2 * hp2.y;
            s2q.x = zdq.x + (R)2 * hq2.x; s2q.y = zdq.y + (R)2 * hq2.y;
            // Re(A w) for plus slots, Re(A conj(w)) for minus slots (kz = -a)
            const R r0s = (Aa.x * p.x - Aa.y * p.y) + (Aa.x * q.x + Aa.y * q.y);
            const R r1s = (Aa.x * zdp.x - Aa.y * zdp.y) - (Aa.x * zdq.x + Aa.y * zdq.y);
            const R r2s = (Aa.x * s2p.x - Aa.y * s2p.y) + (Aa.x * s2q.x + Aa.y * s2q.y);
            const R kx = (R)row.x, ky = (R)row.y;
            m[0] += kx * kx * r0s;
            m[1] += kx * ky * r0s;
            m[2] += ky * ky * r0s;
            m[3] += kx * r1s;
            m[4] += ky * r1s;
            m[5] += r2s;
        }
        for (int k = 0; k < 6; k++) M[k] += (double)m[k];
    }
    for (int k = 0; k < 6; k++) sM[g][k][l] = M[k];
    __syncthreads();
    if (g != 0 || !act) return;
    double t[6] = {0, 0, 0, 0, 0, 0};
    for (int j = 0; j < EW_FG; j++)
        for (int k = 0; k < 6; k++) t[k] += sM[j][k][l];
    const double tx = A.twopi[0], ty = A.twopi[1], tz = A.twopi[2];
    const double xx = t[0] * tx * tx, xy = t[1] * tx * ty, yy = t[2] * ty * ty;
    const double xz = t[3] * tx * tz, yz = t[4] * ty * tz, zz = t[5] * tz * tz;
    const double vx = v[a], vy = v[A.n + a], vz = v[2 * A.n + a];
    const double q = A.q[a];
    out[a] += q * (xx * vx + xy * vy + xz * vz);
    out[A.n + a] += q * (xy * vx + yy * vy + yz * vz);
    out[2 * A.n + a] += q * (xz * vx + yz * vy + zz * vz);
}

// k-force coefficients i cf S^v_k, S^v_k = sum_d k_d SW_d(k), in the layout of k_sk_reduce
// (plus slots conjugated)
template <typename R>
__global__ void k_hvcoef(EwArgs A, const int *__restrict__ slot_row, const double2 *__restrict__ SW,
                         void *__restrict__ coef) {
    typedef typename C2<R>::T T2;
    const int slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= A.nslots) return;
    const int r = slot_row[slot];
    const int4 row = A.rows[r];
    const int local = slot - A.row_slot[r];
    const int a = local >> 1, minus = local & 1;
    const bool valid = a <= row.z && !(minus && (a == 0 || row.w)) && !(row.w && a == 0);
    T2 c;
    c.x = c.y = (R)0;
    if (valid) {
        const double kz = minus ? -a : a;
        const double k0 = A.twopi[0] * row.x, k1 = A.twopi[1] * row.y, k2 = A.twopi[2] * kz;
        const double rksq = k0 * k0 + k1 * k1 + k2 * k2;
        const double cf = 4.0 * A.vfac * A.coul * exp(-A.bfac * rksq) / rksq;
        const double2 sx = SW[slot], sy = SW[A.nslots + slot], sz = SW[2 * A.nslots + slot];
        const double vr = k0 * sx.x + k1 * sy.x + k2 * sz.x, vi = k0 * sx.y + k1 * sy.y + k2 * sz.y;
        // X = i cf S^v = cf (-vi, vr); plus slots hold conj(X)
        c.x = (R)(-cf * vi);
        c.y = (R)(minus ? cf * vr : -cf * vr);
    }
    ((T2 *)coef)[slot] = c;
}

}  // namespace

// adds the directional derivative of the reciprocal-space force along v ([3][n]) to out,
// given SW[3][nslots], the structure factors with weights q_j v_j,d, and scratch for one
// coefficient array (nslots complex values of the working precision)
mg_status mg_ewald_jvp(mg_ctx *c, const double *v, const double2 *SW, void *coef_scratch, double *out) {
    if (c->nrows == 0) return MG_OK;
    const bool fp64 = c->opt.precision == MG_PREC_FP64;
    const size_t esz = fp64 ? sizeof(double2) : sizeof(float2);
    EwArgs A = ew_args(c);
    int maxa = 1;
    for (int r = 0; r < c->nrows; r++) maxa = std::max(maxa, c->h_rows[4 * r + 2] + 1);
    const size_t fsmem = 2 * esz * (size_t)EW_FROWS * maxa;
    const unsigned fblocks = (unsigned)((A.n + EW_FSITES - 1) / EW_FSITES);
    const unsigned sb = (unsigned)((A.nslots + 255) / 256);
    const int *slot_row = (const int *)c->d_row_slot.p + c->nrows;
    cudaStream_t s = c->stream;
    EwArgs B = A;
    B.scoef = coef_scratch;
    B.f = out;
    if (fp64) {
        MG_CUDA(cudaFuncSetAttribute(k_khess<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem));
        k_khess<double><<<fblocks, EW_FG * EW_FSITES, fsmem, s>>>(A, maxa, v, out);
        k_hvcoef<double><<<sb, 256, 0, s>>>(A, slot_row, SW, coef_scratch);
        MG_CUDA(cudaFuncSetAttribute(k_kforce<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem));
        k_kforce<double><<<fblocks, EW_FG * EW_FSITES, fsmem, s>>>(B, maxa);
    } else {
        MG_CUDA(cudaFuncSetAttribute(k_khess<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem));
        k_khess<float><<<fblocks, EW_FG * EW_FSITES, fsmem, s>>>(A, maxa, v, out);
        k_hvcoef<float><<<sb, 256, 0, s>>>(A, slot_row, SW, coef_scratch);
        MG_CUDA(launch_kforce<float>(EW_FG, fblocks, fsmem, s, B, maxa));
    }
    MG_CUDA(cudaGetLastError());
    return MG_OK;
}
