// mg_nblist.cu - cluster build and cluster-pair (Verlet) list on the GPU.
//
// Replaces the O(N^2) site-pair scan of src/frclong.c:56-218 with a list of pairs of
// clusters of at most 8 sites. The list is a deterministic function of the FP64
// positions:
//   1. sites are binned into an ncx x ncy grid of columns by their wrapped FP64
//      position (x - L*floor(x/L)); the column width is min((8/density)^(1/3),
//      0.75*rlist), so clusters stay compact even in dilute systems;
//   2. each column is sorted by (wrapped z, site index) on chip and cut into clusters
//      of consecutive sites: a new cluster starts after 8 sites or when a site lies more
//      than the column width above the cluster's first site;
//   3. an i-cluster lists j-cluster J under periodic image s when the FP64 distance
//      between their bounding boxes is below rlist = max(rcutoff, rcutoffelec) + skin.
// The search runs one warp per i-cluster and one lane per candidate column; inside a
// column the z-sorted clusters are bracketed by binary search. Each candidate is first
// tested in FP32 against rlist^2 -/+ a margin that bounds the FP32 rounding error;
// only candidates inside that band are decided by the FP64 predicate, evaluated with
// explicit round-to-nearest intrinsics in the same order as the CPU builder of
// oracle/nblist_oracle.c, so the two lists agree bit for bit. No step waits for the
// host: capacities are checked on the device and reported in the status word, and with
// a Verlet skin the rebuild decision (any site moved more than skin/2) is taken on the
// device too. Boxes too small for one image per cluster pair use an all-cluster-pairs
// list with the minimum image applied per site pair in the pair kernel.
#include <math.h>

#include <algorithm>

#include "mg_internal.cuh"

// d_meta layout (int units): [0] ncl (0 when the clusters overflowed their buffers),
// [1] max column count, [2] need-rebuild flag, [3] builds since creation, [4..5] (64-bit)
// entries written, [6] clusters the build asked for
#define META_NCL 0
#define META_MAXCOL 1
#define META_NEED 2
#define META_BUILDS 3
#define META_NPAIRS 4
#define META_NCL_TOTAL 6
#define MG_WIN_MARGIN 1e-9  // columns added on each side of a search window

namespace {

// Image count and column index by a product with the reciprocal rounded once on the host
// (a division takes many FP64 instructions, and FP64 is slow on this part). The CPU builder
// uses the same products, so the two stay bit-identical; a wrapped coordinate may lie an
// ulp outside [0, L), which the column clamp and the cluster boxes take as it is.
__device__ __forceinline__ double wrap_coord(double x, double L, double invL, double *img) {
    double n = floor(__dmul_rn(x, invL));
    *img = __dmul_rn(n, L);
    return __dsub_rn(x, *img);
}

__device__ __forceinline__ int column_of(double w, double icw, int nc) {
    int c = (int)floor(__dmul_rn(w, icw));
    return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

// counter[key] += 1 for every calling lane, one atomic per distinct key of the warp (sites in
// molecule order put about three a warp in each column); returns the lane's value of the
// counter before its own increment (lanes of one key in lane order)
__device__ __forceinline__ int warp_add1(int *__restrict__ counter, int key) {
    const unsigned act = __activemask();
    const unsigned peers = __match_any_sync(act, key);
    const int lane = (int)(threadIdx.x & 31), leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&counter[key], __popc(peers));
    base = __shfl_sync(act, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

__global__ void k_bin(int n, int ncol, const double *__restrict__ x, const double *__restrict__ y,
                      const double *__restrict__ z, double lx, double ly, double lz, double ilx, double ily,
                      double ilz, double icwx, double icwy, int ncx, int ncy, double *__restrict__ xb,
                      double *__restrict__ img, int *__restrict__ col_of, int *__restrict__ col_count,
                      const int *__restrict__ meta) {
    if (!meta[META_NEED]) return;
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    double ix, iy, iz;
    double wx = wrap_coord(x[a], lx, ilx, &ix), wy = wrap_coord(y[a], ly, ily, &iy), wz = wrap_coord(z[a], lz, ilz, &iz);
    xb[a] = wx;
    xb[n + a] = wy;
    xb[2 * n + a] = wz;
    img[a] = ix;
    img[n + a] = iy;
    img[2 * n + a] = iz;
    int col = column_of(wy, icwy, ncy) * ncx + column_of(wx, icwx, ncx);
    col_of[a] = col;
    warp_add1(col_count, col);
}

__global__ void k_zero(int *__restrict__ p, int count, const int *__restrict__ meta) {
    if (!meta[META_NEED]) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) p[i] = 0;
}

// Single-block exclusive scan of count[0..nc) into start (start[nc] = total); also resets
// `fill`, and with max_out != null stores the largest count. *total_out gets the total,
// or 0 when it exceeds cap (cap >= 0): a cluster count above the buffers' capacity leaves
// the build empty, so no later kernel of the call reads a cluster that was not written,
// and the call is repeated with larger buffers sized from *total_raw.
__global__ void k_scan(int nc, const int *__restrict__ count, int *__restrict__ start, int *__restrict__ fill,
                       int *__restrict__ total_out, int *__restrict__ max_out, int cap, int *__restrict__ total_raw,
                       const int *__restrict__ meta) {
    if (!meta[META_NEED]) return;
    __shared__ int s_sum[32], s_max[32];
    const int t = threadIdx.x, nt = blockDim.x, lane = t & 31, w = t >> 5;
    const int per = (nc + nt - 1) / nt;
    const int b = t * per, e = min(nc, b + per);
    int sum = 0, mx = 0;
    for (int i = b; i < e; i++) {
        sum += count[i];
        mx = max(mx, count[i]);
    }
    // exclusive scan of the per-thread sums: within each warp by shuffles, then over the
    // warps' totals by the first warp
    int incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    int wm = mx;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wm = max(wm, __shfl_xor_sync(0xffffffffu, wm, o));
    if (lane == 31) s_sum[w] = incl;
    if (lane == 0) s_max[w] = wm;
    __syncthreads();
    if (w == 0) {
        const int nw = nt >> 5;
        int v = lane < nw ? s_sum[lane] : 0, m = lane < nw ? s_max[lane] : 0;
        int vi = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int u = __shfl_up_sync(0xffffffffu, vi, o);
            if (lane >= o) vi += u;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane < nw) s_sum[lane] = vi - v;  // exclusive prefix of the warps
        if (lane == 31) {
            const int a = vi;  // the total (warps beyond nw add zero)
            start[nc] = a;
            if (total_out) *total_out = (cap >= 0 && a > cap) ? 0 : a;
            if (total_raw) *total_raw = a;
            if (max_out) *max_out = m;
        }
    }
    __syncthreads();
    int a = s_sum[w] + incl - sum;
    for (int i = b; i < e; i++) {
        start[i] = a;
        if (fill) fill[i] = 0;
        a += count[i];
    }
}

__global__ void k_scatter(int n, const int *__restrict__ col_of, const int *__restrict__ start,
                          int *__restrict__ fill, int *__restrict__ sorted, const int *__restrict__ meta) {
    if (!meta[META_NEED]) return;
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    int col = col_of[a];
    int slot = warp_add1(fill, col);  // the order within a column is undone by the z sort
    sorted[start[col] + slot] = a;
}

// A 64-bit integer with the order of the FP64 value d (and -0 equal to +0): comparisons of
// these run on the integer pipes, those of doubles on the slow FP64 pipe.
__device__ __forceinline__ long long order_key(double d) {
    const long long b = __double_as_longlong(d);
    return (b << 1) == 0 ? 0 : (b < 0 ? b ^ 0x7fffffffffffffffLL : b);
}

// One block per column: sort its sites by (wrapped z, index) in place (bitonic, on integer
// keys with the order of z), count the clusters the cutting rule makes and record where
// each starts (cut[start + k] = first sorted position of the column's cluster k). The rule
// (a cluster ends after MG_CL sites or before the first site more than zcap above its first
// one) is sequential; each position's successor cut is found in parallel first, so that
// the walk from cut to cut is a chain of table reads.
__global__ void k_sort_columns(int n, const int *__restrict__ start, int *__restrict__ sorted,
                               const double *__restrict__ xb, double zcap, int *__restrict__ col_ncl,
                               int *__restrict__ cut, unsigned *__restrict__ flags, const int *__restrict__ meta) {
    if (!meta[META_NEED]) return;
    __shared__ long long kk[MG_MAX_COLUMN];  // order keys of z, then the sorted z themselves
    __shared__ int ki[MG_MAX_COLUMN];
    __shared__ short nxt[MG_MAX_COLUMN];
    int col = blockIdx.x;
    int s0 = start[col], cnt = start[col + 1] - s0;
    if (cnt > MG_MAX_COLUMN) {
        if (threadIdx.x == 0) {
            atomicOr(flags, MG_FLAG_COLUMN_OVERFLOW);
            col_ncl[col] = 0;
        }
        return;
    }
    int pow2 = 1;
    while (pow2 < cnt) pow2 <<= 1;
    for (int i = threadIdx.x; i < pow2; i += blockDim.x) {
        if (i < cnt) {
            int a = sorted[s0 + i];
            ki[i] = a;
            kk[i] = order_key(xb[2 * (size_t)n + a]);
        } else {
            ki[i] = 0x7fffffff;
            kk[i] = 0x7fffffffffffffffLL;
        }
    }
    __syncthreads();
    for (int k = 2; k <= pow2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < pow2; i += blockDim.x) {
                int p = i ^ j;
                if (p > i) {
                    bool up = (i & k) == 0;
                    const long long bi = kk[i], bp = kk[p];
                    const int ii = ki[i], ip = ki[p];
                    bool gt = (bi > bp) || (bi == bp && ii > ip);
                    if (gt == up) {
                        kk[i] = bp;
                        kk[p] = bi;
                        ki[i] = ip;
                        ki[p] = ii;
                    }
                }
            }
            __syncthreads();
        }
    }
    double *kz = reinterpret_cast<double *>(kk);  // the sorted z, over the keys
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        const int a = ki[i];
        sorted[s0 + i] = a;
        kz[i] = xb[2 * (size_t)n + a];
    }
    __syncthreads();
    // the successor cut of a cluster starting at i: i + MG_CL, or the first site within the
    // next MG_CL - 1 that lies more than zcap above site i (the CPU builder's FP64 test)
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
        int nx = min(i + MG_CL, cnt);
        for (int j = i + 1; j < nx; j++)
            if (__dsub_rn(kz[j], kz[i]) > zcap) {
                nx = j;
                break;
            }
        nxt[i] = (short)nx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int ncl = 0;
        for (int first = 0; first < cnt; first = nxt[first]) cut[s0 + ncl++] = first;
        col_ncl[col] = ncl;
    }
}

// One block per column, eight lanes per cluster of the column (one per site): write the
// clusters (sites, FP64 and FP32 boxes, centre) from the cuts k_sort_columns recorded, the
// box bounds as the exact FP64 minimum and maximum over the eight lanes; then, one thread
// per z bucket b (z in [b lz / MG_ZB, (b + 1) lz / MG_ZB)), the range of the column's
// clusters that can overlap the bucket: from the first whose top lies above the bucket's
// bottom to the last whose bottom lies below the bucket's top, both widened by zmarg. Along a
// column the clusters are runs of z-sorted sites, so both bounds grow with the cluster index.
__global__ void __launch_bounds__(256) k_write_clusters(int n, const int *__restrict__ start, const int *__restrict__ sorted,
                                 const int *__restrict__ cut, const int *__restrict__ col_ncl,
                                 const int *__restrict__ cl_start, const double *__restrict__ xb, int cl_cap,
                                 int *__restrict__ cl_atom, double *__restrict__ cl_ref, float *__restrict__ cl_refh,
                                 double *__restrict__ cl_bb,
                                 float *__restrict__ cl_bbf, float lzf, float zmarg, int2 *__restrict__ col_bkt,
                                 unsigned *__restrict__ flags, const int *__restrict__ meta) {
    if (!meta[META_NEED]) return;
    __shared__ float s_zlo[MG_MAX_COLUMN], s_zhi[MG_MAX_COLUMN];
    const int col = blockIdx.x;
    const int s0 = start[col], cnt = start[col + 1] - s0;
    if (cnt > MG_MAX_COLUMN) return;
    const int ncl = col_ncl[col], c0 = cl_start[col];
    const int nw = max(0, min(ncl, cl_cap - c0));
    if (threadIdx.x == 0 && ncl > nw) atomicOr(flags, MG_FLAG_LIST_OVERFLOW);
    const int sl = threadIdx.x & 7;
    for (int k0 = 0; k0 < nw; k0 += blockDim.x >> 3) {  // whole warps stay in the loop (shuffles)
        const int k = k0 + (int)(threadIdx.x >> 3), c = c0 + k;
        const bool on = k < nw;
        const int first = on ? cut[s0 + k] : 0, end = on ? (k + 1 < ncl ? cut[s0 + k + 1] : cnt) : 0;
        const int idx = first + sl;
        const int a = on && idx < end ? sorted[s0 + idx] : -1;
        if (on) cl_atom[(size_t)c * MG_CL + sl] = a;
        double lo[3], hi[3];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const double v = a >= 0 ? xb[(size_t)d * n + a] : 0.0;
            lo[d] = a >= 0 ? v : INFINITY;
            hi[d] = a >= 0 ? v : -INFINITY;
#pragma unroll
            for (int o = 1; o < 8; o <<= 1) {  // over the cluster's eight lanes
                lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
                hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
            }
        }
        if (on && sl < 3) {
            const int d = sl;
            const double l = d == 0 ? lo[0] : d == 1 ? lo[1] : lo[2], h = d == 0 ? hi[0] : d == 1 ? hi[1] : hi[2];
            cl_bb[(size_t)c * 6 + d] = l;
            cl_bb[(size_t)c * 6 + 3 + d] = h;
            cl_bbf[(size_t)c * 6 + d] = (float)l;
            cl_bbf[(size_t)c * 6 + 3 + d] = (float)h;
            if (d == 2) {
                s_zlo[k] = (float)l;
                s_zhi[k] = (float)h;
            }
            const double r = __dmul_rn(0.5, __dadd_rn(l, h));
            cl_ref[(size_t)c * 3 + d] = r;
            const float rh = __double2float_rn(r);
            cl_refh[(size_t)c * 6 + d] = rh;
            cl_refh[(size_t)c * 6 + 3 + d] = __double2float_rn(__dsub_rn(r, (double)rh));
        }
    }
    __syncthreads();  // the column's z bounds are in shared memory
    for (int b = threadIdx.x; b < MG_ZB; b += blockDim.x) {
        const float z0 = (float)b * (lzf / MG_ZB) - zmarg, z1 = (float)(b + 1) * (lzf / MG_ZB) + zmarg;
        int lo = nw, hi = -1;
        for (int k = 0; k < nw; k++) {
            if (lo == nw && s_zhi[k] >= z0) lo = k;
            if (s_zlo[k] <= z1) hi = k;
        }
        col_bkt[(size_t)col * MG_ZB + b] = make_int2(c0 + lo, c0 + hi);
    }
}

// FP64 squared gap between two boxes along one axis, J shifted by s (same op order as
// the CPU builder)
__device__ __forceinline__ double gap2(double loi, double hii, double loj, double hij, double s) {
    double a = __dsub_rn(__dadd_rn(loj, s), hii);
    double b = __dsub_rn(loi, __dadd_rn(hij, s));
    double g = fmax(0.0, fmax(a, b));
    return __dmul_rn(g, g);
}

__device__ __forceinline__ float gap2f(float loi, float hii, float loj, float hij, float s) {
    float a = (loj + s) - hii;
    float b = loi - (hij + s);
    float g = fmaxf(0.f, fmaxf(a, b));
    return g * g;
}

struct SearchArgs {
    int ncx, ncy;
    double lx, ly, lz, cwx, cwy, icwx, icwy, rlist, rlist2;
    double nlx, nly, nlz;         // -lx, -ly, -lz: image shifts picked without FP64 arithmetic
    float lxf, lyf, lzf, cwxf, cwyf;  // FP32 copies for the prefilters
    float flo, fhi, fmarg;  // FP32 band [rlist^2 - m, rlist^2 + m] and a length margin
    const int *meta;
    int *meta_w;
    const double *bb, *ref;
    const float *refh;            // cluster references as FP32 hi, lo pairs [ncl][6]
    float lxh, lyh, lzh, lxl, lyl, lzl;  // box lengths as FP32 hi + lo
    const float *bbf;
    const int *col_cl_start;
    const int2 *col_bkt;          // per column and z bucket: cluster range (k_write_clusters)
    float zr, zbs;                // rlist + margin; buckets per unit z
    int *pair_start, *pair_cnt, *pair_j, *pair_img;
    void *pair_shift;
    unsigned long long *counter;
    long long cap;
    int fp64;
    unsigned *flags;
};

// Images iz = -1, 0, 1 (bits 0, 1, 2) in which j-cluster J lies within rlist of i-cluster
// I, for the column image (sx, sy): an FP32 band decides all but the borderline pairs,
// which the exact FP64 predicate of the CPU builder decides.
__device__ __forceinline__ unsigned cluster_images(const SearchArgs &A, const double *bi, const float *bif, int J,
                                                   double sx, double sy, float sxf, float syf) {
    const float *bjf = A.bbf + (size_t)J * 6;
    const float dxyf = gap2f(bif[0], bif[3], bjf[0], bjf[3], sxf) + gap2f(bif[1], bif[4], bjf[1], bjf[4], syf);
    if (dxyf > A.fhi) return 0u;
    unsigned m = 0u;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float d2f = dxyf + gap2f(bif[2], bif[5], bjf[2], bjf[5], (float)(k - 1) * A.lzf);
        bool hit;
        if (d2f < A.flo) {
            hit = true;
        } else if (d2f > A.fhi) {
            hit = false;
        } else {  // FP64 decides, as the CPU builder does
            const double *bj = A.bb + (size_t)J * 6;
            const double sz = k == 1 ? 0.0 : (k == 2 ? A.lz : A.nlz);
            double dxy = __dadd_rn(gap2(bi[0], bi[3], bj[0], bj[3], sx), gap2(bi[1], bi[4], bj[1], bj[4], sy));
            double d2 = __dadd_rn(dxy, gap2(bi[2], bi[5], bj[2], bj[5], sz));
            hit = d2 < A.rlist2;
        }
        if (hit) m |= 1u << k;
    }
    return m;
}

#define SEARCH_WPB 4     // warps (i-clusters) per block of k_search
#define SEARCH_CAP 512   // entries one warp keeps in shared memory before it falls back

// column number c of the window of an i-cluster: wrapped column indices, image offsets and
// the conservative FP32 rejection of the column's x/y slab
struct ColumnView {
    int col, ix, iy;
    float sxf, syf;
    bool reject;
};

__device__ __forceinline__ ColumnView column_view(const SearchArgs &A, const float *bif, int cx0, int cy0, int nx,
                                                  int c) {
    ColumnView v;
    const int uy = cy0 + c / nx, ux = cx0 + c % nx;
    int wy = uy % A.ncy;
    if (wy < 0) wy += A.ncy;
    v.iy = (uy - wy) / A.ncy;
    int wx = ux % A.ncx;
    if (wx < 0) wx += A.ncx;
    v.ix = (ux - wx) / A.ncx;
    // image offsets (ix, iy in {-1, 0, 1}): exact in FP32 as (float)ix * (float)L
    v.sxf = (float)v.ix * A.lxf;
    v.syf = (float)v.iy * A.lyf;
    // the column's sites lie within its x/y slab; the FP32 error of the slab edges
    // (~1e-5 A) is far inside the margin fmarg
    const float cx_lo = fmaf((float)wx, A.cwxf, v.sxf) - A.fmarg, cx_hi = fmaf((float)(wx + 1), A.cwxf, v.sxf) + A.fmarg;
    const float cy_lo = fmaf((float)wy, A.cwyf, v.syf) - A.fmarg, cy_hi = fmaf((float)(wy + 1), A.cwyf, v.syf) + A.fmarg;
    const float gx = fmaxf(0.f, fmaxf(cx_lo - bif[3], bif[0] - cx_hi));
    const float gy = fmaxf(0.f, fmaxf(cy_lo - bif[4], bif[1] - cy_hi));
    v.reject = gx * gx + gy * gy > A.fhi;
    v.col = wy * A.ncx + wx;
    return v;
}

__device__ __forceinline__ double image_shift(int i, double l, double nl) { return i == 0 ? 0.0 : (i > 0 ? l : nl); }

// a + b = s + e exactly (Knuth's two-sum, FP32)
__device__ __forceinline__ float two_sum(float a, float b, float &e) {
    const float s = __fadd_rn(a, b), bp = __fsub_rn(s, a), ap = __fsub_rn(s, bp);
    e = __fadd_rn(__fsub_rn(a, ap), __fsub_rn(b, bp));
    return s;
}

// ref_i - (ref_j + img L) from FP32 hi + lo pairs: the large parts subtracted exactly by
// two-sums, the small ones added, one final rounding (within about an ulp of the FP64 value
// rounded to FP32), with no FP64 instruction
__device__ __forceinline__ float shift_f32(float ih, float il, float jh, float jl, int img, float lh, float ll) {
    float e1, e2;
    const float h = two_sum(ih, -jh, e1);
    const float h2 = two_sum(h, img == 0 ? 0.f : (img > 0 ? -lh : lh), e2);
    const float lo = __fadd_rn(__fadd_rn(__fsub_rn(il, jl), img == 0 ? 0.f : (img > 0 ? -ll : ll)), __fadd_rn(e1, e2));
    return __fadd_rn(h2, lo);
}

// writes entry o: j-cluster J in image (ix, iy, iz) of i-cluster I (reference point ri, and
// rih as FP32 hi, lo); the FP64 path's shift in FP64, the mixed path's from the FP32 pairs
__device__ __forceinline__ void put_entry(const SearchArgs &A, long long o, const double *ri, const float *rih, int J,
                                          int ix, int iy, int iz) {
    A.pair_j[o] = J;
    A.pair_img[o] = ((ix + 512) & 1023) | (((iy + 512) & 1023) << 10) | (((iz + 512) & 1023) << 20);
    if (A.fp64) {
        const double *rj = A.ref + (size_t)J * 3;
        const double s0 = __dsub_rn(ri[0], __dadd_rn(rj[0], image_shift(ix, A.lx, A.nlx)));
        const double s1 = __dsub_rn(ri[1], __dadd_rn(rj[1], image_shift(iy, A.ly, A.nly)));
        const double s2 = __dsub_rn(ri[2], __dadd_rn(rj[2], image_shift(iz, A.lz, A.nlz)));
        ((double4 *)A.pair_shift)[o] = make_double4(s0, s1, s2, 0.0);
    } else {
        const float *rj = A.refh + (size_t)J * 6;
        ((float4 *)A.pair_shift)[o] =
            make_float4(shift_f32(rih[0], rih[3], rj[0], rj[3], ix, A.lxh, A.lxl),
                        shift_f32(rih[1], rih[4], rj[1], rj[4], iy, A.lyh, A.lyl),
                        shift_f32(rih[2], rih[5], rj[2], rj[5], iz, A.lzh, A.lzl), 0.f);
    }
}

// The clusters of column col that can lie within rlist of an i-cluster with FP32 box bif in
// z, in any of the images J + s, s = +lz, 0, -lz: for each image the z interval J must reach,
// mapped through the column's bucket table to a cluster range (a superset of the clusters
// that overlap it), the ranges merged in increasing cluster order (their starts already run
// that way). Up to three ranges (ra[k], rn[k] clusters), zero-length at the end.
__device__ __forceinline__ void column_ranges(const SearchArgs &A, int col, const float *bif, int (&ra)[3],
                                              int (&rn)[3]) {
    const int2 *bk = A.col_bkt + (size_t)col * MG_ZB;
    int s[3], e[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {  // s = +lz, 0, -lz
        const float sh = (float)(1 - k) * A.lzf;
        const float q0 = fmaxf(bif[2] - A.zr - sh, 0.f), q1 = fminf(bif[5] + A.zr - sh, A.lzf);
        s[k] = 0;
        e[k] = -1;
        if (q0 <= q1) {
            const int b0 = min(max((int)(q0 * A.zbs), 0), MG_ZB - 1), b1 = min(max((int)(q1 * A.zbs), 0), MG_ZB - 1);
            s[k] = bk[b0].x;
            e[k] = bk[b1].y;
        }
    }
    int m = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        ra[k] = 0;
        rn[k] = 0;
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        if (s[k] > e[k]) continue;  // empty
        // merge into the last range when it overlaps or touches
        bool merged = false;
#pragma unroll
        for (int r = 0; r < 3; r++)
            if (r == m - 1 && s[k] <= ra[r] + rn[r]) {
                rn[r] = max(ra[r] + rn[r], e[k] + 1) - ra[r];
                merged = true;
            }
        if (!merged) {
#pragma unroll
            for (int r = 0; r < 3; r++)
                if (r == m) {
                    ra[r] = s[k];
                    rn[r] = e[k] - s[k] + 1;
                }
            m++;
        }
    }
}

// One warp per i-cluster. Entries are ordered by candidate column (row-major over the
// column window), then j-cluster, then z image (-1, 0, 1), as the CPU builder orders them.
// The warp takes 32 columns at a time (one lane per column: its rejection test and the
// ranges of its clusters that can reach the i-cluster in z), lays those clusters out in that
// order and tests 32 of them at a time, one per lane, so that many loads are in flight. Hits go to a shared-memory buffer and
// are written after one reservation; a warp whose buffer would overflow counts and writes
// in two passes instead.
__global__ void __launch_bounds__(SEARCH_WPB * 32) k_search(SearchArgs A) {
    __shared__ int s_j[SEARCH_WPB][SEARCH_CAP];
    __shared__ int s_code[SEARCH_WPB][SEARCH_CAP];  // image bits: (ix+1) | (iy+1) << 2 | (iz+1) << 4
    if (!A.meta[META_NEED]) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int I = blockIdx.x * SEARCH_WPB + w;
    if (I >= A.meta[META_NCL]) return;
    double bi[6];
    float bif[6];
    for (int d = 0; d < 6; d++) {
        bi[d] = A.bb[(size_t)I * 6 + d];
        bif[d] = A.bbf[(size_t)I * 6 + d];
    }
    // the column window, widened by MG_WIN_MARGIN columns against the rounding of the product
    // (an extra column holds no cluster within rlist, so the entries and their order stay)
    const int cx0 = (int)floor(__dsub_rn(__dmul_rn(__dsub_rn(bi[0], A.rlist), A.icwx), MG_WIN_MARGIN));
    const int cx1 = (int)floor(__dadd_rn(__dmul_rn(__dadd_rn(bi[3], A.rlist), A.icwx), MG_WIN_MARGIN));
    const int cy0 = (int)floor(__dsub_rn(__dmul_rn(__dsub_rn(bi[1], A.rlist), A.icwy), MG_WIN_MARGIN));
    const int cy1 = (int)floor(__dadd_rn(__dmul_rn(__dadd_rn(bi[4], A.rlist), A.icwy), MG_WIN_MARGIN));
    const int nx = cx1 - cx0 + 1, ny = cy1 - cy0 + 1;
    if (nx > A.ncx || ny > A.ncy) {  // a column would be visited twice: small-box mode
        if (lane == 0) {
            atomicOr(A.flags, MG_FLAG_SMALL_BOX);
            A.pair_start[I] = 0;  // the pair kernel of this (repeated) call sees no entries
            A.pair_cnt[I] = 0;
        }
        return;
    }
    const int ncand = nx * ny;
    const double *ri = A.ref + (size_t)I * 3;
    float rih[6];
    if (!A.fp64)
        for (int d = 0; d < 6; d++) rih[d] = A.refh[(size_t)I * 6 + d];
    // mode 0: into shared memory; 1: count only (buffer too small); 2: write from run
    long long run = 0;
    bool multi = false;
    for (int mode = 0; mode < 3; mode++) {
        for (int base = 0; base < ncand; base += 32) {
            const int c = base + lane;
            int cnt = 0;
            int ra[3] = {0, 0, 0}, rn[3] = {0, 0, 0};
            ColumnView v;
            v.ix = v.iy = 0;
            v.sxf = v.syf = 0.f;
            if (c < ncand) {
                v = column_view(A, bif, cx0, cy0, nx, c);
                if (!v.reject) {
                    column_ranges(A, v.col, bif, ra, rn);
                    cnt = rn[0] + rn[1] + rn[2];
                }
            }
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            const int excl = incl - cnt, T = __shfl_sync(0xffffffffu, incl, 31);
            for (int t0 = 0; t0 < T; t0 += 32) {
                const int t = t0 + lane;
                int k = 0;  // the column lane of item t: the number of columns with incl <= t
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int probe = __shfl_sync(0xffffffffu, incl, k + step - 1);
                    if (probe <= t) k += step;
                }
                k = min(k, 31);
                const int ek = __shfl_sync(0xffffffffu, excl, k);
                const int a0 = __shfl_sync(0xffffffffu, ra[0], k), n0 = __shfl_sync(0xffffffffu, rn[0], k);
                const int a1 = __shfl_sync(0xffffffffu, ra[1], k), n1 = __shfl_sync(0xffffffffu, rn[1], k);
                const int a2 = __shfl_sync(0xffffffffu, ra[2], k);
                const int ixk = __shfl_sync(0xffffffffu, v.ix, k), iyk = __shfl_sync(0xffffffffu, v.iy, k);
                const float sxf = __shfl_sync(0xffffffffu, v.sxf, k), syf = __shfl_sync(0xffffffffu, v.syf, k);
                const int off = t - ek;  // the item's place among its column's clusters
                const int J = off < n0 ? a0 + off : (off < n0 + n1 ? a1 + off - n0 : a2 + off - n0 - n1);
                unsigned m = 0u;
                if (t < T)
                    m = cluster_images(A, bi, bif, J, image_shift(ixk, A.lx, A.nlx), image_shift(iyk, A.ly, A.nly),
                                       sxf, syf);
                const int h = __popc(m);
                multi |= h > 1;
                int hi = h;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int q = __shfl_up_sync(0xffffffffu, hi, o);
                    if (lane >= o) hi += q;
                }
                if (h > 0) {
                    long long o = run + hi - h;
                    for (int b = 0; b < 3; b++) {
                        if (!(m & (1u << b))) continue;
                        if (mode == 0) {
                            if (o < SEARCH_CAP) {
                                s_j[w][o] = J;
                                s_code[w][o] = (ixk + 1) | ((iyk + 1) << 2) | (b << 4);
                            }
                        } else if (mode == 2) {
                            put_entry(A, o, ri, rih, J, ixk, iyk, b - 1);
                        }
                        o++;
                    }
                }
                run += __shfl_sync(0xffffffffu, hi, 31);
            }
        }
        if (mode == 2) return;
        if (mode == 1 || run <= SEARCH_CAP) {
            if (__any_sync(0xffffffffu, multi) && lane == 0) atomicOr(A.flags, MG_FLAG_SMALL_BOX);
            const long long total = run;
            unsigned long long off = 0;
            if (lane == 0) off = atomicAdd(A.counter, (unsigned long long)total);
            off = __shfl_sync(0xffffffffu, off, 0);
            if (lane == 0) {
                A.pair_start[I] = (int)off;
                A.pair_cnt[I] = (int)total;
            }
            if ((long long)(off + total) > A.cap) {
                if (lane == 0) {
                    atomicOr(A.flags, MG_FLAG_LIST_OVERFLOW);
                    A.pair_cnt[I] = 0;
                }
                return;
            }
            if (mode == 0) {  // the buffer holds every entry: write them out
                __syncwarp();
                for (int e = lane; e < (int)total; e += 32) {
                    const int code = s_code[w][e];
                    put_entry(A, (long long)off + e, ri, rih, s_j[w][e], (code & 3) - 1, ((code >> 2) & 3) - 1,
                              ((code >> 4) & 3) - 1);
                }
                return;
            }
            run = (long long)off;
            mode = 1;  // next: the writing pass
        } else {
            run = 0;   // too many entries for the buffer: count again, then write
        }
    }
}

// Inner sub-list for the short (RESPA inner) pair pass: per i-cluster, in list order, the
// entries whose cluster boxes (at build positions, in the entry's image) lie within
// rsub = respa_split + skin. Any site pair closer than respa_split now was closer than
// rsub at the build, because no site has moved by more than skin/2 since; the FP32 test
// has a small positive margin, so it keeps every such entry. One warp per i-cluster:
// a counting pass, one reservation, an order-keeping compaction pass.
__global__ void k_sublist(const int *__restrict__ meta, const int *__restrict__ pair_start,
                          const int *__restrict__ pair_cnt, const int *__restrict__ pair_j,
                          const void *__restrict__ pair_shift, const int *__restrict__ pair_img,
                          const float *__restrict__ bbf, float lx, float ly, float lz, float rsub2, int fp64,
                          int *__restrict__ sub_start, int *__restrict__ sub_cnt, int *__restrict__ sub_j,
                          void *__restrict__ sub_shift, int *__restrict__ sub_img,
                          unsigned long long *__restrict__ counter) {
    if (!meta[META_NEED]) return;
    const int lane = threadIdx.x & 31;
    const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (I >= meta[META_NCL]) return;
    const int e0 = pair_start[I], n = pair_cnt[I];
    float bi[6];
    for (int d = 0; d < 6; d++) bi[d] = bbf[(size_t)I * 6 + d];
    auto keep = [&](int k) -> bool {
        if (k >= n) return false;
        const int e = e0 + k, J = pair_j[e], img = pair_img[e];
        const float sh[3] = {(float)((img & 1023) - 512) * lx, (float)(((img >> 10) & 1023) - 512) * ly,
                             (float)(((img >> 20) & 1023) - 512) * lz};
        float d2 = 0.f;
        for (int d = 0; d < 3; d++) {
            const float lo = bbf[(size_t)J * 6 + d] + sh[d], hi = bbf[(size_t)J * 6 + 3 + d] + sh[d];
            const float g = fmaxf(0.f, fmaxf(lo - bi[3 + d], bi[d] - hi));
            d2 += g * g;
        }
        return d2 < rsub2;
    };
    int cnt = 0;
    for (int b = 0; b < n; b += 32) cnt += __popc(__ballot_sync(0xffffffffu, keep(b + lane)));
    unsigned long long off = 0;
    if (lane == 0) off = atomicAdd(counter, (unsigned long long)cnt);
    off = __shfl_sync(0xffffffffu, off, 0);
    if (lane == 0) {
        sub_start[I] = (int)off;
        sub_cnt[I] = cnt;
    }
    long long run = (long long)off;
    for (int b = 0; b < n; b += 32) {
        const bool k = keep(b + lane);
        const unsigned m = __ballot_sync(0xffffffffu, k);
        if (k) {
            const long long o = run + __popc(m & ((1u << lane) - 1u));
            const int e = e0 + b + lane;
            sub_j[o] = pair_j[e];
            sub_img[o] = pair_img[e];
            if (fp64)
                ((double4 *)sub_shift)[o] = ((const double4 *)pair_shift)[e];
            else
                ((float4 *)sub_shift)[o] = ((const float4 *)pair_shift)[e];
        }
        run += __popc(m);
    }
}

__global__ void k_set_int(int *p, int v) { *p = v; }

// small boxes: every (I, J) pair once, no image (minimum image per site pair later)
__global__ void k_all_pairs(const int *__restrict__ meta, const double *__restrict__ ref, int *__restrict__ pair_start,
                            int *__restrict__ pair_cnt, int *__restrict__ pair_j, void *pair_shift,
                            int *__restrict__ pair_img, int fp64, long long cap, unsigned *__restrict__ flags) {
    if (!meta[META_NEED]) return;
    const int ncl = meta[META_NCL];
    if ((long long)ncl * ncl > cap) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(flags, MG_FLAG_LIST_OVERFLOW);
        return;
    }
    const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x, stride = (long long)gridDim.x * blockDim.x;
    for (long long i = t0; i < ncl; i += stride) {
        pair_start[i] = (int)(i * ncl);
        pair_cnt[i] = ncl;
    }
    for (long long e = t0; e < (long long)ncl * ncl; e += stride) {
        int I = (int)(e / ncl), J = (int)(e % ncl);
        double s0 = __dsub_rn(ref[I * 3 + 0], ref[J * 3 + 0]);
        double s1 = __dsub_rn(ref[I * 3 + 1], ref[J * 3 + 1]);
        double s2 = __dsub_rn(ref[I * 3 + 2], ref[J * 3 + 2]);
        pair_j[e] = J;
        pair_img[e] = 512 | (512 << 10) | (512 << 20);
        if (fp64)
            ((double4 *)pair_shift)[e] = make_double4(s0, s1, s2, 0.0);
        else
            ((float4 *)pair_shift)[e] = make_float4((float)s0, (float)s1, (float)s2, 0.f);
    }
}

__global__ void k_finish(int *__restrict__ meta, const unsigned long long *__restrict__ counter) {
    if (!meta[META_NEED]) return;
    meta[META_BUILDS] += 1;
    *(long long *)(meta + META_NPAIRS) = (long long)*counter;
}

// any site moved more than skin/2 since the build -> rebuild
__global__ void k_displacement(int n, const double *__restrict__ x, const double *__restrict__ y,
                               const double *__restrict__ z, const double *__restrict__ xb,
                               const double *__restrict__ img, double half_skin2, int *__restrict__ meta) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    bool move = false;
    if (a < n) {
        double dx = (x[a] - img[a]) - xb[a];
        double dy = (y[a] - img[n + a]) - xb[n + a];
        double dz = (z[a] - img[2 * n + a]) - xb[2 * n + a];
        move = !(dx * dx + dy * dy + dz * dz <= half_skin2);
    }
    if (__any_sync(0xffffffffu, move) && (threadIdx.x & 31) == 0) atomicOr(&meta[META_NEED], 1);
}

// the info word (molecule << 2 | flags) carried in the fourth lane of a packed position
__device__ __forceinline__ float info_lane(int v, float) { return __int_as_float(v); }
__device__ __forceinline__ double info_lane(int v, double) { return __longlong_as_double((long long)v); }

// Pack the per-slot pair-kernel operands from the current positions: pos (x, y, z relative
// to the cluster reference, charge), lj (half-sigma, sqrt-epsilon) and info for the FP64 pair
// kernel and the adjoint passes; xi (x, y, z, info bits) and qp (charge, half-sigma,
// sqrt-epsilon, 0) for the mixed-precision pair kernel, which stages both rows into shared
// memory as they are.
template <typename R4, typename R2, typename R>
__global__ void k_pack(int n, const int *__restrict__ meta, const int *__restrict__ cl_atom,
                       const double *__restrict__ cl_ref, const double *__restrict__ x, const double *__restrict__ y,
                       const double *__restrict__ z, const double *__restrict__ img, const double *__restrict__ q,
                       const double *__restrict__ hsig, const double *__restrict__ seps,
                       const int *__restrict__ mol, const int *__restrict__ sflags, R4 *__restrict__ pos,
                       R2 *__restrict__ lj, int *__restrict__ info, R4 *__restrict__ xi, R4 *__restrict__ qp) {
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= meta[META_NCL] * MG_CL) return;
    int a = cl_atom[s];
    int cl = s / MG_CL;
    if (a < 0) {
        R4 p;
        p.x = p.y = p.z = p.w = (R)0;
        pos[s] = p;
        R2 l;
        l.x = l.y = (R)0;
        lj[s] = l;
        info[s] = MG_SITE_DEAD;
        qp[s] = p;
        p.w = info_lane(MG_SITE_DEAD, (R)0);
        xi[s] = p;
        return;
    }
    R4 p;
    p.x = (R)((x[a] - img[a]) - cl_ref[cl * 3 + 0]);
    p.y = (R)((y[a] - img[n + a]) - cl_ref[cl * 3 + 1]);
    p.z = (R)((z[a] - img[2 * n + a]) - cl_ref[cl * 3 + 2]);
    p.w = (R)q[a];
    pos[s] = p;
    R2 l;
    l.x = (R)hsig[a];
    l.y = (R)seps[a];
    lj[s] = l;
    int f = sflags[a];
    const int inf = (mol[a] << 2) | (f & (MG_SITE_LJ | MG_SITE_DEAD));
    info[s] = inf;
    R4 v = p;
    v.w = info_lane(inf, (R)0);
    xi[s] = v;
    v.x = p.w;
    v.y = l.x;
    v.z = l.y;
    v.w = (R)0;
    qp[s] = v;
}

}  // namespace

// ---------------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------------
static void choose_grid(mg_ctx *c, double rlist) {
    double vol = c->lx * c->ly * c->lz;
    double cw = std::min(cbrt(8.0 * vol / c->natom), 0.75 * rlist) * c->tune.cell_scale / pow(1.5, c->col_refine);
    c->ncx = std::max(1, (int)floor(c->lx / cw));
    c->ncy = std::max(1, (int)floor(c->ly / cw));
    c->zcap = cw * c->tune.zcap_scale;
    c->small_box = c->small_box_forced || c->lx < 2.0 * rlist + 2.0 * (c->lx / c->ncx) ||
                   c->ly < 2.0 * rlist + 2.0 * (c->ly / c->ncy) || c->lz < 2.0 * rlist + 2.0 * std::max(cw, c->zcap);
}

// Size every list buffer for the current grid; called when the grid or capacity changes.
static mg_status size_list(mg_ctx *c) {
    int n = c->natom, ncol = c->ncx * c->ncy;
    if (c->cl_cap < n / 4 + ncol + 16) c->cl_cap = n / 4 + ncol + 16;
    if (c->cl_cap > n + ncol + 16) c->cl_cap = n + ncol + 16;
    long long ncl = c->cl_cap;
    if (c->small_box) {
        if (c->pair_cap < ncl * ncl) c->pair_cap = ncl * ncl;
    } else if (c->pair_cap == 0) {
        double rho = n / (c->lx * c->ly * c->lz);
        double r = c->list_rlist + 2.0 * c->zcap;
        c->pair_cap = (long long)(ncl * (1.5 * 4.18879 * r * r * r * rho / MG_CL + 64));
    }
    if (c->pair_cap > 0x7fffffffLL) return mg_fail(c, MG_ERR_CAPACITY, "cluster-pair list exceeds 2^31 entries");
    bool fp64 = c->opt.precision == MG_PREC_FP64;
    size_t ent = fp64 ? sizeof(double4) : sizeof(float4);
    if (!mg_ensure(c, c->d_col_count, sizeof(int) * (ncol + 1)) || !mg_ensure(c, c->d_col_start, sizeof(int) * (ncol + 1)) ||
        !mg_ensure(c, c->d_col_fill, sizeof(int) * (ncol + 1)) || !mg_ensure(c, c->d_col_cl_start, sizeof(int) * (ncol + 1)) ||
        !mg_ensure(c, c->d_col_bkt, sizeof(int2) * (size_t)ncol * MG_ZB) ||
        !mg_ensure(c, c->d_col_ncl, sizeof(int) * (ncol + 1)) || !mg_ensure(c, c->d_col_sorted, sizeof(int) * (size_t)n * 2) ||
        !mg_ensure(c, c->d_xbuild, sizeof(double) * 3 * (size_t)n) || !mg_ensure(c, c->d_img, sizeof(double) * 3 * (size_t)n) ||
        !mg_ensure(c, c->d_cl_atom, sizeof(int) * (size_t)ncl * MG_CL) || !mg_ensure(c, c->d_cl_ref, sizeof(double) * 3 * (size_t)ncl) ||
        !mg_ensure(c, c->d_cl_refh, sizeof(float) * 6 * (size_t)ncl) ||
        !mg_ensure(c, c->d_cl_bb, sizeof(double) * 6 * (size_t)ncl) || !mg_ensure(c, c->d_cl_bbf, sizeof(float) * 6 * (size_t)ncl) ||
        !mg_ensure(c, c->d_pair_start, sizeof(int) * (size_t)(ncl + 1)) || !mg_ensure(c, c->d_pair_count, sizeof(int) * (size_t)(ncl + 1)) ||
        !mg_ensure(c, c->d_pair_j, sizeof(int) * (size_t)c->pair_cap) || !mg_ensure(c, c->d_pair_shift, ent * (size_t)c->pair_cap) ||
        !mg_ensure(c, c->d_pair_img, sizeof(int) * (size_t)c->pair_cap) || !mg_ensure(c, c->d_counter, 64))
        return MG_ERR_ALLOC;
    return MG_OK;
}

mg_status mg_list_update(mg_ctx *c, const double *dx, const double *dy, const double *dz) {
    const mg_params &p = c->params;
    cudaStream_t s = c->stream;
    const int n = c->natom;
    double rlist = std::max(p.rcutoff, p.rcutoffelec) + std::max(c->opt.skin, 0.0);
    if (!mg_ensure(c, c->d_meta, 64)) return MG_ERR_ALLOC;
    int *meta = (int *)c->d_meta.p;
    bool geometry = !c->list_valid || c->list_lx != c->lx || c->list_ly != c->ly || c->list_lz != c->lz ||
                    c->list_rlist != rlist;
    if (geometry) {
        c->list_rlist = rlist;
        c->list_lx = c->lx;
        c->list_ly = c->ly;
        c->list_lz = c->lz;
        choose_grid(c, rlist);
        mg_status st = size_list(c);
        if (st) return st;
    }
    if (geometry || !(c->opt.skin > 0)) {
        k_set_int<<<1, 1, 0, s>>>(meta + META_NEED, 1);
        c->launches += 1;
    } else {
        MG_CUDA(cudaMemsetAsync(meta + META_NEED, 0, sizeof(int), s));
        double hs = 0.5 * c->opt.skin;
        k_displacement<<<(n + 255) / 256, 256, 0, s>>>(n, dx, dy, dz, (double *)c->d_xbuild.p, (double *)c->d_img.p,
                                                        hs * hs, meta);
        c->launches += 1;
    }
    const int ncx = c->ncx, ncy = c->ncy, ncol = ncx * ncy;
    const double cwx = c->lx / ncx, cwy = c->ly / ncy;
    int *col_of = (int *)c->d_col_sorted.p + n;
    const bool fp64 = c->opt.precision == MG_PREC_FP64;
    k_zero<<<(ncol + 255) / 256, 256, 0, s>>>((int *)c->d_col_count.p, ncol + 1, meta);
    k_zero<<<1, 32, 0, s>>>((int *)c->d_counter.p, 4, meta);
    k_bin<<<(n + 255) / 256, 256, 0, s>>>(n, ncol, dx, dy, dz, c->lx, c->ly, c->lz, 1.0 / c->lx, 1.0 / c->ly,
                                           1.0 / c->lz, 1.0 / cwx, 1.0 / cwy, ncx, ncy,
                                           (double *)c->d_xbuild.p, (double *)c->d_img.p, col_of,
                                           (int *)c->d_col_count.p, meta);
    k_scan<<<1, 1024, 0, s>>>(ncol, (int *)c->d_col_count.p, (int *)c->d_col_start.p, (int *)c->d_col_fill.p, nullptr,
                              meta + META_MAXCOL, -1, nullptr, meta);
    k_scatter<<<(n + 255) / 256, 256, 0, s>>>(n, col_of, (int *)c->d_col_start.p, (int *)c->d_col_fill.p,
                                              (int *)c->d_col_sorted.p, meta);
    // the cluster cuts reuse col_of's storage, which k_scatter was the last to read
    int *cut = col_of;
    k_sort_columns<<<ncol, 256, 0, s>>>(n, (int *)c->d_col_start.p, (int *)c->d_col_sorted.p, (double *)c->d_xbuild.p,
                                       c->zcap, (int *)c->d_col_ncl.p, cut, (unsigned *)c->d_flags.p, meta);
    k_scan<<<1, 1024, 0, s>>>(ncol, (int *)c->d_col_ncl.p, (int *)c->d_col_cl_start.p, nullptr, meta + META_NCL, nullptr,
                              c->cl_cap, meta + META_NCL_TOTAL, meta);
    // z margin of the bucket tables and queries: far above the FP32 rounding of boxes and
    // bounds (a few ulp of the box length)
    const float zmarg = (float)(64.0 * 5.960464477539063e-08 * 2.0 * std::max(c->lx, std::max(c->ly, c->lz)) + 1e-4 * rlist);
    k_write_clusters<<<ncol, 256, 0, s>>>(n, (int *)c->d_col_start.p, (int *)c->d_col_sorted.p, cut,
                                         (int *)c->d_col_ncl.p, (int *)c->d_col_cl_start.p, (double *)c->d_xbuild.p,
                                         c->cl_cap, (int *)c->d_cl_atom.p, (double *)c->d_cl_ref.p, (float *)c->d_cl_refh.p,
                                         (double *)c->d_cl_bb.p, (float *)c->d_cl_bbf.p, (float)c->lz, zmarg,
                                         (int2 *)c->d_col_bkt.p, (unsigned *)c->d_flags.p, meta);
    if (c->small_box) {
        long long tot = (long long)c->cl_cap * c->cl_cap;
        unsigned blocks = (unsigned)std::min<long long>((tot + 255) / 256, 65535);
        k_all_pairs<<<blocks, 256, 0, s>>>(meta, (double *)c->d_cl_ref.p, (int *)c->d_pair_start.p,
                                           (int *)c->d_pair_count.p, (int *)c->d_pair_j.p, c->d_pair_shift.p,
                                           (int *)c->d_pair_img.p, fp64, c->pair_cap, (unsigned *)c->d_flags.p);
    } else {
        SearchArgs A;
        A.ncx = ncx;
        A.ncy = ncy;
        A.lx = c->lx;
        A.ly = c->ly;
        A.lz = c->lz;
        A.cwx = cwx;
        A.cwy = cwy;
        A.icwx = 1.0 / cwx;
        A.icwy = 1.0 / cwy;
        A.nlx = -c->lx;
        A.nly = -c->ly;
        A.nlz = -c->lz;
        A.lxf = (float)c->lx;
        A.lyf = (float)c->ly;
        A.lzf = (float)c->lz;
        A.cwxf = (float)cwx;
        A.cwyf = (float)cwy;
        A.rlist = rlist;
        A.rlist2 = rlist * rlist;
        // FP32 rounding of the boxes, shifts and gaps is below 8 u max(L) per gap
        // (u = 2^-24); the band is four times the resulting bound on d^2
        double L = std::max(c->lx, std::max(c->ly, c->lz));
        double u = 5.960464477539063e-08;
        double m = 4.0 * (3.0 * 2.0 * rlist * 8.0 * u * 2.0 * L + 6.0 * u * rlist * rlist) + 1e-30;
        A.flo = (float)(rlist * rlist - m);
        A.fhi = (float)(rlist * rlist + m);
        A.fmarg = (float)(64.0 * u * 2.0 * L + 1e-6 * rlist);
        A.meta = meta;
        A.meta_w = meta;
        A.bb = (double *)c->d_cl_bb.p;
        A.bbf = (float *)c->d_cl_bbf.p;
        A.ref = (double *)c->d_cl_ref.p;
        A.refh = (const float *)c->d_cl_refh.p;
        A.lxh = (float)c->lx;
        A.lyh = (float)c->ly;
        A.lzh = (float)c->lz;
        A.lxl = (float)(c->lx - (double)A.lxh);
        A.lyl = (float)(c->ly - (double)A.lyh);
        A.lzl = (float)(c->lz - (double)A.lzh);
        A.col_cl_start = (int *)c->d_col_cl_start.p;
        A.col_bkt = (const int2 *)c->d_col_bkt.p;
        A.zr = (float)rlist + zmarg;
        A.zbs = (float)MG_ZB / (float)c->lz;
        A.pair_start = (int *)c->d_pair_start.p;
        A.pair_cnt = (int *)c->d_pair_count.p;
        A.pair_j = (int *)c->d_pair_j.p;
        A.pair_img = (int *)c->d_pair_img.p;
        A.pair_shift = c->d_pair_shift.p;
        A.counter = (unsigned long long *)c->d_counter.p;
        A.cap = c->pair_cap;
        A.fp64 = fp64;
        A.flags = (unsigned *)c->d_flags.p;
        unsigned blocks = (unsigned)(((long long)c->cl_cap + SEARCH_WPB - 1) / SEARCH_WPB);
        k_search<<<blocks, SEARCH_WPB * 32, 0, s>>>(A);
    }
    k_finish<<<1, 1, 0, s>>>(meta, (unsigned long long *)c->d_counter.p);
    c->sub_ready = false;
    if (p.respa_split > 0 && !c->small_box) {
        // the inner sub-list of the distance split, rebuilt whenever the list is
        const size_t ent = fp64 ? sizeof(double4) : sizeof(float4);
        if (!mg_ensure(c, c->d_sub_start, sizeof(int) * ((size_t)c->cl_cap + 1)) ||
            !mg_ensure(c, c->d_sub_count, sizeof(int) * ((size_t)c->cl_cap + 1)) ||
            !mg_ensure(c, c->d_sub_j, sizeof(int) * (size_t)c->pair_cap) ||
            !mg_ensure(c, c->d_sub_shift, ent * (size_t)c->pair_cap) ||
            !mg_ensure(c, c->d_sub_img, sizeof(int) * (size_t)c->pair_cap))
            return MG_ERR_ALLOC;
        const double rsub = p.respa_split + std::max(c->opt.skin, 0.0);
        const float rsub2 = (float)(rsub * rsub) * 1.0001f + 1e-4f;
        const unsigned blocks = (unsigned)(((long long)c->cl_cap * 32 + 127) / 128);
        k_sublist<<<blocks, 128, 0, s>>>(meta, (int *)c->d_pair_start.p, (int *)c->d_pair_count.p,
                                         (int *)c->d_pair_j.p, c->d_pair_shift.p, (int *)c->d_pair_img.p,
                                         (float *)c->d_cl_bbf.p, (float)c->lx, (float)c->ly, (float)c->lz, rsub2,
                                         fp64 ? 1 : 0, (int *)c->d_sub_start.p, (int *)c->d_sub_count.p,
                                         (int *)c->d_sub_j.p, c->d_sub_shift.p, (int *)c->d_sub_img.p,
                                         (unsigned long long *)c->d_counter.p + 1);
        c->launches += 1;
        c->sub_ready = true;
    }
    MG_CUDA(cudaGetLastError());
    c->launches += 10;
    c->list_valid = true;
    return MG_OK;
}

mg_status mg_pack_clusters(mg_ctx *c, const double *dx, const double *dy, const double *dz) {
    int n = c->natom;
    bool fp64 = c->opt.precision == MG_PREC_FP64;
    size_t slots = (size_t)c->cl_cap * MG_CL;
    if (!mg_ensure(c, c->d_pack_pos, slots * (fp64 ? sizeof(double4) : sizeof(float4))) ||
        !mg_ensure(c, c->d_pack_lj, slots * (fp64 ? sizeof(double2) : sizeof(float2))) ||
        !mg_ensure(c, c->d_pack_info, slots * sizeof(int)) ||
        !mg_ensure(c, c->d_pack_xi, slots * (fp64 ? sizeof(double4) : sizeof(float4))) ||
        !mg_ensure(c, c->d_pack_qp, slots * (fp64 ? sizeof(double4) : sizeof(float4))))
        return MG_ERR_ALLOC;
    unsigned blocks = (unsigned)((slots + 255) / 256);
    const int *meta = (const int *)c->d_meta.p;
    if (fp64)
        k_pack<double4, double2, double><<<blocks, 256, 0, c->stream>>>(
            n, meta, (int *)c->d_cl_atom.p, (double *)c->d_cl_ref.p, dx, dy, dz, (double *)c->d_img.p,
            (double *)c->d_site_q.p, (double *)c->d_site_hsig.p, (double *)c->d_site_seps.p, (int *)c->d_site_mol.p,
            (int *)c->d_site_flags.p, (double4 *)c->d_pack_pos.p, (double2 *)c->d_pack_lj.p, (int *)c->d_pack_info.p,
            (double4 *)c->d_pack_xi.p, (double4 *)c->d_pack_qp.p);
    else
        k_pack<float4, float2, float><<<blocks, 256, 0, c->stream>>>(
            n, meta, (int *)c->d_cl_atom.p, (double *)c->d_cl_ref.p, dx, dy, dz, (double *)c->d_img.p,
            (double *)c->d_site_q.p, (double *)c->d_site_hsig.p, (double *)c->d_site_seps.p, (int *)c->d_site_mol.p,
            (int *)c->d_site_flags.p, (float4 *)c->d_pack_pos.p, (float2 *)c->d_pack_lj.p, (int *)c->d_pack_info.p,
            (float4 *)c->d_pack_xi.p, (float4 *)c->d_pack_qp.p);
    MG_CUDA(cudaGetLastError());
    c->launches += 1;
    return MG_OK;
}

// Adjust the list set-up after a call whose status word asked for it; returns true when
// the call must be repeated.
bool mg_list_retry(mg_ctx *c, unsigned flags, const int *meta_host) {
    bool retry = false;
    if (flags & MG_FLAG_COLUMN_OVERFLOW) {
        c->col_refine += 1;
        retry = true;
    }
    if (flags & MG_FLAG_SMALL_BOX) {
        c->small_box_forced = true;
        retry = true;
    }
    if (flags & MG_FLAG_LIST_OVERFLOW) {
        long long need = *(const long long *)(meta_host + META_NPAIRS);
        int ncl = meta_host[META_NCL_TOTAL];
        if (ncl > c->cl_cap) {  // the clusters overflowed and the search did not run
            int grown = ncl + ncl / 8 + 16;
            c->pair_cap = (long long)((double)c->pair_cap * grown / c->cl_cap) + 1024;
            c->cl_cap = grown;
        } else if (need > c->pair_cap) {
            c->pair_cap = need + need / 4 + 1024;
        } else {
            c->pair_cap = c->pair_cap * 2;
        }
        retry = true;
    }
    if (retry) c->list_valid = false;
    return retry;
}

extern "C" mg_status mg_debug_get_list(mg_ctx *c, int *ncl, long long *npairs, int *grid, double *zcap,
                                       int *cluster_atoms, int *pairs, int *shifts) {
    if (!c || !ncl || !npairs) return MG_ERR_INVALID;
    cudaSetDevice(c->device);
    *ncl = 0;
    *npairs = 0;
    if (zcap) *zcap = c->zcap;
    if (grid) {
        grid[0] = c->ncx;
        grid[1] = c->ncy;
        grid[2] = c->small_box ? 1 : 0;
    }
    if (!c->list_valid) return MG_OK;
    int meta[8];
    MG_CUDA(cudaStreamSynchronize(c->stream));
    MG_CUDA(cudaMemcpy(meta, c->d_meta.p, sizeof(meta), cudaMemcpyDeviceToHost));
    int n = meta[META_NCL];
    std::vector<int> start(n), cnt(n);
    MG_CUDA(cudaMemcpy(start.data(), c->d_pair_start.p, sizeof(int) * n, cudaMemcpyDeviceToHost));
    MG_CUDA(cudaMemcpy(cnt.data(), c->d_pair_count.p, sizeof(int) * n, cudaMemcpyDeviceToHost));
    long long tot = 0;
    for (int I = 0; I < n; I++) tot += cnt[I];
    *ncl = n;
    *npairs = tot;
    if (cluster_atoms)
        MG_CUDA(cudaMemcpy(cluster_atoms, c->d_cl_atom.p, sizeof(int) * (size_t)n * MG_CL, cudaMemcpyDeviceToHost));
    if (pairs || shifts) {
        long long used = *(long long *)(meta + META_NPAIRS);
        if (c->small_box) used = (long long)n * n;
        std::vector<int> pj(used), img(used);
        MG_CUDA(cudaMemcpy(pj.data(), c->d_pair_j.p, sizeof(int) * used, cudaMemcpyDeviceToHost));
        MG_CUDA(cudaMemcpy(img.data(), c->d_pair_img.p, sizeof(int) * used, cudaMemcpyDeviceToHost));
        long long o = 0;
        for (int I = 0; I < n; I++)
            for (int e = start[I]; e < start[I] + cnt[I]; e++, o++) {
                if (pairs) {
                    pairs[2 * o] = I;
                    pairs[2 * o + 1] = pj[e];
                }
                if (shifts) {
                    shifts[3 * o] = (img[e] & 1023) - 512;
                    shifts[3 * o + 1] = ((img[e] >> 10) & 1023) - 512;
                    shifts[3 * o + 2] = ((img[e] >> 20) & 1023) - 512;
                }
            }
    }
    return MG_OK;
}
