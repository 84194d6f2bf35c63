// Empirical variogram estimators (vario_estimate / vario_estimate_axis).
//
// The reference estimates variograms with the external gstools-cython
// kernels unstructured, directional, structured and ma_structured
// (src/gstools/variogram/variogram.py:48-124, gstools-cython >= 1, < 2):
//
//   estimator  'm' (Matheron): d^2                 'c' (Cressie): |d|^0.5
//   normalise  'm': g / (2 N)
//              'c': 0.5 (g / N)^4 / (0.457 + 0.494 / N + 0.045 / N^2)
//              with N = max(count, 1)
//
// over the point pairs j < k whose distance falls in [edge_i, edge_{i+1})
// (per direction for the directional estimator: angle to the direction
// below angles_tol and, for bandwidth > 0, distance to its line below the
// bandwidth; separate_dirs stops at the first matching direction), for every
// field whose two values are not NaN.  Their loop runs the bins outermost
// and so evaluates every pair once per bin; here every pair is evaluated
// once, over 128 x 128 tiles of the upper triangle of the pair matrix.
// Euclidean omnidirectional estimates with up to 1024 bins take the fast path
// (vario_omni_kernel): FP32 squared distances from hi + lo coordinate splits
// with a proven error bound, a bin table, the exact FP64 distance only near
// an edge, per-warp histograms, and for one field the binned pairs queued
// per warp so the FP64 terms run on full warps.  Directional, haversine and
// many-bin estimates use vario_pairs_kernel (FP64 distances, FP32 binning
// with the same exact fallback, shared-memory histograms).  Sums of positive
// terms in a different order: equal to the reference within rounding;
// counts exact.
// The structured estimator runs one CTA per (lag, column chunk), partial
// sums reduced in a fixed order (deterministic).
#include <algorithm>
#include <cmath>

#include "gst_common.cuh"

namespace gst {
namespace {

constexpr int kPairTile = 128;
constexpr int kVarioThreads = 256;
constexpr int kMaxDims = 3;

__device__ __forceinline__ double estimate(int est, double d) {
    return est == 'c' ? sqrt(fabs(d)) : d * d;
}

// The reference's angle test, "if tt < 1: ok = acos(tt) < tol" with
// tt = |s| / dist, decided exactly: with a correctly rounded acos,
// RN(acos(tt)) < tol holds iff acos(tt) lies below the midpoint b of tol and
// its predecessor, i.e. iff tt > cos(b) (acos decreases).  cos(b) is formed
// once per call in double-double (angle_boundary) and compared here exactly,
// so no device acos (whose last bit may differ from the host's) decides a
// pair on the tolerance cone.  tt >= 1 always passes, as in the reference.
__device__ __forceinline__ bool angle_ok(double tt, double c_hi, double c_lo) {
    return tt > c_hi || (tt == c_hi && c_lo < 0.0);
}

__device__ __forceinline__ double haversine(double lat_j, double lon_j, double lat_k,
                                            double lon_k) {
    const double deg = 3.14159265358979323846 / 180.0;
    const double dlat = (lat_k - lat_j) * deg;
    const double dlon = (lon_k - lon_j) * deg;
    const double sa = sin(dlat / 2.0), so = sin(dlon / 2.0);
    const double a = sa * sa + cos(lat_j * deg) * cos(lat_k * deg) * so * so;
    return 2.0 * atan2(sqrt(a), sqrt(1.0 - a));
}

// Bin of distance `dist` given as its square d2 (exact sqrt on demand):
// last i with edge[i] <= dist < edge[i + 1], or -1.  The search runs in
// FP32 on the squared edges (GB300's FP64 rate is 1/64 of its FP32 rate);
// within 2^-20 (relative) of a squared edge, where FP32 rounding could
// change the order, the exact FP64 distance decides.
__device__ __forceinline__ int find_bin(double d2, const double *edges,
                                        const float *edges2f, int n_bins,
                                        double &dist, bool &have_dist) {
    if (!(d2 >= 0.0)) return -1;
    const float f2 = __double2float_rn(d2);
    constexpr float kGuard = 9.5367431640625e-07f;   // 2^-20
    // beyond the last edge: no bin (the common case for far pairs)
    if (f2 > edges2f[n_bins] * (1.0f + kGuard)) return -1;
    int lo = -1, hi = n_bins + 1;   // edges2f[lo] <= f2 < edges2f[hi] (virtual)
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (edges2f[mid] <= f2) lo = mid; else hi = mid;
    }
    bool near = false;
    if (lo >= 0 && fabsf(f2 - edges2f[lo]) <= kGuard * edges2f[lo]) near = true;
    if (lo + 1 <= n_bins && fabsf(f2 - edges2f[lo + 1]) <= kGuard * edges2f[lo + 1])
        near = true;
    if (near) {
        if (!have_dist) {
            dist = sqrt(d2);
            have_dist = true;
        }
        lo = -1;
        hi = n_bins + 1;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (edges[mid] <= dist) lo = mid; else hi = mid;
        }
    }
    return (lo >= 0 && lo < n_bins) ? lo : -1;
}

struct VarioArgs {
    int dim;
    int64_t n;
    int64_t f_max;
    const double *f;      // f_max x n
    const double *pos;    // dim x n
    int n_bins;
    const double *edges;  // n_bins + 1
    int est;              // 'm' or 'c'
    int haversine;        // distance type 'h'
    int d_max;            // 0: omnidirectional
    const double *dirs;   // d_max x dim (unit vectors)
    double angles_tol;
    double cos_hi, cos_lo;   // angle test boundary, see angle_boundary()
    double bandwidth;
    int separate_dirs;
    double *sums;         // max(d_max, 1) x n_bins, raw sums
    unsigned long long *counts;
};

// Dynamic shared memory: edges, squared edges, then the histograms.
__global__ void __launch_bounds__(kVarioThreads)
    vario_pairs_kernel(VarioArgs a, int64_t n_tiles) {
    extern __shared__ double sh[];
    const int nb = a.n_bins;
    const int nh = (a.d_max > 0 ? a.d_max : 1) * nb;
    double *edges = sh;
    float *edges2f = reinterpret_cast<float *>(edges + (nb + 1));
    double *h_sum = edges + 2 * (nb + 1);
    unsigned long long *h_cnt = reinterpret_cast<unsigned long long *>(h_sum + nh);
    // upper-triangle tile (tj <= tk) from the linear block index
    const int64_t t = blockIdx.x;
    int64_t tj = static_cast<int64_t>((sqrt(8.0 * static_cast<double>(t) + 1.0) - 1.0) / 2.0);
    while ((tj + 1) * (tj + 2) / 2 <= t) ++tj;
    while (tj * (tj + 1) / 2 > t) --tj;
    const int64_t tk_rev = t - tj * (tj + 1) / 2;   // 0..tj
    // map (row tj of the lower triangle) -> pair tile (j-tile tk_rev, k-tile tj)
    const int64_t jt = tk_rev, kt = tj;
    if (kt >= n_tiles) return;
    for (int i = threadIdx.x; i <= nb; i += blockDim.x) {
        const double e = a.edges[i];
        edges[i] = e;
        // non-positive edges lie below every distance: keep the squared
        // table monotonic
        edges2f[i] = e > 0.0 ? __double2float_rn(e * e) : -1.0f;
    }
    for (int i = threadIdx.x; i < nh; i += blockDim.x) {
        h_sum[i] = 0.0;
        h_cnt[i] = 0ull;
    }
    __syncthreads();
    const int64_t j0 = jt * kPairTile, k0 = kt * kPairTile;
    // thread -> one j of the tile and half of the k range
    const int jl = threadIdx.x % kPairTile;
    const int half = threadIdx.x / kPairTile;
    const int64_t j = j0 + jl;
    if (j < a.n) {
        double pj[kMaxDims] = {0.0, 0.0, 0.0};
        for (int d = 0; d < a.dim; ++d) pj[d] = a.pos[d * a.n + j];
        const int64_t kb = k0 + half * (kPairTile / 2);
        const int64_t ke = min(kb + kPairTile / 2, a.n);
        for (int64_t k = max(kb, j + 1); k < ke; ++k) {
            // unfused products and sums: the squared distance has the same
            // bits as the reference's, so bins match exactly
            double diffv[kMaxDims] = {0.0, 0.0, 0.0};
            double d2 = 0.0;
            for (int d = 0; d < a.dim; ++d) {
                diffv[d] = pj[d] - a.pos[d * a.n + k];
                d2 = __dadd_rn(d2, __dmul_rn(diffv[d], diffv[d]));
            }
            double dist = 0.0;
            bool have_dist = false;
            int bin;
            if (a.haversine) {
                dist = haversine(pj[0], pj[1], a.pos[k], a.pos[a.n + k]);
                have_dist = true;
                int lo = -1, hi = nb + 1;
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (edges[mid] <= dist) lo = mid; else hi = mid;
                }
                bin = (lo >= 0 && lo < nb) ? lo : -1;
            } else {
                bin = find_bin(d2, edges, edges2f, nb, dist, have_dist);
            }
            if (bin < 0) continue;
            if (a.d_max == 0) {
                for (int64_t m = 0; m < a.f_max; ++m) {
                    const double fa = a.f[m * a.n + k], fb = a.f[m * a.n + j];
                    if (isnan(fa) || isnan(fb)) continue;
                    atomicAdd(&h_sum[bin], estimate(a.est, fa - fb));
                    atomicAdd(&h_cnt[bin], 1ull);
                }
                continue;
            }
            if (!have_dist) {
                dist = sqrt(d2);
                have_dist = true;
            }
            for (int dd = 0; dd < a.d_max; ++dd) {
                const double *dir = a.dirs + dd * a.dim;
                double s_prod = 0.0;
                for (int d = 0; d < a.dim; ++d)
                    s_prod = __dadd_rn(s_prod, __dmul_rn(diffv[d], dir[d]));
                bool ok = true;
                if (a.bandwidth > 0.0) {
                    double b_dist = 0.0;
                    for (int d = 0; d < a.dim; ++d) {
                        const double tt = __dsub_rn(diffv[d], __dmul_rn(s_prod, dir[d]));
                        b_dist = __dadd_rn(b_dist, __dmul_rn(tt, tt));
                    }
                    ok = b_dist < __dmul_rn(a.bandwidth, a.bandwidth);
                }
                if (ok && dist > 0.0) ok = angle_ok(fabs(s_prod) / dist, a.cos_hi, a.cos_lo);
                if (!ok) continue;
                for (int64_t m = 0; m < a.f_max; ++m) {
                    const double fa = a.f[m * a.n + k], fb = a.f[m * a.n + j];
                    if (isnan(fa) || isnan(fb)) continue;
                    atomicAdd(&h_sum[dd * nb + bin], estimate(a.est, fa - fb));
                    atomicAdd(&h_cnt[dd * nb + bin], 1ull);
                }
                if (a.separate_dirs) break;
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nh; i += blockDim.x) {
        if (h_cnt[i] != 0ull) {
            atomicAdd(&a.sums[i], h_sum[i]);
            atomicAdd(&a.counts[i], h_cnt[i]);
        }
    }
}

// ------------------------------------------------ omnidirectional, fast path --
//
// Euclidean omnidirectional estimator with at most kOmniMaxBins bins.  The
// squared distance is formed in FP32 from hi + lo splits of the coordinates
// (x = hi + lo + r, |r| <= 2^-48 |x|).  Each difference is then off by at
// most 2^-23 |dx| + 2^-46 X (X the largest |coordinate| of the tile), and
// the squared distance, against the reference's FP64 value, by at most
//     B = 2^-21 d2 + 2^-44 X sqrt(d2) + 2^-90 X^2
// (checked on 3000 random point clouds, offsets 1e-6 .. 1e12, close and far
// pairs: largest error 0.72 B).  A pair whose FP32 value lies within
//     G_i = 2^-19 e_i^2 + 2^-41 X e_i + 2^-88 X^2
// (at least four times B at d2 = e_i^2) of a squared edge is binned from the
// exact FP64 distance instead, so every pair lands in the reference's bin.
// Each warp adds its pairs' FP64 terms into its own histogram in shared
// memory (shared FP64 atomics: measured 185 G adds/s over 40 random bins on
// GB300, against the ~55 G/s this kernel needs; per-thread histograms, 2.7x
// faster to update, held the SM to 12 warps); the CTAs are persistent over
// the upper-triangle tiles and flush their histograms (warps in a fixed
// order, one global atomic per bin) once at the end, or sooner if a 32-bit
// count could overflow.
constexpr int kOmniThreads = 128;
constexpr int kOmniWarps = kOmniThreads / 32;
constexpr int kOmniMaxBins = 1024;
constexpr int kOmniTab = 1024;   // cells of the squared-distance bin table
constexpr float kGuardRel = 1.9073486328125e-06f;     // 2^-19
constexpr float kGuardAbs = 4.547473508864641e-13f;   // 2^-41
constexpr float kGuardSq = 3.2311742677852644e-27f;   // 2^-88

constexpr int kOmniMaxDirs = 32;
constexpr float kDirGuardAbs = 2.2737367544323206e-13f;   // 2^-42

struct OmniArgs {
    int64_t n;
    int64_t f_max;
    const double *f;      // f_max x n
    const double *pos;    // dim x n
    int n_bins;
    const double *edges;  // n_bins + 1
    int est;
    int64_t n_tiles;      // 128-point tiles per axis
    int64_t n_tri;        // upper-triangle tiles
    double *sums;         // max(d_max, 1) x n_bins
    unsigned long long *counts;
    // directional estimator (d_max > 0): unit directions, angle tolerance
    // in (0, pi], bandwidth (<= 0: none), first matching direction only
    int d_max;
    const double *dirs;   // d_max x dim
    double angles_tol;
    double cos_hi, cos_lo;   // angle test boundary, see angle_boundary()
    double bandwidth;
    int separate_dirs;
};

__host__ __device__ constexpr size_t omni_smem_bytes(int nb, int nh) {
    return sizeof(double) * (nb + 1)                        // edges
           + sizeof(float) * 2 * (nb + 1)                   // squared edges, guards
           + sizeof(float4) * kOmniThreads * 2              // k-tile hi/lo, |x| max
           + sizeof(double) * kOmniThreads                  // k-tile field 0
           + sizeof(float) * 4                              // tile |x| max per warp
           + sizeof(double) * kOmniThreads                  // field 0 at j, per lane
           + sizeof(unsigned int) * 2 * kOmniThreads        // per-warp queues (64)
           + sizeof(short) * kOmniTab                       // bin table
           + sizeof(float) * 3 * kOmniMaxDirs               // FP32 directions
           + (sizeof(double) + sizeof(unsigned int)) * nh * kOmniWarps;
}

__device__ __forceinline__ void tile_of(int64_t t, int64_t &jt, int64_t &kt) {
    int64_t r = static_cast<int64_t>((sqrt(8.0 * static_cast<double>(t) + 1.0) - 1.0) / 2.0);
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    while (r * (r + 1) / 2 > t) --r;
    jt = t - r * (r + 1) / 2;   // 0..r
    kt = r;
}

template <int DIM>
__device__ __forceinline__ double exact_d2(double p0, double p1, double p2,
                                           const double *pos, int64_t n, int64_t k) {
    double dd = p0 - pos[k];
    double d2 = __dadd_rn(0.0, __dmul_rn(dd, dd));
    if (DIM > 1) {
        dd = p1 - pos[n + k];
        d2 = __dadd_rn(d2, __dmul_rn(dd, dd));
    }
    if (DIM > 2) {
        dd = p2 - pos[2 * n + k];
        d2 = __dadd_rn(d2, __dmul_rn(dd, dd));
    }
    return d2;
}

// Bin of pair (j, k) or -1: FP32 squared distance against the squared
// edges, the exact FP64 distance within the guard of an edge (or for every
// pair of a tile whose coordinates are out of the FP32 bound's range).
template <int DIM>
__device__ __forceinline__ int pair_bin(int kl, const float *jh, const float *jl,
                                        const double *pj, const float4 *k_hi,
                                        const float4 *k_lo, const float *e2f,
                                        const float *guard, const double *edges, int nb,
                                        float lim, const short *tab, float tscale,
                                        bool exact_only, const double *pos, int64_t n,
                                        int64_t k) {
    bool exact = exact_only;
    int bin = -1;
    if (!exact) {
        const float4 kh = k_hi[kl], klo = k_lo[kl];
        const float dx = (jh[0] - kh.x) + (jl[0] - klo.x);
        float f2 = dx * dx;
        if (DIM > 1) {
            const float dy = (jh[1] - kh.y) + (jl[1] - klo.y);
            f2 = fmaf(dy, dy, f2);
        }
        if (DIM > 2) {
            const float dz = (jh[2] - kh.z) + (jl[2] - klo.z);
            f2 = fmaf(dz, dz, f2);
        }
        if (!(f2 <= lim)) return -1;   // beyond the last edge (or NaN)
        // last lo with e2f[lo] <= f2: table guess, then exact steps
        int lo = tab[min(__float2int_rz(f2 * tscale), kOmniTab - 1)];
        while (lo >= 0 && e2f[lo] > f2) --lo;
        while (lo < nb && e2f[lo + 1] <= f2) ++lo;
        exact = (lo >= 0 && fabsf(f2 - e2f[lo]) <= guard[lo]) ||
                (lo + 1 <= nb && fabsf(f2 - e2f[lo + 1]) <= guard[lo + 1]);
        bin = (lo >= 0 && lo < nb) ? lo : -1;
    }
    if (exact) {
        const double d2 = exact_d2<DIM>(pj[0], pj[1], pj[2], pos, n, k);
        if (!(d2 >= 0.0)) return -1;
        const double dist = sqrt(d2);
        int lo = -1, hi = nb + 1;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (edges[mid] <= dist) lo = mid; else hi = mid;
        }
        bin = (lo >= 0 && lo < nb) ? lo : -1;
    }
    return bin;
}

// Directional form of pair_bin: the bin (or -1) and, in `mask`, the
// directions that accept the pair (bit dd; only the first with
// separate_dirs).  The FP32 projections decide unless a quantity lies within
// its guard of a threshold: the angle test |s| / dist > cos(tol) within
// 2^-19 + 2^-42 X / dist, the bandwidth test within the distance guard at
// d2; then the whole pair is evaluated in FP64 the reference's way
// (unfused sums, acos of |s| / dist against the tolerance).
template <int DIM>
__device__ __forceinline__ int pair_bin_dirs(int kl, const float *jh, const float *jl,
                                             const double *pj, const float4 *k_hi,
                                             const float4 *k_lo, const float *e2f,
                                             const float *guard, const double *edges,
                                             int nb, float lim, const short *tab,
                                             float tscale, bool exact_only, float X,
                                             const float *dirf, const OmniArgs &a,
                                             float ctol, float bw2f, int64_t k,
                                             unsigned int &mask) {
    mask = 0u;
    bool exact = exact_only;
    int bin = -1;
    if (!exact) {
        const float4 kh = k_hi[kl], klo = k_lo[kl];
        float dx[3] = {0.f, 0.f, 0.f};
        dx[0] = (jh[0] - kh.x) + (jl[0] - klo.x);
        float f2 = dx[0] * dx[0];
        if (DIM > 1) {
            dx[1] = (jh[1] - kh.y) + (jl[1] - klo.y);
            f2 = fmaf(dx[1], dx[1], f2);
        }
        if (DIM > 2) {
            dx[2] = (jh[2] - kh.z) + (jl[2] - klo.z);
            f2 = fmaf(dx[2], dx[2], f2);
        }
        if (!(f2 <= lim)) return -1;
        int lo = tab[min(__float2int_rz(f2 * tscale), kOmniTab - 1)];
        while (lo >= 0 && e2f[lo] > f2) --lo;
        while (lo < nb && e2f[lo + 1] <= f2) ++lo;
        exact = (lo >= 0 && fabsf(f2 - e2f[lo]) <= guard[lo]) ||
                (lo + 1 <= nb && fabsf(f2 - e2f[lo + 1]) <= guard[lo + 1]);
        bin = (lo >= 0 && lo < nb) ? lo : -1;
        if (!exact && bin < 0) return -1;
        if (!exact && !(f2 >= 1e-30f)) exact = true;   // (near) zero distance
        if (!exact) {
            const float dist = sqrtf(f2);
            const float gx = kGuardRel + kDirGuardAbs * X / dist;
            const float gb = kGuardRel * f2 + kGuardAbs * X * dist + kGuardSq * X * X;
            for (int dd = 0; dd < a.d_max; ++dd) {
                const float *dv = dirf + 3 * dd;
                float sp = dx[0] * dv[0];
                if (DIM > 1) sp = fmaf(dx[1], dv[1], sp);
                if (DIM > 2) sp = fmaf(dx[2], dv[2], sp);
                bool ok = true;
                if (bw2f > 0.0f) {
                    float b = 0.0f;
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        const float t = dx[d] - sp * dv[d];
                        b = fmaf(t, t, b);
                    }
                    if (fabsf(b - bw2f) <= gb) {
                        exact = true;
                        break;
                    }
                    ok = b < bw2f;
                }
                if (ok) {
                    const float x = fabsf(sp) / dist;
                    if (fabsf(x - ctol) <= gx) {
                        exact = true;
                        break;
                    }
                    ok = x > ctol;
                }
                if (ok) {
                    mask |= 1u << dd;
                    if (a.separate_dirs) break;
                }
            }
        }
    }
    if (exact) {
        mask = 0u;
        double diffv[3] = {0.0, 0.0, 0.0};
        double d2 = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
            diffv[d] = pj[d] - a.pos[d * a.n + k];
            d2 = __dadd_rn(d2, __dmul_rn(diffv[d], diffv[d]));
        }
        if (!(d2 >= 0.0)) return -1;
        const double dist = sqrt(d2);
        int lo = -1, hi = nb + 1;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (edges[mid] <= dist) lo = mid; else hi = mid;
        }
        if (lo < 0 || lo >= nb) return -1;
        bin = lo;
        for (int dd = 0; dd < a.d_max; ++dd) {
            const double *dir = a.dirs + dd * DIM;
            double s_prod = 0.0;
#pragma unroll
            for (int d = 0; d < DIM; ++d)
                s_prod = __dadd_rn(s_prod, __dmul_rn(diffv[d], dir[d]));
            bool ok = true;
            if (a.bandwidth > 0.0) {
                double b_dist = 0.0;
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    const double tt = __dsub_rn(diffv[d], __dmul_rn(s_prod, dir[d]));
                    b_dist = __dadd_rn(b_dist, __dmul_rn(tt, tt));
                }
                ok = b_dist < __dmul_rn(a.bandwidth, a.bandwidth);
            }
            if (ok && dist > 0.0) ok = angle_ok(fabs(s_prod) / dist, a.cos_hi, a.cos_lo);
            if (ok) {
                mask |= 1u << dd;
                if (a.separate_dirs) break;
            }
        }
    }
    return mask != 0u ? bin : -1;
}

template <bool CRESSIE>
__device__ __forceinline__ double estimate_t(double d) {
    return CRESSIE ? sqrt(fabs(d)) : d * d;
}

template <int DIM, bool CRESSIE, bool DIRS>
__global__ void __launch_bounds__(kOmniThreads, 8)
    vario_omni_kernel(const OmniArgs a) {
    extern __shared__ __align__(16) double sh[];
    const int nb = a.n_bins;
    const int nh = DIRS ? a.d_max * nb : nb;   // histogram cells: direction x bin
    const int tid = threadIdx.x;
    double *edges = sh;
    float *e2f = reinterpret_cast<float *>(edges + (nb + 1));
    float *guard = e2f + (nb + 1);
    // 16-byte aligned region after the edge tables
    const size_t off = (sizeof(double) * (nb + 1) + sizeof(float) * 2 * (nb + 1) + 15) / 16 * 16;
    float4 *k_hi = reinterpret_cast<float4 *>(reinterpret_cast<unsigned char *>(sh) + off);
    float4 *k_lo = k_hi + kOmniThreads;
    double *k_f = reinterpret_cast<double *>(k_lo + kOmniThreads);
    float *w_max = reinterpret_cast<float *>(k_f + kOmniThreads);
    double *w_fj = reinterpret_cast<double *>(w_max + 4);
    unsigned int *w_queue = reinterpret_cast<unsigned int *>(w_fj + kOmniThreads);
    double *h_sum = reinterpret_cast<double *>(w_queue + 2 * kOmniThreads);
    unsigned int *h_cnt = reinterpret_cast<unsigned int *>(h_sum + nh * kOmniWarps);
    short *tab = reinterpret_cast<short *>(h_cnt + nh * kOmniWarps);
    float *dirf = reinterpret_cast<float *>(tab + kOmniTab);   // [dir][3]
    const float ctol = DIRS ? static_cast<float>(cos(a.angles_tol)) : 0.0f;
    const float bw2f =
        (DIRS && a.bandwidth > 0.0) ? static_cast<float>(a.bandwidth * a.bandwidth) : 0.0f;
    if (DIRS)
        for (int i = tid; i < 3 * a.d_max; i += kOmniThreads)
            dirf[i] = (i % 3 < DIM) ? static_cast<float>(a.dirs[(i / 3) * DIM + i % 3]) : 0.0f;

    for (int i = tid; i <= nb; i += kOmniThreads) {
        const double e = a.edges[i];
        edges[i] = e;
        e2f[i] = e > 0.0 ? __double2float_rn(e * e) : -1.0f;
    }
    for (int i = tid; i < nh * kOmniWarps; i += kOmniThreads) {
        h_sum[i] = 0.0;
        h_cnt[i] = 0u;
    }
    __syncthreads();
    // tab[c]: last bin lo with e2f[lo] <= c / tscale (cell c of [0, e2f[nb]])
    const float tscale = e2f[nb] > 0.0f ? static_cast<float>(kOmniTab) / e2f[nb] : 0.0f;
    for (int c = tid; c < kOmniTab; c += kOmniThreads) {
        const float v = tscale > 0.0f ? static_cast<float>(c) / tscale : 0.0f;
        int lo = -1, hi = nb + 1;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (e2f[mid] <= v) lo = mid; else hi = mid;
        }
        tab[c] = static_cast<short>(lo > nb ? nb : lo);
    }
    // tiles between flushes such that no 32-bit count overflows: a warp
    // adds at most 32 x kOmniThreads pairs per field, direction and tile
    const int64_t per_tile = static_cast<int64_t>(32 * kOmniThreads) *
                             (a.f_max > 1 ? a.f_max : 1) *
                             (DIRS && a.d_max > 1 ? a.d_max : 1);
    const int64_t flush_every = per_tile >= 0xffffffffLL ? 1 : 0xffffffffLL / per_tile;
    int64_t since_flush = 0;

    auto flush = [&]() {
        __syncthreads();
        for (int b = tid; b < nh; b += kOmniThreads) {
            double g = 0.0;
            unsigned long long c = 0ull;
            for (int w = 0; w < kOmniWarps; ++w) {
                g += h_sum[w * nh + b];
                c += h_cnt[w * nh + b];
                h_sum[w * nh + b] = 0.0;
                h_cnt[w * nh + b] = 0u;
            }
            if (c != 0ull) {
                atomicAdd(&a.sums[b], g);
                atomicAdd(&a.counts[b], c);
            }
        }
        __syncthreads();
    };

    for (int64_t t = blockIdx.x; t < a.n_tri; t += gridDim.x) {
        int64_t jt, kt;
        tile_of(t, jt, kt);
        const int64_t j = jt * kOmniThreads + tid;
        const int64_t kstage = kt * kOmniThreads + tid;
        __syncthreads();   // the previous tile's readers are done
        float xmax = 0.0f;
        {
            float4 hi = make_float4(0.f, 0.f, 0.f, 0.f), lo = hi;
            if (kstage < a.n) {
                float h[3] = {0.f, 0.f, 0.f}, l[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    const double x = a.pos[d * a.n + kstage];
                    h[d] = __double2float_rn(x);
                    l[d] = __double2float_rn(x - static_cast<double>(h[d]));
                    xmax = fmaxf(xmax, fabsf(h[d]));
                }
                // w: 1 when field 0 of this point is a number
                const double fk = a.f_max > 0 ? a.f[kstage] : 0.0;
                hi = make_float4(h[0], h[1], h[2],
                                 (a.f_max > 0 && !isnan(fk)) ? 1.f : 0.f);
                lo = make_float4(l[0], l[1], l[2], 0.f);
                k_f[tid] = fk;
            }
            k_hi[tid] = hi;
            k_lo[tid] = lo;
        }
        double pj[3] = {0.0, 0.0, 0.0};
        float jh[3] = {0.f, 0.f, 0.f}, jl[3] = {0.f, 0.f, 0.f};
        if (j < a.n) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                pj[d] = a.pos[d * a.n + j];
                jh[d] = __double2float_rn(pj[d]);
                jl[d] = __double2float_rn(pj[d] - static_cast<double>(jh[d]));
                xmax = fmaxf(xmax, fabsf(jh[d]));
            }
        }
        // tile maximum of |x| (NaN propagates as "not finite" below)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            xmax = fmaxf(xmax, __shfl_xor_sync(0xffffffffu, xmax, o));
        if ((tid & 31) == 0) w_max[tid >> 5] = xmax;
        __syncthreads();
        const float X = fmaxf(fmaxf(w_max[0], w_max[1]), fmaxf(w_max[2], w_max[3]));
        // the FP32 bound holds for moderate coordinates; otherwise every
        // pair of the tile takes the exact FP64 distance
        const bool exact_only = !(X >= 1e-18f && X <= 1e18f);
        for (int i = tid; i <= nb; i += kOmniThreads) {
            const float e = __double2float_rn(fabs(edges[i]));
            guard[i] = edges[i] > 0.0
                           ? kGuardRel * e2f[i] + kGuardAbs * X * e + kGuardSq * X * X
                           : 0.0f;
        }
        __syncthreads();
        const float lim = e2f[nb] + guard[nb];
        const int64_t rest = a.n - kt * kOmniThreads;
        const int kl1 = rest < kOmniThreads ? static_cast<int>(rest) : kOmniThreads;
        const double fj = (j < a.n && a.f_max > 0) ? a.f[j] : 0.0;
        if (a.f_max == 1) {
            // One field: the lanes run the same k sequence, and the pairs
            // that fall in a bin (about 40 % of them) are queued per warp, so
            // the FP64 terms run on full warps.  Queue entry: bin << 16 |
            // k << 5 | lane of j.
            const int lane = tid & 31, warp = tid >> 5;
            unsigned int *q = w_queue + warp * 64;
            w_fj[tid] = fj;
            const bool row_ok = j < a.n && !isnan(fj);
            const int kl_first = (jt == kt) ? warp * 32 + 1 : 0;
            int qn = 0;
            // queue the pair (bin >= 0) and run the FP64 terms of a full round
            auto enqueue = [&](int bin, int kl) {
                const unsigned int m = __ballot_sync(0xffffffffu, bin >= 0);
                if (bin >= 0)
                    q[qn + __popc(m & ((1u << lane) - 1u))] =
                        (static_cast<unsigned int>(bin) << 16) |
                        (static_cast<unsigned int>(kl) << 5) | lane;
                qn += __popc(m);
                if (qn >= 32) {
                    __syncwarp();
                    const unsigned int e = q[lane];
                    const double d = k_f[(e >> 5) & 127u] - w_fj[warp * 32 + (e & 31u)];
                    atomicAdd(&h_sum[warp * nh + (e >> 16)], estimate_t<CRESSIE>(d));
                    atomicAdd(&h_cnt[warp * nh + (e >> 16)], 1u);
                    __syncwarp();
                    if (lane < qn - 32) q[lane] = q[32 + lane];
                    __syncwarp();
                    qn -= 32;
                }
            };
            // bin of pair (j, k), and its accepted directions (DIRS)
            auto bin_of = [&](int kl, unsigned int &mask) {
                mask = 1u;
                if (kl < kl1 && row_ok && (jt != kt || kl > tid) && k_hi[kl].w != 0.f) {
                    if (DIRS)
                        return pair_bin_dirs<DIM>(kl, jh, jl, pj, k_hi, k_lo, e2f, guard,
                                                  edges, nb, lim, tab, tscale, exact_only,
                                                  X, dirf, a, ctol, bw2f,
                                                  kt * kOmniThreads + kl, mask);
                    return pair_bin<DIM>(kl, jh, jl, pj, k_hi, k_lo, e2f, guard, edges, nb,
                                         lim, tab, tscale, exact_only, a.pos, a.n,
                                         kt * kOmniThreads + kl);
                }
                return -1;
            };
            // one queue entry per accepted direction (cell dir * nb + bin)
            auto enqueue_dirs = [&](int bin, unsigned int mask, int kl) {
                if constexpr (DIRS) {
                    for (int dd = 0; dd < a.d_max; ++dd)
                        enqueue((bin >= 0 && ((mask >> dd) & 1u)) ? dd * nb + bin : -1, kl);
                } else {
                    enqueue(bin, kl);
                }
            };
            if (__any_sync(0xffffffffu, row_ok)) {
                // two independent pairs per step for latency hiding (four
                // measured no faster)
                for (int kl = kl_first; kl < kl1; kl += 2) {
                    unsigned int m0, m1;
                    const int b0 = bin_of(kl, m0);
                    const int b1 = bin_of(kl + 1, m1);
                    enqueue_dirs(b0, m0, kl);
                    enqueue_dirs(b1, m1, kl + 1);
                }
            }
            __syncwarp();
            if (lane < qn) {
                const unsigned int e = q[lane];
                const double d = k_f[(e >> 5) & 127u] - w_fj[warp * 32 + (e & 31u)];
                atomicAdd(&h_sum[warp * nh + (e >> 16)], estimate_t<CRESSIE>(d));
                atomicAdd(&h_cnt[warp * nh + (e >> 16)], 1u);
            }
        } else if (j < a.n) {
            // no field or several fields: per-lane terms
            const bool fj_ok = a.f_max > 0 && !isnan(fj);
            const int kl0 = (jt == kt) ? tid + 1 : 0;
            for (int kl = kl0; kl < kl1; ++kl) {
                const int64_t k = kt * kOmniThreads + kl;
                unsigned int mask = 1u;
                const int bin =
                    DIRS ? pair_bin_dirs<DIM>(kl, jh, jl, pj, k_hi, k_lo, e2f, guard, edges,
                                              nb, lim, tab, tscale, exact_only, X, dirf, a,
                                              ctol, bw2f, k, mask)
                         : pair_bin<DIM>(kl, jh, jl, pj, k_hi, k_lo, e2f, guard, edges, nb,
                                         lim, tab, tscale, exact_only, a.pos, a.n, k);
                if (bin < 0) continue;
                double g = 0.0;
                unsigned int c = 0u;
                if (fj_ok && k_hi[kl].w != 0.f) {
                    g = estimate_t<CRESSIE>(k_f[kl] - fj);
                    c = 1u;
                }
                for (int64_t m = 1; m < a.f_max; ++m) {
                    const double fa = a.f[m * a.n + k], fb = a.f[m * a.n + j];
                    if (isnan(fa) || isnan(fb)) continue;
                    g += estimate_t<CRESSIE>(fa - fb);
                    ++c;
                }
                if (c != 0u) {
                    for (int dd = 0; dd < (DIRS ? a.d_max : 1); ++dd) {
                        if (!((mask >> dd) & 1u)) continue;
                        atomicAdd(&h_sum[(tid >> 5) * nh + dd * nb + bin], g);
                        atomicAdd(&h_cnt[(tid >> 5) * nh + dd * nb + bin], c);
                    }
                }
            }
        }
        if (++since_flush >= flush_every) {
            flush();
            since_flush = 0;
        }
    }
    flush();
}

__device__ __forceinline__ double normalise(int est, double g, unsigned long long c) {
    const double cnt = c > 1ull ? static_cast<double>(c) : 1.0;
    if (est == 'c') {
        const double q = g / cnt;
        return 0.5 * (q * q) * (q * q) / (0.457 + 0.494 / cnt + 0.045 / (cnt * cnt));
    }
    return g / (2.0 * cnt);
}

__global__ void vario_normalise_kernel(int est, int64_t n, double *sums,
                                       const unsigned long long *counts) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i < n) sums[i] = normalise(est, sums[i], counts[i]);
}

// Structured: one CTA per (lag k, chunk of 256 columns); each thread one
// column, sums over i; CTA partial -> partials[k * n_chunks + chunk].
__global__ void __launch_bounds__(256)
    vario_structured_kernel(int64_t n0, int64_t rest, const double *__restrict__ f,
                            const unsigned char *__restrict__ mask, int est,
                            int64_t n_chunks, double *__restrict__ part_sum,
                            unsigned long long *__restrict__ part_cnt) {
    __shared__ double s_sum[256];
    __shared__ unsigned long long s_cnt[256];
    const int64_t k = blockIdx.y + 1;
    const int64_t chunk = blockIdx.x;
    const int64_t j = chunk * 256 + threadIdx.x;
    double g = 0.0;
    unsigned long long c = 0;
    if (j < rest) {
        for (int64_t i = 0; i + k < n0; ++i) {
            if (mask && (mask[i * rest + j] || mask[(i + k) * rest + j])) continue;
            ++c;
            g += estimate(est, f[i * rest + j] - f[(i + k) * rest + j]);
        }
    }
    s_sum[threadIdx.x] = g;
    s_cnt[threadIdx.x] = c;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            s_sum[threadIdx.x] += s_sum[threadIdx.x + w];
            s_cnt[threadIdx.x] += s_cnt[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part_sum[(k - 1) * n_chunks + chunk] = s_sum[0];
        part_cnt[(k - 1) * n_chunks + chunk] = s_cnt[0];
    }
}

// Structured, tiled: one CTA per block of 32 columns, the whole block
// (n0 <= kTiledMaxRows rows) in shared memory.  Warp g handles the lags
// k = g + 1, g + 9, ...; lane c one column: per lag it sums the pairs
// (i, i + k) of its column in row order, the warp adds its 32 column sums
// in a fixed order (shuffle tree) and lane 0 writes the CTA's partial for k.
// Per pair two shared loads, one DADD and one DFMA: the FP64 pipe bounds it.
constexpr int kTiledCols = 32;
constexpr int kTiledWarps = 8;
constexpr int kTiledMaxRows = 512;

template <bool CRESSIE, bool MASKED>
__global__ void __launch_bounds__(kTiledCols * kTiledWarps)
    vario_structured_tiled_kernel(int64_t n0, int64_t rest, const double *__restrict__ f,
                                  const unsigned char *__restrict__ mask, int64_t n_chunks,
                                  double *__restrict__ part_sum,
                                  unsigned long long *__restrict__ part_cnt) {
    extern __shared__ __align__(16) double fs[];   // [n0][32], then mask bytes
    unsigned char *ms = reinterpret_cast<unsigned char *>(fs + n0 * kTiledCols);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t chunk = blockIdx.x;
    const int64_t col = chunk * kTiledCols + lane;
    const bool col_ok = col < rest;
    for (int64_t i = warp; i < n0; i += kTiledWarps) {
        fs[i * kTiledCols + lane] = col_ok ? f[i * rest + col] : 0.0;
        if (MASKED) ms[i * kTiledCols + lane] = col_ok ? mask[i * rest + col] : 1;
    }
    __syncthreads();
    for (int64_t k = warp + 1; k < n0; k += kTiledWarps) {
        double acc = 0.0;
        unsigned int cnt = 0u;
        if (col_ok) {
            for (int64_t i = 0; i + k < n0; ++i) {
                const double d = fs[i * kTiledCols + lane] - fs[(i + k) * kTiledCols + lane];
                if (MASKED) {
                    if (ms[i * kTiledCols + lane] | ms[(i + k) * kTiledCols + lane]) continue;
                    ++cnt;
                }
                if (CRESSIE) acc += sqrt(fabs(d));
                else acc = fma(d, d, acc);
            }
            if (!MASKED) cnt = static_cast<unsigned int>(n0 - k);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            acc += __shfl_down_sync(0xffffffffu, acc, o);
            cnt += __shfl_down_sync(0xffffffffu, cnt, o);
        }
        if (lane == 0) {
            part_sum[(k - 1) * n_chunks + chunk] = acc;
            part_cnt[(k - 1) * n_chunks + chunk] = cnt;
        }
    }
}

__global__ void vario_structured_finish(int64_t n0, int64_t n_chunks, int est,
                                        const double *part_sum,
                                        const unsigned long long *part_cnt,
                                        double *vario) {
    const int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (k >= n0) return;
    if (k == 0) {
        vario[0] = 0.0;
        return;
    }
    double g = 0.0;
    unsigned long long c = 0;
    for (int64_t ch = 0; ch < n_chunks; ++ch) {
        g += part_sum[(k - 1) * n_chunks + ch];
        c += part_cnt[(k - 1) * n_chunks + ch];
    }
    vario[k] = normalise(est, g, c);
}

// ---------------------------------------------- double-double angle bound --

struct DD {
    double hi, lo;
};

DD dd_two_sum(double a, double b) {
    const double s = a + b;
    const double bb = s - a;
    return DD{s, (a - (s - bb)) + (b - bb)};
}

DD dd_add(DD a, DD b) {
    DD s = dd_two_sum(a.hi, b.hi);
    s.lo += a.lo + b.lo;
    return dd_two_sum(s.hi, s.lo);
}

DD dd_mul(DD a, DD b) {
    const double p = a.hi * b.hi;
    const double e = std::fma(a.hi, b.hi, -p) + (a.hi * b.lo + a.lo * b.hi);
    return dd_two_sum(p, e);
}

DD dd_div_d(DD a, double d) {
    const double q1 = a.hi / d;
    // remainder a - q1 d, exact in double-double
    const double p = q1 * d;
    const double e = std::fma(q1, d, -p);
    const double r = ((a.hi - p) - e) + a.lo;
    const double q2 = r / d;
    return dd_two_sum(q1, q2);
}

// cos(tol - delta) in double-double, delta half the gap from tol down to the
// next double: the boundary of "RN(acos(tt)) < tol".  Taylor series in
// double-double (|x| <= 2, terms below 1e-40 dropped).  tol <= 0 or NaN:
// only tt >= 1 passes; tol > 2 (beyond pi / 2 + 0.4): every tt in [0, 1]
// passes.
void angle_boundary(double tol, double &c_hi, double &c_lo) {
    if (!(tol > 0.0)) {
        c_hi = 1.0;
        c_lo = -1e-30;
        return;
    }
    if (tol > 2.0) {
        c_hi = -2.0;
        c_lo = 0.0;
        return;
    }
    const double below = std::nextafter(tol, 0.0);
    const DD x = dd_two_sum(tol, -(tol - below) * 0.5);   // exact: tol - delta
    const DD x2 = dd_mul(x, x);
    DD sum{1.0, 0.0}, term{1.0, 0.0};
    for (int n = 1; n < 40; ++n) {
        term = dd_div_d(dd_mul(term, x2), static_cast<double>((2 * n - 1) * (2 * n)));
        const DD signed_term = (n & 1) ? DD{-term.hi, -term.lo} : term;
        sum = dd_add(sum, signed_term);
        if (std::fabs(term.hi) < 1e-40) break;
    }
    c_hi = sum.hi;
    c_lo = sum.lo;
}

template <int DIM, bool CRESSIE, bool DIRS>
cudaError_t launch_omni_t(const OmniArgs &o, cudaStream_t s) {
    const int nh = DIRS ? o.d_max * o.n_bins : o.n_bins;
    const size_t smem = omni_smem_bytes(o.n_bins, nh) + 16;
    cudaError_t e = cudaFuncSetAttribute(vario_omni_kernel<DIM, CRESSIE, DIRS>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, vario_omni_kernel<DIM, CRESSIE, DIRS>, kOmniThreads, smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = std::min<int64_t>(
        o.n_tri, static_cast<int64_t>(std::max(per_sm, 1)) * sm_count());
    vario_omni_kernel<DIM, CRESSIE, DIRS>
        <<<static_cast<unsigned>(grid), kOmniThreads, smem, s>>>(o);
    return cudaGetLastError();
}

template <int DIM>
cudaError_t launch_omni(const OmniArgs &o, cudaStream_t s) {
    if (o.d_max > 0)
        return o.est == 'c' ? launch_omni_t<DIM, true, true>(o, s)
                            : launch_omni_t<DIM, false, true>(o, s);
    return o.est == 'c' ? launch_omni_t<DIM, true, false>(o, s)
                        : launch_omni_t<DIM, false, false>(o, s);
}

int pairs_impl(const VarioArgs &args, double *vario, int64_t *counts, cudaStream_t s) {
    const int nh = (args.d_max > 0 ? args.d_max : 1) * args.n_bins;
    VarioArgs a = args;
    angle_boundary(a.angles_tol, a.cos_hi, a.cos_lo);
    a.sums = vario;   // raw sums, normalised in place at the end
    a.counts = reinterpret_cast<unsigned long long *>(counts);
    GST_TRY_CUDA(cudaMemsetAsync(a.sums, 0, sizeof(double) * nh, s));
    GST_TRY_CUDA(cudaMemsetAsync(a.counts, 0, sizeof(unsigned long long) * nh, s));
    // Fast path: Euclidean; omnidirectional, or up to 32 directions with an
    // angle tolerance in (0, pi]; at most 1024 histogram cells.
    const bool fast_dirs =
        a.d_max == 0 || (a.d_max <= kOmniMaxDirs && a.angles_tol > 0.0 &&
                         a.angles_tol <= 3.14159265358979323846);
    if (!a.haversine && fast_dirs && nh <= kOmniMaxBins) {
        OmniArgs o{};
        o.n = a.n;
        o.f_max = a.f_max;
        o.f = a.f;
        o.pos = a.pos;
        o.n_bins = a.n_bins;
        o.edges = a.edges;
        o.est = a.est;
        o.n_tiles = ceil_div(a.n, kOmniThreads);
        o.n_tri = o.n_tiles * (o.n_tiles + 1) / 2;
        o.sums = a.sums;
        o.counts = a.counts;
        o.d_max = a.d_max;
        o.dirs = a.dirs;
        o.angles_tol = a.angles_tol;
        o.cos_hi = a.cos_hi;
        o.cos_lo = a.cos_lo;
        o.bandwidth = a.bandwidth;
        o.separate_dirs = a.separate_dirs;
        if (o.n_tri > 0) {
            cudaError_t e = a.dim == 1   ? launch_omni<1>(o, s)
                            : a.dim == 2 ? launch_omni<2>(o, s)
                                         : launch_omni<3>(o, s);
            GST_TRY_CUDA(e);
        }
        vario_normalise_kernel<<<static_cast<unsigned>(ceil_div(nh, 256)), 256, 0, s>>>(
            a.est, nh, a.sums, a.counts);
        GST_TRY_CUDA(cudaGetLastError());
        return GST_OK;
    }
    const int64_t n_tiles = ceil_div(args.n, kPairTile);
    const int64_t blocks = n_tiles * (n_tiles + 1) / 2;
    if (blocks > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    const size_t smem = sizeof(double) * (2 * (args.n_bins + 1) + nh) +
                        sizeof(unsigned long long) * nh;
    if (smem > 200 * 1024) return GST_ERR_TOO_LARGE;
    if (smem > 48 * 1024)
        GST_TRY_CUDA(cudaFuncSetAttribute(vario_pairs_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          static_cast<int>(smem)));
    if (blocks > 0)
        vario_pairs_kernel<<<static_cast<unsigned>(blocks), kVarioThreads, smem, s>>>(
            a, n_tiles);
    GST_TRY_CUDA(cudaGetLastError());
    vario_normalise_kernel<<<static_cast<unsigned>(ceil_div(nh, 256)), 256, 0, s>>>(
        a.est, nh, a.sums, a.counts);
    GST_TRY_CUDA(cudaGetLastError());
    return GST_OK;
}

bool valid_est(int est) { return est == 'm' || est == 'c'; }

}  // namespace
}  // namespace gst

extern "C" {

int gst_vario_unstructured(int dim, int64_t n, int64_t f_max, const double *f,
                           int64_t n_bins, const double *bin_edges, const double *pos,
                           int estimator, int distance_type, double *vario,
                           int64_t *counts, void *stream) {
    if (dim < 1 || dim > gst::kMaxDims) return GST_ERR_UNSUPPORTED_DIM;
    if (n < 0 || f_max < 0 || n_bins < 0 || n_bins > 0x7fffffffLL)
        return GST_ERR_INVALID_ARGUMENT;
    if (!gst::valid_est(estimator) || (distance_type != 'e' && distance_type != 'h'))
        return GST_ERR_INVALID_ARGUMENT;
    if (distance_type == 'h' && dim != 2) return GST_ERR_UNSUPPORTED_DIM;
    if (n_bins == 0) return GST_OK;
    if (bin_edges == nullptr || vario == nullptr || counts == nullptr ||
        (n > 0 && (pos == nullptr || (f_max > 0 && f == nullptr))))
        return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    gst::VarioArgs a{};
    a.dim = dim;
    a.n = n;
    a.f_max = f_max;
    a.f = f;
    a.pos = pos;
    a.n_bins = static_cast<int>(n_bins);
    a.edges = bin_edges;
    a.est = estimator;
    a.haversine = distance_type == 'h';
    a.d_max = 0;
    return gst::pairs_impl(a, vario, counts, static_cast<cudaStream_t>(stream));
}

int gst_vario_directional(int dim, int64_t n, int64_t f_max, const double *f,
                          int64_t n_bins, const double *bin_edges, const double *pos,
                          int64_t n_dirs, const double *directions, double angles_tol,
                          double bandwidth, int separate_dirs, int estimator,
                          double *vario, int64_t *counts, void *stream) {
    if (dim < 1 || dim > gst::kMaxDims) return GST_ERR_UNSUPPORTED_DIM;
    if (n < 0 || f_max < 0 || n_bins < 0 || n_dirs < 0 || n_bins > 0x7fffffffLL ||
        n_dirs > 0x7fffffffLL)
        return GST_ERR_INVALID_ARGUMENT;
    if (!gst::valid_est(estimator)) return GST_ERR_INVALID_ARGUMENT;
    if (n_bins == 0 || n_dirs == 0) return GST_OK;
    if (bin_edges == nullptr || vario == nullptr || counts == nullptr ||
        directions == nullptr || (n > 0 && (pos == nullptr || (f_max > 0 && f == nullptr))))
        return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    gst::VarioArgs a{};
    a.dim = dim;
    a.n = n;
    a.f_max = f_max;
    a.f = f;
    a.pos = pos;
    a.n_bins = static_cast<int>(n_bins);
    a.edges = bin_edges;
    a.est = estimator;
    a.haversine = 0;
    a.d_max = static_cast<int>(n_dirs);
    a.dirs = directions;
    a.angles_tol = angles_tol;
    a.bandwidth = bandwidth;
    a.separate_dirs = separate_dirs ? 1 : 0;
    return gst::pairs_impl(a, vario, counts, static_cast<cudaStream_t>(stream));
}

int gst_vario_angle_boundary(double angles_tol, double *cos_hi, double *cos_lo) {
    if (cos_hi == nullptr || cos_lo == nullptr) return GST_ERR_INVALID_ARGUMENT;
    gst::angle_boundary(angles_tol, *cos_hi, *cos_lo);
    return GST_OK;
}

int gst_vario_structured(int64_t n0, int64_t rest, const double *f,
                         const unsigned char *mask, int estimator, double *vario,
                         void *stream) {
    if (n0 < 0 || rest < 0) return GST_ERR_INVALID_ARGUMENT;
    if (!gst::valid_est(estimator)) return GST_ERR_INVALID_ARGUMENT;
    if (n0 == 0) return GST_OK;
    if (vario == nullptr || (rest > 0 && f == nullptr)) return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool tiled = n0 <= gst::kTiledMaxRows;
    const int64_t n_chunks =
        std::max<int64_t>(1, gst::ceil_div(rest, tiled ? gst::kTiledCols : 256));
    const int64_t lags = n0 - 1;
    if (lags > 65535 || n_chunks > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    gst::StreamScratch scratch;
    const size_t parts = static_cast<size_t>(std::max<int64_t>(lags, 1)) * n_chunks;
    GST_TRY_CUDA(scratch.alloc(parts * (sizeof(double) + sizeof(unsigned long long)), s));
    double *psum = static_cast<double *>(scratch.ptr);
    auto *pcnt = reinterpret_cast<unsigned long long *>(psum + parts);
    if (lags > 0 && tiled) {
        if (rest == 0) {
            GST_TRY_CUDA(cudaMemsetAsync(psum, 0, parts * sizeof(double), s));
            GST_TRY_CUDA(cudaMemsetAsync(pcnt, 0, parts * sizeof(unsigned long long), s));
        } else {
            const size_t smem = static_cast<size_t>(n0) * gst::kTiledCols *
                                (sizeof(double) + (mask ? 1 : 0));
            auto *kern = estimator == 'c'
                             ? (mask ? gst::vario_structured_tiled_kernel<true, true>
                                     : gst::vario_structured_tiled_kernel<true, false>)
                             : (mask ? gst::vario_structured_tiled_kernel<false, true>
                                     : gst::vario_structured_tiled_kernel<false, false>);
            GST_TRY_CUDA(cudaFuncSetAttribute(
                kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
            kern<<<static_cast<unsigned>(n_chunks), gst::kTiledCols * gst::kTiledWarps,
                   smem, s>>>(n0, rest, f, mask, n_chunks, psum, pcnt);
            GST_TRY_CUDA(cudaGetLastError());
        }
    } else if (lags > 0) {
        const dim3 grid(static_cast<unsigned>(n_chunks), static_cast<unsigned>(lags));
        gst::vario_structured_kernel<<<grid, 256, 0, s>>>(n0, rest, f, mask, estimator,
                                                          n_chunks, psum, pcnt);
        GST_TRY_CUDA(cudaGetLastError());
    }
    gst::vario_structured_finish<<<static_cast<unsigned>(gst::ceil_div(n0, 256)), 256, 0,
                                   s>>>(n0, n_chunks, estimator, psum, pcnt, vario);
    GST_TRY_CUDA(cudaGetLastError());
    return GST_OK;
}

}  // extern "C"
