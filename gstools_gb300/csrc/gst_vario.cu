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
// once: CTAs own 128 x 128 tiles of the upper triangle of the pair matrix,
// bin by binary search over the squared edges (the exact square root is
// taken only when the squared distance is within a few ulps of a squared
// edge, so bins match the reference's sqrt-then-compare), and add into
// shared-memory histograms flushed with atomics.  Sums of positive terms in
// a different order: equal to the reference within rounding; counts exact.
// The structured estimator runs one CTA per (lag, column chunk), partial
// sums reduced in a fixed order (deterministic).
#include <algorithm>

#include "gst_common.cuh"

namespace gst {
namespace {

constexpr int kPairTile = 128;
constexpr int kVarioThreads = 256;
constexpr int kMaxDims = 3;

__device__ __forceinline__ double estimate(int est, double d) {
    return est == 'c' ? sqrt(fabs(d)) : d * d;
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
                if (ok && dist > 0.0) {
                    const double tt = fabs(s_prod) / dist;
                    if (tt < 1.0) ok = acos(tt) < a.angles_tol;
                }
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

int pairs_impl(const VarioArgs &args, double *vario, int64_t *counts, cudaStream_t s) {
    const int nh = (args.d_max > 0 ? args.d_max : 1) * args.n_bins;
    VarioArgs a = args;
    a.sums = vario;   // raw sums, normalised in place at the end
    a.counts = reinterpret_cast<unsigned long long *>(counts);
    GST_TRY_CUDA(cudaMemsetAsync(a.sums, 0, sizeof(double) * nh, s));
    GST_TRY_CUDA(cudaMemsetAsync(a.counts, 0, sizeof(unsigned long long) * nh, s));
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

int gst_vario_structured(int64_t n0, int64_t rest, const double *f,
                         const unsigned char *mask, int estimator, double *vario,
                         void *stream) {
    if (n0 < 0 || rest < 0) return GST_ERR_INVALID_ARGUMENT;
    if (!gst::valid_est(estimator)) return GST_ERR_INVALID_ARGUMENT;
    if (n0 == 0) return GST_OK;
    if (vario == nullptr || (rest > 0 && f == nullptr)) return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int64_t n_chunks = std::max<int64_t>(1, gst::ceil_div(rest, 256));
    const int64_t lags = n0 - 1;
    if (lags > 65535 || n_chunks > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    gst::StreamScratch scratch;
    const size_t parts = static_cast<size_t>(std::max<int64_t>(lags, 1)) * n_chunks;
    GST_TRY_CUDA(scratch.alloc(parts * (sizeof(double) + sizeof(unsigned long long)), s));
    double *psum = static_cast<double *>(scratch.ptr);
    auto *pcnt = reinterpret_cast<unsigned long long *>(psum + parts);
    if (lags > 0) {
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
