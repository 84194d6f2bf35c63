// Kriging field and error variance from the inverted kriging matrix.
//
// The reference's Krige (src/gstools/krige/base.py:307-320, through the
// wrappers at :42-60) hands the inverted kriging matrix M (K x K), the
// right-hand sides V (K x n: covariances between the K conditions and n
// target points, plus unbiasedness / drift rows) and the condition values c
// to the external gstools-cython kernels calc_field_krige(_and_variance)
// (gstools-cython >= 1, < 2), which compute per target point k
//
//     f_k = sum_i c_i (M v_k)_i,        e_k = sum_i v_ik (M v_k)_i,
//
// a K^2 n FP64 contraction.  With the variance, one CTA owns 64 target
// points and walks the rows of M in blocks of 64: the 64 x 64 block of M V is
// accumulated in registers (4 x 4 per thread) from shared-memory tiles of M
// and V, and reduced at once against c and the matching rows of V, so M V is
// never stored.  GB300's FP64 FMA rate (~1/64 of FP32) bounds that kernel.
// The field alone is f = (M^T c)^T V: the weights u = M^T c (K^2 flops) and
// one pass over V (K n flops, bound by HBM) give it without the K^2 n
// contraction; the sums run in another order than the nested loops, with the
// same FP64 error bound (relative to sum_i |c_i| sum_j |M_ij| |v_jk|).
// Every partial sum is kept per thread in a fixed order and reduced in a
// fixed order: results are deterministic.
#include "gst_common.cuh"

namespace gst {
namespace {

constexpr int kKT = 64;   // target points per CTA
constexpr int kIT = 64;   // rows of M per block
constexpr int kJT = 16;   // inner-dimension chunk
constexpr int kThreadsK = 256;

__global__ void __launch_bounds__(kThreadsK)
    krige_kernel(int64_t K, int64_t n, const double *__restrict__ mat,
                 const double *__restrict__ vecs, const double *__restrict__ cond,
                 double *__restrict__ field, double *__restrict__ error) {
    __shared__ double ms[kIT][kJT + 1];
    __shared__ double vs[kJT][kKT];
    __shared__ double red[2][16][kKT];
    const int tx = threadIdx.x & 15;   // columns tx + 16 c
    const int ty = threadIdx.x >> 4;   // rows ty + 16 r
    const int64_t k0 = blockIdx.x * static_cast<int64_t>(kKT);
    double f_part[4] = {0.0, 0.0, 0.0, 0.0};
    double e_part[4] = {0.0, 0.0, 0.0, 0.0};
    for (int64_t i0 = 0; i0 < K; i0 += kIT) {
        double acc[4][4] = {};
        for (int64_t j0 = 0; j0 < K; j0 += kJT) {
            // M tile: 64 rows x 16 columns; V tile: 16 rows x 64 columns
            for (int t = threadIdx.x; t < kIT * kJT; t += kThreadsK) {
                const int r = t / kJT, c = t % kJT;
                const int64_t i = i0 + r, j = j0 + c;
                ms[r][c] = (i < K && j < K) ? mat[i * K + j] : 0.0;
            }
            for (int t = threadIdx.x; t < kJT * kKT; t += kThreadsK) {
                const int r = t / kKT, c = t % kKT;
                const int64_t j = j0 + r, k = k0 + c;
                vs[r][c] = (j < K && k < n) ? vecs[j * n + k] : 0.0;
            }
            __syncthreads();
#pragma unroll
            for (int jj = 0; jj < kJT; ++jj) {
                double a[4], b[4];
#pragma unroll
                for (int r = 0; r < 4; ++r) a[r] = ms[ty + 16 * r][jj];
#pragma unroll
                for (int c = 0; c < 4; ++c) b[c] = vs[jj][tx + 16 * c];
#pragma unroll
                for (int r = 0; r < 4; ++r)
#pragma unroll
                    for (int c = 0; c < 4; ++c) acc[r][c] = fma(a[r], b[c], acc[r][c]);
            }
            __syncthreads();
        }
        // fold this block of M V against c and the matching rows of V
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int64_t i = i0 + ty + 16 * r;
            if (i >= K) continue;
            const double ci = cond[i];
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int64_t k = k0 + tx + 16 * c;
                f_part[c] = fma(ci, acc[r][c], f_part[c]);
                if (error != nullptr && k < n)
                    e_part[c] = fma(vecs[i * n + k], acc[r][c], e_part[c]);
            }
        }
    }
    // reduce over the 16 row groups in a fixed order
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        red[0][ty][tx + 16 * c] = f_part[c];
        red[1][ty][tx + 16 * c] = e_part[c];
    }
    __syncthreads();
    if (threadIdx.x < kKT) {
        const int col = threadIdx.x;
        const int64_t k = k0 + col;
        if (k < n) {
            double f = 0.0, e = 0.0;
            for (int g = 0; g < 16; ++g) {
                f += red[0][g][col];
                e += red[1][g][col];
            }
            field[k] = f;
            if (error != nullptr) error[k] = e;
        }
    }
}

// out_k = sum_j u_j A_jk for a row-major K x n matrix A: thread (g, c) of a
// CTA sums the rows j = g (mod GROUPS) of column k0 + c (COLS contiguous
// doubles per warp and row, four loads in flight), then the GROUPS partial
// sums are added in group order.  Used twice: u = M^T c (A = M, many row
// groups for the few columns) and f = V^T u (A = V).
template <int COLS, int GROUPS>
__global__ void __launch_bounds__(COLS * GROUPS)
    krige_colsum_kernel(int64_t K, int64_t n, const double *__restrict__ u,
                        const double *__restrict__ a, double *__restrict__ out) {
    __shared__ double part[GROUPS][COLS];
    const int c = threadIdx.x % COLS;
    const int g = threadIdx.x / COLS;
    const int64_t k = blockIdx.x * static_cast<int64_t>(COLS) + c;
    double acc = 0.0;
    if (k < n) {
        int64_t j = g;
        for (; j + 3 * GROUPS < K; j += 4 * GROUPS) {
            const double v0 = a[j * n + k];
            const double v1 = a[(j + GROUPS) * n + k];
            const double v2 = a[(j + 2 * GROUPS) * n + k];
            const double v3 = a[(j + 3 * GROUPS) * n + k];
            acc = fma(u[j], v0, acc);
            acc = fma(u[j + GROUPS], v1, acc);
            acc = fma(u[j + 2 * GROUPS], v2, acc);
            acc = fma(u[j + 3 * GROUPS], v3, acc);
        }
        for (; j < K; j += GROUPS) acc = fma(u[j], a[j * n + k], acc);
    }
    part[g][c] = acc;
    __syncthreads();
    if (g == 0 && k < n) {
        double f = part[0][c];
#pragma unroll
        for (int q = 1; q < GROUPS; ++q) f += part[q][c];
        out[k] = f;
    }
}

template <int COLS, int GROUPS>
cudaError_t launch_colsum(int64_t K, int64_t n, const double *u, const double *a,
                          double *out, cudaStream_t s) {
    const int64_t blocks = ceil_div(n, COLS);
    if (blocks > 0x7fffffffLL) return cudaErrorInvalidConfiguration;
    krige_colsum_kernel<COLS, GROUPS>
        <<<static_cast<unsigned>(blocks), COLS * GROUPS, 0, s>>>(K, n, u, a, out);
    return cudaGetLastError();
}

}  // namespace
}  // namespace gst

extern "C" {

int gst_calc_field_krige(int64_t n_cond, int64_t n_pts, const double *krig_mat,
                         const double *krig_vecs, const double *cond, double *field,
                         double *error, void *stream) {
    if (n_cond < 0 || n_pts < 0) return GST_ERR_INVALID_ARGUMENT;
    if (n_pts == 0) return GST_OK;
    if (field == nullptr) return GST_ERR_INVALID_ARGUMENT;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    if (n_cond == 0) {
        GST_TRY_CUDA(cudaMemsetAsync(field, 0, sizeof(double) * n_pts, s));
        if (error != nullptr)
            GST_TRY_CUDA(cudaMemsetAsync(error, 0, sizeof(double) * n_pts, s));
        return GST_OK;
    }
    if (krig_mat == nullptr || krig_vecs == nullptr || cond == nullptr)
        return GST_ERR_INVALID_ARGUMENT;
    if (error == nullptr) {
        // field only: u = M^T c, then f = V^T u
        if (gst::ceil_div(n_pts, 64) > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
        gst::StreamScratch u;
        GST_TRY_CUDA(u.alloc(sizeof(double) * n_cond, s));
        double *du = static_cast<double *>(u.ptr);
        GST_TRY_CUDA((gst::launch_colsum<32, 32>(n_cond, n_cond, cond, krig_mat, du, s)));
        GST_TRY_CUDA((gst::launch_colsum<64, 4>(n_cond, n_pts, du, krig_vecs, field, s)));
        return GST_OK;
    }
    const int64_t blocks = gst::ceil_div(n_pts, gst::kKT);
    if (blocks > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    gst::krige_kernel<<<static_cast<unsigned>(blocks), gst::kThreadsK, 0, s>>>(
        n_cond, n_pts, krig_mat, krig_vecs, cond, field, error);
    GST_TRY_CUDA(cudaGetLastError());
    return GST_OK;
}

}  // extern "C"
