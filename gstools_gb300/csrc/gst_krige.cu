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
#include <cublas_v2.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <climits>
#include <mutex>
#include <utility>
#include <vector>

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

// ------------------------------------------------- FP64 by error-free slices --
//
// The quadratic forms e_k = sum_i v_ik (M v_k)_i need W = M V, a K x K by
// K x n FP64 product -- on GB300, whose FP64 rate is ~1/64 of FP32, the
// bulk of the kriging time.  It runs on the FP16 tensor cores instead by
// error-free slicing (the Ozaki scheme): every row i of M is scaled by 2^-a_i
// (a_i: its largest magnitude's exponent) and every column k of V by 2^-b_k,
// and each scaled value x in (-1, 1) is cut into S integer slices of
// kBeta bits, x = sum_s q_s 2^(-kBeta s) + (a remainder of at most
// 2^(-kBeta S - 1)): the balanced base-2^kBeta digits of rint(x 2^(kBeta S))
// (slice_digits); |q_1| <= 2^kBeta, |q_s| <= 2^(kBeta-1) after, all exact in
// FP16.  A product of two slices is at most 2^(2 kBeta) = 2^12, so a sum
// of up to 2^24 / 2^12 = 4096 of them is an integer below 2^24 and an FP16
// GEMM with FP32 accumulation computes slice products exactly, whatever
// order its tensor cores add in.  With
//
//     W_ik = 2^(a_i + b_k) sum_{s+t <= S+1} 2^(-kBeta (s+t)) (Q^M_s Q^V_t)_ik
//
// (the pairs with s + t > S + 1 lie below FP64 resolution), the slice pairs of
// one level L = s + t share a scale and are contracted together as one GEMM
// over the concatenated inner dimension (as many pairs as keep the bound
// K sum |q_s| |q_t| <= 2^24: all of a level for K ~ 1000), and each GEMM's
// exact FP32 result P is folded straight into
//
//     e_k = 2^b_k sum_L 2^(-kBeta L) sum_i (v_ik 2^a_i) P_ik
//
// in FP64 (fixed order: deterministic).  The products are plain GEMMs, run
// by cuBLAS; slicing and folding are the kernels below.

constexpr int kBeta = 6;      // bits per slice
constexpr int kSlices = 9;    // kBeta (kSlices + 1) = 60 bits
constexpr int64_t kOzakiMaxInner = (int64_t(1) << 24) >> (2 * kBeta);   // 4096

// Largest magnitude of slice s: 2^kBeta for the leading digit, 2^(kBeta-1)
// for the balanced digits after it (slice_digits).
constexpr int64_t slice_bound(int s) { return s == 1 ? (1 << kBeta) : (1 << (kBeta - 1)); }
// Lowest level accumulated in FP32 (see krige_variance_ozaki).
constexpr int kChainLevel = 7;
static_assert(24 + kBeta * (kChainLevel - 2) >= 53, "FP32 chain above FP64 resolution");

// Exponent a with |x| < 2^a for the largest |x| of row i (one warp per
// row) and the scale 2^a; a non-finite value sets *bad.
__global__ void row_exponent_kernel(int64_t K, const double *__restrict__ m, int *expo,
                                    double *scale, unsigned int *bad) {
    const int64_t i = (blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= K) return;
    double mx = 0.0;
    bool finite = true;
    for (int64_t j = lane; j < K; j += 32) {
        const double v = m[i * K + j];
        finite = finite && isfinite(v);
        mx = fmax(mx, fabs(v));
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (!__all_sync(0xffffffffu, finite) && lane == 0) atomicOr(bad, 1u);
    if (lane == 0) {
        int e = 0;
        if (mx > 0.0 && mx < INFINITY) frexp(mx, &e);
        expo[i] = e;
        scale[i] = ldexp(1.0, e);
    }
}

// Same per column k of the row-major K x n matrix v; a column holding a
// non-finite value gets the marker exponent INT_MIN.  Also writes v scaled
// by M's row scales, vs_jk = v_jk 2^a_j, the weights of the fold below.
// 32 columns per CTA, 8 groups of rows (i = g mod 8) per column, maxima
// and finiteness combined through shared memory.
__global__ void __launch_bounds__(256)
    col_exponent_kernel(int64_t K, int64_t n, const double *__restrict__ v,
                        const double *__restrict__ row_scale, int *expo,
                        double *__restrict__ vs) {
    __shared__ double s_mx[8][32];
    __shared__ int s_fin[8][32];
    const int c = threadIdx.x & 31, g = threadIdx.x >> 5;
    const int64_t k = blockIdx.x * static_cast<int64_t>(32) + c;
    double mx = 0.0;
    bool finite = true;
    if (k < n)
        for (int64_t j = g; j < K; j += 8) {
            const double x = v[j * n + k];
            finite = finite && isfinite(x);
            mx = fmax(mx, fabs(x));
            vs[j * n + k] = x * row_scale[j];
        }
    s_mx[g][c] = mx;
    s_fin[g][c] = finite ? 1 : 0;
    __syncthreads();
    if (g == 0 && k < n) {
        for (int q = 1; q < 8; ++q) {
            mx = fmax(mx, s_mx[q][c]);
            finite = finite && s_fin[q][c];
        }
        int e = 0;
        if (mx > 0.0 && finite) frexp(mx, &e);
        expo[k] = finite ? e : INT_MIN;
    }
}

// The slices of x 2^-e (|x| < 2^e): X = rint(x 2^(kBeta S - e)), an integer
// below 2^(kBeta S) (the rounding is below the slices' resolution), cut into
// balanced base-2^kBeta digits from the least significant one, d in
// [-2^(kBeta-1), 2^(kBeta-1)), so X = sum_s q_s 2^(kBeta (S - s)) with |q_1|
// <= 2^kBeta and |q_s| <= 2^(kBeta-1) after -- integer work instead of S
// FP64 multiply-round-subtract steps.  q[s - 1] receives slice s.
__device__ __forceinline__ void slice_digits(double x, int e, __half (&q)[kSlices]) {
    long long X = isfinite(x) ? __double2ll_rn(ldexp(x, kBeta * kSlices - e)) : 0;
    constexpr long long kHalf = 1LL << (kBeta - 1), kMask = (1LL << kBeta) - 1;
#pragma unroll
    for (int s = kSlices - 1; s >= 1; --s) {
        const long long d = ((X + kHalf) & kMask) - kHalf;
        q[s] = __int2half_rn(static_cast<int>(d));
        X = (X - d) >> kBeta;
    }
    q[0] = __int2half_rn(static_cast<int>(X));
}

// Slices of M: element (i, j) to slot (s - 1) Kp + j of row i of the
// K x (S Kp) array qm (slice s = 1..S side by side, each padded with zeros
// from K to Kp columns: the tensor-core GEMMs want 16-byte aligned blocks).
__global__ void slice_rows_kernel(int64_t K, int64_t Kp, const double *__restrict__ m,
                                  const int *__restrict__ expo, __half *qm) {
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= K * K) return;
    const int64_t i = t / K, j = t % K;
    __half q[kSlices];
    slice_digits(m[t], expo[i], q);
    __half *row = qm + i * (kSlices * Kp) + j;
#pragma unroll
    for (int s = 0; s < kSlices; ++s) row[s * Kp] = q[s];
}

// Slices of V: element (j, k) of slice t = 1..S to row (S - t) Kp + j,
// column k of the (S Kp) x np array qv (slices in decreasing t, so that the
// partners of the increasing slices 1, 2, ... of M at a level are
// consecutive rows; rows K..Kp-1 of a slice and columns n..np-1 stay zero).
__global__ void slice_cols_kernel(int64_t K, int64_t Kp, int64_t n, int64_t np,
                                  const double *__restrict__ v,
                                  const int *__restrict__ expo, __half *qv) {
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= K * n) return;
    const int64_t j = t / n, k = t % n;
    const int e = expo[k];
    __half q[kSlices];
    slice_digits(e != INT_MIN ? v[t] : 0.0, e, q);
#pragma unroll
    for (int s = 1; s <= kSlices; ++s) qv[((kSlices - s) * Kp + j) * np + k] = q[s - 1];
}

// d_k (+)= scale sum_i vs_ik P_ik (vs_ik = v_ik 2^a_i) for the row-major K x n FP32 result
// P of one GEMM: thread (g, c) sums the rows i = g (mod GROUPS) of column
// k0 + c, the GROUPS partial sums are added in group order (deterministic).
template <int COLS, int GROUPS>
__global__ void __launch_bounds__(COLS * GROUPS)
    fold_kernel(int64_t K, int64_t n, int64_t np, const double *__restrict__ vs,
                const float *__restrict__ p, double scale, int first,
                double *__restrict__ d) {
    __shared__ double part[GROUPS][COLS];
    const int c = threadIdx.x % COLS;
    const int g = threadIdx.x / COLS;
    const int64_t k = blockIdx.x * static_cast<int64_t>(COLS) + c;
    double acc = 0.0;
    if (k < n)
        for (int64_t i = g; i < K; i += GROUPS)
            acc = fma(vs[i * n + k], static_cast<double>(p[i * np + k]), acc);
    part[g][c] = acc;
    __syncthreads();
    if (g == 0 && k < n) {
        double f = part[0][c];
#pragma unroll
        for (int q = 1; q < GROUPS; ++q) f += part[q][c];
        d[k] = first ? scale * f : fma(scale, f, d[k]);
    }
}

// e_k = 2^b_k d_k; NaN where V's column or M held a non-finite value.
__global__ void ozaki_finish_kernel(int64_t n, const double *__restrict__ d,
                                    const int *__restrict__ col_expo,
                                    const unsigned int *__restrict__ bad, double *e) {
    const int64_t k = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (k >= n) return;
    const int b = col_expo[k];
    e[k] = (*bad != 0u || b == INT_MIN) ? NAN : ldexp(d[k], b);
}

// One cuBLAS handle and one side stream (the folds run there, beside the
// next GEMM) per device, created on first use.
std::mutex g_blas_mutex;
cublasHandle_t g_blas[64];
cudaStream_t g_fold_stream[64];

int blas_handle(cublasHandle_t *h, cudaStream_t *side) {
    const int dev = current_device();
    if (dev < 0 || dev >= 64) return GST_ERR_NO_DEVICE;
    if (g_blas[dev] == nullptr) {
        if (cublasCreate(&g_blas[dev]) != CUBLAS_STATUS_SUCCESS) return GST_ERR_CUDA;
    }
    if (g_fold_stream[dev] == nullptr)
        GST_TRY_CUDA(cudaStreamCreateWithFlags(&g_fold_stream[dev], cudaStreamNonBlocking));
    *h = g_blas[dev];
    *side = g_fold_stream[dev];
    return GST_OK;
}

// Events of one variance call (destroyed when it has issued its work).
struct FoldEvents {
    cudaEvent_t ev[5] = {};
    cudaError_t create() {
        for (auto &e : ev) {
            const cudaError_t r = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
            if (r != cudaSuccess) return r;
        }
        return cudaSuccess;
    }
    ~FoldEvents() {
        for (auto e : ev)
            if (e) cudaEventDestroy(e);
    }
};

// When the variance runs through the slices: the inner dimension fits one
// slice pair per GEMM, and the product is large enough for the fixed costs
// (slicing passes, ~15 GEMMs) to pay off.
bool use_ozaki(int64_t K, int64_t n) {
    return K >= 64 && static_cast<int64_t>(align_up(static_cast<size_t>(K), 8)) <= kOzakiMaxInner &&
           static_cast<double>(K) * static_cast<double>(K) * static_cast<double>(n) >= 4e9;
}

int krige_variance_ozaki(int64_t K, int64_t n, const double *mat, const double *vecs,
                         double *error, cudaStream_t s) {
    const int64_t Kp = align_up(static_cast<size_t>(K), 8);
    const int64_t np = align_up(static_cast<size_t>(n), 8);

    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = align_up(off + bytes, 256);
        return o;
    };
    const size_t o_qm = take(sizeof(__half) * kSlices * Kp * K);
    const size_t o_qv = take(sizeof(__half) * kSlices * Kp * np);
    const size_t o_p = take(sizeof(float) * K * np * 2);   // two GEMM results in turn
    const size_t o_re = take(sizeof(int) * K);
    const size_t o_ce = take(sizeof(int) * n);
    const size_t o_d = take(sizeof(double) * n);
    const size_t o_rs = take(sizeof(double) * K);
    const size_t o_vs = take(sizeof(double) * K * n);
    const size_t o_bad = take(sizeof(unsigned int));
    StreamScratch ws;
    GST_TRY_CUDA(ws.alloc(off, s));
    unsigned char *base = static_cast<unsigned char *>(ws.ptr);
    __half *qm = reinterpret_cast<__half *>(base + o_qm);
    __half *qv = reinterpret_cast<__half *>(base + o_qv);
    float *p = reinterpret_cast<float *>(base + o_p);
    int *re = reinterpret_cast<int *>(base + o_re);
    int *ce = reinterpret_cast<int *>(base + o_ce);
    double *d = reinterpret_cast<double *>(base + o_d);
    double *rs = reinterpret_cast<double *>(base + o_rs);
    double *vsc = reinterpret_cast<double *>(base + o_vs);
    unsigned int *bad = reinterpret_cast<unsigned int *>(base + o_bad);

    GST_TRY_CUDA(cudaMemsetAsync(bad, 0, sizeof(unsigned int), s));
    if (Kp != K || np != n) {   // the padding rows and columns stay zero
        GST_TRY_CUDA(cudaMemsetAsync(qm, 0, sizeof(__half) * kSlices * Kp * K, s));
        GST_TRY_CUDA(cudaMemsetAsync(qv, 0, sizeof(__half) * kSlices * Kp * np, s));
    }
    row_exponent_kernel<<<static_cast<unsigned>(ceil_div(K * 32, 256)), 256, 0, s>>>(
        K, mat, re, rs, bad);
    col_exponent_kernel<<<static_cast<unsigned>(ceil_div(n, 32)), 256, 0, s>>>(K, n, vecs,
                                                                               rs, ce, vsc);
    slice_rows_kernel<<<static_cast<unsigned>(ceil_div(K * K, 256)), 256, 0, s>>>(K, Kp, mat,
                                                                                  re, qm);
    slice_cols_kernel<<<static_cast<unsigned>(ceil_div(K * n, 256)), 256, 0, s>>>(
        K, Kp, n, np, vecs, ce, qv);
    GST_TRY_CUDA(cudaGetLastError());

    cublasHandle_t h = nullptr;
    cudaStream_t side = nullptr;
    std::lock_guard<std::mutex> lock(g_blas_mutex);
    int rc = blas_handle(&h, &side);
    if (rc) return rc;
    if (cublasSetStream(h, s) != CUBLAS_STATUS_SUCCESS) return GST_ERR_CUDA;
    // GEMM g writes result buffer g & 1 on s; its fold reads it on `side`
    // (in order: the FP64 sums are deterministic) while GEMM g + 1 runs;
    // GEMM g + 2 waits for that fold.  ev: [0, 1] GEMM done, [2, 3] fold
    // done, [4] inputs ready.
    FoldEvents fe;
    GST_TRY_CUDA(fe.create());
    GST_TRY_CUDA(cudaEventRecord(fe.ev[4], s));
    GST_TRY_CUDA(cudaStreamWaitEvent(side, fe.ev[4], 0));
    const float one = 1.0f;
    bool first = true;
    int gi = 0;           // GEMMs issued
    int last_fold = -1;   // buffer of the last fold queued
    // on a failure after folds were queued, s still waits for them: the
    // scratch they use is released on s
    auto bail = [&](int code) {
        if (last_fold >= 0) cudaStreamWaitEvent(s, fe.ev[2 + last_fold], 0);
        return code;
    };
    // The GEMM groups of level L: as many pairs as keep every sum an integer
    // below 2^24 (Kp sum_pairs |q_s| |q_t| <= 2^24).
    auto groups_of = [&](int L) {
        std::vector<std::pair<int, int>> g;
        const int s_lo = std::max(1, L - kSlices), s_hi = std::min(kSlices, L - 1);
        for (int s1 = s_lo, s2; s1 <= s_hi; s1 = s2 + 1) {
            int64_t bound = slice_bound(s1) * slice_bound(L - s1);
            s2 = s1;
            while (s2 + 1 <= s_hi &&
                   Kp * (bound + slice_bound(s2 + 1) * slice_bound(L - s2 - 1)) <=
                       (int64_t(1) << 24)) {
                ++s2;
                bound += slice_bound(s2) * slice_bound(L - s2);
            }
            g.emplace_back(s1, s2);
        }
        return g;
    };
    bool pending[2] = {false, false};   // a fold still reads this buffer
    // P[buf] = QM[:, s1..s2 blocks] QV[rows of t = L - s1 .. L - s2]
    // (+ beta P[buf]); row-major, so cuBLAS sees the column-major
    // transposes: P^T = QV^T QM^T
    auto gemm = [&](int L, int s1, int s2, float beta, int buf) -> int {
        const int64_t inner = static_cast<int64_t>(s2 - s1 + 1) * Kp;
        const __half *a = qv + static_cast<int64_t>(kSlices - L + s1) * Kp * np;
        const __half *b = qm + static_cast<int64_t>(s1 - 1) * Kp;
        float *pb = p + static_cast<int64_t>(buf) * K * np;
        if (pending[buf] && cudaStreamWaitEvent(s, fe.ev[2 + buf], 0) != cudaSuccess)
            return GST_ERR_CUDA;
        pending[buf] = false;
        if (cublasGemmEx(h, CUBLAS_OP_N, CUBLAS_OP_N, static_cast<int>(np),
                         static_cast<int>(K), static_cast<int>(inner), &one, a,
                         CUDA_R_16F, static_cast<int>(np), b, CUDA_R_16F,
                         static_cast<int>(kSlices * Kp), &beta, pb, CUDA_R_32F,
                         static_cast<int>(np), CUBLAS_COMPUTE_32F,
                         CUBLAS_GEMM_DEFAULT) != CUBLAS_STATUS_SUCCESS)
            return GST_ERR_CUDA;
        ++gi;
        return GST_OK;
    };
    // d (+)= 2^(-kBeta L) sum_i vs_ik P[buf]_ik on `side`, after the GEMMs
    auto fold = [&](int L, int buf) -> int {
        if (cudaEventRecord(fe.ev[buf], s) != cudaSuccess ||
            cudaStreamWaitEvent(side, fe.ev[buf], 0) != cudaSuccess)
            return GST_ERR_CUDA;
        fold_kernel<64, 4><<<static_cast<unsigned>(ceil_div(n, 64)), 256, 0, side>>>(
            K, n, np, vsc, p + static_cast<int64_t>(buf) * K * np, ldexp(1.0, -kBeta * L),
            first ? 1 : 0, d);
        if (cudaGetLastError() != cudaSuccess ||
            cudaEventRecord(fe.ev[2 + buf], side) != cudaSuccess)
            return GST_ERR_CUDA;
        pending[buf] = true;
        last_fold = buf;
        first = false;
        return GST_OK;
    };
    // Levels kChainLevel..S+1 accumulate in FP32, each new level scaling the
    // sum so far by 2^-kBeta (beta of the GEMM): the rounding, at most
    // 2^-24 of a level-kChainLevel term, lies below FP64 resolution
    // relative to the leading level 2 (2^-24 2^(-kBeta (kChainLevel - 2))
    // <= 2^-53); one fold takes them all.  The levels below are exact
    // integer GEMMs, one fold each.
    bool started = false;
    for (int L = kSlices + 1; L >= kChainLevel; --L) {
        bool level_first = true;
        for (const auto &g : groups_of(L)) {
            const float beta = !started ? 0.0f : (level_first ? 1.0f / (1 << kBeta) : 1.0f);
            if (gemm(L, g.first, g.second, beta, 0)) return bail(GST_ERR_CUDA);
            started = true;
            level_first = false;
        }
    }
    if (started && fold(kChainLevel, 0)) return bail(GST_ERR_CUDA);
    int buf = 1;
    for (int L = kChainLevel - 1; L >= 2; --L)
        for (const auto &g : groups_of(L)) {
            if (gemm(L, g.first, g.second, 0.0f, buf) || fold(L, buf))
                return bail(GST_ERR_CUDA);
            buf ^= 1;
        }
    // every fold done (they run in order on `side`) before the result and
    // before the scratch is released on s
    if (last_fold >= 0) GST_TRY_CUDA(cudaStreamWaitEvent(s, fe.ev[2 + last_fold], 0));
    ozaki_finish_kernel<<<static_cast<unsigned>(ceil_div(n, 256)), 256, 0, s>>>(n, d, ce,
                                                                                bad, error);
    GST_TRY_CUDA(cudaGetLastError());
    return GST_OK;
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
    if (gst::use_ozaki(n_cond, n_pts) && n_pts <= 0x7fffffffLL) {
        // field as above, the variance through FP16 slice products
        gst::StreamScratch u;
        GST_TRY_CUDA(u.alloc(sizeof(double) * n_cond, s));
        double *du = static_cast<double *>(u.ptr);
        GST_TRY_CUDA((gst::launch_colsum<32, 32>(n_cond, n_cond, cond, krig_mat, du, s)));
        GST_TRY_CUDA((gst::launch_colsum<64, 4>(n_cond, n_pts, du, krig_vecs, field, s)));
        return gst::krige_variance_ozaki(n_cond, n_pts, krig_mat, krig_vecs, error, s);
    }
    const int64_t blocks = gst::ceil_div(n_pts, gst::kKT);
    if (blocks > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    gst::krige_kernel<<<static_cast<unsigned>(blocks), gst::kThreadsK, 0, s>>>(
        n_cond, n_pts, krig_mat, krig_vecs, cond, field, error);
    GST_TRY_CUDA(cudaGetLastError());
    return GST_OK;
}

}  // extern "C"
