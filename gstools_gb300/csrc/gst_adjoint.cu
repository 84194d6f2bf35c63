// Adjoint (vector-Jacobian product) of the randomization-method sum with
// respect to the modes.
//
// Forward (src/gstools/field/generator.py:193-199):
//     u_i = sum_j z1_j cos(phi_ij) + z2_j sin(phi_ij),   phi_ij = <k_j, x_i>
// Given g_i = dL/du_i:
//     dL/dz1_j   = sum_i g_i cos(phi_ij)
//     dL/dz2_j   = sum_i g_i sin(phi_ij)
//     dL/dk_jd   = z2_j sum_i g_i x_id cos(phi_ij) - z1_j sum_i g_i x_id sin(phi_ij)
// (dL/dx is the pointwise kind kGradPos in gst_pointwise.cu.)
//
// The sums run over points for every mode -- the transpose of the forward
// reduction.  A CTA keeps 512 modes in registers (2 per thread) and streams a
// slice of the points through shared memory in chunks of 256; sin/cos are
// recomputed from the phase instead of stored.  Point slices are spread over
// blockIdx.y and the FP64 partial sums are added in slice order by a second
// kernel, which also forms dL/dk.  FP64 (parity) and mixed precision (the
// turn reduction of gst_mixed.cuh, SFU sin/cos, FP32 sums per chunk, FP64
// across chunks) variants.
#include <algorithm>

#include "gst_common.cuh"
#include "gst_mixed.cuh"

namespace gst {
namespace {

constexpr int kThreads = 256;
constexpr int kModesPerThread = 2;
constexpr int kModesPerCta = kThreads * kModesPerThread;
constexpr int kChunk = 256;

enum Prec { kF64 = 0, kMixed = 1 };

struct VjpArgs {
    int64_t n_modes, n_pts;
    const double *cov, *pos, *g;
    int64_t pts_per_split;
    double *partial;  // [split][n_modes][2 + 2 dim]
};

template <int DIM, int PREC>
__global__ void __launch_bounds__(kThreads) vjp_modes_kernel(const VjpArgs a) {
    constexpr int NA = 2 + 2 * DIM;  // C, S, Cx[d], Sx[d]
    __shared__ double s_x[DIM][kChunk];
    __shared__ double s_g[kChunk];
    __shared__ float s_xh[DIM][kChunk], s_xl[DIM][kChunk], s_xf[DIM][kChunk];
    __shared__ float s_gf[kChunk];

    const int tid = threadIdx.x;
    int64_t mode[kModesPerThread];
    double k[kModesPerThread][DIM];
    float qh[kModesPerThread][3], ql[kModesPerThread][3];
#pragma unroll
    for (int m = 0; m < kModesPerThread; ++m) {
        mode[m] = static_cast<int64_t>(blockIdx.x) * kModesPerCta + m * kThreads + tid;
#pragma unroll
        for (int d = 0; d < DIM; ++d)
            k[m][d] = mode[m] < a.n_modes ? a.cov[d * a.n_modes + mode[m]] : 0.0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            constexpr double kInv2Pi = 0.15915494309189533576888376337251436;
            const double q = d < DIM ? k[m][d] * kInv2Pi : 0.0;
            qh[m][d] = split_hi12(q);
            ql[m][d] = static_cast<float>(q - static_cast<double>(qh[m][d]));
        }
    }
    double acc[kModesPerThread][NA];
#pragma unroll
    for (int m = 0; m < kModesPerThread; ++m)
#pragma unroll
        for (int c = 0; c < NA; ++c) acc[m][c] = 0.0;

    const int64_t p_begin = static_cast<int64_t>(blockIdx.y) * a.pts_per_split;
    const int64_t p_end = min(p_begin + a.pts_per_split, a.n_pts);
    // mixed: positions relative to the first point (the finish kernel
    // rotates the sums back, gst_mixed.cuh)
    double x0[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) x0[d] = PREC == kMixed ? origin_coord(a.pos + d * a.n_pts) : 0.0;
    for (int64_t c0 = p_begin; c0 < p_end; c0 += kChunk) {
        const int64_t i = c0 + tid;
        const bool in = i < p_end;
        double xv[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) xv[d] = in ? a.pos[d * a.n_pts + i] - x0[d] : 0.0;
        const double gv = in ? a.g[i] : 0.0;  // g = 0 pads the chunk
        if (PREC == kF64) {
#pragma unroll
            for (int d = 0; d < DIM; ++d) s_x[d][tid] = xv[d];
            s_g[tid] = gv;
        } else {
            const MixedPoint<DIM> mp = mixed_split_point<DIM>(xv);
#pragma unroll
            for (int d = 0; d < DIM; ++d) {
                s_xh[d][tid] = mp.xh[d];
                s_xl[d][tid] = mp.xl[d];
                s_xf[d][tid] = mp.xf[d];
            }
            s_gf[tid] = static_cast<float>(gv);
        }
        __syncthreads();
        const int n = static_cast<int>(min(static_cast<int64_t>(kChunk), p_end - c0));
        if (PREC == kF64) {
            for (int p = 0; p < n; ++p) {
                const double gp = s_g[p];
                double xp[DIM];
#pragma unroll
                for (int d = 0; d < DIM; ++d) xp[d] = s_x[d][p];
#pragma unroll
                for (int m = 0; m < kModesPerThread; ++m) {
                    double ph = k[m][0] * xp[0];
#pragma unroll
                    for (int d = 1; d < DIM; ++d) ph = fma(k[m][d], xp[d], ph);
                    double sn, cs;
                    sincos(ph, &sn, &cs);
                    const double gc = gp * cs, gs = gp * sn;
                    acc[m][0] += gc;
                    acc[m][1] += gs;
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        acc[m][2 + d] = fma(gc, xp[d], acc[m][2 + d]);
                        acc[m][2 + DIM + d] = fma(gs, xp[d], acc[m][2 + DIM + d]);
                    }
                }
            }
        } else {
            float af[kModesPerThread][NA];
#pragma unroll
            for (int m = 0; m < kModesPerThread; ++m)
#pragma unroll
                for (int c = 0; c < NA; ++c) af[m][c] = 0.0f;
            for (int p = 0; p < n; ++p) {
                MixedPoint<DIM> mp;
#pragma unroll
                for (int d = 0; d < DIM; ++d) {
                    mp.xh[d] = s_xh[d][p];
                    mp.xl[d] = s_xl[d][p];
                    mp.xf[d] = s_xf[d][p];
                }
                const float gp = s_gf[p];
#pragma unroll
                for (int m = 0; m < kModesPerThread; ++m) {
                    float sn, cs;
                    mixed_sincos<DIM>(qh[m], ql[m], mp, &sn, &cs);
                    const float gc = gp * cs, gs = gp * sn;
                    af[m][0] += gc;
                    af[m][1] += gs;
#pragma unroll
                    for (int d = 0; d < DIM; ++d) {
                        af[m][2 + d] = fmaf(gc, mp.xf[d], af[m][2 + d]);
                        af[m][2 + DIM + d] = fmaf(gs, mp.xf[d], af[m][2 + DIM + d]);
                    }
                }
            }
#pragma unroll
            for (int m = 0; m < kModesPerThread; ++m)
#pragma unroll
                for (int c = 0; c < NA; ++c) acc[m][c] += static_cast<double>(af[m][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int m = 0; m < kModesPerThread; ++m) {
        if (mode[m] >= a.n_modes) continue;
        double *dst = a.partial + (static_cast<int64_t>(blockIdx.y) * a.n_modes + mode[m]) * NA;
#pragma unroll
        for (int c = 0; c < NA; ++c) dst[c] = acc[m][c];
    }
}

// Sums the slices in order and forms the gradients.  With `shifted` (mixed
// path) the sums ran over phases <k, x - x0> and positions x - x0, x0 the
// first point; with a = <k, x0>:
//   C  = cos(a) C' - sin(a) S',     S  = sin(a) C' + cos(a) S',
//   Cx = x0 C + cos(a) C'x - sin(a) S'x,   Sx = x0 S + sin(a) C'x + cos(a) S'x.
__global__ void vjp_modes_finish_kernel(int dim, int64_t n_modes, int64_t n_split,
                                        const double *__restrict__ partial,
                                        const double *__restrict__ z1,
                                        const double *__restrict__ z2,
                                        const double *__restrict__ cov,
                                        const double *__restrict__ pos, int64_t n_pts,
                                        int shifted, double *grad_z1, double *grad_z2,
                                        double *grad_cov) {
    const int64_t j = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (j >= n_modes) return;
    const int na = 2 + 2 * dim;
    double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int64_t k = 0; k < n_split; ++k) {
        const double *src = partial + (k * n_modes + j) * na;
        for (int c = 0; c < na; ++c) s[c] += src[c];
    }
    if (shifted) {
        double k[4] = {0.0, 0.0, 0.0, 0.0}, x0[3] = {0.0, 0.0, 0.0};
        for (int d = 0; d < dim; ++d) {
            k[d] = cov[d * n_modes + j];
            x0[d] = origin_coord(pos + d * n_pts);
        }
        double ca = 1.0, sa = 0.0;   // (cos a, sin a) from rotating (1, 0)
        double one = 1.0, zero = 0.0;
        rotate_to_origin(k, dim, x0, one, zero);   // (cos a, -sin a)
        ca = one;
        sa = -zero;
        const double c = ca * s[0] - sa * s[1];
        const double sn = sa * s[0] + ca * s[1];
        double t[8];
        for (int d = 0; d < dim; ++d) {
            t[2 + d] = x0[d] * c + ca * s[2 + d] - sa * s[2 + dim + d];
            t[2 + dim + d] = x0[d] * sn + sa * s[2 + d] + ca * s[2 + dim + d];
        }
        s[0] = c;
        s[1] = sn;
        for (int d = 0; d < dim; ++d) {
            s[2 + d] = t[2 + d];
            s[2 + dim + d] = t[2 + dim + d];
        }
    }
    if (grad_z1) grad_z1[j] = s[0];
    if (grad_z2) grad_z2[j] = s[1];
    if (grad_cov)
        for (int d = 0; d < dim; ++d)
            grad_cov[d * n_modes + j] = z2[j] * s[2 + d] - z1[j] * s[2 + dim + d];
}

template <int PREC>
cudaError_t launch_vjp(int dim, dim3 grid, const VjpArgs &args, cudaStream_t s) {
    switch (dim) {
        case 1: vjp_modes_kernel<1, PREC><<<grid, kThreads, 0, s>>>(args); break;
        case 2: vjp_modes_kernel<2, PREC><<<grid, kThreads, 0, s>>>(args); break;
        case 3: vjp_modes_kernel<3, PREC><<<grid, kThreads, 0, s>>>(args); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

int run_vjp_modes(int prec, int dim, int64_t n_modes, int64_t n_pts,
                  const double *cov, const double *z1, const double *z2,
                  const double *pos, const double *g, double *grad_z1,
                  double *grad_z2, double *grad_cov, cudaStream_t s) {
    if (dim < 1 || dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    if (n_modes < 0 || n_pts < 0) return GST_ERR_INVALID_ARGUMENT;
    if (n_modes == 0) return GST_OK;
    if (cov == nullptr || z1 == nullptr || z2 == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (current_device() < 0) return GST_ERR_NO_DEVICE;
    if (n_pts == 0) {
        if (grad_z1) GST_TRY_CUDA(cudaMemsetAsync(grad_z1, 0, 8 * n_modes, s));
        if (grad_z2) GST_TRY_CUDA(cudaMemsetAsync(grad_z2, 0, 8 * n_modes, s));
        if (grad_cov) GST_TRY_CUDA(cudaMemsetAsync(grad_cov, 0, 8 * n_modes * dim, s));
        return GST_OK;
    }
    if (pos == nullptr || g == nullptr) return GST_ERR_INVALID_ARGUMENT;
    const int64_t mode_blocks = ceil_div(n_modes, kModesPerCta);
    if (mode_blocks > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    // slices of points: about four CTAs per SM, each slice >= one chunk
    const int64_t target = static_cast<int64_t>(sm_count()) * 4;
    int64_t n_split = std::max<int64_t>(1, ceil_div(target, mode_blocks));
    n_split = std::min<int64_t>(n_split, ceil_div(n_pts, kChunk));
    n_split = std::min<int64_t>(n_split, 65535);
    const int64_t per = ceil_div(ceil_div(n_pts, n_split), kChunk) * kChunk;
    n_split = ceil_div(n_pts, per);
    const int na = 2 + 2 * dim;

    StreamScratch ws;
    GST_TRY_CUDA(ws.alloc(sizeof(double) * n_split * n_modes * na, s));
    VjpArgs args{n_modes, n_pts, cov, pos, g, per, static_cast<double *>(ws.ptr)};
    const dim3 grid(static_cast<unsigned>(mode_blocks), static_cast<unsigned>(n_split));
    GST_TRY_CUDA(prec == kF64 ? launch_vjp<kF64>(dim, grid, args, s)
                              : launch_vjp<kMixed>(dim, grid, args, s));
    vjp_modes_finish_kernel<<<static_cast<unsigned>(ceil_div(n_modes, 256)), 256, 0, s>>>(
        dim, n_modes, n_split, args.partial, z1, z2, cov, pos, n_pts,
        prec == kMixed ? 1 : 0, grad_z1, grad_z2, grad_cov);
    GST_TRY_CUDA(cudaGetLastError());
    return GST_OK;
}

// The mode map of a differentiable field: mt = M(angles, anis)^T
// (len_scale_ref / len_scale) with M = diag(1, 1/anis) R_0 R_1 ..., R_i the
// Givens rotation of plane i ((0,1), (0,2), (1,2)) by (-1)^i (-angles_i) --
// the reference's isometrize construction (src/gstools/tools/geometric.py:
// 184-294) -- and its Jacobian jac[a][p] = d mt_a / d params_p (a = row-major
// index of mt), params = [len_scale, anis..., angles...].  One thread: dim
// <= 3, a few hundred flops.
__device__ void mat3_mul(const double (&a)[3][3], const double (&b)[3][3], double (&c)[3][3]) {
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double t = 0.0;
            for (int k = 0; k < 3; ++k) t += a[i][k] * b[k][j];
            c[i][j] = t;
        }
}

__global__ void mode_map_kernel(int dim, const double *__restrict__ params,
                                double len_scale_ref, double *mt, double *jac) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int n_anis = dim - 1, n_ang = dim * (dim - 1) / 2;
    const int n_par = 1 + n_anis + n_ang;
    const double ls = params[0];
    const double r = len_scale_ref / ls;
    // Givens factors and their derivatives (3 x 3, identity beyond dim)
    double g[3][3][3], dg[3][3][3];
    int planes[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int i = 0; i < n_ang; ++i) {
        const double th = ((i & 1) ? 1.0 : -1.0) * params[1 + n_anis + i];
        const double c = cos(th), sn = sin(th);
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                g[i][a][b] = a == b ? 1.0 : 0.0;
                dg[i][a][b] = 0.0;
            }
        const int p = planes[i][0], q = planes[i][1];
        g[i][p][p] = g[i][q][q] = c;
        g[i][p][q] = -sn;
        g[i][q][p] = sn;
        dg[i][p][p] = dg[i][q][q] = -sn;
        dg[i][p][q] = -c;
        dg[i][q][p] = c;
    }
    auto product = [&](int skip, double (&out)[3][3]) {
        // G_0 ... G_{n-1} with factor `skip` replaced by its derivative
        double acc[3][3], tmp[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) acc[a][b] = a == b ? 1.0 : 0.0;
        for (int i = 0; i < n_ang; ++i) {
            mat3_mul(acc, i == skip ? dg[i] : g[i], tmp);
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) acc[a][b] = tmp[a][b];
        }
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) out[a][b] = acc[a][b];
    };
    double rot[3][3];
    product(-1, rot);
    double st[3] = {1.0, 1.0, 1.0};
    for (int j = 0; j < n_anis; ++j) st[j + 1] = 1.0 / params[1 + j];
    // mt[a][b] = M[b][a] r = st[b] rot[b][a] r
    for (int a = 0; a < dim; ++a)
        for (int b = 0; b < dim; ++b) {
            const double v = st[b] * rot[b][a] * r;
            mt[a * dim + b] = v;
            jac[(a * dim + b) * n_par + 0] = -v / ls;   // d / d len_scale
        }
    for (int j = 0; j < n_anis; ++j)   // d / d anis_j: row j + 1 of M
        for (int a = 0; a < dim; ++a)
            for (int b = 0; b < dim; ++b)
                jac[(a * dim + b) * n_par + 1 + j] =
                    b == j + 1 ? -rot[b][a] * r / (params[1 + j] * params[1 + j]) : 0.0;
    for (int i = 0; i < n_ang; ++i) {   // d / d angles_i
        double drot[3][3];
        product(i, drot);
        const double dth = (i & 1) ? 1.0 : -1.0;
        for (int a = 0; a < dim; ++a)
            for (int b = 0; b < dim; ++b)
                jac[(a * dim + b) * n_par + 1 + n_anis + i] = st[b] * drot[b][a] * r * dth;
    }
}

struct GatherGeom {
    int dim;
    int64_t n[3];     // grid axis lengths
    int64_t off[3];   // offsets of the axes in the concatenated array
    int64_t n_grid, n_extra;
};

// Coordinates and cotangent of point idx[t] (a grid point in "ij" order, or
// point idx - n_grid of the extra points).
__global__ void gather_points_kernel(GatherGeom gg, const double *__restrict__ axes,
                                     const double *__restrict__ x_extra, int64_t n_idx,
                                     const int64_t *__restrict__ idx,
                                     const double *__restrict__ g, double *xs,
                                     double *gs) {
    const int64_t t = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (t >= n_idx) return;
    const int64_t i = idx[t];
    const bool ok = i >= 0 && i < gg.n_grid + gg.n_extra;
    if (ok && i < gg.n_grid) {
        int64_t rest = i;
        for (int d = gg.dim - 1; d >= 0; --d) {
            const int64_t n = d == 0 ? gg.n[0] : (d == 1 ? gg.n[1] : gg.n[2]);
            const int64_t o = d == 0 ? gg.off[0] : (d == 1 ? gg.off[1] : gg.off[2]);
            xs[d * n_idx + t] = axes[o + rest % n];
            rest /= n;
        }
    } else {
        for (int d = 0; d < gg.dim; ++d)
            xs[d * n_idx + t] = ok ? x_extra[d * gg.n_extra + (i - gg.n_grid)] : 0.0;
    }
    gs[t] = ok ? g[i] : 0.0;
}

}  // namespace
}  // namespace gst

extern "C" {

int gst_mode_map(int dim, const double *params, double len_scale_ref, double *mt,
                 double *jac, void *stream) {
    if (dim < 1 || dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    if (params == nullptr || mt == nullptr || jac == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    gst::mode_map_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(
        dim, params, len_scale_ref, mt, jac);
    GST_TRY_CUDA(cudaGetLastError());
    return GST_OK;
}

int gst_gather_points(int dim, const int64_t *axis_len, const double *axes,
                      int64_t n_extra, const double *x_extra, int64_t n_idx,
                      const int64_t *idx, const double *g, double *xs,
                      double *gs, void *stream) {
    using namespace gst;
    if (dim < 1 || dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    if (axis_len == nullptr || n_extra < 0 || n_idx < 0) return GST_ERR_INVALID_ARGUMENT;
    if (n_idx == 0) return GST_OK;
    GatherGeom geo{};
    geo.dim = dim;
    geo.n_grid = 1;
    int64_t off = 0;
    for (int d = 0; d < dim; ++d) {
        if (axis_len[d] < 0) return GST_ERR_INVALID_ARGUMENT;
        geo.n[d] = axis_len[d];
        geo.off[d] = off;
        off += axis_len[d];
        geo.n_grid *= axis_len[d];
    }
    geo.n_extra = n_extra;
    if (idx == nullptr || g == nullptr || xs == nullptr || gs == nullptr ||
        (geo.n_grid > 0 && axes == nullptr) || (n_extra > 0 && x_extra == nullptr))
        return GST_ERR_INVALID_ARGUMENT;
    if (current_device() < 0) return GST_ERR_NO_DEVICE;
    const int64_t blocks = ceil_div(n_idx, 256);
    if (blocks > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    gather_points_kernel<<<static_cast<unsigned>(blocks), 256, 0,
                           static_cast<cudaStream_t>(stream)>>>(geo, axes, x_extra, n_idx,
                                                                idx, g, xs, gs);
    GST_TRY_CUDA(cudaGetLastError());
    return GST_OK;
}

int gst_summate_vjp_modes_f64(int dim, int64_t n_modes, int64_t n_pts,
                              const double *cov_samples, const double *z_1,
                              const double *z_2, const double *pos,
                              const double *grad_out, double *grad_z1,
                              double *grad_z2, double *grad_cov, void *stream) {
    return gst::run_vjp_modes(gst::kF64, dim, n_modes, n_pts, cov_samples, z_1,
                              z_2, pos, grad_out, grad_z1, grad_z2, grad_cov,
                              static_cast<cudaStream_t>(stream));
}

int gst_summate_vjp_modes_mixed(int dim, int64_t n_modes, int64_t n_pts,
                                const double *cov_samples, const double *z_1,
                                const double *z_2, const double *pos,
                                const double *grad_out, double *grad_z1,
                                double *grad_z2, double *grad_cov, void *stream) {
    return gst::run_vjp_modes(gst::kMixed, dim, n_modes, n_pts, cov_samples, z_1,
                              z_2, pos, grad_out, grad_z1, grad_z2, grad_cov,
                              static_cast<cudaStream_t>(stream));
}

}  // extern "C"
