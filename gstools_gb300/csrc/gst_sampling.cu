// Device-side spectral sampling for ensembles.
//
// The reference draws every realization's modes on the host
// (RandMeth.reset_seed, src/gstools/field/generator.py:346-387, with the RNG
// of src/gstools/random/rng.py:38-203): amplitudes z1, z2 ~ N(0, 1),
// directions uniform on the unit sphere, and radii from the model's radial
// spectral law.  For an ensemble of hundreds of realizations that host loop
// costs far more than the summation, so this file draws all modes of all
// realizations in one launch, from a counter-based stream:
//
//   key (seed_r, 0), counter (j, b, 0, 0) -> Philox4x64-10 -> 4 x uint64
//
// for mode j of realization r and block b (Salmon, Moraes, Dror and Shaw,
// "Parallel random numbers: as easy as 1, 2, 3", SC 2011).  Every mode is an
// independent function of (seed_r, j), so the draw is order-free and
// reproducible.  It is not the reference's MT19937 stream; the distributions
// are the reference's (the radial laws are the exact analytic samplers of the
// host mirror: Gaussian normal, Exponential multivariate t with 1 degree of
// freedom, Matern nu multivariate t with 2 nu degrees of freedom).
//
// Block use per mode:
//   b = 0: (z1, z2) = BoxMuller(x0, x1); direction from u(x2), u(x3)
//          (the reference's sphere formulas, rng.py:142-193)
//   b = 1: normals (n0, n1), (n2, n3) = BoxMuller(x0, x1), BoxMuller(x2, x3);
//          g = |(n_0 .. n_{d-1})|
//          Gaussian     rho = sqrt(2) / ls * g
//          Exponential  rho = g / |n_d| / ls
//          Matern(nu)   rho = g / sqrt(chi2 / (2 nu)) / (sqrt(2) ls),
//                       chi2 = 2 Gamma(nu)
//   b = 2: u(x0) for the shape boost Gamma(a) = Gamma(a + 1) u^(1/a), a < 1
//   b = 3 + i: iteration i of Marsaglia and Tsang's gamma sampler
//          (ACM TOMS 26(3), 2000): x = BoxMuller(x0, x1).first, u = u(x2);
//          at most 16 iterations (each accepts with probability > 0.95; the
//          mean d is returned after 16 rejections).
// u(x) = ((x >> 11) + 1) 2^-53 lies in (0, 1], so log(u) is finite.
#include "gst_common.cuh"

namespace gst {
namespace {

constexpr uint64_t kPhiloxM0 = 0xD2E7470EE14C6C93ull;
constexpr uint64_t kPhiloxM1 = 0xCA5A826395121157ull;
constexpr uint64_t kPhiloxW0 = 0x9E3779B97F4A7C15ull;   // golden ratio
constexpr uint64_t kPhiloxW1 = 0xBB67AE8584CAA73Bull;   // sqrt(3) - 1
constexpr int kGammaIters = 16;
constexpr double kTwoPi = 6.283185307179586476925286766559;
constexpr double kSqrt2 = 1.4142135623730950488016887242097;

struct U64x4 {
    uint64_t v[4];
};

__device__ __forceinline__ U64x4 philox4x64(uint64_t c0, uint64_t c1, uint64_t c2,
                                            uint64_t c3, uint64_t k0, uint64_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t hi0 = __umul64hi(kPhiloxM0, c0), lo0 = kPhiloxM0 * c0;
        const uint64_t hi1 = __umul64hi(kPhiloxM1, c2), lo1 = kPhiloxM1 * c2;
        const uint64_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += kPhiloxW0;
        k1 += kPhiloxW1;
    }
    return U64x4{{c0, c1, c2, c3}};
}

__device__ __forceinline__ double unit(uint64_t x) {
    return static_cast<double>((x >> 11) + 1) * 0x1.0p-53;
}

__device__ __forceinline__ void box_muller(uint64_t xa, uint64_t xb, double &a,
                                           double &b) {
    const double rho = sqrt(-2.0 * log(unit(xa)));
    const double th = kTwoPi * unit(xb);
    double s, c;
    sincos(th, &s, &c);
    a = rho * c;
    b = rho * s;
}

// Gamma(shape, 1) from the mode's blocks 2.. of the stream.
__device__ double gamma_draw(double shape, uint64_t j, uint64_t k0) {
    double boost = 1.0;
    if (shape < 1.0) {
        const U64x4 q = philox4x64(j, 2, 0, 0, k0, 0);
        boost = exp(log(unit(q.v[0])) / shape);
        shape += 1.0;
    }
    const double d = shape - 1.0 / 3.0;
    const double c = 1.0 / sqrt(9.0 * d);
    for (int i = 0; i < kGammaIters; ++i) {
        const U64x4 q = philox4x64(j, 3 + static_cast<uint64_t>(i), 0, 0, k0, 0);
        double x, unused;
        box_muller(q.v[0], q.v[1], x, unused);
        const double t = 1.0 + c * x;
        if (t <= 0.0) continue;
        const double v = t * t * t;
        const double u = unit(q.v[2]);
        if (log(u) < 0.5 * x * x + d - d * v + d * log(v)) return d * v * boost;
    }
    return d * boost;
}

__global__ void sample_modes_kernel(int dim, int64_t n_items, int64_t total,
                                    const int64_t *__restrict__ mode_off, int model,
                                    double nu, const uint64_t *__restrict__ seeds,
                                    const double *__restrict__ len_rescaled,
                                    double *__restrict__ cov, double *__restrict__ z1,
                                    double *__restrict__ z2) {
    const int64_t m = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (m >= total) return;
    // realization owning global mode m: last r with mode_off[r] <= m
    int64_t lo = 0, hi = n_items;
    while (hi - lo > 1) {
        const int64_t mid = (lo + hi) >> 1;
        if (mode_off[mid] <= m) lo = mid; else hi = mid;
    }
    const int64_t r = lo;
    const uint64_t j = static_cast<uint64_t>(m - mode_off[r]);
    const uint64_t key = seeds[r];
    const double ls = len_rescaled[r];

    const U64x4 q0 = philox4x64(j, 0, 0, 0, key, 0);
    double a, b;
    box_muller(q0.v[0], q0.v[1], a, b);
    z1[m] = a;
    z2[m] = b;
    double dir[3] = {0.0, 0.0, 0.0};
    if (dim == 1) {
        dir[0] = unit(q0.v[2]) <= 0.5 ? -1.0 : 1.0;
    } else {
        const double phi = kTwoPi * unit(q0.v[2]);
        double s, c;
        sincos(phi, &s, &c);
        if (dim == 2) {
            dir[0] = c;
            dir[1] = s;
        } else {
            const double h = 2.0 * unit(q0.v[3]) - 1.0;
            const double w = sqrt(1.0 - h * h);
            dir[0] = w * c;
            dir[1] = w * s;
            dir[2] = h;
        }
    }
    const U64x4 q1 = philox4x64(j, 1, 0, 0, key, 0);
    double n[4];
    box_muller(q1.v[0], q1.v[1], n[0], n[1]);
    box_muller(q1.v[2], q1.v[3], n[2], n[3]);
    double g2 = 0.0;
    for (int i = 0; i < dim; ++i) g2 += n[i] * n[i];
    const double g = sqrt(g2);
    double rho;
    if (model == GST_MODEL_GAUSSIAN) {
        rho = kSqrt2 / ls * g;
    } else if (model == GST_MODEL_EXPONENTIAL) {
        rho = g / fabs(n[dim]) / ls;
    } else {
        const double chi2 = 2.0 * gamma_draw(nu, j, key);
        rho = g / sqrt(chi2 / (2.0 * nu)) / (kSqrt2 * ls);
    }
    for (int i = 0; i < dim; ++i) cov[i * total + m] = rho * dir[i];
}

__global__ void philox_fill_kernel(uint64_t k0, uint64_t k1, int64_t n_blocks,
                                   uint64_t ctr1, uint64_t *__restrict__ out) {
    const int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    if (i >= n_blocks) return;
    const U64x4 q = philox4x64(static_cast<uint64_t>(i), ctr1, 0, 0, k0, k1);
    for (int t = 0; t < 4; ++t) out[4 * i + t] = q.v[t];
}

}  // namespace
}  // namespace gst

extern "C" {

int gst_batch_sample_modes(int dim, int64_t n_items, int64_t total_modes,
                           const int64_t *mode_offsets, int model, double nu,
                           const uint64_t *seeds, const double *len_rescaled,
                           double *cov, double *z_1, double *z_2, void *stream) {
    if (dim < 1 || dim > 3) return GST_ERR_UNSUPPORTED_DIM;
    if (n_items < 0 || total_modes < 0) return GST_ERR_INVALID_ARGUMENT;
    if (model != GST_MODEL_GAUSSIAN && model != GST_MODEL_EXPONENTIAL &&
        model != GST_MODEL_MATERN)
        return GST_ERR_INVALID_ARGUMENT;
    if (model == GST_MODEL_MATERN && !(nu > 0.0 && nu <= 20.0))
        return GST_ERR_INVALID_ARGUMENT;
    if (total_modes == 0) return GST_OK;
    if (n_items == 0 || mode_offsets == nullptr || seeds == nullptr ||
        len_rescaled == nullptr || cov == nullptr || z_1 == nullptr || z_2 == nullptr)
        return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    const int threads = 128;
    const int64_t blocks = gst::ceil_div(total_modes, threads);
    if (blocks > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    gst::sample_modes_kernel<<<static_cast<unsigned>(blocks), threads, 0,
                               static_cast<cudaStream_t>(stream)>>>(
        dim, n_items, total_modes, mode_offsets, model, nu, seeds, len_rescaled, cov,
        z_1, z_2);
    GST_TRY_CUDA(cudaGetLastError());
    return GST_OK;
}

int gst_philox4x64_fill(uint64_t key0, uint64_t key1, int64_t n_blocks,
                        uint64_t counter1, uint64_t *out, void *stream) {
    if (n_blocks < 0) return GST_ERR_INVALID_ARGUMENT;
    if (n_blocks == 0) return GST_OK;
    if (out == nullptr) return GST_ERR_INVALID_ARGUMENT;
    if (gst::current_device() < 0) return GST_ERR_NO_DEVICE;
    const int threads = 256;
    const int64_t blocks = gst::ceil_div(n_blocks, threads);
    if (blocks > 0x7fffffffLL) return GST_ERR_TOO_LARGE;
    gst::philox_fill_kernel<<<static_cast<unsigned>(blocks), threads, 0,
                              static_cast<cudaStream_t>(stream)>>>(key0, key1, n_blocks,
                                                                   counter1, out);
    GST_TRY_CUDA(cudaGetLastError());
    return GST_OK;
}

}  // extern "C"
