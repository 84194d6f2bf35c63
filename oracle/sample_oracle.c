/* CPU restatement of the device spectral sampler (test infrastructure only).
 *
 * Restates gst_batch_sample_modes (gstools_gb300/csrc/gst_sampling.cu) in
 * plain C with libm: Philox4x64-10 (Salmon, Moraes, Dror and Shaw, SC 2011)
 * keyed by (seed_r, 0) with counter (j, b, 0, 0) for mode j and block b,
 * Box-Muller normals, the sphere formulas of the reference
 * (src/gstools/random/rng.py:142-193) and the analytic radial laws of the
 * covariance models (Gaussian, Exponential, Matern), Matern's chi-square via
 * Marsaglia and Tsang's gamma sampler.  The Philox stream is pinned to
 * numpy's own Philox bit generator by the tests; the transforms agree with
 * the device to the last few ulps (libm and CUDA round log/sin/cos
 * differently in the last place).
 */
#include <math.h>
#include <stdint.h>

#define PHILOX_M0 0xD2E7470EE14C6C93ull
#define PHILOX_M1 0xCA5A826395121157ull
#define PHILOX_W0 0x9E3779B97F4A7C15ull
#define PHILOX_W1 0xBB67AE8584CAA73Bull
#define GAMMA_ITERS 16
#define TWO_PI 6.283185307179586476925286766559
#define SQRT2 1.4142135623730950488016887242097

enum { MODEL_GAUSSIAN = 0, MODEL_EXPONENTIAL = 1, MODEL_MATERN = 2 };

void oracle_philox4x64(uint64_t c0, uint64_t c1, uint64_t c2, uint64_t c3,
                       uint64_t k0, uint64_t k1, uint64_t out[4])
{
    for (int r = 0; r < 10; ++r) {
        const unsigned __int128 p0 = (unsigned __int128)PHILOX_M0 * c0;
        const unsigned __int128 p1 = (unsigned __int128)PHILOX_M1 * c2;
        const uint64_t hi0 = (uint64_t)(p0 >> 64), lo0 = (uint64_t)p0;
        const uint64_t hi1 = (uint64_t)(p1 >> 64), lo1 = (uint64_t)p1;
        const uint64_t n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
        c0 = n0;
        c1 = lo1;
        c2 = n2;
        c3 = lo0;
        k0 += PHILOX_W0;
        k1 += PHILOX_W1;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

static double unit(uint64_t x) { return (double)((x >> 11) + 1) * 0x1.0p-53; }

static void box_muller(uint64_t xa, uint64_t xb, double *a, double *b)
{
    const double rho = sqrt(-2.0 * log(unit(xa)));
    const double th = TWO_PI * unit(xb);
    *a = rho * cos(th);
    *b = rho * sin(th);
}

static double gamma_draw(double shape, uint64_t j, uint64_t k0)
{
    uint64_t q[4];
    double boost = 1.0;
    if (shape < 1.0) {
        oracle_philox4x64(j, 2, 0, 0, k0, 0, q);
        boost = exp(log(unit(q[0])) / shape);
        shape += 1.0;
    }
    const double d = shape - 1.0 / 3.0;
    const double c = 1.0 / sqrt(9.0 * d);
    for (int i = 0; i < GAMMA_ITERS; ++i) {
        oracle_philox4x64(j, 3 + (uint64_t)i, 0, 0, k0, 0, q);
        double x, unused;
        box_muller(q[0], q[1], &x, &unused);
        const double t = 1.0 + c * x;
        if (t <= 0.0) continue;
        const double v = t * t * t;
        const double u = unit(q[2]);
        if (log(u) < 0.5 * x * x + d - d * v + d * log(v)) return d * v * boost;
    }
    return d * boost;
}

int oracle_sample_modes(int dim, int64_t n_items, int64_t total,
                        const int64_t *mode_off, int model, double nu,
                        const uint64_t *seeds, const double *len_rescaled,
                        double *cov, double *z1, double *z2)
{
    if (dim < 1 || dim > 3 || n_items < 0 || total < 0) return 1;
    if (model == MODEL_MATERN && !(nu > 0.0 && nu <= 20.0)) return 1;
#pragma omp parallel for schedule(static)
    for (int64_t m = 0; m < total; ++m) {
        int64_t lo = 0, hi = n_items;
        while (hi - lo > 1) {
            const int64_t mid = (lo + hi) >> 1;
            if (mode_off[mid] <= m) lo = mid; else hi = mid;
        }
        const uint64_t j = (uint64_t)(m - mode_off[lo]);
        const uint64_t key = seeds[lo];
        const double ls = len_rescaled[lo];
        uint64_t q[4];
        oracle_philox4x64(j, 0, 0, 0, key, 0, q);
        double a, b;
        box_muller(q[0], q[1], &a, &b);
        z1[m] = a;
        z2[m] = b;
        double dir[3] = {0.0, 0.0, 0.0};
        if (dim == 1) {
            dir[0] = unit(q[2]) <= 0.5 ? -1.0 : 1.0;
        } else {
            const double phi = TWO_PI * unit(q[2]);
            const double s = sin(phi), c = cos(phi);
            if (dim == 2) {
                dir[0] = c;
                dir[1] = s;
            } else {
                const double h = 2.0 * unit(q[3]) - 1.0;
                const double w = sqrt(1.0 - h * h);
                dir[0] = w * c;
                dir[1] = w * s;
                dir[2] = h;
            }
        }
        oracle_philox4x64(j, 1, 0, 0, key, 0, q);
        double n[4];
        box_muller(q[0], q[1], &n[0], &n[1]);
        box_muller(q[2], q[3], &n[2], &n[3]);
        double g2 = 0.0;
        for (int i = 0; i < dim; ++i) g2 += n[i] * n[i];
        const double g = sqrt(g2);
        double rho;
        if (model == MODEL_GAUSSIAN) {
            rho = SQRT2 / ls * g;
        } else if (model == MODEL_EXPONENTIAL) {
            rho = g / fabs(n[dim]) / ls;
        } else {
            const double chi2 = 2.0 * gamma_draw(nu, j, key);
            rho = g / sqrt(chi2 / (2.0 * nu)) / (SQRT2 * ls);
        }
        for (int i = 0; i < dim; ++i) cov[i * total + m] = rho * dir[i];
    }
    return 0;
}
