/*
 * TEST INFRASTRUCTURE ONLY -- the FP64 CPU oracle for the randomization-method
 * summation.  Nothing in the gstools_gb300 product path links, loads or calls
 * this file; only tests/, __graft_entry__.smoke() and the CPU-baseline leg of
 * bench.py use it, as the checker and as the timed CPU baseline.
 *
 * The reference's arithmetic lives in the external package gstools-cython
 * (pinned `gstools-cython>=1,<2`, pyproject.toml:47; imported at
 * src/gstools/field/generator.py:22-24), which is not vendored in the
 * reference tree.  This file restates the published formulas instead:
 *
 *   summate          src/gstools/field/generator.py:193-199
 *       out[i] = sum_j z1[j] cos(<k_j, x_i>) + z2[j] sin(<k_j, x_i>)
 *   summate_incompr  src/gstools/field/generator.py:479-495
 *       out[c, i] = sum_j (delta_{c0} - k_cj k_0j / |k_j|^2)
 *                         (z1[j] cos(<k_j, x_i>) + z2[j] sin(<k_j, x_i>))
 *   summate_fourier  src/gstools/field/generator.py:682-689, 852-862
 *       out[i] = sum_j f[j] (z1[j] cos(<k_j, x_i>) + z2[j] sin(<k_j, x_i>))
 *
 * Loop order is the one the formulas imply and the reference's call sites
 * assume (generator.py:266-270): parallel over points, sequential over modes,
 * the phase accumulated over the dimensions in order, one libm cos and sin
 * per (mode, point).  Layouts follow the reference's arrays: cov_samples is
 * (dim, N) row-major, pos is (dim, n) row-major, out is (n,) or (dim, n).
 *
 * Parity status: pinned -- tests/golden/ holds vectors produced by the
 * reference's own Python (RNG, models, SRF) driving this restatement, and
 * tests/test_oracle.py checks them against the literal golden values of the
 * reference's tests (tests/test_randmeth.py, tests/test_incomprrandmeth.py,
 * tests/test_srf.py).
 */
#include <math.h>
#include <stdint.h>

#ifdef _OPENMP
#include <omp.h>
#endif

static void set_threads(int n_threads)
{
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
}

int oracle_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* summate: generator.py:193-199 */
int oracle_summate(int dim, int64_t n_modes, int64_t n_pts,
                   const double *cov, const double *z1, const double *z2,
                   const double *pos, double *out, int n_threads)
{
    if (dim < 1 || n_modes < 0 || n_pts < 0) return 1;
    set_threads(n_threads);
    int64_t i;
#pragma omp parallel for schedule(static)
    for (i = 0; i < n_pts; ++i) {
        double acc = 0.0;
        for (int64_t j = 0; j < n_modes; ++j) {
            double phase = 0.0;
            for (int d = 0; d < dim; ++d)
                phase += cov[d * n_modes + j] * pos[d * n_pts + i];
            acc += z1[j] * cos(phase) + z2[j] * sin(phase);
        }
        out[i] = acc;
    }
    return 0;
}

/* summate_incompr: generator.py:479-495 (projector p(k) = e1 - k k_1/|k|^2) */
int oracle_summate_incompr(int dim, int64_t n_modes, int64_t n_pts,
                           const double *cov, const double *z1,
                           const double *z2, const double *pos, double *out,
                           int n_threads)
{
    if (dim < 2 || dim > 3 || n_modes < 0 || n_pts < 0) return 1;
    set_threads(n_threads);
    int64_t i;
#pragma omp parallel for schedule(static)
    for (i = 0; i < n_pts; ++i) {
        double acc[3] = {0.0, 0.0, 0.0};
        for (int64_t j = 0; j < n_modes; ++j) {
            double k2 = 0.0, phase = 0.0;
            for (int d = 0; d < dim; ++d) {
                double k = cov[d * n_modes + j];
                k2 += k * k;
                phase += k * pos[d * n_pts + i];
            }
            double amp = z1[j] * cos(phase) + z2[j] * sin(phase);
            double k0 = cov[j];
            for (int d = 0; d < dim; ++d) {
                double e = (d == 0) ? 1.0 : 0.0;
                double proj = e - cov[d * n_modes + j] * k0 / k2;
                acc[d] += proj * amp;
            }
        }
        for (int d = 0; d < dim; ++d) out[d * n_pts + i] = acc[d];
    }
    return 0;
}

/* summate_fourier: generator.py:682-689 (spectrum_factor weights each mode) */
int oracle_summate_fourier(int dim, int64_t n_modes, int64_t n_pts,
                           const double *spectrum_factor, const double *modes,
                           const double *z1, const double *z2,
                           const double *pos, double *out, int n_threads)
{
    if (dim < 1 || n_modes < 0 || n_pts < 0) return 1;
    set_threads(n_threads);
    int64_t i;
#pragma omp parallel for schedule(static)
    for (i = 0; i < n_pts; ++i) {
        double acc = 0.0;
        for (int64_t j = 0; j < n_modes; ++j) {
            double phase = 0.0;
            for (int d = 0; d < dim; ++d)
                phase += modes[d * n_modes + j] * pos[d * n_pts + i];
            acc += spectrum_factor[j] *
                   (z1[j] * cos(phase) + z2[j] * sin(phase));
        }
        out[i] = acc;
    }
    return 0;
}
