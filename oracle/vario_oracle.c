/* CPU restatement of the variogram estimators (test infrastructure only).
 *
 * The reference's vario_estimate / vario_estimate_axis
 * (src/gstools/variogram/variogram.py:151-470, 473-575) call the external
 * gstools-cython kernels unstructured, directional, structured and
 * ma_structured through the wrappers at :48-124 (gstools-cython pinned
 * >= 1, < 2 in pyproject.toml:47, absent from the reference tree).  Their
 * published algorithm, restated with the same loop order:
 *
 *   estimator  'm' (Matheron): d^2                 'c' (Cressie): |d|^0.5
 *   normalise  'm': g / (2 N)
 *              'c': 0.5 (g / N)^4 / (0.457 + 0.494 / N + 0.045 / N^2)
 *              with N = max(count, 1)
 *   unstructured: per bin, pairs j < k with edge[i] <= dist < edge[i + 1],
 *              every field m whose two values are not NaN
 *   directional: the same per direction, for pairs whose connecting vector
 *              is within angles_tol of the direction (and, for bandwidth >
 *              0, closer than bandwidth to its line); separate_dirs stops at
 *              the first matching direction
 *   structured / ma_structured: lags k >= 1 along axis 0 of f (n0, rest),
 *              skipping masked values
 *
 * The angle test stays "acos(|s| / dist) < angles_tol" with the host libm's
 * acos, as in the reference; pairs on the tolerance cone (lattice points at
 * exactly the tolerance angle) then depend on libm's last bit.  The GPU
 * kernels decide the same test as a correctly rounded acos would, so the
 * two agree wherever libm's acos is correctly rounded.
 */
#include <math.h>
#include <stdint.h>

static double estimate(char est, double d)
{
    return est == 'c' ? sqrt(fabs(d)) : d * d;
}

static void normalize(char est, int64_t n, double *g, const int64_t *counts)
{
    for (int64_t i = 0; i < n; ++i) {
        const double cnt = counts[i] > 1 ? (double)counts[i] : 1.0;
        if (est == 'c')
            g[i] = 0.5 * pow(g[i] / cnt, 4.0) / (0.457 + 0.494 / cnt + 0.045 / (cnt * cnt));
        else
            g[i] /= 2.0 * cnt;
    }
}

static double dist_euclid(int dim, const double *pos, int64_t n, int64_t j, int64_t k)
{
    double s = 0.0;
    for (int d = 0; d < dim; ++d) {
        const double t = pos[d * n + j] - pos[d * n + k];
        s += t * t;
    }
    return sqrt(s);
}

static double dist_haversine(const double *pos, int64_t n, int64_t j, int64_t k)
{
    const double deg = 3.14159265358979323846 / 180.0;
    const double dlat = (pos[k] - pos[j]) * deg;
    const double dlon = (pos[n + k] - pos[n + j]) * deg;
    const double a = pow(sin(dlat / 2.0), 2.0) +
                     cos(pos[j] * deg) * cos(pos[k] * deg) * pow(sin(dlon / 2.0), 2.0);
    return 2.0 * atan2(sqrt(a), sqrt(1.0 - a));
}

int oracle_vario_unstructured(int dim, int64_t n, int64_t f_max, const double *f,
                              int64_t n_bins, const double *edges, const double *pos,
                              char est, char dist_type, double *vario, int64_t *counts)
{
    if (dim < 1 || n < 0 || f_max < 0 || n_bins < 0) return 1;
    if (dist_type == 'h' && dim != 2) return 1;
#pragma omp parallel for schedule(dynamic)
    for (int64_t i = 0; i < n_bins; ++i) {
        double g = 0.0;
        int64_t c = 0;
        for (int64_t j = 0; j < n; ++j) {
            for (int64_t k = j + 1; k < n; ++k) {
                const double dist = dist_type == 'h' ? dist_haversine(pos, n, j, k)
                                                     : dist_euclid(dim, pos, n, j, k);
                if (!(dist >= edges[i] && dist < edges[i + 1])) continue;
                for (int64_t m = 0; m < f_max; ++m) {
                    const double a = f[m * n + k], b = f[m * n + j];
                    if (isnan(a) || isnan(b)) continue;
                    ++c;
                    g += estimate(est, a - b);
                }
            }
        }
        vario[i] = g;
        counts[i] = c;
    }
    normalize(est, n_bins, vario, counts);
    return 0;
}

static int dir_test(int dim, const double *pos, int64_t n, const double *dir, double dist,
                    int64_t j, int64_t k, double angles_tol, double bandwidth)
{
    double s_prod = 0.0, b_dist = 0.0;
    int in_band = 1, in_angle = 1;
    for (int i = 0; i < dim; ++i) s_prod += (pos[i * n + j] - pos[i * n + k]) * dir[i];
    if (bandwidth > 0.0) {
        for (int i = 0; i < dim; ++i) {
            const double t = (pos[i * n + j] - pos[i * n + k]) - s_prod * dir[i];
            b_dist += t * t;
        }
        in_band = b_dist < bandwidth * bandwidth;
    }
    if (dist > 0.0) {
        const double t = fabs(s_prod) / dist;
        if (t < 1.0) in_angle = acos(t) < angles_tol;
    }
    return in_band && in_angle;
}

int oracle_vario_directional(int dim, int64_t n, int64_t f_max, const double *f,
                             int64_t n_bins, const double *edges, const double *pos,
                             int64_t d_max, const double *dirs, double angles_tol,
                             double bandwidth, int separate_dirs, char est,
                             double *vario, int64_t *counts)
{
    if (dim < 1 || n < 0 || f_max < 0 || n_bins < 0 || d_max < 0) return 1;
#pragma omp parallel for schedule(dynamic)
    for (int64_t i = 0; i < n_bins; ++i) {
        for (int64_t d = 0; d < d_max; ++d) {
            vario[d * n_bins + i] = 0.0;
            counts[d * n_bins + i] = 0;
        }
        for (int64_t j = 0; j < n; ++j) {
            for (int64_t k = j + 1; k < n; ++k) {
                const double dist = dist_euclid(dim, pos, n, j, k);
                if (!(dist >= edges[i] && dist < edges[i + 1])) continue;
                for (int64_t d = 0; d < d_max; ++d) {
                    if (!dir_test(dim, pos, n, dirs + d * dim, dist, j, k, angles_tol,
                                  bandwidth))
                        continue;
                    for (int64_t m = 0; m < f_max; ++m) {
                        const double a = f[m * n + k], b = f[m * n + j];
                        if (isnan(a) || isnan(b)) continue;
                        ++counts[d * n_bins + i];
                        vario[d * n_bins + i] += estimate(est, a - b);
                    }
                    if (separate_dirs) break;
                }
            }
        }
    }
    for (int64_t d = 0; d < d_max; ++d)
        normalize(est, n_bins, vario + d * n_bins, counts + d * n_bins);
    return 0;
}

int oracle_vario_structured(int64_t n0, int64_t rest, const double *f,
                            const unsigned char *mask, char est, double *vario)
{
    if (n0 < 0 || rest < 0) return 1;
#pragma omp parallel for schedule(dynamic)
    for (int64_t k = 0; k < n0; ++k) {
        double g = 0.0;
        int64_t c = 0;
        if (k > 0) {
            for (int64_t j = 0; j < rest; ++j) {
                for (int64_t i = 0; i + k < n0; ++i) {
                    if (mask && (mask[i * rest + j] || mask[(i + k) * rest + j])) continue;
                    ++c;
                    g += estimate(est, f[i * rest + j] - f[(i + k) * rest + j]);
                }
            }
        }
        const double cnt = c > 1 ? (double)c : 1.0;
        if (est == 'c')
            vario[k] = 0.5 * pow(g / cnt, 4.0) / (0.457 + 0.494 / cnt + 0.045 / (cnt * cnt));
        else
            vario[k] = g / (2.0 * cnt);
    }
    return 0;
}
