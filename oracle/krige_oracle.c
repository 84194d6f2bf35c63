/* CPU restatement of the kriging kernels (test infrastructure only).
 *
 * The reference's Krige (src/gstools/krige/base.py:307-320, wrappers at
 * :42-60) calls calc_field_krige(_and_variance) of the external
 * gstools-cython package (pinned gstools-cython >= 1, < 2 in
 * pyproject.toml:47), absent from the reference tree.  Its published
 * algorithm, restated here with the same loop order: for every target point
 * k (parallel), for every row i of the inverted kriging matrix M,
 *
 *     fac    = sum_j M[i, j] V[j, k]          (j ascending)
 *     err[k] += V[i, k] * fac
 *     fld[k] += cond[i] * fac                  (i ascending)
 */
#include <stdint.h>

int oracle_krige(int64_t n_cond, int64_t n_pts, const double *mat,
                 const double *vecs, const double *cond, double *field,
                 double *error)
{
    if (n_cond < 0 || n_pts < 0) return 1;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n_pts; ++k) {
        double f = 0.0, e = 0.0;
        for (int64_t i = 0; i < n_cond; ++i) {
            double fac = 0.0;
            for (int64_t j = 0; j < n_cond; ++j) fac += mat[i * n_cond + j] * vecs[j * n_pts + k];
            e += vecs[i * n_pts + k] * fac;
            f += cond[i] * fac;
        }
        field[k] = f;
        if (error) error[k] = e;
    }
    return 0;
}
