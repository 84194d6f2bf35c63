"""Mixed-precision summate of large unstructured point sets (the sorted
amplitude-phase path of gst_summate_mixed) against the FP64 oracle.

``gst_summate_mixed`` sends sums of at least 1e9 mode-points, or in 2-D /
3-D of at least 4e8 over at least 2e5 points (and at most 16 384 modes),
through the path the ensembles use: points sorted spatially,
modes by |k|_1, one SFU cosine per mode and point, per-warp origins, FP32
phases where they stay small and the exact split turn reduction elsewhere.
The cases cover the direct store (enough point tiles) and the mode range
split over FP64 partial sums (few point tiles), 1-D to 3-D, points 1e5 from
the origin, and a heavy-tailed spectrum (multivariate t with 1 degree of
freedom, the Exponential model's law) whose large |k| run the exact path.
Bar: RMS of the scaled field <= 1e-5 sigma against the oracle on a fixed
subsample of 2048 points.
"""

import numpy as np
import pytest

import gstools_gb300 as gg
import oracle

pytestmark = pytest.mark.gpu

RMS_SIGMA = 1e-5


def _modes(rng, dim, n_modes, ls, heavy):
    if heavy:
        g = rng.normal(size=(dim, n_modes))
        chi = np.sqrt(rng.chisquare(1, size=n_modes))
        cov = g / chi / ls
    else:
        cov = rng.normal(size=(dim, n_modes)) * np.sqrt(2.0) / ls
    return cov, rng.normal(size=n_modes), rng.normal(size=n_modes)


CASES = [
    # (dim, modes, points, extent, offset, len_scale, heavy)
    (2, 2000, 600_000, 1000.0, 0.0, 10.0, False),   # direct store
    (3, 16384, 100_000, 200.0, 0.0, 8.0, False),    # mode split, partials
    (1, 4000, 300_000, 5000.0, 0.0, 20.0, False),
    (2, 2000, 600_000, 500.0, 1.0e5, 10.0, False),  # far from the origin
    (2, 4000, 400_000, 500.0, 0.0, 5.0, True),      # heavy tail: exact chunks
    (3, 2048, 600_000, 300.0, 3.0e4, 20.0, True),
    (2, 1000, 450_000, 400.0, 0.0, 10.0, False),     # 4.5e8 over 4.5e5 points
]


@pytest.mark.parametrize("case", CASES)
def test_sorted_mixed_path_vs_oracle(cuda_lib, case):
    dim, n_modes, n_pts, extent, offset, ls, heavy = case
    assert n_modes * n_pts >= 1e9 or (dim >= 2 and n_modes * n_pts >= 4e8
                                      and n_pts >= 200_000)
    rng = np.random.RandomState(n_modes + n_pts + dim)
    cov, z1, z2 = _modes(rng, dim, n_modes, ls, heavy)
    pos = offset + rng.uniform(0.0, extent, size=(dim, n_pts))
    got = gg.summate(cov, z1, z2, pos, precision="mixed")
    idx = np.sort(rng.choice(n_pts, size=2048, replace=False))
    ref = oracle.c_summate(cov, z1, z2, np.ascontiguousarray(pos[:, idx]))
    rms = np.sqrt(np.mean((got[idx] - ref) ** 2)) / np.sqrt(n_modes)
    assert rms <= RMS_SIGMA, rms
    # deterministic: the sorts are stable and the partial sums ordered
    again = gg.summate(cov, z1, z2, pos, precision="mixed")
    np.testing.assert_array_equal(got, again)


def test_sorted_mixed_path_float32_and_nan(cuda_lib):
    rng = np.random.RandomState(5)
    cov, z1, z2 = _modes(rng, 2, 2000, 10.0, False)
    pos = rng.uniform(0.0, 800.0, size=(2, 600_000))
    pos[:, 1234] = np.nan
    got = gg.summate(cov, z1, z2, pos, precision="mixed", out_dtype="float32")
    assert got.dtype == np.float32
    assert np.isnan(got[1234]) and np.isfinite(np.delete(got, 1234)).all()
    idx = np.arange(0, 600_000, 293)
    idx = idx[idx != 1234]
    ref = oracle.c_summate(cov, z1, z2, np.ascontiguousarray(pos[:, idx]))
    rms = np.sqrt(np.mean((got[idx].astype(np.float64) - ref) ** 2)) / np.sqrt(2000)
    assert rms <= RMS_SIGMA, rms
