"""The host RNG mirror against the reference's own ``RNG`` (CPU side).

Same seed, same draws: the direction sampler of src/gstools/random/rng.py:
142-193 for every dimension (1-3 by their closed forms, higher dimensions as
normalised Gaussian vectors) and for scalar, vector and array sample sizes.
Skipped where the reference tree is not present.
"""

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import reference_import  # noqa: E402

from gstools_gb300.rng import RNG  # noqa: E402


@pytest.fixture(scope="module")
def ref_rng():
    if not reference_import.available():
        pytest.skip("reference tree not present")
    gs = reference_import.import_gstools()
    return gs.random.RNG


@pytest.mark.parametrize("dim", [1, 2, 3, 4, 5, 7])
@pytest.mark.parametrize("size", [None, 1, 1000, (3, 4)])
def test_sample_sphere_matches_reference(ref_rng, dim, size):
    for seed in (1, 20170519):
        ours = RNG(seed).sample_sphere(dim, size)
        theirs = ref_rng(seed).sample_sphere(dim, size)
        np.testing.assert_array_equal(ours, theirs)
