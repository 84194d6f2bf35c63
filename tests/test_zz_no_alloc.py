"""The allocation-free FP64 summate entry point, through the C ABI.

``gst_summate_f64_noalloc`` is for callers that cannot let a library
allocate device memory (hosts that reserve all GPU memory for their own pool,
latency-critical loops that cannot pay for an allocator call).  Its scratch
lives in a fixed device array inside the library and keeps the previous
call's contents, so the test runs two different calls in a row and checks
each against ``gst_summate_f64`` (which allocates its scratch per call)
within the FP64 bar of the other tests: max|diff| <= 1e-12 * max|ref|.

This file is collected last so that a failure here cannot hide the other
tests in a run that stops at the first failure.
"""

import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

F64_REL = 1e-12


def _case(seed, dim, n_modes, n_pts):
    rng = np.random.RandomState(seed)
    cov = rng.standard_t(3, size=(dim, n_modes)) * 0.3
    z1, z2 = rng.normal(size=n_modes), rng.normal(size=n_modes)
    pos = rng.uniform(0.0, 200.0, size=(dim, n_pts))
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda()
            for a in (cov, z1, z2, pos)]


def _call(lib, name, dim, arrays, n_modes, n_pts):
    out = torch.full((n_pts,), float("nan"), dtype=torch.float64,
                     device="cuda")
    ptrs = [ctypes.c_void_p(a.data_ptr()) for a in arrays]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = getattr(lib, name)(dim, n_modes, n_pts, *ptrs,
                            ctypes.c_void_p(out.data_ptr()), stream)
    torch.cuda.synchronize()
    return rc, out.cpu().numpy()


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    from gstools_gb300 import _native, build

    build.build()
    return _native.load()


def test_noalloc_matches_allocating_entry_point_twice(lib):
    # two calls in a row with different sizes: the second must not see the
    # first call's table or partial sums
    for seed, dim, n_modes, n_pts in ((11, 3, 2000, 50_000),
                                      (12, 2, 777, 3001)):
        arrays = _case(seed, dim, n_modes, n_pts)
        rc_ref, ref = _call(lib, "gst_summate_f64", dim, arrays, n_modes,
                            n_pts)
        rc, got = _call(lib, "gst_summate_f64_noalloc", dim, arrays, n_modes,
                        n_pts)
        assert rc_ref == 0 and rc == 0
        assert np.all(np.isfinite(got))
        assert np.max(np.abs(got - ref)) <= F64_REL * np.max(np.abs(ref))


def test_noalloc_rejects_too_many_modes(lib):
    from gstools_gb300 import _native

    arrays = _case(13, 2, 16385, 10)
    rc, _ = _call(lib, "gst_summate_f64_noalloc", 2, arrays, 16385, 10)
    assert rc == _native.GST_ERR_TOO_LARGE
