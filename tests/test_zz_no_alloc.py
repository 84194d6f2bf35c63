"""The allocation-free FP64 summate entry point, through the C ABI.

``gst_summate_f64_noalloc`` is for callers that cannot let a library
allocate device memory (hosts that reserve all GPU memory for their own pool,
latency-critical loops that cannot pay for an allocator call).  Its scratch
lives in a fixed device array inside the library and keeps the previous
call's contents, so the test runs different calls in a row and checks each
against ``gst_summate_f64`` (which allocates its scratch per call) and
against the FP64 C oracle on a subsample of the points, within the FP64 bar
of the other tests: max|diff| <= 1e-12 * max|ref|.  The cases cover the
three ways the call splits its work: mode range split over CTAs with the
partial sums in the fixed array (2000 x 50 000, 777 x 3001, 4096 x 150 000),
and the full 16 384-mode table on 300 000 points, where the partial sums
would not fit and the kernel writes straight to ``out`` (no split).

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


def _oracle_check(arrays, got, stride):
    """FP64 C oracle on every `stride`-th point."""
    import oracle

    cov, z1, z2, pos = (a.cpu().numpy() for a in arrays)
    sub = np.ascontiguousarray(pos[:, ::stride])
    ref = oracle.c_summate(cov, z1, z2, sub)
    err = np.max(np.abs(got[::stride] - ref))
    assert err <= F64_REL * np.max(np.abs(ref)), err


def test_noalloc_matches_allocating_entry_point_twice(lib):
    # calls in a row with different sizes: none may see the previous call's
    # table or partial sums
    for seed, dim, n_modes, n_pts, stride in ((11, 3, 2000, 50_000, 7),
                                              (12, 2, 777, 3001, 1),
                                              (14, 3, 16384, 300_000, 101),
                                              (15, 2, 4096, 150_000, 37)):
        arrays = _case(seed, dim, n_modes, n_pts)
        rc_ref, ref = _call(lib, "gst_summate_f64", dim, arrays, n_modes,
                            n_pts)
        rc, got = _call(lib, "gst_summate_f64_noalloc", dim, arrays, n_modes,
                        n_pts)
        assert rc_ref == 0 and rc == 0
        assert np.all(np.isfinite(got))
        assert np.max(np.abs(got - ref)) <= F64_REL * np.max(np.abs(ref))
        _oracle_check(arrays, got, stride)


def test_noalloc_rejects_too_many_modes(lib):
    from gstools_gb300 import _native

    arrays = _case(13, 2, 16385, 10)
    rc, _ = _call(lib, "gst_summate_f64_noalloc", 2, arrays, 16385, 10)
    assert rc == _native.GST_ERR_TOO_LARGE
