"""Variogram estimators (gstools-cython's unstructured, directional,
structured, ma_structured).

Fixtures: the arrays the reference's vario_estimate / vario_estimate_axis
hand to those kernels (setups of tests/test_variogram_unstructured.py and
test_variogram_structured.py: the literature 1-D series, a 2-D field with
no-data values, Cressie, three axis directions with a bandwidth, a 45 degree
direction, masked and unmasked axis variograms, haversine distances),
recorded by tests/golden/make_golden.py with the C oracle as the kernels
after reproducing the reference's literal values 0.4917 / 0.7625.
CPU: the oracle against a brute-force numpy witness; the reference's own
variogram and kriging test files pass with the oracle as gstools-cython
(except the ones tied to emcee's random stream); the hook routes and
restores the reference's variogram wrappers.
GPU: counts exact, variograms within 1e-12 relative (sums of positive terms
in another order), binning exact on integer grids where distances fall on
the bin edges.
"""

import os
import subprocess
import sys

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import reference_import  # noqa: E402

REL = 1e-12
# a variogram fit on a field drawn through emcee's MCMC stream (its outcome
# depends on that stream, which the stand-in sampler does not reproduce)
MCMC_DEPENDENT = ["test_fit_directional"]


def _cases(ref_goldens):
    return sorted({k.split("/")[0] for k in ref_goldens.files
                   if k.startswith("vario_")})


def _call_oracle(name, c):
    if name.endswith("_unstructured") and not name.endswith("ma_structured"):
        return oracle.c_vario_unstructured(c["f"], c["bin_edges"], c["pos"],
                                           str(c["estimator_type"]),
                                           str(c["distance_type"]))
    if name.endswith("_directional"):
        return oracle.c_vario_directional(
            c["f"], c["bin_edges"], c["pos"], c["direction"],
            float(c["angles_tol"]), float(c["bandwidth"]),
            bool(c["separate_dirs"]), str(c["estimator_type"]))
    if name.endswith("_ma_structured"):
        return oracle.c_vario_structured(c["f"], str(c["estimator_type"]),
                                         mask=c["mask"])
    return oracle.c_vario_structured(c["f"], str(c["estimator_type"]))


def _call_gpu(name, c):
    import gstools_gb300.variogram as gv

    if name.endswith("_unstructured") and not name.endswith("ma_structured"):
        return gv.unstructured(c["f"], c["bin_edges"], c["pos"],
                               str(c["estimator_type"]), str(c["distance_type"]))
    if name.endswith("_directional"):
        return gv.directional(c["f"], c["bin_edges"], c["pos"], c["direction"],
                              float(c["angles_tol"]), float(c["bandwidth"]),
                              bool(c["separate_dirs"]), str(c["estimator_type"]))
    if name.endswith("_ma_structured"):
        return gv.ma_structured(c["f"], c["mask"], str(c["estimator_type"]))
    return gv.structured(c["f"], str(c["estimator_type"]))


def _np_unstructured(f, edges, pos, est):
    f = np.atleast_2d(f)
    d = np.sqrt(((pos[:, :, None] - pos[:, None, :]) ** 2).sum(axis=0))
    j, k = np.triu_indices(pos.shape[1], 1)
    dist = d[j, k]
    g = np.zeros(len(edges) - 1)
    c = np.zeros(len(edges) - 1, dtype=np.int64)
    for i in range(len(edges) - 1):
        sel = (dist >= edges[i]) & (dist < edges[i + 1])
        diff = f[:, k[sel]] - f[:, j[sel]]
        diff = diff[~np.isnan(diff)]
        c[i] = diff.size
        g[i] = (diff ** 2).sum() if est == "m" else np.sqrt(np.abs(diff)).sum()
    cnt = np.maximum(c, 1).astype(float)
    if est == "m":
        return g / (2 * cnt), c
    return 0.5 * (g / cnt) ** 4 / (0.457 + 0.494 / cnt + 0.045 / cnt ** 2), c


def test_fixtures_cover_all_kernels(ref_goldens):
    names = _cases(ref_goldens)
    kinds = {n.split("_", 2)[2] for n in names}
    assert kinds == {"unstructured", "directional", "structured", "ma_structured"}
    c = ref_goldens.case(names[0])
    np.testing.assert_allclose(c["vario"][:2], [0.4917, 0.7625], atol=5e-5)


@pytest.mark.parametrize("est", ["m", "c"])
def test_oracle_matches_numpy_witness(est):
    rng = np.random.RandomState(7)
    pos = rng.uniform(0, 10, size=(2, 150))
    pos[:, :40] = np.round(pos[:, :40])   # distances on integer edges too
    f = rng.normal(size=(2, 150))
    f[0, ::13] = np.nan
    edges = np.arange(0.0, 9.0, 1.0)
    g, c = oracle.c_vario_unstructured(f, edges, pos, est)
    g2, c2 = _np_unstructured(f, edges, pos, est)
    np.testing.assert_array_equal(c, c2)
    np.testing.assert_allclose(g, g2, rtol=1e-12)


def test_oracle_reproduces_recorded_cases(ref_goldens):
    for name in _cases(ref_goldens):
        c = ref_goldens.case(name)
        res = _call_oracle(name, c)
        if isinstance(res, tuple):
            np.testing.assert_array_equal(res[0], c["vario"])
            np.testing.assert_array_equal(res[1], c["counts"])
        else:
            np.testing.assert_array_equal(res, c["vario"])


def test_reference_tests_pass_with_the_oracle():
    """The reference's own variogram and kriging test files, run with the C
    oracle standing in for gstools-cython."""
    if not reference_import.available():
        pytest.skip("reference tree not present")
    cmd = [sys.executable, os.path.join(HERE, "golden", "run_reference_tests.py"),
           "test_variogram_unstructured.py", "test_variogram_structured.py",
           "test_krige.py", "test_condition.py"]
    cmd += ["-k", " and ".join(f"not {t}" for t in MCMC_DEPENDENT)]
    res = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stdout[-3000:]


def test_hook_routes_variograms_and_restores():
    if not reference_import.available():
        pytest.skip("reference tree not present")
    reference_import.import_gstools()
    import gstools.variogram.variogram as vv

    import gstools_gb300 as gg

    names = ("_unstructured", "_directional", "_structured", "_ma_structured")
    before = {n: getattr(vv, n) for n in names}
    gg.install()
    try:
        for n in names:
            assert getattr(vv, n).__module__ == "gstools_gb300.hook"
    finally:
        gg.uninstall()
    for n, fct in before.items():
        assert getattr(vv, n) is fct


@pytest.mark.gpu
def test_gpu_matches_recorded_cases(cuda_lib, ref_goldens):
    for name in _cases(ref_goldens):
        c = ref_goldens.case(name)
        res = _call_gpu(name, c)
        if isinstance(res, tuple):
            np.testing.assert_array_equal(res[1], c["counts"], err_msg=name)
            np.testing.assert_allclose(res[0], c["vario"], rtol=REL, atol=0,
                                       err_msg=name)
        else:
            np.testing.assert_allclose(res, c["vario"], rtol=REL, atol=0,
                                       err_msg=name)


def test_fp32_distance_error_bound():
    """The fast variogram kernel's squared distance, emulated in numpy
    float32 (hi + lo coordinate splits, the kernel's operation order):
    within B = 2^-21 d2 + 2^-44 X sqrt(d2) + 2^-90 X^2 of the FP64 value
    (X the largest |coordinate|), on clouds from 1e-6 to 1e12 with close
    and far pairs; the kernel's guard is at least 4 B."""
    f32 = np.float32
    rng = np.random.default_rng(7)
    worst = 0.0
    for trial in range(400):
        off = 10.0 ** rng.uniform(-6, 12)
        spread = off * 10.0 ** rng.uniform(-12, 1) + 1e-3 * rng.uniform()
        dim = int(rng.integers(1, 4))
        xj = off + spread * rng.uniform(-1, 1, (dim, 500))
        xk = off + spread * rng.uniform(-1, 1, (dim, 500))
        if trial % 3 == 0:
            xk = xj + spread * 1e-6 * rng.uniform(-1, 1, (dim, 500))
        hj, hk = xj.astype(f32), xk.astype(f32)
        lj = (xj - hj.astype(np.float64)).astype(f32)
        lk = (xk - hk.astype(np.float64)).astype(f32)
        dx = ((hj - hk) + (lj - lk)).astype(f32)
        f2 = (dx[0] * dx[0]).astype(f32)
        for d in range(1, dim):   # fmaf: one rounding of the exact sum
            f2 = (f2.astype(np.float64) + dx[d].astype(np.float64) ** 2).astype(f32)
        d2 = np.zeros(xj.shape[1])
        for d in range(dim):
            d2 = d2 + (xj[d] - xk[d]) ** 2
        big_x = max(np.abs(hj).max(), np.abs(hk).max())
        bound = 2.0**-21 * d2 + 2.0**-44 * big_x * np.sqrt(d2) + 2.0**-90 * big_x**2
        ok = d2 > 0
        if ok.any():
            err = np.abs(f2.astype(np.float64) - d2)[ok] / bound[ok]
            worst = max(worst, float(err.max()))
    assert 0.0 < worst <= 1.0, worst


def test_angle_boundary_double_double():
    """cos of the rounding boundary of the angle tolerance (host code of the
    library, no device): against 200-bit arithmetic, and the decisions it
    gives on the 45-degree lattice pairs equal the host libm's acos test."""
    import ctypes
    import math

    mpmath = pytest.importorskip("mpmath")
    from gstools_gb300 import _native

    lib = _native.load()
    mpmath.mp.prec = 200
    hi, lo = ctypes.c_double(), ctypes.c_double()
    for tol in (math.pi / 4, math.pi / 8, 0.3, math.pi / 2, 1e-5, 1.9, 0.05):
        assert lib.gst_vario_angle_boundary(tol, ctypes.byref(hi), ctypes.byref(lo)) == 0
        b = mpmath.mpf(tol) - (mpmath.mpf(tol) - mpmath.mpf(math.nextafter(tol, 0.0))) / 2
        assert abs(mpmath.mpf(hi.value) + mpmath.mpf(lo.value) - mpmath.cos(b)) < 1e-31
    lib.gst_vario_angle_boundary(math.pi / 4, ctypes.byref(hi), ctypes.byref(lo))
    for k in range(1, 40):
        tt = k / math.sqrt(2.0 * k * k)
        gpu_rule = tt > hi.value or (tt == hi.value and lo.value < 0.0)
        assert gpu_rule == (tt >= 1.0 or math.acos(tt) < math.pi / 4), k
    # tol <= 0 or NaN: only tt >= 1 passes; tol > 2: everything passes
    for tol in (0.0, -1.0, float("nan")):
        lib.gst_vario_angle_boundary(tol, ctypes.byref(hi), ctypes.byref(lo))
        assert not (1.0 - 2**-53 > hi.value) and (1.0 > hi.value or lo.value < 0.0)
    lib.gst_vario_angle_boundary(2.5, ctypes.byref(hi), ctypes.byref(lo))
    assert 0.0 > hi.value


@pytest.mark.gpu
@pytest.mark.parametrize("dim,n,f_max,est", [
    (1, 1, 1, "m"), (1, 500, 1, "c"), (2, 3000, 2, "m"), (3, 2000, 3, "c"),
    (2, 129, 1, "m")])
def test_gpu_unstructured_random(cuda_lib, dim, n, f_max, est):
    import gstools_gb300.variogram as gv

    rng = np.random.RandomState(dim * 1000 + n)
    pos = rng.uniform(0, 30, size=(dim, n))
    pos[:, : n // 3] = np.round(pos[:, : n // 3])   # exact edge hits
    f = rng.normal(size=(f_max, n))
    if n > 10:
        f[0, ::11] = np.nan
    edges = np.concatenate(([-1.0, 0.0], np.arange(1.0, 25.0, 1.0), [25.0, 25.0, 40.0]))
    g, c = gv.unstructured(f, edges, pos, est)
    go, co = oracle.c_vario_unstructured(f, edges, pos, est)
    np.testing.assert_array_equal(c, co)
    np.testing.assert_allclose(g, go, rtol=REL, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["offset", "close_far_out", "bins1024", "bins1025"])
def test_gpu_unstructured_fp32_distance_guard(cuda_lib, case):
    """The FP32 squared distance and its guard: integer coordinates far from
    the origin (every pair distance that is an integer hits an integer edge
    exactly), tiny distances between points at 3e8 (the quadratic guard
    term), and the 1024-bin limit of the fast kernel and one bin past it
    (the general kernel).  Counts exact, sums within 1e-12."""
    import gstools_gb300.variogram as gv

    rng = np.random.RandomState(77)
    n = 1500
    if case == "offset":
        pos = 1.0e6 + np.round(rng.uniform(0, 40, size=(2, n)))
        edges = np.arange(0.0, 31.0)
    elif case == "close_far_out":
        base = 3.0e8 + rng.uniform(0, 1, size=(3, 1))
        pos = base + np.round(rng.uniform(-5, 5, size=(3, n))) * 2.0 ** -22
        edges = np.arange(0.0, 12.0) * 2.0 ** -22
    else:
        nb = 1024 if case == "bins1024" else 1025
        pos = rng.uniform(0, 100, size=(3, n))
        pos[:, : n // 2] = np.round(pos[:, : n // 2])
        edges = np.linspace(0.0, 100.0, nb + 1)
    f = rng.normal(size=(1, n))
    g, c = gv.unstructured(f, edges, pos, "m")
    go, co = oracle.c_vario_unstructured(f, edges, pos, "m")
    assert co.sum() > 0
    np.testing.assert_array_equal(c, co)
    np.testing.assert_allclose(g, go, rtol=REL, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(512, 33), (513, 7), (2, 1), (300, 64)])
def test_gpu_structured_tiled_limits(cuda_lib, shape):
    """Axis variogram at the tiled kernel's row limit (512 rows in shared
    memory), one row past it (per-lag kernel), a single lag, and whole
    32-column blocks; with and without a mask, both estimators."""
    import gstools_gb300.variogram as gv

    rng = np.random.RandomState(shape[0])
    fld = rng.normal(size=shape) + 3.0
    mask = rng.uniform(size=shape) < 0.2
    for est in ("m", "c"):
        np.testing.assert_allclose(gv.structured(fld, est),
                                   oracle.c_vario_structured(fld, est), rtol=REL)
        np.testing.assert_allclose(gv.ma_structured(fld, mask, est),
                                   oracle.c_vario_structured(fld, est, mask=mask),
                                   rtol=REL)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["grid45", "random", "offset", "fallback_tol0",
                                  "fallback_cells"])
def test_gpu_directional_fast_path(cuda_lib, case):
    """Directional estimator on the FP32 fast path: an integer grid with the
    angle tolerance exactly pi/4 from the axis directions (pairs on the
    tolerance cone are decided in FP64 the reference's way), random points
    with several tolerances and bandwidths, points far from the origin; and
    the general kernel for a zero tolerance and for more than 1024
    histogram cells."""
    import gstools_gb300.variogram as gv

    rng = np.random.RandomState(len(case))
    if case == "grid45":
        g1 = np.arange(20.0)
        pos = np.array(np.meshgrid(g1, g1, indexing="ij")).reshape(2, -1)
        dirs = np.array([[1.0, 0.0], [0.0, 1.0]])
        runs = [(np.pi / 4, -1.0), (np.pi / 4, 1.0), (np.pi / 8, 2.0)]
        edges = np.arange(0.0, 15.0, 1.0)
    elif case in ("random", "offset"):
        pos = rng.uniform(0, 40, size=(3, 1200))
        if case == "offset":
            pos += 1e6
        dirs = rng.normal(size=(4, 3))
        dirs /= np.linalg.norm(dirs, axis=1)[:, None]
        runs = [(0.3, -1.0), (0.7, 5.0), (np.pi, 3.0), (np.pi / 2, -1.0)]
        edges = np.linspace(0.0, 30.0, 21)
    elif case == "fallback_tol0":
        pos = rng.uniform(0, 10, size=(2, 300))
        dirs = np.array([[1.0, 0.0]])
        runs = [(0.0, -1.0)]
        edges = np.linspace(0.0, 10.0, 11)
    else:
        pos = rng.uniform(0, 10, size=(2, 300))
        dirs = np.array([[1.0, 0.0], [0.0, 1.0]])
        runs = [(0.4, -1.0)]
        edges = np.linspace(0.0, 10.0, 514)   # 2 x 513 cells
    f = rng.normal(size=(1, pos.shape[1]))
    f[0, ::13] = np.nan
    for tol, bw in runs:
        for separate in (False, True):
            g, c = gv.directional(f, edges, pos, dirs, tol, bw, separate, "m")
            go, co = oracle.c_vario_directional(f, edges, pos, dirs, tol, bw,
                                                separate, "m")
            np.testing.assert_array_equal(c, co, err_msg=f"{tol} {bw} {separate}")
            np.testing.assert_allclose(g, go, rtol=REL, atol=0)


@pytest.mark.gpu
@pytest.mark.parametrize("separate", [False, True])
def test_gpu_directional_random(cuda_lib, separate):
    import gstools_gb300.variogram as gv

    rng = np.random.RandomState(11)
    g1 = np.arange(12.0)
    pos = np.array(np.meshgrid(g1, g1, g1[:6], indexing="ij")).reshape(3, -1)
    f = rng.normal(size=(1, pos.shape[1]))
    dirs = np.array([[1.0, 0, 0], [0, 1.0, 0], [1.0, 1.0, 0]])
    dirs /= np.linalg.norm(dirs, axis=1)[:, None]
    edges = np.arange(0.0, 10.0, 1.5)
    for bw in (-1.0, 0.5):
        g, c = gv.directional(f, edges, pos, dirs, np.pi / 8, bw, separate, "m")
        go, co = oracle.c_vario_directional(f, edges, pos, dirs, np.pi / 8, bw,
                                            separate, "m")
        np.testing.assert_array_equal(c, co)
        np.testing.assert_allclose(g, go, rtol=REL, atol=0)


@pytest.mark.gpu
def test_gpu_haversine_and_structured(cuda_lib):
    import gstools_gb300.variogram as gv

    rng = np.random.RandomState(5)
    latlon = np.array([rng.uniform(-80, 80, 700), rng.uniform(-180, 180, 700)])
    f = rng.normal(size=700)
    edges = np.linspace(0.0, 1.5, 16)
    g, c = gv.unstructured(f, edges, latlon, "m", "h")
    go, co = oracle.c_vario_unstructured(f, edges, latlon, "m", "h")
    np.testing.assert_array_equal(c, co)
    np.testing.assert_allclose(g, go, rtol=1e-11, atol=0)
    fld = rng.normal(size=(50, 40, 30))
    mask = rng.uniform(size=fld.shape) < 0.1
    for est in ("m", "c"):
        np.testing.assert_allclose(gv.structured(fld, est),
                                   oracle.c_vario_structured(fld, est), rtol=REL)
        np.testing.assert_allclose(gv.ma_structured(fld, mask, est),
                                   oracle.c_vario_structured(fld, est, mask=mask),
                                   rtol=REL)
    np.testing.assert_array_equal(gv.structured(np.ones(1)), [0.0])
    g0, c0 = gv.unstructured(np.zeros((1, 0)), edges, np.zeros((2, 0)))
    assert not g0.any() and not c0.any()
