"""Kriging kernels (gstools-cython's calc_field_krige(_and_variance)).

Fixtures: the arrays the reference's Simple / Ordinary / Universal kriging
(tests/test_krige.py:56-153 setups; Gaussian and Exponential, 1-3 D) hands
to the kernels, recorded by tests/golden/make_golden.py with the C oracle as
the kernel, after checking the reference test's own properties (exact at the
conditions, to 2 places).
CPU: the C oracle against the numpy witness; the hook routes the reference's
kriging wrappers (src/gstools/krige/base.py:42-60) and restores them, and
raises without a GPU.
GPU: field and error variance against the oracle (and the field alone,
computed as V^T (M^T c)), scale-aware FP64 bar:
|diff| <= 1e-12 * sum_i (|c_i| + |v_i|) (|M| |v|)_i per point (a different
summation order than the oracle's; rounding scales with the magnitude of the
terms of both nested sums, not with the result, which cancels for the
ill-conditioned kriging matrices of smooth covariances).
"""

import os
import sys

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import reference_import  # noqa: E402

import gstools_gb300 as gg  # noqa: E402

REL = 1e-12


def _cases(ref_goldens):
    return sorted({k.split("/")[0] for k in ref_goldens.files
                   if k.startswith("krige_")})


def _within(got, want, scale):
    return np.all(np.abs(np.asarray(got) - want) <= REL * scale + 1e-300)


def test_oracle_matches_numpy_witness(ref_goldens):
    names = _cases(ref_goldens)
    assert len(names) == 18
    for name in names:
        c = ref_goldens.case(name)
        f, e = oracle.c_krige(c["mat"], c["vecs"], c["cond"])
        f2, e2, scale = oracle.np_krige(c["mat"], c["vecs"], c["cond"])
        assert _within(f, f2, scale) and _within(e, e2, scale), name
        np.testing.assert_array_equal(f, c["field"])
        np.testing.assert_array_equal(e, c["error"])


def test_hook_routes_kriging_and_restores():
    if not reference_import.available():
        pytest.skip("reference tree not present")
    reference_import.import_gstools()
    import gstools.krige.base as kb

    before = {n: getattr(kb, n) for n in ("_calc_field_krige",
                                          "_calc_field_krige_and_variance")}
    gg.install()
    try:
        for name, fct in before.items():
            assert getattr(kb, name) is not fct
            assert getattr(kb, name).__module__ == "gstools_gb300.hook"
        import torch

        if not torch.cuda.is_available():
            with pytest.raises(RuntimeError):
                kb._calc_field_krige(np.eye(2), np.ones((2, 3)), np.ones(2))
    finally:
        gg.uninstall()
    for name, fct in before.items():
        assert getattr(kb, name) is fct


@pytest.mark.gpu
def test_kernel_matches_reference_fixtures(cuda_lib, ref_goldens):
    for name in _cases(ref_goldens):
        c = ref_goldens.case(name)
        _, _, scale = oracle.np_krige(c["mat"], c["vecs"], c["cond"])
        f, e = gg.calc_field_krige_and_variance(c["mat"], c["vecs"], c["cond"])
        assert _within(f, c["field"], scale), name
        assert _within(e, c["error"], scale), name
        f_only = gg.calc_field_krige(c["mat"], c["vecs"], c["cond"])
        assert _within(f_only, c["field"], scale), name


@pytest.mark.gpu
@pytest.mark.parametrize("k,n", [(1, 1), (63, 64), (64, 65), (65, 1000),
                                 (300, 4097), (7, 20000)])
def test_kernel_matches_oracle_random(cuda_lib, k, n):
    rng = np.random.RandomState(k * 7 + n)
    a = rng.normal(size=(k, k))
    mat = a @ a.T / k + np.eye(k)
    vecs = rng.normal(size=(k, n))
    cond = rng.normal(size=k)
    f, e = gg.calc_field_krige_and_variance(mat, vecs, cond)
    fo, eo = oracle.c_krige(mat, vecs, cond)
    _, _, scale = oracle.np_krige(mat, vecs, cond)
    assert _within(f, fo, scale) and _within(e, eo, scale)
    # field only: V^T (M^T c), another summation order under the same bar
    assert _within(gg.calc_field_krige(mat, vecs, cond), fo, scale)


@pytest.mark.gpu
def test_kernel_torch_and_empty(cuda_lib):
    import torch

    rng = np.random.RandomState(2)
    mat, vecs, cond = rng.normal(size=(5, 5)), rng.normal(size=(5, 77)), rng.normal(size=5)
    f, e = gg.calc_field_krige_and_variance(
        torch.from_numpy(mat).cuda(), torch.from_numpy(vecs).cuda(),
        torch.from_numpy(cond).cuda())
    assert f.is_cuda and e.is_cuda
    fo, eo = oracle.c_krige(mat, vecs, cond)
    _, _, scale = oracle.np_krige(mat, vecs, cond)
    assert _within(f.cpu().numpy(), fo, scale)
    z = gg.calc_field_krige(np.zeros((0, 0)), np.zeros((0, 9)), np.zeros(0))
    np.testing.assert_array_equal(z, np.zeros(9))


def _gauss_kriging_system(rng, k, n, dim=2, ls=3.0, nugget=1e-6):
    """Inverted simple-kriging matrix of a Gaussian covariance (smooth,
    ill-conditioned) and the target covariances, as the reference builds
    them (krige/base.py:280-320)."""
    cond_pos = rng.uniform(0.0, 20.0, size=(k, dim))
    tgt_pos = rng.uniform(0.0, 20.0, size=(n, dim))

    def cov(a, b):
        d2 = ((a[:, None, :] - b[None, :, :]) ** 2).sum(-1)
        return np.exp(-d2 / ls ** 2)

    mat = np.linalg.inv(cov(cond_pos, cond_pos) + nugget * np.eye(k))
    vecs = np.ascontiguousarray(cov(cond_pos, tgt_pos))
    return mat, vecs, rng.normal(size=k)


@pytest.mark.gpu
@pytest.mark.parametrize("kind,n", [("random", 4096), ("kriging", 4096),
                                    ("random", 4003)])
def test_sliced_variance_matches_oracle(cuda_lib, kind, n):
    """Large K^2 n variances run as FP16 tensor-core products of error-free
    FP64 slices: same scale-aware FP64 bar against the oracle (K = 1001 and
    n = 4003 exercise the zero padding of both GEMM dimensions)."""
    rng = np.random.RandomState((17 if kind == "random" else 18) + n)
    k = 1001
    if kind == "random":
        a = rng.normal(size=(k, k))
        mat = a @ a.T / k + np.eye(k)
        vecs = rng.normal(size=(k, n)) * np.exp(rng.uniform(-20, 20, size=(1, n)))
        cond = rng.normal(size=k)
    else:
        mat, vecs, cond = _gauss_kriging_system(rng, k, n)
    assert k * k * n >= 4e9
    f, e = gg.calc_field_krige_and_variance(mat, vecs, cond)
    fo, eo = oracle.c_krige(mat, vecs, cond)
    _, _, scale = oracle.np_krige(mat, vecs, cond)
    assert _within(f, fo, scale)
    assert _within(e, eo, scale), np.max(np.abs(e - eo) / scale)
    again = gg.calc_field_krige_and_variance(mat, vecs, cond)[1]
    np.testing.assert_array_equal(e, again)   # deterministic


@pytest.mark.gpu
def test_sliced_variance_non_finite(cuda_lib):
    rng = np.random.RandomState(19)
    k, n = 1001, 4096
    a = rng.normal(size=(k, k))
    mat = a @ a.T / k + np.eye(k)
    vecs = rng.normal(size=(k, n))
    cond = rng.normal(size=k)
    vecs[5, 7] = np.nan
    e = gg.calc_field_krige_and_variance(mat, vecs, cond)[1]
    assert np.isnan(e[7]) and np.isfinite(np.delete(e, 7)).all()
    vecs[5, 7] = 1.0
    mat[3, 4] = np.inf
    e = gg.calc_field_krige_and_variance(mat, vecs, cond)[1]
    assert np.isnan(e).all()
