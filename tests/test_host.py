"""Host-side mirror of the reference's generator stack (no GPU needed).

The RNG streams, radial samplers and isometrize maps must reproduce the
reference's arrays: bit for bit where the reference uses a closed-form ppf,
to scipy's root-finding tolerance where it inverts a cdf numerically.
"""

import numpy as np
import pytest
from scipy import integrate, stats

import gstools_gb300 as gg
from gstools_gb300.geometric import generate_grid, matrix_isometrize
from gstools_gb300.rng import RNG


def _modes(gen):
    return gen._cov_sample, gen._z_1, gen._z_2


def test_rng_normal_streams(ref_goldens):
    # tests/test_rng.py:20-37
    rng = RNG(19031977)
    z1 = rng.random.normal(size=100)
    z2 = rng.random.normal(size=100)
    np.testing.assert_array_equal(z1, ref_goldens["rng_normal/z1"])
    np.testing.assert_array_equal(z2, ref_goldens["rng_normal/z2"])


def _assert_same_modes(gen, case, exact=True):
    cov, z1, z2 = _modes(gen)
    np.testing.assert_array_equal(z1, case["z1"])
    np.testing.assert_array_equal(z2, case["z2"])
    if exact:
        np.testing.assert_array_equal(cov, case["cov"])
    else:
        np.testing.assert_allclose(cov, case["cov"], rtol=1e-9, atol=0)


def test_randmeth_modes_match_reference(ref_goldens):
    # tests/test_randmeth.py:15-71 setup, replayed through the mirror
    cm1 = gg.Gaussian(dim=1, var=1.5, len_scale=3.5)
    cm2 = gg.Gaussian(dim=2, var=1.5, len_scale=3.5)
    rm1 = gg.RandMeth(cm1, mode_no=100, seed=19031977)
    _assert_same_modes(rm1, ref_goldens.case("randmeth_1d"))
    rm2 = gg.RandMeth(cm2, mode_no=100, seed=19031977)
    _assert_same_modes(rm2, ref_goldens.case("randmeth_2d"))
    rm2.seed = 74893621
    _assert_same_modes(rm2, ref_goldens.case("randmeth_2d_reseed"))
    rm2.mode_no = 800
    _assert_same_modes(rm2, ref_goldens.case("randmeth_2d_800"))


def test_incompr_modes_match_reference(ref_goldens):
    cm = gg.Gaussian(dim=2, var=1.5, len_scale=2.5)
    ir = gg.IncomprRandMeth(cm, mode_no=100, seed=19031977)
    _assert_same_modes(ir, ref_goldens.case("incompr_2d"))
    srf = gg.SRF(cm, mean=(0.5, 0), generator="VectorField", seed=198412031)
    _assert_same_modes(srf.generator, ref_goldens.case("vector_mean"))


def test_srf_generator_modes_match_reference(ref_goldens):
    cm = gg.Gaussian(dim=2, var=0.5, len_scale=1.0)
    srf = gg.SRF(cm, mean=0.3, mode_no=100, generator="IncomprRandMeth",
                 mean_velocity=0.5)
    srf.generator.update(cm, 476356)
    _assert_same_modes(srf.generator, ref_goldens.case("srf_incompr_unstruct"))
    srf.generator.update(cm, 4734654)
    _assert_same_modes(srf.generator, ref_goldens.case("srf_incompr_struct"))


def test_workload_modes_match_reference(workloads):
    # 2-D Gaussian (closed-form ppf): exact
    gen = gg.RandMeth(gg.Gaussian(dim=2, var=1.0, len_scale=10.0),
                      mode_no=1000, seed=20170519)
    _assert_same_modes(gen, workloads.case("gau2d"))


@pytest.mark.slow
def test_workload_modes_inversion_3d(workloads):
    # 3-D Exponential via the reference's numerical inversion path
    model = gg.Exponential(dim=3, var=2.0, len_scale=[20.0, 10.0, 5.0])
    gen = gg.RandMeth(model, mode_no=2000, seed=20170519,
                      sampling="inversion")
    _assert_same_modes(gen, workloads.case("exp3d"), exact=False)
    np.testing.assert_allclose(model.isometrize_matrix,
                               workloads["exp3d/isometrize"], rtol=0,
                               atol=1e-15)


def test_isometrize_matches_reference(workloads):
    model = gg.Gaussian(dim=3, var=1.0, len_scale=16.0, anis=[0.8, 0.6],
                        angles=[0.3, 0.2, 0.1])
    np.testing.assert_allclose(model.isometrize_matrix,
                               workloads["gau3d_grad/isometrize"], rtol=0,
                               atol=1e-15)
    m = gg.Exponential(dim=3, var=2.0, len_scale=[20.0, 10.0, 5.0])
    assert m.len_scale == 20.0
    np.testing.assert_allclose(m.anis, [0.5, 0.25])
    np.testing.assert_allclose(m.isometrize_matrix,
                               workloads["exp3d/isometrize"], atol=1e-15)


@pytest.mark.parametrize("name,model", [
    ("gau3", lambda: gg.Gaussian(dim=3, len_scale=8.0)),
    ("exp3", lambda: gg.Exponential(dim=3, len_scale=20.0)),
    ("exp2", lambda: gg.Exponential(dim=2, len_scale=20.0)),
    ("gau2", lambda: gg.Gaussian(dim=2, len_scale=10.0)),
    ("mat2", lambda: gg.Matern(dim=2, nu=1.5, len_scale=10.0)),
    ("mat3", lambda: gg.Matern(dim=3, nu=1.5, len_scale=10.0)),
])
def test_spectral_law_matches_reference(workloads, name, model):
    m = model()
    r = workloads[f"spectral/{name}/r"]
    assert m.len_rescaled == pytest.approx(
        float(workloads[f"spectral/{name}/len_rescaled"]), rel=1e-15)
    np.testing.assert_allclose(m.spectral_rad_pdf(r),
                               workloads[f"spectral/{name}/pdf"], rtol=1e-13)
    key = f"spectral/{name}/cdf"
    if key in workloads.files:
        np.testing.assert_allclose(m.spectral_rad_cdf(r), workloads[key],
                                   rtol=1e-13, atol=1e-300)


def _numeric_cdf(model):
    def cdf(r):
        r = np.atleast_1d(r)
        out = np.empty_like(r, dtype=float)
        for i, ri in enumerate(r):
            out[i] = integrate.quad(lambda s: model.spectral_rad_pdf(s)[0],
                                    0.0, ri, limit=200)[0]
        return out
    return cdf


@pytest.mark.parametrize("model", [
    gg.Gaussian(dim=3, len_scale=8.0),
    gg.Gaussian(dim=2, len_scale=8.0),
    gg.Exponential(dim=3, len_scale=[20.0, 10.0, 5.0]),
    gg.Exponential(dim=2, len_scale=5.0),
    gg.Matern(dim=2, nu=1.5, len_scale=12.0),
    gg.Matern(dim=3, nu=0.7, len_scale=3.0),
])
def test_analytic_radius_sampler_follows_spectral_law(model):
    """KS test of the exact samplers against the reference's radial law."""
    rad = model.sample_radius(np.random.RandomState(1234), 4000)
    cdf = model.spectral_rad_cdf if model.has_cdf else _numeric_cdf(model)
    if not model.has_cdf:
        rad = rad[:800]
    res = stats.kstest(rad, cdf)
    assert res.pvalue > 1e-3, res


def test_generate_grid_order():
    g = generate_grid([np.arange(2.0), np.arange(3.0) + 10])
    np.testing.assert_array_equal(g[0], [0, 0, 0, 1, 1, 1])
    np.testing.assert_array_equal(g[1], [10, 11, 12, 10, 11, 12])


def test_isometrize_transpose_identity():
    """<k, M x> == <M^T k, x>: the identity the grid kernels rely on."""
    rng = np.random.RandomState(3)
    m = matrix_isometrize(3, [0.4, -0.2, 1.1], [0.7, 0.3])
    k = rng.normal(size=(3, 50))
    x = rng.uniform(0, 100, size=(3, 40))
    np.testing.assert_allclose(k.T @ (m @ x), (m.T @ k).T @ x, rtol=1e-12,
                               atol=1e-10)


def test_generator_argument_errors():
    with pytest.raises(ValueError):
        gg.IncomprRandMeth(gg.Gaussian(dim=1))
    with pytest.raises(ValueError):
        gg.RandMeth(gg.Gaussian(dim=2), sampling="nope")
    rm = gg.RandMeth(gg.Gaussian(dim=2), mode_no=10, seed=1)
    with pytest.raises(ValueError):
        rm.update("not a model")
    with pytest.raises(ValueError):
        gg.RandMeth(gg.Gaussian(dim=2), precision="f16")


def test_zero_var_modes():
    rm = gg.RandMeth(gg.Gaussian(dim=2, var=0.0), mode_no=10, seed=5)
    assert np.all(rm.cov_samples == 0.0)
    out = rm(np.zeros((2, 4)), add_nugget=False)
    np.testing.assert_array_equal(out, np.zeros(4))


def test_reseed_semantics():
    model = gg.Gaussian(dim=2, var=1.0, len_scale=4.0)
    rm = gg.RandMeth(model, mode_no=50, seed=11)
    a = rm.cov_samples.copy()
    rm.update(model, np.nan)  # same model, keep seed: nothing redrawn
    np.testing.assert_array_equal(a, rm.cov_samples)
    rm.update(seed=12)
    assert not np.array_equal(a, rm.cov_samples)
    rm.update(seed=11)
    np.testing.assert_array_equal(a, rm.cov_samples)


def test_summators_refuse_without_gpu():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(RuntimeError):
        gg.summate(np.ones((2, 3)), np.ones(3), np.ones(3), np.ones((2, 4)))
    # every public compute entry point fails loudly: there is no CPU fallback
    import gstools_gb300.variogram as gv

    k, z, x = np.ones((2, 3)), np.ones(3), np.ones((2, 4))
    axes = [np.arange(4.0), np.arange(5.0)]
    calls = [
        lambda: gg.summate(k, z, z, x, precision="mixed"),
        lambda: gg.summate_incompr(k, z, z, x),
        lambda: gg.summate_fourier(z, k, z, z, x),
        lambda: gg.summate_grid(k, z, z, axes, precision="mixed"),
        lambda: gg.summate_incompr_grid(k, z, z, axes, precision="mixed"),
        lambda: gg.summate_fourier_grid(z, k, z, z, axes),
        lambda: gg.calc_field_krige(np.eye(2), np.ones((2, 3)), np.ones(2)),
        lambda: gg.calc_field_krige_and_variance(np.eye(2), np.ones((2, 3)), np.ones(2)),
        lambda: gv.unstructured(np.ones((1, 4)), np.arange(3.0), x),
        lambda: gv.directional(np.ones((1, 4)), np.arange(3.0), x, np.eye(2), 0.3),
        lambda: gv.structured(np.ones((4, 3))),
        lambda: gg.BatchedSummator(2, [3], [4]),
    ]
    for i, call in enumerate(calls):
        with pytest.raises(RuntimeError):
            call()


def test_torch_isometrize_matches_numpy():
    import torch

    from gstools_gb300.grad import isometrize_matrix

    for dim, angles, anis in ((2, [0.7], [0.4]), (3, [0.3, 0.2, 0.1], [0.8, 0.6]),
                              (3, [-1.1, 0.5, 2.0], [1.3, 0.2])):
        ref = matrix_isometrize(dim, angles, anis)
        got = isometrize_matrix(dim, torch.tensor(angles, dtype=torch.float64),
                                torch.tensor(anis, dtype=torch.float64))
        np.testing.assert_allclose(got.numpy(), ref, rtol=0, atol=1e-15)
