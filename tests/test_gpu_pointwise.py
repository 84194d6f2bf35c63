"""GPU parity of the pointwise kernels against the FP64 oracle.

Bars (written into each assertion):
* FP64 kernels: max|gpu - oracle| <= 1e-12 * max|oracle| (the relative
  measure for fields with zero crossings), plus the reference tests' literal
  goldens to 7 places;
* mixed precision: RMS(gpu - oracle) <= 1e-5 * sigma of the scaled field,
  with sigma = sqrt(var) and the field scaled by sqrt(var / N).
"""

import numpy as np
import pytest
import torch

import gstools_gb300 as gg
import oracle

pytestmark = pytest.mark.gpu

F64_REL = 1e-12
MIXED_RMS_SIGMA = 1e-5


def rel_err(got, ref):
    return np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-300)


def rms_sigma(got, ref, n_modes, var=1.0):
    """RMS error of the scaled field, in units of sigma."""
    scale = np.sqrt(var / n_modes)
    return np.sqrt(np.mean((scale * (got - ref)) ** 2)) / np.sqrt(var)


def random_case(seed, dim, n_modes, n_pts, k_scale=0.3, extent=100.0):
    rng = np.random.RandomState(seed)
    cov = rng.standard_t(3, size=(dim, n_modes)) * k_scale
    z1, z2 = rng.normal(size=n_modes), rng.normal(size=n_modes)
    pos = rng.uniform(0.0, extent, size=(dim, n_pts))
    return cov, z1, z2, pos


# ------------------------------------------------------------- goldens --

@pytest.mark.parametrize("name", ["randmeth_1d", "randmeth_2d",
                                  "randmeth_2d_reseed", "randmeth_2d_800"])
def test_randmeth_goldens_f64(cuda_lib, ref_goldens, name):
    c = ref_goldens.case(name)
    summed = gg.summate(c["cov"], c["z1"], c["z2"], c["pos"])
    ref = oracle.c_summate(c["cov"], c["z1"], c["z2"], c["pos"])
    assert rel_err(summed, ref) <= F64_REL
    field = np.sqrt(c["var"] / c["cov"].shape[1]) * summed
    for exp, idx in zip(c["expected"], c["index"]):
        assert round(abs(field[tuple(idx)] - exp), 7) == 0


def test_incompr_golden_f64(cuda_lib, ref_goldens):
    c = ref_goldens.case("incompr_2d")
    summed = gg.summate_incompr(c["cov"], c["z1"], c["z2"], c["pos"])
    ref = oracle.c_summate_incompr(c["cov"], c["z1"], c["z2"], c["pos"])
    assert rel_err(summed, ref) <= F64_REL
    field = (np.array([[1.0], [0.0]])
             + np.sqrt(c["var"] / c["cov"].shape[1]) * summed)
    for exp, idx in zip(c["expected"], c["index"]):
        assert round(abs(field[tuple(idx)] - exp), 7) == 0


def test_randmeth_mirror_end_to_end(cuda_lib):
    # tests/test_randmeth.py:33-41 through the standalone mirror
    x = np.linspace(0.0, 10.0, 10)
    y = np.linspace(-5.0, 5.0, 10)
    rm1 = gg.RandMeth(gg.Gaussian(dim=1, var=1.5, len_scale=3.5), mode_no=100,
                      seed=19031977)
    m = rm1((x,))
    assert round(abs(m[0] - 3.19799030), 7) == 0
    assert round(abs(m[1] - 2.44848295), 7) == 0
    rm2 = gg.RandMeth(gg.Gaussian(dim=2, var=1.5, len_scale=3.5), mode_no=100,
                      seed=19031977)
    m = rm2((x, y))
    assert round(abs(m[0] - 1.67318010), 7) == 0
    assert round(abs(m[1] - 2.12310269), 7) == 0


def test_srf_incompr_end_to_end(cuda_lib):
    # tests/test_srf.py:259-275 and tests/test_incomprrandmeth.py:50-59
    rng = np.random.RandomState(123018)
    xs, ys = rng.uniform(0.0, 10, 100), rng.uniform(0.0, 10, 100)
    srf = gg.SRF(gg.Gaussian(dim=2, var=0.5, len_scale=1.0), mean=0.3,
                 mode_no=100, generator="IncomprRandMeth", mean_velocity=0.5)
    f = srf((xs, ys), seed=476356)
    assert round(abs(f[0, 0] - 1.23693272), 7) == 0
    assert round(abs(f[0, 1] - 0.89242284), 7) == 0
    f = srf((np.linspace(0.0, 12.0, 48), np.linspace(0.0, 10.0, 46)),
            seed=4734654, mesh_type="structured")
    assert round(abs(f[0, 0, 0] - 1.07812013), 7) == 0
    assert round(abs(f[0, 1, 0] - 1.06180674), 7) == 0
    srf = gg.SRF(gg.Gaussian(dim=2, var=1.5, len_scale=2.5), mean=(0.5, 0),
                 generator="VectorField", seed=198412031)
    f = srf.structured((np.linspace(0.0, 10.0, 9), np.linspace(-5.0, 5.0, 16)))
    assert round(abs(np.mean(f[0]) - 1.3025621393180298), 7) == 0
    assert round(abs(np.mean(f[1]) + 0.04729596839446052), 7) == 0


# ------------------------------------------------------ workload parity --

def test_gau2d_full_workload_f64_and_mixed(cuda_lib, workloads):
    """2-D Gaussian, 1000 modes, 100 000 points in [0, 100]^2."""
    c = workloads.case("gau2d")
    pos = np.random.RandomState(20170519).uniform(0.0, 100.0, (2, 100_000))
    np.testing.assert_array_equal(pos[:, :4096], c["pos_head"])
    ref = oracle.c_summate(c["cov"], c["z1"], c["z2"], pos)
    np.testing.assert_array_equal(ref[:4096], c["summed_head"])
    got = gg.summate(c["cov"], c["z1"], c["z2"], pos)
    assert rel_err(got, ref) <= F64_REL
    mixed = gg.summate(c["cov"], c["z1"], c["z2"], pos, precision="mixed")
    assert rms_sigma(mixed, ref, 1000) <= MIXED_RMS_SIGMA
    assert rel_err(mixed, ref) <= 1e-5


def test_exp3d_grid_subsample(cuda_lib, workloads):
    """3-D anisotropic Exponential: grid entry points vs the oracle on the
    isometrized, materialised sub-grid."""
    c = workloads.case("exp3d")
    axes = [c["sub_x"], c["sub_y"], c["sub_z"]]
    kprime = c["isometrize"].T @ c["cov"]
    ref = c["summed_sub"].reshape([len(a) for a in axes])
    got = gg.summate_grid(kprime, c["z1"], c["z2"], axes)
    assert rel_err(got, ref) <= F64_REL
    mixed = gg.summate_grid(kprime, c["z1"], c["z2"], axes, precision="mixed")
    assert rms_sigma(mixed, ref, 2000, var=2.0) <= MIXED_RMS_SIGMA
    grid = np.array(np.meshgrid(*axes, indexing="ij")).reshape(3, -1)
    pw = gg.summate(c["cov"], c["z1"], c["z2"], c["isometrize"] @ grid)
    assert rel_err(pw, ref.ravel()) <= F64_REL


def test_incompr3d_grid_subsample(cuda_lib, workloads):
    c = workloads.case("incompr3d")
    axes = [c["sub_x"], c["sub_y"], c["sub_z"]]
    ref = c["summed_sub"].reshape((3,) + tuple(len(a) for a in axes))
    got = gg.summate_incompr_grid(c["cov"], c["z1"], c["z2"], axes)
    assert rel_err(got, ref) <= F64_REL
    mixed = gg.summate_incompr_grid(c["cov"], c["z1"], c["z2"], axes,
                                    precision="mixed", out_dtype="float32")
    assert mixed.dtype == np.float32
    assert rms_sigma(mixed.astype(np.float64), ref, 2000) <= MIXED_RMS_SIGMA


def test_incompressible_divergence_free(cuda_lib, workloads):
    """Central differences of the FP64 field: div u = O(h^2)."""
    c = workloads.case("incompr3d")
    h = 1e-3
    base = np.array([[10.0, 20.0, 30.0], [55.5, 3.25, 100.0]]).T  # (3, 2)
    div = np.zeros(base.shape[1])
    for d in range(3):
        e = np.zeros((3, 1))
        e[d] = h
        up = gg.summate_incompr(c["cov"], c["z1"], c["z2"], base + e)
        dn = gg.summate_incompr(c["cov"], c["z1"], c["z2"], base - e)
        div += (up[d] - dn[d]) / (2 * h)
    ref = gg.summate_incompr(c["cov"], c["z1"], c["z2"], base)
    kmax = np.max(np.linalg.norm(c["cov"], axis=0))
    assert np.max(np.abs(div)) <= 1e-5 * np.max(np.abs(ref)) * max(kmax, 1.0)


# ----------------------------------------------------------- edge cases --

@pytest.mark.parametrize("dim", [1, 2, 3, 4])
@pytest.mark.parametrize("n_modes,n_pts", [(1, 1), (129, 257), (1000, 3001),
                                           (300, 70_000)])
def test_random_shapes_f64(cuda_lib, dim, n_modes, n_pts):
    cov, z1, z2, pos = random_case(dim * 100 + n_modes, dim, n_modes, n_pts)
    ref = oracle.c_summate(cov, z1, z2, pos)
    got = gg.summate(cov, z1, z2, pos)
    assert got.shape == (n_pts,)
    assert rel_err(got, ref) <= F64_REL


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("n_modes,n_pts", [(1, 1), (257, 1025), (2000, 5003)])
def test_random_shapes_mixed(cuda_lib, dim, n_modes, n_pts):
    cov, z1, z2, pos = random_case(dim * 7 + n_modes, dim, n_modes, n_pts,
                                   extent=500.0)
    ref = oracle.c_summate(cov, z1, z2, pos)
    got = gg.summate(cov, z1, z2, pos, precision="mixed")
    assert rms_sigma(got, ref, n_modes) <= MIXED_RMS_SIGMA
    got32 = gg.summate(cov, z1, z2, pos, precision="mixed", out_dtype="float32")
    assert got32.dtype == np.float32
    assert rms_sigma(got32.astype(np.float64), ref, n_modes) <= MIXED_RMS_SIGMA


@pytest.mark.parametrize("dim", [2, 3])
def test_random_incompr_f64_and_mixed(cuda_lib, dim):
    cov, z1, z2, pos = random_case(dim, dim, 777, 9001)
    ref = oracle.c_summate_incompr(cov, z1, z2, pos)
    got = gg.summate_incompr(cov, z1, z2, pos)
    assert got.shape == (dim, 9001)
    assert rel_err(got, ref) <= F64_REL
    mixed = gg.summate_incompr(cov, z1, z2, pos, precision="mixed")
    assert rms_sigma(mixed, ref, 777) <= MIXED_RMS_SIGMA


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_fourier_f64(cuda_lib, dim):
    cov, z1, z2, pos = random_case(40 + dim, dim, 500, 2001)
    fac = np.random.RandomState(dim).uniform(0.1, 2.0, size=500)
    ref = oracle.c_summate_fourier(fac, cov, z1, z2, pos)
    got = gg.summate_fourier(fac, cov, z1, z2, pos)
    assert rel_err(got, ref) <= F64_REL


def test_large_phases_f64_and_mixed(cuda_lib):
    """Heavy-tailed wave numbers on a 5000-wide domain: phases ~1e5 rad."""
    cov, z1, z2, pos = random_case(99, 2, 500, 4000, k_scale=2.0,
                                   extent=5000.0)
    ref = oracle.c_summate(cov, z1, z2, pos)
    assert rel_err(gg.summate(cov, z1, z2, pos), ref) <= F64_REL
    mixed = gg.summate(cov, z1, z2, pos, precision="mixed")
    assert rms_sigma(mixed, ref, 500) <= MIXED_RMS_SIGMA


def test_empty_inputs(cuda_lib):
    out = gg.summate(np.zeros((2, 0)), np.zeros(0), np.zeros(0),
                     np.ones((2, 7)))
    np.testing.assert_array_equal(out, np.zeros(7))
    out = gg.summate(np.ones((3, 5)), np.ones(5), np.ones(5), np.zeros((3, 0)))
    assert out.shape == (0,)
    out = gg.summate_incompr(np.zeros((3, 0)), np.zeros(0), np.zeros(0),
                             np.ones((3, 4)), precision="mixed")
    np.testing.assert_array_equal(out, np.zeros((3, 4)))


def test_invalid_arguments_raise(cuda_lib):
    with pytest.raises(ValueError):
        gg.summate(np.ones((5, 3)), np.ones(3), np.ones(3), np.ones((5, 2)))
    with pytest.raises(ValueError):
        gg.summate(np.ones((4, 3)), np.ones(3), np.ones(3), np.ones((4, 2)),
                   precision="mixed")
    with pytest.raises(ValueError):
        gg.summate_incompr(np.ones((1, 3)), np.ones(3), np.ones(3),
                           np.ones((1, 2)))
    with pytest.raises(ValueError):
        gg.summate(np.ones((2, 3)), np.ones(2), np.ones(3), np.ones((2, 2)))


def test_torch_inputs_stay_on_device(cuda_lib):
    cov, z1, z2, pos = random_case(5, 3, 300, 1000)
    t = [torch.from_numpy(a).cuda() for a in (cov, z1, z2, pos)]
    out = gg.summate(*t)
    assert isinstance(out, torch.Tensor) and out.is_cuda
    ref = oracle.c_summate(cov, z1, z2, pos)
    assert rel_err(out.cpu().numpy(), ref) <= F64_REL


def test_deterministic_repeat(cuda_lib):
    cov, z1, z2, pos = random_case(8, 2, 1500, 20_000)
    a = gg.summate(cov, z1, z2, pos)
    b = gg.summate(cov, z1, z2, pos)
    np.testing.assert_array_equal(a, b)


def test_no_device_error_recorded(cuda_lib):
    from gstools_gb300 import _native

    assert _native.read_device_error() == 0


def test_hook_drives_installed_summators(cuda_lib, ref_goldens):
    """install() on a stand-in of gstools.field.generator: the rebound
    globals are called exactly as RandMeth.__call__ calls them
    (generator.py:266-270) and reproduce the reference goldens."""
    import types

    mod = types.SimpleNamespace(_summate=None, _summate_incompr=None,
                                _summate_fourier=None)
    gg.install(mod)
    try:
        c = ref_goldens.case("randmeth_2d")
        summed = mod._summate(c["cov"], c["z1"], c["z2"], c["pos"], None)
        field = np.sqrt(c["var"] / c["cov"].shape[1]) * summed
        for exp, idx in zip(c["expected"], c["index"]):
            assert round(abs(field[tuple(idx)] - exp), 7) == 0
        c = ref_goldens.case("incompr_2d")
        summed = mod._summate_incompr(c["cov"], c["z1"], c["z2"], c["pos"], 4)
        ref = oracle.c_summate_incompr(c["cov"], c["z1"], c["z2"], c["pos"])
        assert rel_err(summed, ref) <= F64_REL
    finally:
        gg.uninstall(mod)
    assert mod._summate is None
