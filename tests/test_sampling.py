"""Device-side spectral sampling for ensembles (gst_batch_sample_modes).

CPU: the oracle's Philox4x64-10 matches numpy's own Philox bit generator and
the Random123 known answer; the oracle sampler's amplitudes, directions and
radii follow N(0, 1), the uniform sphere and the models' radial spectral laws
(KS tests, the laws pinned to the reference in test_host.py); a
realization's modes do not depend on the batch around it.
GPU: the device Philox stream is bit-identical to numpy's; the device sampler
matches the oracle to a few ulps (libm and CUDA round log/sin/cos differently
in the last place; bar 1e-13 relative); an ensemble sampled and summed on the
device matches the oracle's sum of the oracle's modes (mixed-precision bar
RMS <= 1e-5 sigma).
"""

import ctypes

import numpy as np
import pytest
from scipy import integrate, stats

import gstools_gb300 as gg
import oracle

MODELS = [
    ("Gaussian", 1, 0.0), ("Gaussian", 2, 0.0), ("Gaussian", 3, 0.0),
    ("Exponential", 2, 0.0), ("Exponential", 3, 0.0),
    ("Matern", 2, 1.5), ("Matern", 3, 0.7), ("Matern", 2, 0.4),
]


def _model(name, dim, nu, len_scale=1.0):
    if name == "Matern":
        return gg.Matern(dim=dim, nu=nu, len_scale=len_scale)
    return getattr(gg, name)(dim=dim, len_scale=len_scale)


def _numeric_cdf(model):
    # log-spaced out to 1e7 / len_rescaled: Matern's radial law has a
    # k^-(1 + 2 nu) tail, heavy for small nu
    r = np.concatenate(([0.0], np.logspace(-7, 7, 200001) / model.len_rescaled))
    pdf = model.spectral_rad_pdf(r)
    cdf = integrate.cumulative_trapezoid(pdf, r, initial=0.0)
    cdf /= cdf[-1]
    return lambda x: np.interp(x, r, cdf)


def test_oracle_philox_matches_numpy_and_known_answer():
    # Random123 known answer: counter 0, key 0
    np.testing.assert_array_equal(
        oracle.c_philox4x64((0, 0, 0, 0), (0, 0)),
        np.array([0x16554d9eca36314c, 0xdb20fe9d672d0fdc, 0xd7e772cee186176b,
                  0x7e68b68aec7ba23b], dtype=np.uint64))
    rng = np.random.RandomState(5)
    for _ in range(20):
        key = rng.randint(0, 2**62, size=2).astype(np.uint64)
        ctr = rng.randint(0, 2**62, size=4).astype(np.uint64)
        bg = np.random.Philox(key=key, counter=ctr)
        ref = bg.random_raw(4)          # numpy increments the counter first
        ctr1 = ctr.copy()
        ctr1[0] += np.uint64(1)
        np.testing.assert_array_equal(oracle.c_philox4x64(ctr1, key), ref)


@pytest.mark.parametrize("name,dim,nu", MODELS)
def test_oracle_sampler_distributions(name, dim, nu):
    model = _model(name, dim, nu, len_scale=3.0)
    n = 6000
    cov, z1, z2 = oracle.c_sample_modes(dim, [n], name, nu, [20240611],
                                        [model.len_rescaled])
    assert stats.kstest(z1, "norm").pvalue > 1e-3
    assert stats.kstest(z2, "norm").pvalue > 1e-3
    rad = np.linalg.norm(cov, axis=0)
    cdf = model.spectral_rad_cdf if model.has_cdf else _numeric_cdf(model)
    assert stats.kstest(rad, cdf).pvalue > 1e-3
    unit = cov / rad
    if dim == 2:
        ang = np.arctan2(unit[1], unit[0])
        assert stats.kstest(ang, stats.uniform(-np.pi, 2 * np.pi).cdf).pvalue > 1e-3
    elif dim == 3:
        assert stats.kstest(unit[2], stats.uniform(-1, 2).cdf).pvalue > 1e-3
    else:
        assert abs(np.mean(np.sign(unit[0]))) < 0.05


def test_oracle_sampler_is_batch_independent():
    counts, seeds, ls = [300, 0, 120, 77], [9, 10, 11, 12], [1.0, 2.0, 3.0, 4.0]
    cov, z1, z2 = oracle.c_sample_modes(3, counts, "Matern", 1.5, seeds, ls)
    alone = oracle.c_sample_modes(3, [120], "Matern", 1.5, [11], [3.0])
    np.testing.assert_array_equal(cov[:, 300:420], alone[0])
    np.testing.assert_array_equal(z1[300:420], alone[1])
    np.testing.assert_array_equal(z2[300:420], alone[2])


def test_sampler_argument_errors():
    with pytest.raises(ValueError):
        oracle.c_sample_modes(2, [10], "Matern", 25.0, [1], [1.0])


@pytest.mark.gpu
def test_device_philox_matches_numpy(cuda_lib):
    import torch

    key = (0x123456789ABCDEF0, 42)
    n = 1000
    out = torch.empty(4 * n, dtype=torch.int64, device="cuda")
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert cuda_lib.gst_philox4x64_fill(key[0], key[1], n, 3,
                                        ctypes.c_void_p(out.data_ptr()), stream) == 0
    got = out.cpu().numpy().view(np.uint64)
    bg = np.random.Philox(key=np.array(key, dtype=np.uint64),
                          counter=np.array([2**64 - 1, 2, 0, 0], dtype=np.uint64))
    np.testing.assert_array_equal(got, bg.random_raw(4 * n))


@pytest.mark.gpu
@pytest.mark.parametrize("name,dim,nu", MODELS)
def test_device_sampler_matches_oracle(cuda_lib, name, dim, nu):
    counts = [1000, 1, 0, 2500, 333]
    seeds = [1, 2**63 + 5, 7, 123456789012345, 99]
    ls = [0.5, 2.0, 3.0, 10.0, 40.0]
    model = _model(name, dim, nu)
    bs = gg.BatchedSummator(dim, counts, [1] * len(counts))
    bs.sample(model, seeds, len_scales=ls)
    ref = oracle.c_sample_modes(dim, counts, name, nu, seeds,
                                np.asarray(ls) / model.rescale)
    for got, want in zip((bs.cov, bs.z1, bs.z2), ref):
        g = got.cpu().numpy()
        np.testing.assert_allclose(g, want, rtol=1e-13, atol=1e-300)


@pytest.mark.gpu
def test_device_sampled_ensemble_matches_oracle_sum(cuda_lib):
    rng = np.random.RandomState(3)
    n_items = 24
    counts = rng.choice([500, 1000, 2000], size=n_items)
    points = rng.randint(100, 3000, size=n_items)
    seeds = rng.randint(1, 2**62, size=n_items).astype(np.uint64)
    ls = np.exp(rng.uniform(np.log(2.0), np.log(50.0), size=n_items))
    model = gg.Matern(dim=2, nu=1.5, var=1.3)
    pos = [rng.uniform(0.0, 500.0, size=(2, p)) for p in points]
    bs = gg.BatchedSummator(2, counts, points, out_dtype="float64")
    bs.sample(model, seeds, len_scales=ls)
    bs.load_points(pos)
    bs.run()
    fields = bs.split()
    cov, z1, z2 = oracle.c_sample_modes(2, counts, "Matern", 1.5, seeds,
                                        ls / model.rescale)
    off = np.concatenate(([0], np.cumsum(counts)))
    for r in range(0, n_items, 5):
        m0, m1 = off[r], off[r + 1]
        ref = np.sqrt(1.3 / counts[r]) * oracle.c_summate(
            cov[:, m0:m1], z1[m0:m1], z2[m0:m1], pos[r])
        d = fields[r] - ref
        assert np.sqrt(np.mean(d ** 2)) <= 1e-5 * np.sqrt(1.3), r
