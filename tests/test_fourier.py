"""The Fourier generator (src/gstools/field/generator.py:595-919).

CPU: the oracle reproduces the reference's own goldens
(tests/test_fouriergen.py:47-57) from the fixture inputs, and the mirror
``Fourier`` draws the same wave-vector grid, amplitudes and spectrum factors
as the reference for the same seed; setter and argument semantics.
GPU: ``SRF(model, generator="Fourier")`` on structured 1-D / 2-D / 3-D grids
reproduces the reference's fields (FP64 bar max|diff| <= 1e-12 max|ref|, the
literal goldens to 7 places), is periodic, and the tensor-core grid path
(precision="mixed") keeps the mixed-precision bar.
"""

import numpy as np
import pytest

import gstools_gb300 as gg
import oracle

F64_REL = 1e-12
DIMS = (1, 2, 3)


def _case(ref_goldens, d):
    c = ref_goldens.case(f"fourier_{d}d")
    axes = [c[f"axis{i}"] for i in range(d)]
    model = gg.Gaussian(dim=d, var=float(c["var"]), len_scale=float(c["len_scale"]))
    return c, axes, model


@pytest.mark.parametrize("d", DIMS)
def test_oracle_reproduces_fourier_goldens(ref_goldens, d):
    c, axes, _ = _case(ref_goldens, d)
    grid = np.array(np.meshgrid(*axes, indexing="ij")).reshape(d, -1)
    field = oracle.c_summate_fourier(c["spectrum_factor"], c["modes"], c["z1"],
                                     c["z2"], grid).reshape(c["field"].shape)
    np.testing.assert_allclose(field, c["field"], rtol=0,
                               atol=F64_REL * np.abs(c["field"]).max())
    assert round(abs(field[(0,) * d] - float(c["expected"])), 7) == 0


@pytest.mark.parametrize("d", DIMS)
def test_fourier_modes_match_reference(ref_goldens, d):
    c, _, model = _case(ref_goldens, d)
    gen = gg.Fourier(model, period=c["period"], mode_no=c["mode_no"],
                     seed=int(c["seed"]))
    np.testing.assert_array_equal(gen.modes, c["modes"])
    np.testing.assert_array_equal(gen.z_1, c["z1"])
    np.testing.assert_array_equal(gen.z_2, c["z2"])
    np.testing.assert_allclose(gen.spectrum_factor, c["spectrum_factor"],
                               rtol=1e-13, atol=0)
    assert list(gen.mode_no) == list(c["mode_no"])


def test_fourier_setters_and_errors():
    model = gg.Gaussian(dim=2, var=2.0, len_scale=30.0)
    gen = gg.Fourier(model, period=[80, 30], mode_no=[12, 6], seed=1)
    z_before = gen.z_1.copy()
    gen.period = [5, 10]
    np.testing.assert_almost_equal(gen.period, [5.0, 10.0])
    np.testing.assert_array_equal(gen.z_1, z_before)      # same seed, same z
    gen.mode_no = [6, 6]
    np.testing.assert_almost_equal(gen.mode_no, [6, 6])
    assert gen.modes.shape == (2, 36)
    with pytest.raises(ValueError):
        gg.Fourier(model, period=[80, 30], mode_no=[13, 50], seed=1)
    # period / mode_no filled to dim with their last entry
    gen3 = gg.Fourier(gg.Gaussian(dim=3), period=10.0, mode_no=[4, 6], seed=2)
    np.testing.assert_array_equal(gen3.period, [10.0, 10.0, 10.0])
    assert list(gen3.mode_no) == [4, 6, 6]
    # zero variance: zero spectrum factors, zero field without a kernel call
    zero = gg.Fourier(gg.Gaussian(dim=2, var=0.0), period=4.0, mode_no=4, seed=3)
    assert not zero.spectrum_factor.any()
    assert not zero.structured([np.arange(3.0), np.arange(2.0)]).any()
    assert "Fourier" in gg.srf.GENERATOR


@pytest.mark.gpu
@pytest.mark.parametrize("d", DIMS)
def test_srf_fourier_structured_matches_reference(cuda_lib, ref_goldens, d):
    c, axes, model = _case(ref_goldens, d)
    srf = gg.SRF(model, generator="Fourier", mode_no=list(c["mode_no"]),
                 period=list(c["period"]), seed=int(c["seed"]))
    field = srf(tuple(axes), mesh_type="structured")
    ref = c["field"]
    np.testing.assert_allclose(field, ref, rtol=0, atol=F64_REL * np.abs(ref).max())
    assert round(abs(field[(0,) * d] - float(c["expected"])), 7) == 0
    # periodicity (tests/test_fouriergen.py:59-82): the axes span a period
    for ax in range(d):
        first = np.take(field, 0, axis=ax)
        last = np.take(field, -1, axis=ax)
        np.testing.assert_allclose(first, last, rtol=0, atol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("d", (2, 3))
def test_fourier_mixed_tensor_path(cuda_lib, d):
    model = gg.Gaussian(dim=d, var=1.5, len_scale=12.0, anis=[0.7, 0.5][: d - 1],
                        angles=[0.3, 0.1, 0.2][: d * (d - 1) // 2])
    axes = [np.linspace(0.0, 60.0, n) for n in (40, 33, 21)[:d]]
    f64 = gg.Fourier(model, period=60.0, mode_no=[32, 24, 16][:d], seed=5)
    mixed = gg.Fourier(model, period=60.0, mode_no=[32, 24, 16][:d], seed=5,
                       precision="mixed")
    a = f64.structured(axes, add_nugget=False)
    b = mixed.structured(axes, add_nugget=False)
    sigma = np.sqrt(model.var)
    assert np.sqrt(np.mean((a - b) ** 2)) <= 1e-5 * sigma
    assert np.abs(a - b).max() <= 1e-4 * sigma
