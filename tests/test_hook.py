"""The drop-in hook into an unmodified GSTools (CPU side).

``gstools_gb300.install()`` must rebind the three module globals the
reference resolves at call time (src/gstools/field/generator.py:42-75,
266, 554, 682) and ``uninstall()`` must restore them.  Without a GPU the
installed summators must raise instead of falling back to a CPU path.
"""

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import reference_import  # noqa: E402

import gstools_gb300 as gg  # noqa: E402


@pytest.fixture(scope="module")
def gen_module():
    if not reference_import.available():
        pytest.skip("reference tree not present")
    gs = reference_import.import_gstools()
    import gstools.field.generator as gen

    assert gs is not None
    return gen


def test_install_rebinds_and_uninstall_restores(gen_module):
    before = {n: getattr(gen_module, n) for n in
              ("_summate", "_summate_incompr", "_summate_fourier")}
    gg.install(gen_module)
    try:
        for name, fct in before.items():
            assert getattr(gen_module, name) is not fct
            assert getattr(gen_module, name).__module__ == "gstools_gb300.hook"
    finally:
        gg.uninstall(gen_module)
    for name, fct in before.items():
        assert getattr(gen_module, name) is fct


def test_installed_srf_has_no_cpu_fallback(gen_module):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    import gstools

    gg.install(gen_module)
    try:
        srf = gstools.SRF(gstools.Gaussian(dim=2, var=1.0, len_scale=4.0),
                          mode_no=50)
        with pytest.raises(RuntimeError):
            srf((np.arange(5.0), np.arange(5.0)), seed=3)
    finally:
        gg.uninstall(gen_module)


def test_install_rejects_unknown_precision(gen_module):
    with pytest.raises(ValueError):
        gg.install(gen_module, precision="fp16")


# --------------------------------------------------- structured routing --

def _grid_points(axes):
    return np.array(np.meshgrid(*axes, indexing="ij"),
                    dtype=np.float64).reshape(len(axes), -1)


@pytest.fixture
def grid_spy(gen_module, monkeypatch):
    """Stand-ins for the grid kernels behind ``summate_structured``: they
    record what reaches them and evaluate it in FP64 on the CPU from the
    *mapped* wave vectors on the raw (unisometrized) meshgrid -- the C
    oracle for scalar and Fourier sums, numpy for the incompressible sum
    with its separate projector vectors."""
    import oracle
    from gstools_gb300 import summator

    calls = []

    def grid(cov, z1, z2, axes, *, precision=None, method="auto",
             out_dtype=None, scale=1.0):
        calls.append(("scalar", np.array(cov), axes, precision))
        pts = _grid_points(axes)
        out = oracle.c_summate(cov, z1, z2, pts) * scale
        return out.reshape([len(a) for a in axes])

    def grid_incompr(cov, z1, z2, axes, *, precision=None, out_dtype=None,
                     scale=1.0, method="auto", proj_cov=None):
        calls.append(("incompr", np.array(cov), axes, precision))
        pc = cov if proj_cov is None else np.asarray(proj_cov)
        pts = _grid_points(axes)
        ph = cov.T @ pts
        amp = z1[:, None] * np.cos(ph) + z2[:, None] * np.sin(ph)
        k2 = np.sum(pc * pc, axis=0)
        proj = (np.eye(len(axes))[:, :1] - pc * pc[0] / k2)
        out = (proj @ amp) * scale
        return out.reshape([len(axes)] + [len(a) for a in axes])

    def grid_fourier(fac, modes, z1, z2, axes, *, out_dtype=None, scale=1.0):
        calls.append(("fourier", np.array(modes), axes, None))
        pts = _grid_points(axes)
        out = oracle.c_summate_fourier(fac, modes, z1, z2, pts) * scale
        return out.reshape([len(a) for a in axes])

    monkeypatch.setattr(summator, "summate_grid", grid)
    monkeypatch.setattr(summator, "summate_incompr_grid", grid_incompr)
    monkeypatch.setattr(summator, "summate_fourier_grid", grid_fourier)
    return calls


def _hooked(gen_module, make, call, precision):
    gg.install(precision=precision)
    try:
        return call(make())
    finally:
        gg.uninstall()


def test_structured_srf_reaches_grid_kernels_with_mapped_wave_vectors(
        gen_module, grid_spy):
    import gstools

    axes = (np.linspace(0.0, 9.0, 7), np.linspace(-3.0, 4.0, 6),
            np.linspace(1.0, 5.0, 5))
    model = gstools.Exponential(dim=3, var=2.0, len_scale=[4.0, 3.0, 2.0],
                                angles=[0.4, 0.2, 0.1], nugget=0.1)
    make = lambda: gstools.SRF(model, mean=0.5, mode_no=64, seed=9,
                               sampling="inversion")
    ref_srf = make()
    ref = ref_srf.structured(axes)
    for prec in ("f64", "mixed"):
        grid_spy.clear()
        srf = make()
        gg.install(precision=prec)
        try:
            got = srf.structured(axes)
        finally:
            gg.uninstall()
        # one grid call with M^T k on the raw axes, no meshgrid
        assert len(grid_spy) == 1
        kind, cov, ax, p = grid_spy[0]
        m = model.isometrize(np.eye(3))
        assert kind == "scalar" and p == prec
        np.testing.assert_array_equal(cov, m.T @ srf.generator._cov_sample)
        for a, b in zip(ax, axes):
            np.testing.assert_array_equal(a, b)
        # the reference's reshape, scaling, nugget and mean are applied as on
        # its own meshgrid path
        assert got.shape == ref.shape == (7, 6, 5)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
        assert srf.pos[0] is not None and srf.mesh_type == "structured"


def test_structured_vector_and_fourier_fields_route(gen_module, grid_spy):
    import gstools

    axes = (np.linspace(0.0, 10.0, 9), np.linspace(-5.0, 5.0, 8))
    model = gstools.Gaussian(dim=2, var=1.5, len_scale=2.5, angles=0.3,
                             anis=0.7)
    make_v = lambda: gstools.SRF(model, generator="VectorField", mode_no=50,
                                 seed=198412031, mean_velocity=0.5)
    ref = make_v().structured(axes)
    got = _hooked(gen_module, make_v, lambda s: s.structured(axes), "mixed")
    assert [c[0] for c in grid_spy] == ["incompr"]
    assert got.shape == ref.shape == (2, 9, 8)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())

    grid_spy.clear()
    fmodel = gstools.Gaussian(dim=2, var=2.0, len_scale=30.0)
    fa = (np.linspace(0, 30, 31), np.linspace(0, 30, 17))
    make_f = lambda: gstools.SRF(fmodel, generator="Fourier", mode_no=[6, 6],
                                 period=[30, 30], seed=19900408)
    ref = make_f().structured(fa)
    got = _hooked(gen_module, make_f, lambda s: s.structured(fa), "mixed")
    assert [c[0] for c in grid_spy] == ["fourier"]
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_structured_cond_srf_routes(gen_module, grid_spy, monkeypatch):
    import gstools
    import oracle
    from gstools_gb300 import hook

    monkeypatch.setattr(hook, "calc_field_krige_and_variance",
                        lambda m, v, c, num_threads=None: oracle.c_krige(m, v, c))
    cond_pos = [0.3, 1.9, 1.1, 3.3, 4.7]
    cond_val = [0.47, 0.56, 0.74, 1.47, 1.74]
    axes = (np.linspace(0.0, 5.0, 11), np.linspace(0.0, 4.0, 9))
    model = gstools.Gaussian(dim=2, var=0.5, len_scale=2.0)

    def make():
        krige = gstools.krige.Ordinary(model, (cond_pos, cond_pos[::-1]),
                                       cond_val)
        return gstools.CondSRF(krige, mode_no=40, seed=20170519)

    ref = make().structured(axes)
    got = _hooked(gen_module, make, lambda s: s.structured(axes), "f64")
    assert [c[0] for c in grid_spy] == ["scalar"]
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_structured_routing_leaves_other_cases_alone(gen_module, grid_spy):
    import gstools
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    axes = (np.arange(5.0), np.arange(5.0) * 0.5)
    cases = [
        # FP64 Fourier sums have no grid kernel
        (lambda: gstools.SRF(gstools.Gaussian(dim=2, len_scale=3.0),
                             generator="Fourier", mode_no=[4, 4],
                             period=[5, 5], seed=1), "f64", "structured"),
        # unstructured positions
        (lambda: gstools.SRF(gstools.Gaussian(dim=2, len_scale=3.0),
                             mode_no=20, seed=1), "mixed", "unstructured"),
        # latlon models isometrize non-linearly
        (lambda: gstools.SRF(gstools.Gaussian(latlon=True, len_scale=300.0,
                                              geo_scale=gstools.KM_SCALE),
                             mode_no=20, seed=1), "mixed", "structured"),
    ]
    for make, prec, mesh in cases:
        gg.install(precision=prec)
        try:
            with pytest.raises(RuntimeError):   # the GPU summators, no device
                make()(axes, mesh_type=mesh)
        finally:
            gg.uninstall()
        assert grid_spy == []


def test_structured_uninstall_restores_classes(gen_module):
    import gstools.field.base as fb
    import gstools.field.cond_srf as fc
    import gstools.field.srf as fs

    before = (fb.Field.__dict__["pre_pos"], fs.SRF.__dict__["__call__"],
              fc.CondSRF.__dict__["__call__"])
    gg.install()
    try:
        assert fb.Field.__dict__["pre_pos"] is not before[0]
        assert fs.SRF.__dict__["__call__"].__wrapped__ is before[1]
    finally:
        gg.uninstall()
    after = (fb.Field.__dict__["pre_pos"], fs.SRF.__dict__["__call__"],
             fc.CondSRF.__dict__["__call__"])
    assert after == before
