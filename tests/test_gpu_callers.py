"""The reference's own callers, replayed through ``install()`` on the GPU.

``tests/golden/callers.npz`` (made by ``tests/golden/make_callers.py`` from
the reference itself) holds the calls that ``SRF`` (RandMeth,
IncomprRandMeth, Fourier), ``CondSRF``, ``Krige`` and ``vario_estimate`` /
``vario_estimate_axis`` made into the module globals that ``install()``
rebinds -- positional arguments and keywords exactly as passed (argument
order of ``_summate_fourier``, ``num_threads`` positions, the kriging
matrix / vector shapes, the variogram keywords) -- with the C oracle's
results.  Here those calls go, unchanged, into the functions ``install()``
puts on stand-in modules of the same names, and the results must match the
recorded ones at the bars of the kernel tests:

* summators (``precision="f64"``): max|diff| <= 1e-12 max|ref|;
* kriging: |diff| <= 1e-12 * sum_i (|c_i| + |v_ik|)(|M||v_k|)_i per point;
* variograms: counts exact, values within 1e-12 relative.

The grid cases replay structured ``SRF`` evaluations through the routed path
of ``install()``: a placeholder grid registered as ``Field.pre_pos`` does
it, handed to the installed summator as the reference's generator hands its
positions.  FP64 results meet the FP64 bar; mixed precision (tensor cores on
2-D / 3-D grids) meets RMS <= 1e-5 sigma of the scaled field.
"""

import os
import types

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

F64_REL = 1e-12
KRIGE_REL = 1e-12
VARIO_REL = 1e-12
MIXED_RMS_SIGMA = 1e-5

GEN_NAMES = ("_summate", "_summate_incompr", "_summate_fourier")
KRIGE_NAMES = ("_calc_field_krige", "_calc_field_krige_and_variance")
VARIO_NAMES = ("_unstructured", "_directional", "_structured", "_ma_structured")


def _value(tag, a):
    if tag == "n":
        return None
    if tag == "b":
        return bool(a)
    if tag == "i":
        return int(a)
    if tag == "f":
        return float(a)
    if tag == "s":
        return str(a)
    return np.array(a)


def _load():
    return np.load(os.path.join(GOLDEN, "callers.npz"))


def _calls(data):
    out = []
    for i in range(int(data["calls/count"])):
        k = f"call{i:03d}"
        tags = str(data[f"{k}/argtags"])
        args = [_value(t, data[f"{k}/arg{j}"]) for j, t in enumerate(tags)]
        names = [n for n in str(data[f"{k}/kwnames"]).split(",") if n]
        ktags = str(data[f"{k}/kwtags"])
        kwargs = {n: _value(t, data[f"{k}/kw_{n}"]) for n, t in zip(names, ktags)}
        res = [np.array(data[f"{k}/result{j}"])
               for j in range(int(data[f"{k}/nresults"]))]
        out.append(dict(family=str(data[f"{k}/family"]),
                        name=str(data[f"{k}/name"]), args=args, kwargs=kwargs,
                        results=res))
    return out


FAMILIES = ("randmeth_2d", "randmeth_3d_aniso", "incompr", "fourier",
            "cond_srf", "krige_field_only", "vario")


def _not_rebound(*args, **kwargs):
    raise AssertionError("install() did not rebind this name")


def _stand_ins():
    gen = types.ModuleType("gstools_field_generator_stand_in")
    krige = types.ModuleType("gstools_krige_base_stand_in")
    vario = types.ModuleType("gstools_variogram_stand_in")
    for mod, names in ((gen, GEN_NAMES), (krige, KRIGE_NAMES),
                       (vario, VARIO_NAMES)):
        for n in names:
            setattr(mod, n, _not_rebound)
    return gen, krige, vario


@pytest.fixture(scope="module")
def callers():
    return _calls(_load())


def test_fixture_covers_every_hooked_name(callers):
    seen = {c["name"] for c in callers}
    assert seen == set(GEN_NAMES + KRIGE_NAMES + VARIO_NAMES)
    assert {c["family"] for c in callers} == set(FAMILIES)


@pytest.mark.parametrize("family", FAMILIES)
def test_replay_reference_calls(cuda_lib, callers, family):
    import gstools_gb300 as gg
    import oracle

    gen, krige, vario = _stand_ins()
    gg.install(gen, precision="f64", krige_module=krige, vario_module=vario)
    try:
        calls = [c for c in callers if c["family"] == family]
        assert calls
        for c in calls:
            name = c["name"]
            mod = gen if name in GEN_NAMES else (
                krige if name in KRIGE_NAMES else vario)
            res = getattr(mod, name)(*c["args"], **c["kwargs"])
            res = res if isinstance(res, tuple) else (res,)
            assert len(res) == len(c["results"]), name
            if name in GEN_NAMES:
                got, ref = np.asarray(res[0]), c["results"][0]
                assert got.shape == ref.shape, name
                assert np.max(np.abs(got - ref)) <= F64_REL * np.max(np.abs(ref)), name
            elif name in KRIGE_NAMES:
                _, _, scale = oracle.np_krige(*c["args"][:3])
                for got, ref in zip(res, c["results"]):
                    got = np.asarray(got)
                    assert got.shape == ref.shape, name
                    assert np.all(np.abs(got - ref) <= KRIGE_REL * scale + 1e-300), name
            else:
                got, ref = np.asarray(res[0]), c["results"][0]
                assert got.shape == ref.shape, name
                np.testing.assert_allclose(got, ref, rtol=VARIO_REL, atol=0,
                                           err_msg=name)
                if len(res) > 1:
                    np.testing.assert_array_equal(np.asarray(res[1]),
                                                  c["results"][1], err_msg=name)
    finally:
        gg.uninstall(gen, krige_module=krige, vario_module=vario)
    assert gen._summate is _not_rebound and krige._calc_field_krige is _not_rebound


def _grid_case(data, name):
    g = {k[len(name) + 1:]: data[k] for k in data.files
         if k.startswith(name + "/")}
    g["axes"] = [g[f"axis{d}"] for d in range(int(g["ndim"]))]
    return g


GRID_NAMES = ("grid_exp3d_aniso", "grid_gau2d", "grid_gau1d", "grid_vector2d",
              "grid_vector3d_iso", "grid_fourier3d")


@pytest.mark.parametrize("name", GRID_NAMES)
@pytest.mark.parametrize("precision", ["f64", "mixed"])
def test_routed_structured_calls(cuda_lib, name, precision):
    """The installed summator, given the placeholder ``pre_pos`` registers
    for a structured grid, returns the reference's sum on its meshgrid."""
    import gstools_gb300 as gg
    from gstools_gb300 import hook

    data = _load()
    assert set(str(data["grids/names"]).split(",")) == set(GRID_NAMES)
    g = _grid_case(data, name)
    kind = str(g["kind"])
    dim = int(g["ndim"])
    if not gg.summator.structured_supported(kind, dim, precision, g["iso"]):
        # the reference's meshgrid path runs instead (covered by the replay
        # tests above); FP64 Fourier and anisotropic FP64 vector fields
        assert (kind == "fourier" and precision == "f64") or (
            kind == "incompr" and precision == "f64")
        return
    gen, krige, vario = _stand_ins()
    gg.install(gen, precision=precision, krige_module=krige,
               vario_module=vario)
    grid = hook.GridPlaceholder(g["axes"], g["iso"], kind, precision)
    token = grid.register()
    try:
        # the generator's own call: pos = np.asarray(pos, dtype=np.double)
        pos = np.asarray(token, dtype=np.double)
        assert pos is token
        if kind == "fourier":
            got = gen._summate_fourier(g["spectrum_factor"], g["cov"], g["z1"],
                                       g["z2"], pos, None)
        elif kind == "incompr":
            got = gen._summate_incompr(g["cov"], g["z1"], g["z2"], pos, None)
        else:
            got = gen._summate(g["cov"], g["z1"], g["z2"], pos, None)
    finally:
        grid.release()
        gg.uninstall(gen, krige_module=krige, vario_module=vario)
    ref = g["summed"]
    assert got.shape == ref.shape and got.dtype == np.float64
    if precision == "f64":
        assert np.max(np.abs(got - ref)) <= F64_REL * np.max(np.abs(ref))
    else:
        # the field is sqrt(var / N) * sum (generator.py:270); RMS vs sigma
        n_modes = int(g["mode_no"])
        scale = 1.0 / np.sqrt(n_modes) if kind != "fourier" else 1.0 / np.sqrt(
            float(g["var"]))
        rms = np.sqrt(np.mean((scale * (got - ref)) ** 2))
        assert rms <= MIXED_RMS_SIGMA, rms
