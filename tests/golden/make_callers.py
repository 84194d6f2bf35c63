"""Record the calls the reference's own callers make into the summator,
kriging and variogram hooks, for replay on the GPU.

Run from the repository root, where the reference tree is available:

    python tests/golden/make_callers.py

The reference's Python (``reference_import``: the C oracle stands in for the
absent gstools-cython kernels) runs a set of its own entry points --
``SRF`` with ``RandMeth`` / ``IncomprRandMeth`` / ``Fourier``, ``CondSRF``,
``Krige`` with and without the variance, ``vario_estimate`` and
``vario_estimate_axis`` -- while recorders sit on the module globals that
``gstools_gb300.install()`` rebinds:

* ``gstools.field.generator._summate`` / ``_summate_incompr`` /
  ``_summate_fourier`` (called at src/gstools/field/generator.py:266, 554,
  682);
* ``gstools.krige.base._calc_field_krige`` /
  ``_calc_field_krige_and_variance`` (called by ``Krige._summate``,
  src/gstools/krige/base.py:307-320; ``CondSRF`` reaches it through
  src/gstools/field/cond_srf.py:132);
* ``gstools.variogram.variogram._unstructured`` / ``_directional`` /
  ``_structured`` / ``_ma_structured`` (src/gstools/variogram/
  variogram.py:48-124).

Each recorded call keeps its positional arguments and keywords exactly as
the caller passed them (with a type tag per value) and the oracle's result.
Structured SRF evaluations are also stored as grid cases: axis arrays, the
model's isometrize matrix, the generator kind, the modes and the sum the
reference's summator returned on its own meshgrid path, for the routed
(no-meshgrid) path of ``install()``.

Output: ``callers.npz`` beside this script.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from reference_import import import_gstools  # noqa: E402

TARGETS = (
    ("gstools.field.generator", "_summate"),
    ("gstools.field.generator", "_summate_incompr"),
    ("gstools.field.generator", "_summate_fourier"),
    ("gstools.krige.base", "_calc_field_krige"),
    ("gstools.krige.base", "_calc_field_krige_and_variance"),
    ("gstools.variogram.variogram", "_unstructured"),
    ("gstools.variogram.variogram", "_directional"),
    ("gstools.variogram.variogram", "_structured"),
    ("gstools.variogram.variogram", "_ma_structured"),
)


def _tag(v):
    """(type tag, array) of one argument value."""
    if v is None:
        return "n", np.zeros(0)
    if isinstance(v, (bool, np.bool_)):
        return "b", np.asarray(bool(v))
    if isinstance(v, (int, np.integer)):
        return "i", np.asarray(int(v))
    if isinstance(v, (float, np.floating)):
        return "f", np.asarray(float(v))
    if isinstance(v, str):
        return "s", np.asarray(v)
    return "a", np.asarray(v)


class Recorder:
    def __init__(self):
        self.family = None
        self.calls = []
        self.saved = {}

    def install(self):
        for modname, name in TARGETS:
            mod = sys.modules[modname]
            orig = getattr(mod, name)
            self.saved[(modname, name)] = orig

            def rec(*args, _orig=orig, _name=name, **kwargs):
                res = _orig(*args, **kwargs)
                self.calls.append((self.family, _name, args, kwargs, res))
                return res

            setattr(mod, name, rec)

    def uninstall(self):
        for (modname, name), fct in self.saved.items():
            setattr(sys.modules[modname], name, fct)


def scenarios(gs):
    """(family, callable) pairs: each runs reference entry points."""
    rng = np.random.RandomState(20240601)
    x2 = rng.uniform(0.0, 20.0, (2, 300))
    x3 = rng.uniform(0.0, 12.0, (3, 200))
    cond_pos = ([0.3, 1.9, 1.1, 3.3, 4.7], [1.2, 0.6, 3.2, 4.4, 3.8])
    cond_val = [0.47, 0.56, 0.74, 1.47, 1.74]

    def randmeth_2d():
        srf = gs.SRF(gs.Gaussian(dim=2, var=1.5, len_scale=3.5), mode_no=100,
                     seed=19031977)
        srf((x2[0], x2[1]))
        srf((x2[0], x2[1]), seed=74893621)

    def randmeth_3d_aniso():
        model = gs.Exponential(dim=3, var=2.0, len_scale=[4.0, 3.0, 2.0],
                               angles=[0.4, 0.2, 0.1], nugget=0.1)
        srf = gs.SRF(model, mean=0.5, mode_no=64, seed=9, sampling="inversion")
        srf(tuple(x3))

    def incompr():
        # tests/test_srf.py:259-275
        r = np.random.RandomState(123018)
        xs, ys = r.uniform(0.0, 10, 100), r.uniform(0.0, 10, 100)
        srf = gs.SRF(gs.Gaussian(dim=2, var=0.5, len_scale=1.0), mean=0.3,
                     mode_no=100, generator="IncomprRandMeth",
                     mean_velocity=0.5)
        srf((xs, ys), seed=476356)

    def fourier():
        # tests/test_fouriergen.py:14-57 (2-D case)
        srf = gs.SRF(gs.Gaussian(dim=2, var=2.0, len_scale=30.0),
                     generator="Fourier", mode_no=[6, 6], period=[30, 30],
                     seed=19900408)
        srf((np.linspace(0, 30, 31), np.linspace(0, 30, 17)),
            mesh_type="structured")

    def cond_srf():
        krige = gs.krige.Ordinary(gs.Gaussian(dim=2, var=0.5, len_scale=2.0),
                                  cond_pos, cond_val)
        csrf = gs.CondSRF(krige, mode_no=40, seed=20170519)
        csrf((x2[0] * 0.25, x2[1] * 0.25))
        csrf((x2[0] * 0.25, x2[1] * 0.25), seed=4)   # reuses the kriging

    def krige_field_only():
        krige = gs.krige.Universal(
            gs.Exponential(dim=2, var=2.0, len_scale=3.0, anis=0.8,
                           angles=0.5), cond_pos, cond_val, "linear")
        krige((x2[0] * 0.25, x2[1] * 0.25), return_var=False)
        krige.structured((np.linspace(0, 5, 21), np.linspace(0, 5, 16)))

    def vario():
        r = np.random.RandomState(1479373475)
        xs, ys = r.uniform(0, 100, 500), r.uniform(0, 100, 500)
        fld = r.normal(0, 2.0, size=(2, 500))
        fld[1, ::17] = np.nan
        gs.vario_estimate((xs, ys), fld, np.linspace(0, 40, 21))
        gs.vario_estimate((xs, ys), fld[0], np.linspace(0, 40, 21),
                          estimator="cressie")
        gs.vario_estimate((xs, ys), fld[0], np.linspace(0, 40, 11),
                          angles=[0.3, 1.2], angles_tol=np.pi / 6,
                          bandwidth=8.0)
        grid = np.arange(10.0)
        f3 = r.normal(size=(10, 10, 10))
        f3m = np.ma.array(f3, mask=np.abs(f3) < 0.1)
        gs.vario_estimate((grid, grid, grid), f3m, range(10),
                          direction=((1, 0, 0), (0, 1, 0), (0, 0, 1)),
                          bandwidth=0.25, mesh_type="structured")
        gs.vario_estimate_axis(f3m, "y")
        gs.vario_estimate_axis(f3, "z", estimator="cressie")

    return [("randmeth_2d", randmeth_2d), ("randmeth_3d_aniso", randmeth_3d_aniso),
            ("incompr", incompr), ("fourier", fourier), ("cond_srf", cond_srf),
            ("krige_field_only", krige_field_only), ("vario", vario)]


def grid_cases(gs):
    """Structured evaluations for the routed path: (name, srf, axes, kind)."""
    return [
        ("grid_exp3d_aniso", gs.SRF(
            gs.Exponential(dim=3, var=2.0, len_scale=[20.0, 10.0, 5.0],
                           angles=[0.4, 0.2, 0.1]),
            mode_no=500, seed=20170519, sampling="inversion"),
         (np.arange(48.0), np.arange(40.0) * 1.5, np.arange(3.0, 35.0)),
         "scalar"),
        ("grid_gau2d", gs.SRF(gs.Gaussian(dim=2, var=1.0, len_scale=10.0),
                              mode_no=1000, seed=20170519),
         (np.linspace(0.0, 100.0, 160), np.linspace(-20.0, 80.0, 128)),
         "scalar"),
        ("grid_gau1d", gs.SRF(gs.Gaussian(dim=1, var=1.0, len_scale=3.0),
                              mode_no=300, seed=5),
         (np.linspace(0.0, 50.0, 1000),), "scalar"),
        ("grid_vector2d", gs.SRF(
            gs.Gaussian(dim=2, var=1.5, len_scale=2.5, anis=0.7, angles=0.3),
            generator="VectorField", mode_no=400, seed=198412031,
            mean_velocity=0.5),
         (np.linspace(0.0, 10.0, 90), np.linspace(-5.0, 5.0, 70)), "incompr"),
        ("grid_vector3d_iso", gs.SRF(
            gs.Gaussian(dim=3, var=1.0, len_scale=8.0),
            generator="VectorField", mode_no=300, seed=7, sampling="inversion",
            mean_velocity=1.0),
         (np.arange(24.0), np.arange(20.0), np.arange(18.0)), "incompr"),
        ("grid_fourier3d", gs.SRF(
            gs.Gaussian(dim=3, var=2.1, len_scale=21.0), generator="Fourier",
            mode_no=[14, 14, 14], period=[91, 91, 91], seed=19900408),
         (np.linspace(0, 91, 40), np.linspace(0, 91, 33),
          np.linspace(0, 91, 26)), "fourier"),
    ]


def main():
    gs = import_gstools()
    rec = Recorder()
    rec.install()
    try:
        for family, run in scenarios(gs):
            rec.family = family
            run()
        grids = []
        for name, srf, axes, kind in grid_cases(gs):
            rec.family = name
            n0 = len(rec.calls)
            field = srf.structured(axes)
            (fam, fname, args, kwargs, res), = rec.calls[n0:]
            del rec.calls[n0:]
            grids.append((name, srf, axes, kind, fname, args, res, field))
    finally:
        rec.uninstall()

    out = {}
    families = []
    for i, (family, name, args, kwargs, res) in enumerate(rec.calls):
        key = f"call{i:03d}"
        families.append(family)
        out[f"{key}/family"] = np.asarray(family)
        out[f"{key}/name"] = np.asarray(name)
        tags = []
        for j, v in enumerate(args):
            t, a = _tag(v)
            tags.append(t)
            out[f"{key}/arg{j}"] = a
        out[f"{key}/argtags"] = np.asarray("".join(tags))
        kwnames = sorted(kwargs)
        out[f"{key}/kwnames"] = np.asarray(",".join(kwnames))
        ktags = []
        for k in kwnames:
            t, a = _tag(kwargs[k])
            ktags.append(t)
            out[f"{key}/kw_{k}"] = a
        out[f"{key}/kwtags"] = np.asarray("".join(ktags))
        results = res if isinstance(res, tuple) else (res,)
        out[f"{key}/nresults"] = np.asarray(len(results))
        for j, r in enumerate(results):
            out[f"{key}/result{j}"] = np.asarray(r)
    out["calls/count"] = np.asarray(len(rec.calls))
    for name, srf, axes, kind, fname, args, res, field in grids:
        model = srf.model
        out[f"{name}/kind"] = np.asarray(kind)
        out[f"{name}/hook"] = np.asarray(fname)
        out[f"{name}/iso"] = np.asarray(model.isometrize(np.eye(model.dim)))
        for d, a in enumerate(axes):
            out[f"{name}/axis{d}"] = np.asarray(a, dtype=np.float64)
        out[f"{name}/ndim"] = np.asarray(len(axes))
        if kind == "fourier":
            fac, modes, z1, z2 = args[:4]
            out[f"{name}/spectrum_factor"] = np.asarray(fac)
            out[f"{name}/cov"] = np.asarray(modes)
        else:
            cov, z1, z2 = args[:3]
            out[f"{name}/cov"] = np.asarray(cov)
        out[f"{name}/z1"] = np.asarray(z1)
        out[f"{name}/z2"] = np.asarray(z2)
        out[f"{name}/summed"] = np.asarray(res)
        out[f"{name}/var"] = np.asarray(float(model.var))
        out[f"{name}/mode_no"] = np.asarray(np.size(z1))
    out["grids/names"] = np.asarray(",".join(g[0] for g in grids))
    path = os.path.join(HERE, "callers.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {len(rec.calls)} calls ({sorted(set(families))}) and "
          f"{len(grids)} grid cases to {path} "
          f"({os.path.getsize(path) / 1e6:.2f} MB)")


if __name__ == "__main__":
    main()
