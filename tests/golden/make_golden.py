"""Generate the golden fixtures in this directory from the reference itself.

Run from the repository root, where the reference tree is available:

    python tests/golden/make_golden.py

The reference's Python package (RNG, covariance models, RandMeth,
IncomprRandMeth, SRF) is imported with ``reference_import`` and drives the
FP64 C oracle in place of the absent ``gstools_cython.field`` kernels.  Before
anything is written, every literal golden value that the reference's own tests
assert on this path is reproduced here (``assertAlmostEqual``'s 7 places):

* tests/test_randmeth.py:35-36, 40-41, 50-51, 55-56, 60-61, 70-71
* tests/test_incomprrandmeth.py:36-38, 58-59
* tests/test_srf.py:269-275
* tests/test_rng.py:22-37
* tests/test_fouriergen.py:47-57 (Fourier generator through SRF)
* tests/test_krige.py:56-153 (kriging: exact at the conditions, structured
  equals unstructured), with gstools-cython's kriging kernels restated by
  the C oracle; the arrays each Krige call hands to those kernels are stored

The 3-D RandMeth goldens (test_randmeth.py:45-46, 65-66;
test_incomprrandmeth.py:42-44) need emcee's MCMC sampler, which is absent, so
they cannot be reproduced and are not used.

The workload inputs (cov_samples, z_1, z_2) for the benchmark shapes are drawn
by the reference's own RNG: through the closed-form inversion path where the
model has a ppf (2-D Gaussian), and through ``sampling="inversion"`` (scipy's
numerical ppf of the reference's radial cdf) for the 3-D models.

Outputs: ``reference_goldens.npz`` (tiny cases with their literal goldens) and
``workloads.npz`` (mode sets and oracle outputs on sub-samples of the
benchmark point sets).
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import oracle  # noqa: E402
from reference_import import import_gstools  # noqa: E402

PLACES = 7


def check(value, expected, what, places=None):
    if round(abs(value - expected), PLACES if places is None else places) != 0:
        raise AssertionError(f"{what}: got {value!r}, reference {expected!r}")


def modes_of(gen):
    return {
        "cov": np.array(gen._cov_sample, dtype=np.float64),
        "z1": np.array(gen._z_1, dtype=np.float64),
        "z2": np.array(gen._z_2, dtype=np.float64),
    }


def reference_goldens(gs):
    from gstools.field.generator import IncomprRandMeth, RandMeth
    from gstools.random.rng import RNG

    out = {}

    def store(name, gen, pos, field, expected, idx, var):
        m = modes_of(gen)
        pos = np.atleast_2d(np.asarray(pos, dtype=np.float64))
        for key, val in m.items():
            out[f"{name}/{key}"] = val
        out[f"{name}/pos"] = pos
        out[f"{name}/field"] = np.asarray(field)
        out[f"{name}/expected"] = np.asarray(expected, dtype=np.float64)
        out[f"{name}/index"] = np.asarray(idx, dtype=np.int64)
        out[f"{name}/var"] = np.float64(var)
        out[f"{name}/seed"] = np.int64(gen.seed)
        for e, i in zip(expected, idx):
            check(np.asarray(field)[tuple(i)], e, f"{name}{tuple(i)}")

    # tests/test_randmeth.py:15-71
    cm1 = gs.Gaussian(dim=1, var=1.5, len_scale=3.5)
    cm2 = gs.Gaussian(dim=2, var=1.5, len_scale=3.5)
    seed = 19031977
    x_t = np.linspace(0.0, 10.0, 10)
    y_t = np.linspace(-5.0, 5.0, 10)
    rm1 = RandMeth(cm1, mode_no=100, seed=seed)
    store("randmeth_1d", rm1, (x_t,), rm1((x_t,)),
          [3.19799030, 2.44848295], [[0], [1]], 1.5)
    rm2 = RandMeth(cm2, mode_no=100, seed=seed)
    store("randmeth_2d", rm2, (x_t, y_t), rm2((x_t, y_t)),
          [1.67318010, 2.12310269], [[0], [1]], 1.5)
    rm2.seed = 74893621
    store("randmeth_2d_reseed", rm2, (x_t, y_t), rm2((x_t, y_t)),
          [-1.94278053, -1.12401651], [[0], [1]], 1.5)
    rm2.mode_no = 800
    store("randmeth_2d_800", rm2, (x_t, y_t), rm2((x_t, y_t)),
          [-3.20809251, -2.62032778], [[0], [1]], 1.5)

    # tests/test_incomprrandmeth.py:17-38
    ci2 = gs.Gaussian(dim=2, var=1.5, len_scale=2.5)
    ir2 = IncomprRandMeth(ci2, mode_no=100, seed=seed)
    store("incompr_2d", ir2, (x_t, y_t), ir2((x_t, y_t)),
          [0.50751115, 1.03291018, -0.22003005],
          [[0, 0], [0, 1], [1, 1]], 1.5)

    # tests/test_incomprrandmeth.py:50-59: VectorField mean (structured)
    x_g = np.linspace(0.0, 10.0, 9)
    y_g = np.linspace(-5.0, 5.0, 16)
    srf = gs.SRF(ci2, mean=(0.5, 0), generator="VectorField", seed=198412031)
    fld = srf.structured((x_g, y_g))
    means = [np.mean(fld[0]), np.mean(fld[1])]
    check(means[0], 1.3025621393180298, "vector_mean[0]")
    check(means[1], -0.04729596839446052, "vector_mean[1]")
    m = modes_of(srf.generator)
    for key, val in m.items():
        out[f"vector_mean/{key}"] = val
    out["vector_mean/x"] = x_g
    out["vector_mean/y"] = y_g
    out["vector_mean/var"] = np.float64(1.5)
    out["vector_mean/mean_u"] = np.float64(srf.generator.mean_u)
    out["vector_mean/mean"] = np.array([0.5, 0.0])
    out["vector_mean/expected"] = np.array(
        [1.3025621393180298, -0.04729596839446052])

    # tests/test_srf.py:259-275: IncomprRandMeth through SRF, mean 0.3
    rng = np.random.RandomState(123018)
    xs = rng.uniform(0.0, 10, 100)
    ys = rng.uniform(0.0, 10, 100)
    cm = gs.Gaussian(dim=2, var=0.5, len_scale=1.0)
    srf = gs.SRF(cm, mean=0.3, mode_no=100, generator="IncomprRandMeth",
                 mean_velocity=0.5)
    fld = srf((xs, ys), seed=476356)
    check(fld[0, 0], 1.23693272, "srf_incompr_unstruct[0,0]")
    check(fld[0, 1], 0.89242284, "srf_incompr_unstruct[0,1]")
    m = modes_of(srf.generator)
    for key, val in m.items():
        out[f"srf_incompr_unstruct/{key}"] = val
    out["srf_incompr_unstruct/pos"] = np.array([xs, ys])
    out["srf_incompr_unstruct/expected"] = np.array([1.23693272, 0.89242284])
    out["srf_incompr_unstruct/index"] = np.array([[0, 0], [0, 1]])
    out["srf_incompr_unstruct/field"] = fld
    x_g = np.linspace(0.0, 12.0, 48)
    y_g = np.linspace(0.0, 10.0, 46)
    fld = srf((x_g, y_g), seed=4734654, mesh_type="structured")
    check(fld[0, 0, 0], 1.07812013, "srf_incompr_struct[0,0,0]")
    check(fld[0, 1, 0], 1.06180674, "srf_incompr_struct[0,1,0]")
    m = modes_of(srf.generator)
    for key, val in m.items():
        out[f"srf_incompr_struct/{key}"] = val
    out["srf_incompr_struct/x"] = x_g
    out["srf_incompr_struct/y"] = y_g
    out["srf_incompr_struct/expected"] = np.array([1.07812013, 1.06180674])
    out["srf_incompr_struct/index"] = np.array([[0, 0, 0], [0, 1, 0]])
    out["srf_incompr_struct/field"] = fld

    # tests/test_fouriergen.py:14-57: Fourier generator through SRF,
    # structured 1-D / 2-D / 3-D Gaussian fields
    f_seed = 19900408
    f_models = [gs.Gaussian(dim=1, var=0.5, len_scale=10.0),
                gs.Gaussian(dim=2, var=2.0, len_scale=30.0),
                gs.Gaussian(dim=3, var=2.1, len_scale=21.0)]
    f_period = [80, 30, 91]
    f_axes = [np.linspace(0, f_period[0], 11), np.linspace(0, f_period[1], 31),
              np.linspace(0, f_period[2], 13)]
    f_modes = [12, 6, 14]
    f_expected = [0.6236929351309081, -0.1431996611581266, -1.0433325279452803]
    for d in (1, 2, 3):
        srf = gs.SRF(f_models[d - 1], generator="Fourier", mode_no=f_modes[:d],
                     period=f_period[:d], seed=f_seed)
        fld = srf(tuple(f_axes[:d]), mesh_type="structured")
        check(fld[(0,) * d], f_expected[d - 1], f"fourier_{d}d{(0,) * d}")
        gen = srf.generator
        name = f"fourier_{d}d"
        out[f"{name}/modes"] = np.array(gen.modes, dtype=np.float64)
        out[f"{name}/z1"] = np.array(gen._z_1, dtype=np.float64)
        out[f"{name}/z2"] = np.array(gen._z_2, dtype=np.float64)
        out[f"{name}/spectrum_factor"] = np.array(gen._spectrum_factor,
                                                  dtype=np.float64)
        out[f"{name}/period"] = np.array(f_period[:d], dtype=np.float64)
        out[f"{name}/mode_no"] = np.array(f_modes[:d], dtype=np.int64)
        out[f"{name}/var"] = np.float64(f_models[d - 1].var)
        out[f"{name}/len_scale"] = np.float64(f_models[d - 1].len_scale)
        out[f"{name}/seed"] = np.int64(f_seed)
        for i in range(d):
            out[f"{name}/axis{i}"] = f_axes[i]
        out[f"{name}/field"] = np.asarray(fld)
        out[f"{name}/expected"] = np.float64(f_expected[d - 1])

    # tests/test_krige.py:20-153: Simple / Ordinary / Universal kriging of
    # the test's five conditions; record what Krige hands to the kernels
    import gstools_cython.krige as ck

    data = np.array([[0.3, 1.2, 0.5, 0.47], [1.9, 0.6, 1.0, 0.56],
                     [1.1, 3.2, 1.5, 0.74], [3.3, 4.4, 2.0, 1.47],
                     [4.7, 3.8, 2.5, 1.74]])
    data_idx = tuple(np.array(data[:, :3] * 10, dtype=int).T)
    cond_pos = (data[:, 0], data[:, 1], data[:, 2])
    cond_val = data[:, 3]
    axes = (np.linspace(0, 5, 51), np.linspace(0, 6, 61), np.linspace(0, 7, 71))
    recorded = []
    orig = ck.calc_field_krige_and_variance

    def record(m, v, c, num_threads=None):
        recorded.append((np.array(m), np.array(v), np.array(c)))
        return orig(m, v, c)

    ck.calc_field_krige_and_variance = record
    import gstools.krige.base as kb
    kb_orig = kb._calc_field_krige_and_variance
    kb._calc_field_krige_and_variance = lambda m, v, c, num_threads=None: record(m, v, c)
    try:
        cases = [
            ("simple", lambda mdl, d: gs.krige.Simple(mdl, cond_pos[:d], cond_val,
                                                     np.mean(cond_val)), 2, 2),
            ("ordinary", lambda mdl, d: gs.krige.Ordinary(mdl, cond_pos[:d],
                                                          cond_val), 5, 10),
            ("universal", lambda mdl, d: gs.krige.Universal(mdl, cond_pos[:d],
                                                            cond_val, "linear"),
             2, 10),
        ]
        for kind, make, var, ls in cases:
            for Model in (gs.Gaussian, gs.Exponential):
                for d in (1, 2, 3):
                    mdl = Model(dim=d, var=var, len_scale=ls, anis=[0.9, 0.8],
                                angles=[2, 1, 0.5])
                    krig = make(mdl, d)
                    recorded.clear()
                    fld_s, _ = krig.structured(axes[:d])
                    for i, val in enumerate(cond_val):
                        check(fld_s[data_idx[:d]][i], val, f"krige_{kind}",
                              places=2)
                    name = f"krige_{kind}_{Model.__name__.lower()}_{d}d"
                    m, v, c = recorded[-1]
                    v = v[:, :4000]
                    f, e = oracle.c_krige(m, v, c)
                    out[f"{name}/mat"] = m
                    out[f"{name}/vecs"] = v
                    out[f"{name}/cond"] = c
                    out[f"{name}/field"] = f
                    out[f"{name}/error"] = e
    finally:
        ck.calc_field_krige_and_variance = orig
        kb._calc_field_krige_and_variance = kb_orig

    # variograms: the arrays vario_estimate / vario_estimate_axis hand to
    # gstools-cython's kernels (setups of tests/test_variogram_unstructured.py
    # and test_variogram_structured.py), with the oracle's results
    import gstools.variogram.variogram as vv

    calls = []
    saved = {n: getattr(vv, n) for n in ("unstructured_c", "directional_c",
                                         "structured_c", "ma_structured_c")}

    def recorder(name):
        fct = saved[name]

        def run(*args, **kwargs):
            res = fct(*args, **kwargs)
            calls.append((name, args, kwargs, res))
            return res
        return run

    for n in saved:
        setattr(vv, n, recorder(n))
    try:
        x = np.arange(1, 11, 1, dtype=np.double)
        z = np.array((41.2, 40.2, 39.7, 39.2, 40.1, 38.3, 39.1, 40.0, 41.1, 40.3))
        _, gam = gs.vario_estimate([x], z, np.arange(1, 11, 1.0))
        check(gam[0], 0.4917, "vario_1d[0]", places=4)
        check(gam[1], 0.7625, "vario_1d[1]", places=4)
        rng = np.random.RandomState(1479373475)
        xs, ys = rng.uniform(0, 100, 800), rng.uniform(0, 100, 800)
        fld = rng.normal(0, 2.0, size=(2, 800))
        fld[1, ::17] = np.nan
        gs.vario_estimate((xs, ys), fld, np.linspace(0, 40, 21))
        gs.vario_estimate((xs, ys), fld[0], np.linspace(0, 40, 21),
                          estimator="cressie")
        grid = np.arange(10.0)
        f3 = rng.normal(size=(10, 10, 10))
        f3m = np.ma.array(f3, mask=np.abs(f3) < 0.1)
        gs.vario_estimate((grid, grid, grid), f3m, range(10),
                          direction=((1, 0, 0), (0, 1, 0), (0, 0, 1)),
                          bandwidth=0.25, mesh_type="structured")
        gs.vario_estimate((grid[:8], grid), f3[:8, :, 0], range(0, 10, 2),
                          angles=np.pi / 4, mesh_type="structured")
        for ax in ("x", "y", "z"):
            gs.vario_estimate_axis(f3m, ax)
        gs.vario_estimate_axis(f3, "y", estimator="cressie")
        lat, lon = rng.uniform(-60, 60, 300), rng.uniform(-180, 180, 300)
        gs.vario_estimate((lat, lon), rng.normal(size=300), np.linspace(0, 2000, 11),
                          latlon=True, geo_scale=gs.KM_SCALE)
    finally:
        for n, fct in saved.items():
            setattr(vv, n, fct)
    for i, (name, args, kwargs, res) in enumerate(calls):
        key = f"vario_{i:02d}_{name[:-2]}"
        if name in ("unstructured_c", "directional_c"):
            names = ["f", "bin_edges", "pos"] + (
                ["direction", "angles_tol", "bandwidth", "separate_dirs",
                 "estimator_type"] if name == "directional_c" else
                ["estimator_type", "distance_type"])
        else:
            names = ["f", "mask", "estimator_type"] if name == "ma_structured_c" \
                else ["f", "estimator_type"]
        vals = dict(zip(names, args))
        vals.update(kwargs)
        vals.pop("num_threads", None)
        for k, v in vals.items():
            out[f"{key}/{k}"] = np.asarray(v)
        if isinstance(res, tuple):
            out[f"{key}/vario"], out[f"{key}/counts"] = (np.asarray(r) for r in res)
        else:
            out[f"{key}/vario"] = np.asarray(res)

    # tests/test_rng.py:20-37: normal streams of RNG(19031977)
    rng = RNG(seed)
    z1 = rng.random.normal(size=100)
    z2 = rng.random.normal(size=100)
    for v, e, w in ((z1[0], -1.93013270, "z1[0]"), (z1[1], 0.46330478, "z1[1]"),
                    (z2[0], -0.25536086, "z2[0]"), (z2[1], 0.98298696, "z2[1]")):
        check(v, e, w)
    out["rng_normal/z1"] = z1
    out["rng_normal/z2"] = z2
    return out


def workloads(gs):
    from gstools.field.generator import IncomprRandMeth, RandMeth
    from gstools.tools.geometric import generate_grid, matrix_isometrize

    out = {}
    seed = 20170519

    # 2-D Gaussian, var 1, len_scale 10, 1000 modes, 100 000 points in
    # [0, 100]^2 drawn by RandomState(20170519); oracle on the first 4096.
    model = gs.Gaussian(dim=2, var=1.0, len_scale=10.0)
    gen = RandMeth(model, mode_no=1000, seed=seed)
    pos = np.random.RandomState(seed).uniform(0.0, 100.0, (2, 100_000))
    for key, val in modes_of(gen).items():
        out[f"gau2d/{key}"] = val
    sub = pos[:, :4096]
    out["gau2d/pos_head"] = sub
    out["gau2d/summed_head"] = oracle.c_summate(gen._cov_sample, gen._z_1,
                                               gen._z_2, sub)

    # 3-D Exponential, var 2, len_scale [20, 10, 5], 2000 modes; structured
    # grid 0..255 per axis (unit spacing).  Modes by scipy inversion.
    model = gs.Exponential(dim=3, var=2.0, len_scale=[20.0, 10.0, 5.0])
    gen = RandMeth(model, mode_no=2000, seed=seed, sampling="inversion")
    for key, val in modes_of(gen).items():
        out[f"exp3d/{key}"] = val
    iso = matrix_isometrize(3, model.angles, model.anis)
    out["exp3d/isometrize"] = iso
    axes = [np.arange(0.0, 256.0, 17.0), np.arange(3.0, 256.0, 23.0),
            np.arange(1.0, 256.0, 11.0)]
    grid = model.isometrize(generate_grid(axes))
    out["exp3d/sub_x"], out["exp3d/sub_y"], out["exp3d/sub_z"] = axes
    out["exp3d/summed_sub"] = oracle.c_summate(gen._cov_sample, gen._z_1,
                                              gen._z_2, grid)

    # 3-D Gaussian incompressible, var 1, len_scale 8, 2000 modes, mean
    # velocity 1.0 on a 192^3 unit grid.  Modes by scipy inversion.
    model = gs.Gaussian(dim=3, var=1.0, len_scale=8.0)
    gen = IncomprRandMeth(model, mode_no=2000, seed=seed,
                          sampling="inversion", mean_velocity=1.0)
    for key, val in modes_of(gen).items():
        out[f"incompr3d/{key}"] = val
    axes = [np.arange(0.0, 192.0, 13.0), np.arange(5.0, 192.0, 19.0),
            np.arange(2.0, 192.0, 7.0)]
    grid = model.isometrize(generate_grid(axes))
    out["incompr3d/sub_x"], out["incompr3d/sub_y"], out["incompr3d/sub_z"] = (
        axes)
    out["incompr3d/summed_sub"] = oracle.c_summate_incompr(
        gen._cov_sample, gen._z_1, gen._z_2, grid)

    # 3-D Gaussian for the differentiable case: var 1, len_scale 16,
    # anisotropy [0.8, 0.6], angles [0.3, 0.2, 0.1], 4000 modes.
    model = gs.Gaussian(dim=3, var=1.0, len_scale=16.0, anis=[0.8, 0.6],
                        angles=[0.3, 0.2, 0.1])
    gen = RandMeth(model, mode_no=4000, seed=seed, sampling="inversion")
    for key, val in modes_of(gen).items():
        out[f"gau3d_grad/{key}"] = val
    out["gau3d_grad/isometrize"] = matrix_isometrize(3, model.angles,
                                                     model.anis)
    pts = np.random.RandomState(seed + 1).uniform(0.0, 128.0, (3, 2048))
    out["gau3d_grad/pos"] = pts
    out["gau3d_grad/summed"] = oracle.c_summate(
        gen._cov_sample, gen._z_1, gen._z_2, model.isometrize(pts))

    # Radial spectral densities (pdf/cdf) the host-side samplers must follow.
    r = np.geomspace(1e-3, 10.0, 64)
    for name, mdl in (
        ("gau3", gs.Gaussian(dim=3, len_scale=8.0)),
        ("exp3", gs.Exponential(dim=3, len_scale=20.0)),
        ("exp2", gs.Exponential(dim=2, len_scale=20.0)),
        ("gau2", gs.Gaussian(dim=2, len_scale=10.0)),
        ("mat2", gs.Matern(dim=2, nu=1.5, len_scale=10.0)),
        ("mat3", gs.Matern(dim=3, nu=1.5, len_scale=10.0)),
    ):
        out[f"spectral/{name}/r"] = r
        out[f"spectral/{name}/pdf"] = mdl.spectral_rad_pdf(r)
        if mdl.has_cdf:
            out[f"spectral/{name}/cdf"] = mdl.spectral_rad_cdf(r)
        out[f"spectral/{name}/len_rescaled"] = np.float64(mdl.len_rescaled)
    return out


def main():
    gs = import_gstools()
    golden = reference_goldens(gs)
    np.savez_compressed(os.path.join(HERE, "reference_goldens.npz"), **golden)
    work = workloads(gs)
    np.savez_compressed(os.path.join(HERE, "workloads.npz"), **work)
    print(f"wrote {len(golden)} + {len(work)} arrays to {HERE}")


if __name__ == "__main__":
    main()
