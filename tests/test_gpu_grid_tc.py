"""GPU parity of the separable tensor-core grid path (tcgen05; three-product
FP16 split by default, 3xTF32 selectable).

Bar: RMS(gpu - oracle) of the scaled field <= 1e-5 sigma (sigma = sqrt(var),
field scaled by sqrt(var / N)), and max error <= 1e-4 sigma.
"""

import numpy as np
import pytest

import gstools_gb300 as gg
import oracle

pytestmark = pytest.mark.gpu

RMS_SIGMA = 1e-5
MAX_SIGMA = 1e-4


def grid_ref(cov, z1, z2, axes):
    grid = np.array(np.meshgrid(*axes, indexing="ij")).reshape(len(axes), -1)
    return oracle.c_summate(cov, z1, z2, grid).reshape([len(a) for a in axes])


def errors(got, ref, n_modes, var=1.0):
    d = np.sqrt(var / n_modes) * (np.asarray(got, dtype=np.float64) - ref)
    return (np.sqrt(np.mean(d**2)) / np.sqrt(var),
            np.max(np.abs(d)) / np.sqrt(var))


def case(seed, dim, n_modes, k_scale=0.2):
    rng = np.random.RandomState(seed)
    cov = rng.standard_t(3, size=(dim, n_modes)) * k_scale
    return cov, rng.normal(size=n_modes), rng.normal(size=n_modes)


@pytest.mark.parametrize("shape,n_modes", [
    ((16, 16), 8), ((256, 256), 64), ((37, 300), 13), ((300, 5), 100),
    ((1, 1), 1), ((513, 17), 203)])
def test_tc_2d(cuda_lib, shape, n_modes):
    cov, z1, z2 = case(sum(shape) + n_modes, 2, n_modes)
    axes = [np.linspace(-20.0, 80.0, shape[0]), np.arange(shape[1]) * 0.7]
    ref = grid_ref(cov, z1, z2, axes)
    got = gg.summate_grid(cov, z1, z2, axes, precision="mixed",
                          method="tensor", out_dtype="float32")
    assert got.shape == shape and got.dtype == np.float32
    rms, mx = errors(got, ref, n_modes)
    assert rms <= RMS_SIGMA and mx <= MAX_SIGMA, (rms, mx)


@pytest.mark.parametrize("shape,n_modes", [
    ((16, 16, 16), 8), ((20, 33, 17), 61), ((256, 16, 16), 500),
    ((3, 40, 70), 1000), ((300, 9, 31), 37)])
def test_tc_3d(cuda_lib, shape, n_modes):
    cov, z1, z2 = case(sum(shape) * 3 + n_modes, 3, n_modes)
    axes = [np.arange(float(shape[0])), np.arange(shape[1]) * 1.5 - 7.0,
            np.linspace(0.0, 50.0, shape[2])]
    ref = grid_ref(cov, z1, z2, axes)
    got = gg.summate_grid(cov, z1, z2, axes, precision="mixed",
                          method="tensor")
    assert got.shape == shape and got.dtype == np.float64
    rms, mx = errors(got, ref, n_modes)
    assert rms <= RMS_SIGMA and mx <= MAX_SIGMA, (rms, mx)


@pytest.mark.parametrize("nz,nt", [
    (128, 128), (129, 192), (150, 192), (192, 192), (193, 256), (256, 256),
    (320, 192), (384, 192), (640, 256), (40, 128)])
@pytest.mark.parametrize("dim", [2, 3])
def test_tc_tile_widths(cuda_lib, nz, nt, dim):
    """The z tile (MMA N = 128, 192 or 256) picked from the last axis: every
    width against the oracle, on 2-D and 3-D grids, with partial last tiles
    and both the staged (float32, whole tile) and the direct epilogue."""
    n_modes = 150
    cov, z1, z2 = case(nz + dim, dim, n_modes, k_scale=0.05)
    lead = [np.arange(34.0) * 0.9] + ([np.arange(17.0) - 3.0] if dim == 3 else [])
    axes = lead + [np.linspace(-10.0, 40.0, nz)]
    from gstools_gb300 import _native

    assert _native.grid_tile_cols(nz) == nt
    for out_dtype in ("float32", "float64"):
        got = gg.summate_grid(cov, z1, z2, axes, precision="mixed",
                              method="tensor", out_dtype=out_dtype)
        sub = [a[::3] for a in axes[:-1]] + [axes[-1]]
        ref = grid_ref(cov, z1, z2, sub)
        idx = tuple(slice(None, None, 3) for _ in axes[:-1]) + (slice(None),)
        rms, mx = errors(got[idx], ref, n_modes)
        assert rms <= RMS_SIGMA and mx <= MAX_SIGMA, (out_dtype, rms, mx)


@pytest.mark.parametrize("dim", [2, 3])
def test_tc_far_from_origin(cuda_lib, dim):
    """Axes 1e5 - 3e5 from the origin with heavy-tailed wave numbers: per-axis
    phases up to ~6e5 turns.  Tensor cores: reduced exactly (FP64) in the
    tables; mixed pointwise: relative to the first point."""
    n_modes = 300
    cov, z1, z2 = case(7 * dim, dim, n_modes, k_scale=1.0)
    axes = [1.0e5 + np.arange(40.0) * 0.37, 2.0e5 - np.arange(30.0) * 0.51,
            -3.0e5 + np.arange(36.0) * 0.29][:dim]
    got = gg.summate_grid(cov, z1, z2, axes, precision="mixed", method="tensor")
    ref = grid_ref(cov, z1, z2, axes)
    rms, mx = errors(got, ref, n_modes)
    assert rms <= RMS_SIGMA and mx <= MAX_SIGMA, (rms, mx)
    # the mixed pointwise kernel: phases relative to the grid's first point
    # (amplitudes rotated per mode), so only the grid's extent enters the
    # FP32 split reduction
    got_pw = gg.summate_grid(cov, z1, z2, axes, precision="mixed", method="pointwise")
    rms, mx = errors(got_pw, ref, n_modes)
    assert rms <= RMS_SIGMA and mx <= MAX_SIGMA, ("pointwise", rms, mx)
    # and on the same points as an unstructured set
    pts = np.array(np.meshgrid(*axes, indexing="ij")).reshape(dim, -1)
    got_u = gg.summate(cov, z1, z2, pts[:, ::-1].copy(), precision="mixed")
    rms, mx = errors(got_u[::-1].reshape(ref.shape), ref, n_modes)
    assert rms <= RMS_SIGMA and mx <= MAX_SIGMA, ("unstructured", rms, mx)


def test_tc_exp3d_workload_slab(cuda_lib, workloads):
    """The benchmark's modes (3-D anisotropic Exponential, 2000 modes) on a
    full 256^3 grid, checked against the oracle on scattered slabs."""
    c = workloads.case("exp3d")
    kp = c["isometrize"].T @ c["cov"]
    axes = [np.arange(256.0)] * 3
    full = gg.summate_grid(kp, c["z1"], c["z2"], axes, precision="mixed",
                           method="tensor", out_dtype="float32")
    assert full.shape == (256, 256, 256)
    for ix in (0, 77, 255):
        sub = [axes[0][ix:ix + 1], axes[1][::5], axes[2][::3]]
        ref = grid_ref(kp, c["z1"], c["z2"], sub)
        got = full[ix:ix + 1, ::5, ::3]
        rms, mx = errors(got, ref, 2000, var=2.0)
        assert rms <= RMS_SIGMA and mx <= MAX_SIGMA, (ix, rms, mx)


def test_tc_scale_and_zero_modes(cuda_lib):
    cov, z1, z2 = case(5, 3, 40)
    axes = [np.arange(10.0), np.arange(12.0), np.arange(14.0)]
    a = gg.summate_grid(cov, z1, z2, axes, precision="mixed", method="tensor")
    b = gg.summate_grid(cov, z1, z2, axes, precision="mixed", method="tensor",
                        scale=0.25)
    np.testing.assert_allclose(b, 0.25 * a, rtol=1e-6, atol=1e-9)
    z = gg.summate_grid(np.zeros((3, 0)), np.zeros(0), np.zeros(0), axes,
                        precision="mixed", method="tensor")
    np.testing.assert_array_equal(z, np.zeros((10, 12, 14)))


def test_tc_no_device_error(cuda_lib):
    from gstools_gb300 import _native

    assert _native.read_device_error() == 0


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("aniso", [False, True])
def test_tc_incompressible(cuda_lib, dim, aniso):
    from gstools_gb300.geometric import matrix_isometrize

    cov, z1, z2 = case(40 + dim + 7 * aniso, dim, 333)
    shape = (19, 33, 21)[:dim]
    axes = [np.arange(float(n)) * 0.9 for n in shape]
    m = (matrix_isometrize(dim, [0.4, -0.3, 0.2][: dim * (dim - 1) // 2],
                           [0.6, 0.8][: dim - 1]) if aniso else np.eye(dim))
    grid = np.array(np.meshgrid(*axes, indexing="ij")).reshape(dim, -1)
    ref = oracle.c_summate_incompr(cov, z1, z2, m @ grid).reshape((dim,) + shape)
    got = gg.summate_incompr_grid(m.T @ cov, z1, z2, axes, precision="mixed",
                                  method="tensor", proj_cov=cov)
    assert got.shape == (dim,) + shape
    rms, mx = errors(got, ref, 333)
    assert rms <= RMS_SIGMA and mx <= MAX_SIGMA, (rms, mx)


@pytest.mark.parametrize("dim", [2, 3])
def test_tc_fourier_grid(cuda_lib, dim):
    cov, z1, z2 = case(70 + dim, dim, 257)
    fac = np.random.RandomState(dim).uniform(0.1, 1.5, size=257)
    shape = (23, 17, 40)[:dim]
    axes = [np.linspace(-10.0, 30.0, n) for n in shape]
    grid = np.array(np.meshgrid(*axes, indexing="ij")).reshape(dim, -1)
    ref = oracle.c_summate_fourier(fac, cov, z1, z2, grid).reshape(shape)
    got = gg.summate_fourier_grid(fac, cov, z1, z2, axes)
    d = (got - ref) / np.sqrt(np.sum(fac ** 2))
    assert np.sqrt(np.mean(d ** 2)) <= RMS_SIGMA


def test_incompr_mirror_structured_mixed_matches_f64(cuda_lib):
    """IncomprRandMeth.structured: tensor path (mixed) vs FP64 pointwise,
    anisotropic and rotated model."""
    model = gg.Gaussian(dim=3, var=1.0, len_scale=6.0, anis=[0.7, 0.5],
                        angles=[0.2, 0.1, 0.3])
    axes = [np.arange(20.0), np.arange(18.0), np.arange(22.0)]
    f64 = gg.IncomprRandMeth(model, mode_no=500, seed=3, sampling="analytic")
    mixed = gg.IncomprRandMeth(model, mode_no=500, seed=3, sampling="analytic",
                               precision="mixed")
    a = f64.structured(axes, add_nugget=False)
    b = mixed.structured(axes, add_nugget=False)
    assert np.sqrt(np.mean((a - b) ** 2)) <= RMS_SIGMA


def test_tc_host_output_matches_device_output(cuda_lib):
    """numpy inputs go through gst_summate_grid_tc_host (slabs copied to a
    page-locked result while the next slab computes), torch inputs through
    gst_summate_grid_tc; the two differ only where a partial wave's tiles are
    split over their modes, by the FP32 rounding of the two-part sum."""
    import torch

    cov, z1, z2 = case(11, 3, 400)
    axes = [np.arange(64.0), np.arange(96.0), np.arange(100.0)]
    host = gg.summate_grid(cov, z1, z2, axes, precision="mixed",
                           method="tensor", out_dtype="float32")
    assert isinstance(host, np.ndarray) and host.nbytes >= (1 << 20)
    dev = gg.summate_grid(torch.from_numpy(cov).cuda(), torch.from_numpy(z1).cuda(),
                          torch.from_numpy(z2).cuda(),
                          [torch.from_numpy(a).cuda() for a in axes],
                          precision="mixed", method="tensor", out_dtype="float32")
    np.testing.assert_allclose(host, dev.cpu().numpy(), rtol=0,
                               atol=1e-5 * np.max(np.abs(host)))
    grid = np.array(np.meshgrid(*[a[::9] for a in axes], indexing="ij")).reshape(3, -1)
    ref = oracle.c_summate(cov, z1, z2, grid).reshape([len(a[::9]) for a in axes])
    rms, mx = errors(host[::9, ::9, ::9], ref, 400)
    assert rms <= RMS_SIGMA and mx <= MAX_SIGMA


def _tc_workspace(lib, dim, n_modes, lens, flat, cov, z1, z2):
    import ctypes

    import torch

    nb = ctypes.c_size_t()
    assert lib.gst_grid_tc_workspace_size(dim, n_modes, lens, ctypes.byref(nb)) == 0
    ws = torch.empty(nb.value, dtype=torch.uint8, device="cuda")
    p = [ctypes.c_void_p(t.data_ptr()) for t in (flat, cov, z1, z2, ws)]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.gst_grid_tc_tables(dim, n_modes, lens, *p, nb, stream) == 0
    return ws, nb


@pytest.mark.parametrize("dim,shape", [(3, (100, 24, 40)), (2, (700, 90))])
def test_tc_contract_rows(cuda_lib, dim, shape):
    """Slab-by-slab contraction writes only its rows and, slab by slab,
    gives the whole-grid contraction (up to split-tile rounding)."""
    import ctypes

    import torch

    from gstools_gb300 import _native

    n_modes = 301
    cov, z1, z2 = case(5 + dim, dim, n_modes)
    axes = [np.arange(float(n)) * 0.8 for n in shape]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    flat = t(np.concatenate(axes))
    lens = (ctypes.c_int64 * 4)(*(list(shape) + [1] * (4 - dim)))
    ws, nb = _tc_workspace(cuda_lib, dim, n_modes, lens, flat, t(cov), t(z1), t(z2))
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    wsp = ctypes.c_void_p(ws.data_ptr())
    full = torch.full(shape, float("nan"), dtype=torch.float32, device="cuda")
    assert cuda_lib.gst_grid_tc_contract(dim, n_modes, lens, wsp, nb,
                                         ctypes.c_void_p(full.data_ptr()),
                                         _native.GST_OUT_F32, 0.5, stream) == 0
    xb = 16 if dim == 3 else 256
    cuts = [0, xb, 3 * xb, shape[0]] if dim == 3 else [0, 2 * xb, shape[0]]
    part = torch.full(shape, float("nan"), dtype=torch.float32, device="cuda")
    for k, (x0, x1) in enumerate(zip(cuts[:-1], cuts[1:])):
        assert cuda_lib.gst_grid_tc_contract_rows(
            dim, n_modes, lens, wsp, nb, ctypes.c_void_p(part.data_ptr()),
            _native.GST_OUT_F32, 0.5, x0, x1, stream) == 0
        got = part.cpu().numpy()
        assert not np.isnan(got[:x1]).any() and np.isnan(got[x1:]).all(), k
    ref = full.cpu().numpy()
    np.testing.assert_allclose(got, ref, rtol=0, atol=2e-6 * np.abs(ref).max())
    # misaligned or out-of-range rows are rejected before any launch
    for x0, x1 in ((1, xb), (0, xb + 1), (xb, 0), (0, shape[0] + 1), (-xb, 0)):
        if x1 == shape[0]:
            continue
        rc = cuda_lib.gst_grid_tc_contract_rows(
            dim, n_modes, lens, wsp, nb, ctypes.c_void_p(part.data_ptr()),
            _native.GST_OUT_F32, 0.5, x0, x1, stream)
        assert rc == _native.GST_ERR_INVALID_ARGUMENT, (x0, x1)


@pytest.mark.parametrize("kind", ["scalar", "incompr", "fourier"])
@pytest.mark.parametrize("shape,out_dtype", [
    ((128, 256, 256), "float32"),      # 32 MiB per component: 2 slabs
    ((256, 128, 256), "float64"),      # 64 MiB: 4 slabs
    ((2048, 4096), "float32"),         # 2-D, 32 MiB: 2 slabs of 1024 rows
    ((300, 7, 33), "float64")])        # small: one slab, pageable result
def test_tc_host_entry_points(cuda_lib, kind, shape, out_dtype):
    """The *_grid_tc_host entry points (numpy in, numpy out) against the
    device entry points on the same inputs, and against the oracle on a
    subsample of the grid."""
    import torch

    dim, n_modes = len(shape), 200
    cov, z1, z2 = case(len(kind) + dim, dim, n_modes, k_scale=0.05)
    axes = [np.arange(float(n)) * 0.5 for n in shape]
    fac = np.random.RandomState(3).uniform(0.2, 1.2, size=n_modes)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    if kind == "scalar":
        host = gg.summate_grid(cov, z1, z2, axes, precision="mixed",
                               method="tensor", out_dtype=out_dtype)
        dev = gg.summate_grid(t(cov), t(z1), t(z2), [t(a) for a in axes],
                              precision="mixed", method="tensor",
                              out_dtype=out_dtype)
    elif kind == "incompr":
        host = gg.summate_incompr_grid(cov, z1, z2, axes, precision="mixed",
                                       method="tensor", out_dtype=out_dtype)
        dev = gg.summate_incompr_grid(t(cov), t(z1), t(z2), [t(a) for a in axes],
                                      precision="mixed", method="tensor",
                                      out_dtype=out_dtype)
    else:
        host = gg.summate_fourier_grid(fac, cov, z1, z2, axes,
                                       out_dtype=out_dtype)
        dev = gg.summate_fourier_grid(t(fac), t(cov), t(z1), t(z2),
                                      [t(a) for a in axes], out_dtype=out_dtype)
    assert isinstance(host, np.ndarray) and host.dtype == np.dtype(out_dtype)
    dev = dev.cpu().numpy()
    assert host.shape == dev.shape
    np.testing.assert_allclose(host, dev, rtol=0,
                               atol=2e-6 * np.abs(dev).max())
    sub = [a[:: max(1, len(a) // 12)] for a in axes]
    idx = np.ix_(*[np.arange(0, len(a), max(1, len(a) // 12)) for a in axes])
    grid = np.array(np.meshgrid(*sub, indexing="ij")).reshape(dim, -1)
    sub_shape = [len(a) for a in sub]
    if kind == "scalar":
        ref = oracle.c_summate(cov, z1, z2, grid).reshape(sub_shape)
        got, norm = host[idx], np.sqrt(n_modes)
    elif kind == "incompr":
        ref = oracle.c_summate_incompr(cov, z1, z2, grid).reshape([dim] + sub_shape)
        got, norm = host[(slice(None),) + idx], np.sqrt(n_modes)
    else:
        ref = oracle.c_summate_fourier(fac, cov, z1, z2, grid).reshape(sub_shape)
        got, norm = host[idx], np.sqrt(np.sum(fac ** 2))
    d = (got.astype(np.float64) - ref) / norm
    assert np.sqrt(np.mean(d ** 2)) <= RMS_SIGMA and np.abs(d).max() <= MAX_SIGMA


@pytest.fixture
def tf32_operands(cuda_lib):
    from gstools_gb300 import _native

    prev = _native.set_tc_operands("tf32")
    yield
    _native.set_tc_operands(prev)


@pytest.mark.parametrize("dim,shape,n_modes", [
    (2, (300, 257), 203), (3, (40, 33, 70), 500)])
def test_tc_tf32_operands(tf32_operands, dim, shape, n_modes):
    """The 3xTF32 operand variant keeps the same bar as the default FP16 one."""
    cov, z1, z2 = case(dim * 31 + n_modes, dim, n_modes)
    axes = [np.arange(float(n)) * 0.7 for n in shape]
    ref = grid_ref(cov, z1, z2, axes)
    got = gg.summate_grid(cov, z1, z2, axes, precision="mixed",
                          method="tensor")
    rms, mx = errors(got, ref, n_modes)
    assert rms <= RMS_SIGMA and mx <= MAX_SIGMA, (rms, mx)


@pytest.mark.parametrize("amp", [1e-7, 3e-3, 1.0, 5e4, 1e9])
def test_tc_amplitude_range(cuda_lib, amp):
    """FP16 operands: amplitudes far outside FP16 range are normalised by a
    power of two, so the relative error does not depend on their size."""
    cov, z1, z2 = case(17, 3, 300)
    axes = [np.arange(24.0), np.arange(17.0) * 1.3, np.arange(40.0) * 0.6]
    ref = grid_ref(cov, z1, z2, axes)
    got = gg.summate_grid(cov, amp * z1, amp * z2, axes, precision="mixed",
                          method="tensor")
    rms, mx = errors(got / amp, ref, 300)
    assert rms <= RMS_SIGMA and mx <= MAX_SIGMA, (rms, mx)


def test_tc_fourier_small_spectrum_factor(cuda_lib):
    """summate_fourier with spectrum factors spanning 8 decades (the decay of
    a spectral density) keeps the bar relative to the field's scale."""
    cov, z1, z2 = case(23, 2, 400)
    fac = np.exp(-np.linspace(0.0, 18.0, 400)) * 1e-3
    shape = (60, 70)
    axes = [np.linspace(-10.0, 30.0, n) for n in shape]
    grid = np.array(np.meshgrid(*axes, indexing="ij")).reshape(2, -1)
    ref = oracle.c_summate_fourier(fac, cov, z1, z2, grid).reshape(shape)
    got = gg.summate_fourier_grid(fac, cov, z1, z2, axes)
    d = (got - ref) / np.sqrt(np.sum(fac ** 2))
    assert np.sqrt(np.mean(d ** 2)) <= RMS_SIGMA and np.abs(d).max() <= MAX_SIGMA


def test_tc_full_size_workload(cuda_lib, workloads):
    """The 256^3 x 2000-mode Exponential workload at full size: the oracle at
    4096 random grid points (bar of this file), and two size-independent
    properties: scaling the amplitudes by a power of two scales the field
    exactly (the FP16 normalisation takes out that power), and the field is
    linear in (z_1, z_2) within the bar."""
    import torch

    cov = workloads["exp3d/isometrize"].T @ workloads["exp3d/cov"]
    z1, z2 = workloads["exp3d/z1"], workloads["exp3d/z2"]
    n, n_modes = 256, cov.shape[1]
    axes = [np.arange(float(n))] * 3
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    dax = [t(a) for a in axes]
    run = lambda a, b: gg.summate_grid(t(cov), t(a), t(b), dax, precision="mixed",
                                       method="tensor", out_dtype="float32")
    f = run(z1, z2)
    rng = np.random.RandomState(4)
    idx = rng.randint(0, n, size=(3, 4096))
    ref = oracle.c_summate(cov, z1, z2, idx.astype(np.float64))
    got = f[idx[0], idx[1], idx[2]].double().cpu().numpy()
    rms, mx = errors(got, ref, n_modes, var=2.0)
    assert rms <= RMS_SIGMA and mx <= MAX_SIGMA, (rms, mx)
    f8 = run(8.0 * z1, 8.0 * z2)
    assert torch.equal(f8, 8.0 * f)
    za, zb = rng.normal(size=n_modes), rng.normal(size=n_modes)
    fa, fb, fab = run(za, zb), run(z1 - za, z2 - zb), f
    d = np.sqrt(1.0 / n_modes) * (fa + fb - fab).double().cpu().numpy()
    assert np.sqrt(np.mean(d ** 2)) <= 2 * RMS_SIGMA
