"""GPU adjoint of summate vs float64 torch autograd and finite differences.

Bars: FP64 adjoint within 1e-10 (relative, max norm) of float64 torch
autograd of the same sum; mixed precision within 1e-4; model-parameter
gradients (len_scale, anisotropy, rotation angles) within 1e-5 of central
differences with h = 1e-6 in float64.
"""

import numpy as np
import pytest
import torch

import gstools_gb300 as gg
from gstools_gb300.grad import isometrize_matrix, randmeth_field, summate_torch

pytestmark = pytest.mark.gpu


def torch_reference(cov, z1, z2, pos):
    phase = cov.T @ pos
    return z1 @ torch.cos(phase) + z2 @ torch.sin(phase)


def rel(a, b):
    return (torch.max(torch.abs(a - b)) / torch.max(torch.abs(b))).item()


def leaves(seed, dim, n_modes, n_pts, dev="cuda"):
    g = torch.Generator().manual_seed(seed)
    mk = lambda *s, sc=1.0: (torch.randn(*s, generator=g, dtype=torch.float64)
                             * sc).to(dev).requires_grad_(True)
    cov = mk(dim, n_modes, sc=0.3)
    z1, z2 = mk(n_modes), mk(n_modes)
    pos = (torch.rand(dim, n_pts, generator=g, dtype=torch.float64) * 50).to(
        dev).requires_grad_(True)
    w = torch.randn(n_pts, generator=g, dtype=torch.float64).to(dev)
    return cov, z1, z2, pos, w


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("precision,tol", [("f64", 1e-10), ("mixed", 1e-4)])
def test_vjp_matches_torch_autograd(cuda_lib, dim, precision, tol):
    cov, z1, z2, pos, w = leaves(dim, dim, 257, 1500)
    (torch_reference(cov, z1, z2, pos) * w).sum().backward()
    ref = [t.grad.clone() for t in (cov, z1, z2, pos)]
    for t in (cov, z1, z2, pos):
        t.grad = None
    out = summate_torch(cov, z1, z2, pos, precision)
    assert rel(out, torch_reference(cov, z1, z2, pos).detach()) <= tol
    (out * w).sum().backward()
    for name, t, r in zip(("cov", "z1", "z2", "pos"), (cov, z1, z2, pos), ref):
        assert rel(t.grad, r) <= tol, (name, rel(t.grad, r))


@pytest.mark.parametrize("dim", [2, 3])
def test_vjp_mixed_far_from_origin(cuda_lib, dim):
    """Points 2e5 from the origin: the mixed adjoint sums run relative to the
    first point and are rotated back per mode; gradients match the FP64
    adjoint (cov gradients scale with |x|, so compared on their own norm)."""
    cov, z1, z2, pos, w = leaves(10 + dim, dim, 300, 2000)
    with torch.no_grad():
        pos += 2.0e5
    grads = {}
    for prec in ("f64", "mixed"):
        for t in (cov, z1, z2, pos):
            t.grad = None
        (summate_torch(cov, z1, z2, pos, prec) * w).sum().backward()
        grads[prec] = [t.grad.clone() for t in (cov, z1, z2, pos)]
    for name, a, b in zip(("cov", "z1", "z2", "pos"), grads["mixed"], grads["f64"]):
        assert rel(a, b) <= 1e-4, (name, rel(a, b))


def test_vjp_workload_modes(cuda_lib, workloads):
    """4000 modes of the 3-D Gaussian (reference RNG) at 2048 points."""
    c = workloads.case("gau3d_grad")
    dev = "cuda"
    cov = torch.tensor(c["isometrize"].T @ c["cov"], device=dev, requires_grad=True)
    z1 = torch.tensor(c["z1"], device=dev, requires_grad=True)
    z2 = torch.tensor(c["z2"], device=dev, requires_grad=True)
    pos = torch.tensor(c["pos"], device=dev, requires_grad=True)
    w = torch.randn(pos.shape[1], dtype=torch.float64, device=dev)
    (torch_reference(cov, z1, z2, pos) * w).sum().backward()
    ref = [t.grad.clone() for t in (cov, z1, z2, pos)]
    for t in (cov, z1, z2, pos):
        t.grad = None
    (summate_torch(cov, z1, z2, pos, "f64") * w).sum().backward()
    for t, r in zip((cov, z1, z2, pos), ref):
        assert rel(t.grad, r) <= 1e-10


def test_model_parameter_gradients_vs_finite_differences(cuda_lib, workloads):
    c = workloads.case("gau3d_grad")
    dev = "cuda"
    cov_ref = torch.tensor(c["cov"][:, :500], device=dev)
    z1 = torch.tensor(c["z1"][:500], device=dev)
    z2 = torch.tensor(c["z2"][:500], device=dev)
    rng = np.random.RandomState(5)
    obs = torch.tensor(rng.uniform(0.0, 128.0, (3, 400)), device=dev)
    target = torch.tensor(rng.normal(size=400), device=dev)
    p0 = {"len_scale": 16.0, "anis": [0.8, 0.6], "angles": [0.3, 0.2, 0.1],
          "var": 1.0}

    def loss(p):
        u = randmeth_field(cov_ref, 16.0, z1, z2, obs, precision="f64", **p)
        return torch.mean((u - target) ** 2)

    params = {k: torch.tensor(v, dtype=torch.float64, device=dev,
                              requires_grad=True) for k, v in p0.items()}
    loss(params).backward()
    h = 1e-6
    for name in ("len_scale", "anis", "angles", "var"):
        grad = params[name].grad.reshape(-1)
        base = np.atleast_1d(np.array(p0[name], dtype=np.float64))
        for i in range(base.size):
            vals = []
            for sgn in (1.0, -1.0):
                b = base.copy()
                b[i] += sgn * h
                q = {k: torch.tensor(v, dtype=torch.float64, device=dev)
                     for k, v in p0.items()}
                q[name] = torch.tensor(b if base.size > 1 else b[0],
                                       dtype=torch.float64, device=dev)
                vals.append(loss(q).item())
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(grad[i].item() - fd) <= 1e-5 * max(abs(fd), 1e-3), (
                name, i, grad[i].item(), fd)


def test_vjp_empty_points(cuda_lib):
    cov, z1, z2, _, _ = leaves(3, 2, 40, 10)
    pos = torch.zeros((2, 0), dtype=torch.float64, device="cuda",
                      requires_grad=True)
    out = summate_torch(cov, z1, z2, pos, "f64")
    out.sum().backward()
    assert torch.all(cov.grad == 0) and torch.all(z1.grad == 0)


@pytest.mark.parametrize("precision,tol", [("f64", 1e-12), ("mixed", 1e-5)])
def test_sparse_cotangent_matches_all_points(cuda_lib, precision, tol):
    """A loss on 1 % of the points: the backward that runs the adjoint
    kernels on the points with a nonzero cotangent only gives the gradients
    of the backward over all points (same terms, other summation order)."""
    from gstools_gb300 import grad

    cov, z1, z2, pos, _ = leaves(21, 3, 700, 40_000)
    obs = torch.arange(0, 40_000, 97, device="cuda")
    target = torch.randn(obs.numel(), dtype=torch.float64, device="cuda")
    results = {}
    for sparse in (True, False):
        grad.SPARSE_COTANGENT = sparse
        try:
            for t in (cov, z1, z2, pos):
                t.grad = None
            u = summate_torch(cov, z1, z2, pos, precision)
            torch.mean((u[obs] - target) ** 2).backward()
            results[sparse] = [t.grad.clone() for t in (cov, z1, z2, pos)]
        finally:
            grad.SPARSE_COTANGENT = True
    for name, a, b in zip(("cov", "z1", "z2", "pos"), results[True],
                          results[False]):
        assert rel(a, b) <= tol, (name, rel(a, b))
    # positions off the observation set get exactly zero
    mask = torch.ones(40_000, dtype=torch.bool, device="cuda")
    mask[obs] = False
    assert torch.all(results[True][3][:, mask] == 0)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("sparse", [True, False])
def test_grid_function_matches_point_function(cuda_lib, dim, sparse):
    """The structured-grid form (tensor-core forward in mixed precision, the
    FP64 grid kernel in FP64; adjoint on the grid points gathered from the
    axes) against the point form on the meshgrid of the same axes: fields
    and mode gradients of a loss on a subset (sparse cotangent) or on every
    point (dense)."""
    from gstools_gb300 import grad
    from gstools_gb300.grad import summate_grid_torch

    cov, z1, z2, _, _ = leaves(30 + dim, dim, 600, 10)
    shape = (40, 36, 20)[:dim]
    axes = [torch.linspace(-30.0, 50.0, n, dtype=torch.float64, device="cuda")
            for n in shape]
    mesh = torch.stack([m.reshape(-1) for m in
                        torch.meshgrid(*axes, indexing="ij")]).contiguous()
    n = mesh.shape[1]
    obs = torch.arange(0, n, 37, device="cuda") if sparse else torch.arange(
        n, device="cuda")
    target = torch.randn(obs.numel(), dtype=torch.float64, device="cuda")
    tol = {"f64": (1e-12, 1e-10), "mixed": (2e-5, 1e-4)}
    for prec in ("f64", "mixed"):
        res = {}
        for form in ("grid", "points"):
            for t in (cov, z1, z2):
                t.grad = None
            u = (summate_grid_torch(cov, z1, z2, axes, prec) if form == "grid"
                 else summate_torch(cov, z1, z2, mesh, prec))
            torch.mean((u[obs] - target) ** 2).backward()
            res[form] = [u.detach()] + [t.grad.clone() for t in (cov, z1, z2)]
        assert grad.SPARSE_COTANGENT
        ftol, gtol = tol[prec]
        assert rel(res["grid"][0], res["points"][0]) <= ftol, (prec, "field")
        for name, a, b in zip(("cov", "z1", "z2"), res["grid"][1:],
                              res["points"][1:]):
            assert rel(a, b) <= gtol, (prec, name, rel(a, b))


def test_randmeth_field_grid_and_points(cuda_lib, workloads):
    """randmeth_field on a grid plus scattered points (the grid's values
    first) equals the point form on the meshgrid followed by the points, and
    so do the gradients of the points and the model parameters (FP64)."""
    c = workloads.case("gau3d_grad")
    dev = "cuda"
    cov_ref = torch.tensor(c["cov"][:, :300], device=dev)
    z1 = torch.tensor(c["z1"][:300], device=dev)
    z2 = torch.tensor(c["z2"][:300], device=dev)
    axes = [torch.arange(float(n), dtype=torch.float64, device=dev) * 2.0
            for n in (12, 10, 8)]
    mesh = torch.stack([m.reshape(-1) for m in
                        torch.meshgrid(*axes, indexing="ij")])
    pts = (torch.rand((3, 500), dtype=torch.float64, device=dev) * 24.0
           ).requires_grad_(True)
    p0 = {"len_scale": 16.0, "anis": [0.8, 0.6], "angles": [0.3, 0.2, 0.1],
          "var": 1.0}
    res = {}
    for form in ("grid", "points"):
        pts.grad = None
        params = {k: torch.tensor(v, dtype=torch.float64, device=dev,
                                  requires_grad=True) for k, v in p0.items()}
        if form == "grid":
            u = randmeth_field(cov_ref, 16.0, z1, z2, pts, axes=axes,
                               precision="f64", **params)
        else:
            u = randmeth_field(cov_ref, 16.0, z1, z2, torch.cat([mesh, pts], 1),
                               precision="f64", **params)
        torch.sum(u[::7] ** 2).backward()
        res[form] = [u.detach(), pts.grad.clone()] + [
            params[k].grad.clone() for k in ("len_scale", "anis", "angles", "var")]
    for a, b in zip(res["grid"], res["points"]):
        assert rel(a, b) <= 1e-10


def test_gather_points_kernel(cuda_lib):
    """gst_gather_points: grid points unravelled from the axes ("ij"), extra
    points copied, cotangents picked; an out-of-range index gives zeros."""
    import ctypes

    from gstools_gb300 import _native
    from gstools_gb300.summator import _p, _stream

    dev = torch.device("cuda")
    ax = [torch.linspace(0.0, 1.0, n, dtype=torch.float64, device=dev) + 10.0 * d
          for d, n in enumerate((5, 4, 3))]
    extra = torch.randn(3, 7, dtype=torch.float64, device=dev)
    mesh = torch.stack([m.reshape(-1) for m in torch.meshgrid(*ax, indexing="ij")])
    allx = torch.cat([mesh, extra], 1)
    g = torch.randn(allx.shape[1], dtype=torch.float64, device=dev)
    idx = torch.tensor([0, 7, 59, 60, 66, 3, 67, -1], dtype=torch.int64, device=dev)
    xs = torch.empty(3, idx.numel(), dtype=torch.float64, device=dev)
    gs = torch.empty(idx.numel(), dtype=torch.float64, device=dev)
    lens = (ctypes.c_int64 * 3)(5, 4, 3)
    _native.call("gst_gather_points", 3, lens, _p(torch.cat(ax)), 7, _p(extra),
                 idx.numel(), _p(idx), _p(g), _p(xs), _p(gs), _stream(dev))
    torch.cuda.synchronize()
    good = idx[:6]
    assert torch.equal(xs[:, :6], allx[:, good])
    assert torch.equal(gs[:6], g[good])
    assert torch.all(xs[:, 6:] == 0) and torch.all(gs[6:] == 0)


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_device_mode_map_matches_host(cuda_lib, dim):
    """gst_mode_map (map and Jacobian on the device) against the host map
    and its analytic derivative."""
    from gstools_gb300.grad import _ModeMap, _ModeMapDevice

    rng = np.random.RandomState(40 + dim)
    n_anis, n_ang = dim - 1, dim * (dim - 1) // 2
    for _ in range(4):
        vals = np.concatenate([[rng.uniform(2.0, 40.0)], rng.uniform(0.2, 3.0, n_anis),
                               rng.uniform(-3.0, 3.0, n_ang)])
        weight = torch.tensor(rng.normal(size=(dim, dim)))
        host = torch.tensor(vals, requires_grad=True)
        dev = torch.tensor(vals, device="cuda", requires_grad=True)
        mh = _ModeMap.apply(host, dim, 13.0)
        md = _ModeMapDevice.apply(dev, dim, 13.0)
        assert torch.allclose(md.cpu(), mh, rtol=0, atol=1e-14)
        (mh * weight).sum().backward()
        (md * weight.cuda()).sum().backward()
        assert torch.allclose(dev.grad.cpu(), host.grad, rtol=1e-12, atol=1e-14)
