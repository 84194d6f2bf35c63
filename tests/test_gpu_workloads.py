"""Parity at the full benchmark sizes of the ensemble and gradient workloads.

* 512-realization ensemble (2-D Matern nu=1.5, var 1, len_scale log-uniform
  in [2, 50], 1000 / 2000 / 4000 modes, 1k-200k points each in [0, 500]^2,
  the reference's ensemble loop of examples/01_random_field/
  01_srf_ensemble.py run as one batch): the persistent kernel replayed from
  its CUDA graph, every realization checked against the FP64 C oracle on a
  fixed subsample of 256 of its points.  Bar: RMS <= 1e-5 sigma per
  realization.
* Differentiable field (3-D Gaussian, 4000 modes, 128^3 grid plus 50 000
  points in [0, 128]^3, loss = mean squared misfit at 10 000 observation
  points against a field of another seed): dL/dz_1, dL/dz_2 and dL/dk from
  the adjoint kernels over all 2 147 152 points against float64 torch
  autograd of the same loss (the points off the observation set contribute
  zero), and dL/dlen_scale, dL/danis, dL/dangles against central
  differences with h = 1e-6 of the full loss in float64.  Bars: FP64 adjoint
  1e-10 relative (max norm), mixed precision 1e-4, parameters 1e-5 of the
  difference quotient.
"""

import numpy as np
import pytest
import torch

import gstools_gb300 as gg
import oracle
from gstools_gb300.grad import isometrize_matrix, randmeth_field, summate_torch

pytestmark = pytest.mark.gpu

RMS_SIGMA = 1e-5


def test_ensemble512_every_realization_vs_oracle(cuda_lib):
    import bench

    gens, pos = bench.make_ensemble()
    assert len(gens) == 512
    modes = [g.mode_no for g in gens]
    pts = [p.shape[1] for p in pos]
    assert set(modes) == {1000, 2000, 4000}
    assert 1000 <= min(pts) and max(pts) <= 200_000
    scales = [np.sqrt(1.0 / m) for m in modes]
    bs = gg.BatchedSummator(2, modes, pts, out_dtype="float32", graph=True)
    bs.load([g.cov_samples for g in gens], [g.z_1 for g in gens],
            [g.z_2 for g in gens], pos, scales)
    bs.tune()
    bs.run()
    bs.run()          # graph replay
    torch.cuda.synchronize()
    fields = bs.split()
    rng = np.random.RandomState(3)
    worst = 0.0
    for r, (g, f) in enumerate(zip(gens, fields)):
        idx = np.sort(rng.choice(pts[r], size=min(256, pts[r]), replace=False))
        ref = scales[r] * oracle.c_summate(g.cov_samples, g.z_1, g.z_2,
                                           np.ascontiguousarray(pos[r][:, idx]))
        rms = np.sqrt(np.mean((f[idx].astype(np.float64) - ref) ** 2))
        worst = max(worst, rms)
        assert rms <= RMS_SIGMA, (r, rms)
    assert worst > 0.0


@pytest.fixture(scope="module")
def adjoint_case(workloads):
    c = workloads.case("gau3d_grad")
    dev = "cuda"
    rng = np.random.RandomState(7)
    g = np.arange(128.0)
    grid = np.array(np.meshgrid(g, g, g, indexing="ij")).reshape(3, -1)
    pts = np.concatenate([grid, rng.uniform(0.0, 128.0, (3, 50_000))], axis=1)
    obs = np.sort(rng.choice(pts.shape[1], 10_000, replace=False))
    other = gg.RandMeth(gg.Gaussian(dim=3, var=1.0, len_scale=16.0),
                        mode_no=4000, seed=4242, sampling="analytic")
    target = np.sqrt(1.0 / 4000) * oracle.c_summate(
        other.cov_samples, other.z_1, other.z_2,
        np.ascontiguousarray(pts[:, obs]))
    return dict(cov_ref=torch.tensor(c["cov"], device=dev),
                z1=c["z1"], z2=c["z2"], x=torch.tensor(pts, device=dev),
                obs=torch.tensor(obs, device=dev),
                x_obs=torch.tensor(pts[:, obs], device=dev),
                target=torch.tensor(target, device=dev))


P0 = {"len_scale": 16.0, "anis": [0.8, 0.6], "angles": [0.3, 0.2, 0.1],
      "var": 1.0}


def _k(case, p):
    m = isometrize_matrix(3, p["angles"], p["anis"]).to("cuda")
    return m.T @ (case["cov_ref"] * (16.0 / p["len_scale"]))


@pytest.mark.parametrize("precision,tol", [("f64", 1e-10), ("mixed", 1e-4)])
def test_adjoint_full_size_vs_torch_autograd(cuda_lib, adjoint_case,
                                             precision, tol):
    case = adjoint_case
    p = {k: torch.tensor(v, dtype=torch.float64, device="cuda")
         for k, v in P0.items()}
    k0 = _k(case, p).detach()
    s = np.sqrt(1.0 / 4000)

    def leaves():
        return (k0.clone().requires_grad_(True),
                torch.tensor(case["z1"], device="cuda", requires_grad=True),
                torch.tensor(case["z2"], device="cuda", requires_grad=True))

    # the adjoint kernels: forward on every point, loss at the observations
    k, z1, z2 = leaves()
    u = s * summate_torch(k, z1, z2, case["x"], precision)
    torch.mean((u[case["obs"]] - case["target"]) ** 2).backward()
    got = [t.grad for t in (k, z1, z2)]
    # float64 torch autograd of the same loss (only observed points matter)
    k, z1, z2 = leaves()
    ph = k.T @ case["x_obs"]
    u_ref = s * (z1 @ torch.cos(ph) + z2 @ torch.sin(ph))
    torch.mean((u_ref - case["target"]) ** 2).backward()
    for name, a, b in zip(("dk", "dz1", "dz2"), got, (k.grad, z1.grad, z2.grad)):
        r = (torch.max(torch.abs(a - b)) / torch.max(torch.abs(b))).item()
        assert r <= tol, (name, r)


def test_model_parameters_full_size_vs_finite_differences(cuda_lib,
                                                          adjoint_case):
    case = adjoint_case
    z1 = torch.tensor(case["z1"], device="cuda")
    z2 = torch.tensor(case["z2"], device="cuda")

    def loss(p):
        u = randmeth_field(case["cov_ref"], 16.0, z1, z2, case["x"],
                           precision="f64", **p)
        return torch.mean((u[case["obs"]] - case["target"]) ** 2)

    params = {k: torch.tensor(v, dtype=torch.float64, device="cuda",
                              requires_grad=True) for k, v in P0.items()}
    loss(params).backward()
    h = 1e-6
    for name in ("len_scale", "anis", "angles"):
        grad = params[name].grad.reshape(-1)
        base = np.atleast_1d(np.array(P0[name], dtype=np.float64))
        for i in range(base.size):
            vals = []
            for sgn in (1.0, -1.0):
                b = base.copy()
                b[i] += sgn * h
                q = {kk: torch.tensor(v, dtype=torch.float64, device="cuda")
                     for kk, v in P0.items()}
                q[name] = torch.tensor(b if base.size > 1 else b[0],
                                       dtype=torch.float64, device="cuda")
                with torch.no_grad():
                    vals.append(loss(q).item())
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(grad[i].item() - fd) <= 1e-5 * max(abs(fd), 1e-3), (
                name, i, grad[i].item(), fd)
