"""Host side of the differentiable field (CPU): the analytic derivative of
the mode map M(angles, anis)^T len_scale_ref / len_scale against torch
autograd through the explicit Givens construction of isometrize_matrix
(the reference's src/gstools/tools/geometric.py:184-294)."""

import numpy as np
import pytest
import torch

from gstools_gb300.grad import _ModeMap, isometrize_matrix


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_mode_map_matches_autograd(dim):
    rng = np.random.RandomState(dim)
    n_anis, n_ang = dim - 1, dim * (dim - 1) // 2
    for _ in range(5):
        ls0 = float(rng.uniform(2.0, 40.0))
        anis = torch.tensor(rng.uniform(0.2, 3.0, n_anis), requires_grad=True)
        angles = torch.tensor(rng.uniform(-3.0, 3.0, n_ang), requires_grad=True)
        ls = torch.tensor(float(rng.uniform(2.0, 40.0)), dtype=torch.float64,
                          requires_grad=True)
        weight = torch.tensor(rng.normal(size=(dim, dim)))
        ref = isometrize_matrix(dim, angles, anis).T * (ls0 / ls)
        (ref * weight).sum().backward()
        grads = [torch.zeros(t.numel(), dtype=torch.float64) if t.grad is None
                 else t.grad.reshape(-1) for t in (ls, anis, angles)]
        packed = torch.cat([ls.detach().reshape(1), anis.detach(),
                            angles.detach()]).requires_grad_(True)
        got = _ModeMap.apply(packed, dim, ls0)
        np.testing.assert_allclose(got.detach().numpy(), ref.detach().numpy(),
                                   rtol=0, atol=1e-14)
        (got * weight).sum().backward()
        np.testing.assert_allclose(packed.grad.numpy(), torch.cat(grads).numpy(),
                                   rtol=1e-12, atol=1e-14)
