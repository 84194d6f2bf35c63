"""Differentiable randomization-method fields (torch.autograd).

:class:`SummateFunction` wraps the GPU summation and its hand-written adjoint
(``gst_summate_vjp_modes_*`` for dL/dz_1, dL/dz_2, dL/dk and
``gst_summate_vjp_pos_*`` for dL/dx; include/gstools_gb300.h).  The forward
stores only its inputs; the backward recomputes sin/cos.

:func:`isometrize_matrix` rebuilds the reference's isometrize map
(src/gstools/tools/geometric.py:184-294: derotation by Givens rotations with
alternating Tait-Bryan signs, then diag(1, 1/anis)) from torch tensors, and
:func:`randmeth_field` chains everything the reference's RandMeth does
(generator.py:243-270 with covmodel/base.py:572-582): the field at physical
positions x is

    u(x) = sqrt(var / N) * summate(M^T k(len_scale), z_1, z_2, x)

with M = isometrize_matrix(angles, anis) and k(len_scale) = k_ref *
(len_scale_ref / len_scale) -- the radial law of every model scales its wave
numbers by 1 / len_rescaled (covmodel/models.py:143-186, 226-270), so
gradients reach len_scale, the anisotropy ratios and the rotation angles.
"""

import ctypes

import torch

from . import _native, config
from .summator import _p, _stream, device

__all__ = ["SummateFunction", "summate_torch", "isometrize_matrix",
           "randmeth_field", "SPARSE_COTANGENT"]

# Run the adjoint kernels on the points with a nonzero cotangent only, when
# at most a quarter of the points have one (read at every backward).  The
# gradients are the same sums; points whose cotangent is zero are left out,
# so a non-finite coordinate there no longer turns the mode gradients NaN.
SPARSE_COTANGENT = True


def _dev_f64(t, dev):
    return t.detach().to(device=dev, dtype=torch.float64).contiguous()


class SummateFunction(torch.autograd.Function):
    """``u = summate(cov_samples, z_1, z_2, pos)`` with a GPU adjoint."""

    @staticmethod
    def forward(ctx, cov_samples, z_1, z_2, pos, precision):
        prec = config.check_precision(precision)
        dev = device()
        cov = _dev_f64(cov_samples, dev)
        z1 = _dev_f64(z_1, dev).reshape(-1)
        z2 = _dev_f64(z_2, dev).reshape(-1)
        dim, n_modes = cov.shape
        x = _dev_f64(pos, dev).reshape(dim, -1)
        out = torch.empty(x.shape[1], dtype=torch.float64, device=dev)
        name = "gst_summate_f64" if prec == "f64" else "gst_summate_mixed"
        args = [dim, n_modes, x.shape[1], _p(cov), _p(z1), _p(z2), _p(x), _p(out)]
        if prec == "mixed":
            args.append(_native.GST_OUT_F64)
        _native.call(name, *args, _stream(dev))
        ctx.save_for_backward(cov, z1, z2, x)
        ctx.prec = prec
        ctx.in_devices = [t.device for t in (cov_samples, z_1, z_2, pos)]
        return out.to(pos.device) if pos.device != dev else out

    @staticmethod
    def backward(ctx, grad_out):
        cov, z1, z2, x = ctx.saved_tensors
        dev = cov.device
        dim, n_modes = cov.shape
        n_pts = x.shape[1]
        g = _dev_f64(grad_out, dev).reshape(-1)
        stream = _stream(dev)
        need_cov, need_z1, need_z2, need_pos = ctx.needs_input_grad[:4]
        d_cov = d_z1 = d_z2 = d_pos = None
        # Points whose cotangent is exactly zero add nothing to the mode
        # gradients and get a zero position gradient; when at most a quarter
        # of the points carry one (a loss on a subset of the field) the
        # adjoint kernels run on those points only.
        idx = None
        if SPARSE_COTANGENT and n_pts > 0:
            nnz = int(torch.count_nonzero(g))
            if 4 * nnz <= n_pts:
                idx = torch.nonzero(g).reshape(-1)
        xs, gs = (x, g) if idx is None else (x.index_select(1, idx).contiguous(),
                                             g.index_select(0, idx).contiguous())
        n_sel = xs.shape[1]
        if need_cov or need_z1 or need_z2:
            gz1 = torch.empty(n_modes, dtype=torch.float64, device=dev)
            gz2 = torch.empty(n_modes, dtype=torch.float64, device=dev)
            gk = torch.empty((dim, n_modes), dtype=torch.float64, device=dev)
            _native.call(f"gst_summate_vjp_modes_{ctx.prec}", dim, n_modes,
                         n_sel, _p(cov), _p(z1), _p(z2), _p(xs), _p(gs),
                         _p(gz1), _p(gz2), _p(gk), stream)
            d_cov = gk.to(ctx.in_devices[0]) if need_cov else None
            d_z1 = gz1.to(ctx.in_devices[1]) if need_z1 else None
            d_z2 = gz2.to(ctx.in_devices[2]) if need_z2 else None
        if need_pos:
            v = torch.empty((dim, n_sel), dtype=torch.float64, device=dev)
            _native.call(f"gst_summate_vjp_pos_{ctx.prec}", dim, n_modes,
                         n_sel, _p(cov), _p(z1), _p(z2), _p(xs), _p(v), stream)
            if idx is None:
                d_pos = v * g
            else:
                d_pos = torch.zeros((dim, n_pts), dtype=torch.float64, device=dev)
                d_pos.index_copy_(1, idx, v * gs)
            d_pos = d_pos.to(ctx.in_devices[3])
        return d_cov, d_z1, d_z2, d_pos, None


def summate_torch(cov_samples, z_1, z_2, pos, precision=None):
    """Differentiable ``summate`` on torch tensors (float64 result)."""
    return SummateFunction.apply(cov_samples, z_1, z_2, pos, precision)


def _givens(dim, plane, angle):
    rows = []
    c, s = torch.cos(angle), torch.sin(angle)
    one = torch.ones((), dtype=angle.dtype, device=angle.device)
    zero = torch.zeros((), dtype=angle.dtype, device=angle.device)
    for i in range(dim):
        row = []
        for j in range(dim):
            if (i, j) in ((plane[0], plane[0]), (plane[1], plane[1])):
                row.append(c)
            elif (i, j) == (plane[0], plane[1]):
                row.append(-s)
            elif (i, j) == (plane[1], plane[0]):
                row.append(s)
            else:
                row.append(one if i == j else zero)
        rows.append(torch.stack(row))
    return torch.stack(rows)


def isometrize_matrix(dim, angles, anis):
    """Torch version of the reference's ``matrix_isometrize``.

    ``angles`` has dim*(dim-1)/2 entries, ``anis`` dim-1 entries (tensors).
    """
    angles = torch.as_tensor(angles, dtype=torch.float64).reshape(-1)
    anis = torch.as_tensor(anis, dtype=torch.float64).reshape(-1)
    planes = [(i, j) for j in range(1, dim) for i in range(j)]
    rot = torch.eye(dim, dtype=torch.float64, device=angles.device)
    for i, plane in enumerate(planes):
        rot = rot @ _givens(dim, plane, (-1) ** i * (-angles[i]))
    stretch = torch.diag(torch.cat([torch.ones(1, dtype=torch.float64,
                                               device=anis.device), 1.0 / anis]))
    return stretch @ rot


def randmeth_field(cov_ref, len_scale_ref, z_1, z_2, pos, *, var, len_scale,
                   anis, angles, precision=None):
    """Field at physical positions ``pos`` (dim, n), differentiable in every
    tensor argument (``var``, ``len_scale``, ``anis``, ``angles``, ``z_1``,
    ``z_2``, ``pos``).  ``cov_ref`` are the model's wave vectors drawn at
    ``len_scale_ref``."""
    dim, n_modes = cov_ref.shape
    m = isometrize_matrix(dim, angles, anis).to(cov_ref.device)
    k = m.T @ (cov_ref * (len_scale_ref / len_scale))
    return torch.sqrt(var / n_modes) * summate_torch(k, z_1, z_2, pos,
                                                     precision)
