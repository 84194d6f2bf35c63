"""Differentiable randomization-method fields (torch.autograd).

:class:`SummateFunction` wraps the GPU summation and its hand-written adjoint
(``gst_summate_vjp_modes_*`` for dL/dz_1, dL/dz_2, dL/dk and
``gst_summate_vjp_pos_*`` for dL/dx; include/gstools_gb300.h).  The forward
stores only its inputs; the backward recomputes sin/cos.
:class:`SummateGridFunction` does the same for a structured grid (given by
its axes, forward on the tensor cores in mixed precision), optionally
followed by scattered points; its backward gathers the grid points with a
nonzero cotangent (``gst_gather_points``) into one adjoint call.

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
The map M^T len_scale_ref / len_scale and its Jacobian come from one device
kernel (``gst_mode_map``) for parameters on the GPU, from numpy for host
parameters.
"""

import ctypes

import torch

from . import _native, config
from .summator import _p, _stream, device

__all__ = ["SummateFunction", "SummateGridFunction", "summate_torch",
           "summate_grid_torch", "isometrize_matrix", "randmeth_field",
           "SPARSE_COTANGENT"]

# Run the adjoint kernels on the points with a nonzero cotangent only, when
# at most a quarter of the points have one (read at every backward).  The
# gradients are the same sums; points whose cotangent is zero are left out,
# so a non-finite coordinate there no longer turns the mode gradients NaN.
SPARSE_COTANGENT = True


def _dev_f64(t, dev):
    return t.detach().to(device=dev, dtype=torch.float64).contiguous()


def _cotangent_support(g, n_pts):
    """Indices of the points with a nonzero cotangent when at most a quarter
    of the points have one (one device sync), else None (all points)."""
    if not SPARSE_COTANGENT or n_pts == 0:
        return None
    idx = torch.nonzero(g).reshape(-1)
    return idx if 4 * idx.numel() <= n_pts else None


def _adjoint(ctx, g, cov, z1, z2, n_pts, gather, need_pos):
    """The mode (and position) gradients of ``u = summate(cov, z1, z2, x)``
    for the cotangent g; ``gather(idx)`` gives the coordinates and the
    cotangents of the points idx, or of all points for idx None.  Points
    whose cotangent is exactly zero add nothing to the mode gradients and
    get a zero position gradient; when at most a quarter of the points carry
    one (a loss on a subset of the field) the adjoint kernels run on those
    points only."""
    dev = cov.device
    dim, n_modes = cov.shape
    stream = _stream(dev)
    need_cov, need_z1, need_z2 = ctx.needs_input_grad[:3]
    d_cov = d_z1 = d_z2 = d_pos = None
    idx = _cotangent_support(g, n_pts)
    xs, gs = gather(idx)
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
    return d_cov, d_z1, d_z2, d_pos


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
        g = _dev_f64(grad_out, cov.device).reshape(-1)

        def gather(idx):
            if idx is None:
                return x, g
            return (x.index_select(1, idx).contiguous(),
                    g.index_select(0, idx).contiguous())

        grads = _adjoint(ctx, g, cov, z1, z2, x.shape[1], gather,
                         ctx.needs_input_grad[3])
        return (*grads, None)


class SummateGridFunction(torch.autograd.Function):
    """``u = summate`` on the structured grid spanned by ``axes`` ("ij"
    order, flattened), followed by the points ``pos`` when given,
    differentiable in the modes and in ``pos``.

    Mixed precision runs the grid forward through the separable tensor-core
    contraction, FP64 through the FP64 grid kernel; the points run the
    pointwise kernels.  The backward is one adjoint call, as in
    :class:`SummateFunction`, on the grid points and points with a nonzero
    cotangent (grid coordinates gathered from the axes).  The axes get no
    gradient."""

    @staticmethod
    def forward(ctx, cov_samples, z_1, z_2, pos, axes, precision):
        prec = config.check_precision(precision)
        dev = device()
        cov = _dev_f64(cov_samples, dev)
        z1 = _dev_f64(z_1, dev).reshape(-1)
        z2 = _dev_f64(z_2, dev).reshape(-1)
        dim, n_modes = cov.shape
        ax = [_dev_f64(torch.as_tensor(a), dev).reshape(-1) for a in axes]
        if len(ax) != dim:
            raise ValueError("one axis per dimension of cov_samples")
        x = (torch.empty((dim, 0), dtype=torch.float64, device=dev) if pos is None
             else _dev_f64(pos, dev).reshape(dim, -1))
        n_grid = 1
        for a in ax:
            n_grid *= a.numel()
        # the grid's values, then the points', written in place
        out = torch.empty(n_grid + x.shape[1], dtype=torch.float64, device=dev)
        stream = _stream(dev)
        lens = (ctypes.c_int64 * 4)(*([a.numel() for a in ax] + [1] * (4 - dim)))
        flat = torch.cat(ax)
        if prec == "mixed" and dim in (2, 3):
            _native.call("gst_summate_grid_tc", dim, n_modes, lens, _p(flat), _p(cov),
                         _p(z1), _p(z2), _p(out), _native.GST_OUT_F64, 1.0, stream)
        elif prec == "mixed":
            _native.call("gst_summate_grid_mixed", dim, n_modes, lens, _p(flat),
                         _p(cov), _p(z1), _p(z2), _p(out), _native.GST_OUT_F64, 1.0,
                         stream)
        else:
            _native.call("gst_summate_grid_f64", dim, n_modes, lens, _p(flat),
                         _p(cov), _p(z1), _p(z2), _p(out), stream)
        if x.shape[1] > 0:
            name = "gst_summate_f64" if prec == "f64" else "gst_summate_mixed"
            args = [dim, n_modes, x.shape[1], _p(cov), _p(z1), _p(z2), _p(x),
                    _p(out[n_grid:])]
            if prec == "mixed":
                args.append(_native.GST_OUT_F64)
            _native.call(name, *args, stream)
        ctx.save_for_backward(cov, z1, z2, x, *ax)
        ctx.prec = prec
        ctx.in_devices = [t.device for t in (cov_samples, z_1, z_2)] + [
            dev if pos is None else pos.device]
        ctx.shape = tuple(a.numel() for a in ax)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        cov, z1, z2, x, *ax = ctx.saved_tensors
        g = _dev_f64(grad_out, cov.device).reshape(-1)
        shape = ctx.shape
        n_grid = 1
        for n in shape:
            n_grid *= n

        def gather(idx):
            if idx is None:
                mesh = torch.meshgrid(*ax, indexing="ij")
                grid = torch.stack([m.reshape(-1) for m in mesh])
                return torch.cat([grid, x], 1).contiguous(), g
            # one kernel: grid points unravelled from the axes, extra points
            # copied, cotangents picked
            n = idx.numel()
            xs = torch.empty((len(ax), n), dtype=torch.float64, device=g.device)
            gs = torch.empty(n, dtype=torch.float64, device=g.device)
            lens = (ctypes.c_int64 * 3)(*(list(shape) + [1] * (3 - len(shape))))
            flat = torch.cat(ax)
            _native.call("gst_gather_points", len(ax), lens, _p(flat), x.shape[1],
                         _p(x), n, _p(idx), _p(g), _p(xs), _p(gs), _stream(g.device))
            return xs, gs

        need_pos = ctx.needs_input_grad[3] and x.shape[1] > 0
        d_cov, d_z1, d_z2, d_pos = _adjoint(ctx, g, cov, z1, z2, n_grid + x.shape[1],
                                            gather, need_pos)
        if d_pos is not None:
            d_pos = d_pos[:, n_grid:]
        return d_cov, d_z1, d_z2, d_pos, None, None


def summate_torch(cov_samples, z_1, z_2, pos, precision=None):
    """Differentiable ``summate`` on torch tensors (float64 result)."""
    return SummateFunction.apply(cov_samples, z_1, z_2, pos, precision)


def summate_grid_torch(cov_samples, z_1, z_2, axes, precision=None):
    """Differentiable ``summate`` on the structured grid spanned by ``axes``
    (float64, flattened in "ij" order; no gradient w.r.t. the axes)."""
    return SummateGridFunction.apply(cov_samples, z_1, z_2, None, tuple(axes),
                                     precision)


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


def _givens_np(dim, plane, theta):
    """Givens rotation by theta in `plane` and its derivative in theta."""
    import numpy as np

    p, q = plane
    c, s = np.cos(theta), np.sin(theta)
    g = np.eye(dim)
    dg = np.zeros((dim, dim))
    g[p, p] = g[q, q] = c
    g[p, q], g[q, p] = -s, s
    dg[p, p] = dg[q, q] = -s
    dg[p, q], dg[q, p] = -c, c
    return g, dg


class _ModeMap(torch.autograd.Function):
    """``M(angles, anis)^T * (len_scale_ref / len_scale)`` on the host from
    the packed parameters [len_scale, anis..., angles...] (a CPU float64
    tensor), with its analytic derivative: M = diag(1, 1/anis) R_0 R_1 ...,
    R_i the Givens rotation of plane i by (-1)^i (-angles_i) -- the
    construction of :func:`isometrize_matrix` -- in a few numpy operations
    instead of a few dozen autograd nodes."""

    @staticmethod
    def forward(ctx, packed, dim, len_scale_ref):
        import numpy as np

        v = packed.detach().numpy()
        n_anis = dim - 1
        ls, anis, angles = v[0], v[1:1 + n_anis], v[1 + n_anis:]
        planes = [(i, j) for j in range(1, dim) for i in range(j)]
        gs = [_givens_np(dim, pl, (-1) ** i * (-angles[i]))
              for i, pl in enumerate(planes)]
        rot = np.eye(dim)
        for g, _ in gs:
            rot = rot @ g
        stretch = np.diag(np.concatenate([[1.0], 1.0 / anis]))
        m = stretch @ rot
        r = len_scale_ref / ls
        ctx.parts = (dim, ls, anis, r, gs, rot, stretch, m)
        return torch.from_numpy((m.T * r).copy())

    @staticmethod
    def backward(ctx, grad_mt):
        import numpy as np

        dim, ls, anis, r, gs, rot, stretch, m = ctx.parts
        gmt = grad_mt.detach().to("cpu", torch.float64).numpy()
        d_ls = -np.sum(gmt * m.T) * r / ls
        gm = r * gmt.T                      # dL/dM
        gs_ = gm @ rot.T                    # dL/dstretch
        grot = stretch.T @ gm               # dL/drot
        d_anis = np.array([gs_[j + 1, j + 1] * (-1.0 / anis[j] ** 2)
                           for j in range(dim - 1)])
        d_angles = []
        for i in range(len(gs)):
            left = np.eye(dim)
            for g, _ in gs[:i]:
                left = left @ g
            right = np.eye(dim)
            for g, _ in gs[i + 1:]:
                right = right @ g
            dtheta = np.sum((left.T @ grot @ right.T) * gs[i][1])
            d_angles.append(dtheta * -((-1) ** i))
        grad = np.concatenate([[d_ls], d_anis, np.array(d_angles)])
        return torch.from_numpy(grad), None, None


class _ModeMapDevice(torch.autograd.Function):
    """The same map on the device (``gst_mode_map``: one kernel that also
    writes the Jacobian d mt / d params), for parameters that live there:
    no host round trip in the forward or the backward (the backward is
    ``jac^T vec(grad)``)."""

    @staticmethod
    def forward(ctx, packed, dim, len_scale_ref):
        prm = packed.detach().to(torch.float64).contiguous()
        mt = torch.empty((dim, dim), dtype=torch.float64, device=prm.device)
        jac = torch.empty((dim * dim, prm.numel()), dtype=torch.float64,
                          device=prm.device)
        with torch.cuda.device(prm.device):
            _native.call("gst_mode_map", dim, _p(prm), float(len_scale_ref), _p(mt),
                         _p(jac), _stream(prm.device))
        ctx.save_for_backward(jac)
        return mt

    @staticmethod
    def backward(ctx, grad_mt):
        (jac,) = ctx.saved_tensors
        return jac.T @ grad_mt.reshape(-1).to(jac.dtype), None, None


def randmeth_field(cov_ref, len_scale_ref, z_1, z_2, pos=None, *, var, len_scale,
                   anis, angles, precision=None, axes=None):
    """Field at physical positions ``pos`` (dim, n) and/or on the
    structured grid spanned by ``axes`` (flattened, "ij" order; with both,
    the grid's values come first), differentiable in every tensor argument
    (``var``, ``len_scale``, ``anis``, ``angles``, ``z_1``, ``z_2`` and
    ``pos``; not the axes).  ``cov_ref`` are the model's wave vectors drawn
    at ``len_scale_ref``.  A mixed-precision grid runs the tensor-core
    contraction forward."""
    if pos is None and axes is None:
        raise ValueError("give pos, axes or both")
    dim, n_modes = cov_ref.shape
    # The dim x dim map M^T (len_scale_ref / len_scale) and its derivative
    # come from one kernel when the small parameters live on a CUDA device,
    # else from numpy on the host; either way no chain of scalar autograd
    # nodes, and one dim x dim @ dim x N product on the device.
    small = [torch.as_tensor(t, dtype=torch.float64).reshape(-1)
             for t in (len_scale, anis, angles)]
    if small[1].numel() != dim - 1 or small[2].numel() != dim * (dim - 1) // 2:
        raise ValueError("need dim - 1 anisotropy ratios and dim (dim - 1) / 2 angles")
    devs = {t.device for t in small}
    dev0 = next(iter(devs))
    if len(devs) == 1 and dev0.type == "cuda":
        mt = _ModeMapDevice.apply(torch.cat(small), dim, float(len_scale_ref))
    else:
        host = torch.cat([t.to("cpu") for t in small])
        mt = _ModeMap.apply(host, dim, float(len_scale_ref))
    k = mt.to(device=cov_ref.device, dtype=cov_ref.dtype) @ cov_ref
    if axes is not None:
        u = SummateGridFunction.apply(k, z_1, z_2, pos, tuple(axes), precision)
    else:
        u = summate_torch(k, z_1, z_2, pos, precision)
    return torch.sqrt(torch.as_tensor(var, dtype=torch.float64) / n_modes) * u
