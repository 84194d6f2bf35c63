"""Drop-in kriging kernels with gstools-cython's call signatures.

``calc_field_krige(krig_mat, krig_vecs, cond, num_threads=None)`` and
``calc_field_krige_and_variance(...)`` replace
``gstools_cython.krige.calc_field_krige(_and_variance)`` (imported at
src/gstools/krige/base.py:16-19 and called through the module globals
``_calc_field_krige`` / ``_calc_field_krige_and_variance`` at :42-60 from
``Krige._summate``, :307-320).  For the inverted kriging matrix M (K, K),
the right-hand sides V (K, n) and the condition values c (K,):

    field[k] = sum_i c_i (M v_k)_i,   error[k] = sum_i v_ik (M v_k)_i

computed in FP64 on the current CUDA device by ``gst_calc_field_krige``.
numpy arguments give numpy results; torch tensors give CUDA tensors.
"""

import ctypes

import numpy as np
import torch

from . import _native
from .summator import _is_torch, _on_device, _p, _stream, device

__all__ = ["calc_field_krige", "calc_field_krige_and_variance"]


def _krige(krig_mat, krig_vecs, cond, with_error):
    as_torch = _is_torch(krig_mat, krig_vecs, cond)
    dev = device()
    vecs = _on_device(krig_vecs, dev)
    if vecs.dim() == 1:
        vecs = vecs.reshape(-1, 1)
    n_cond, n_pts = vecs.shape
    mat = _on_device(krig_mat, dev).reshape(-1)
    cnd = _on_device(cond, dev).reshape(-1)
    if mat.numel() != n_cond * n_cond or cnd.numel() != n_cond:
        raise ValueError("krig_mat must be (K, K), krig_vecs (K, n), cond (K,)")
    field = torch.empty(n_pts, dtype=torch.float64, device=dev)
    error = torch.empty(n_pts, dtype=torch.float64, device=dev) if with_error else None
    _native.call("gst_calc_field_krige", n_cond, n_pts, _p(mat), _p(vecs),
                 _p(cnd), _p(field),
                 _p(error) if with_error else ctypes.c_void_p(0), _stream(dev))
    if not as_torch:
        field = field.cpu().numpy()
        error = error.cpu().numpy() if with_error else None
    return (field, error) if with_error else field


def calc_field_krige(krig_mat, krig_vecs, cond, num_threads=None):
    """Kriging field ``cond^T M V`` (num_threads is accepted and ignored)."""
    return _krige(krig_mat, krig_vecs, cond, False)


def calc_field_krige_and_variance(krig_mat, krig_vecs, cond, num_threads=None):
    """Kriging field and the quadratic form ``v_k^T M v_k`` per target point
    (the reference subtracts it from the sill)."""
    return _krige(krig_mat, krig_vecs, cond, True)
