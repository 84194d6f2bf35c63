"""Drop-in variogram estimators with gstools-cython's call signatures.

``unstructured``, ``directional``, ``structured`` and ``ma_structured``
replace ``gstools_cython.variogram``'s kernels of the same names (imported at
src/gstools/variogram/variogram.py:14-17, called through the wrappers at
:48-124 by ``vario_estimate`` and ``vario_estimate_axis``): same arguments,
same (variogram, counts) results, computed on the current CUDA device.
numpy arguments give numpy results.  Bin edges must be non-decreasing (the
reference's standard bins always are).
"""

import ctypes

import numpy as np
import torch

from . import _native
from .summator import _p, _stream, device

__all__ = ["unstructured", "directional", "structured", "ma_structured"]


def _est(estimator_type):
    e = str(estimator_type)
    if e not in ("m", "c"):
        raise ValueError(f"unknown estimator type {estimator_type!r}")
    return ord(e)


def _dev(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).to(dev)


def _pairs_inputs(f, bin_edges, pos):
    pos = np.atleast_2d(np.asarray(pos, dtype=np.float64))
    dim, n = pos.shape
    f = np.asarray(f, dtype=np.float64).reshape(-1, n) if n else \
        np.zeros((np.atleast_2d(f).shape[0], 0))
    edges = np.asarray(bin_edges, dtype=np.float64).reshape(-1)
    if edges.size > 1 and np.any(np.diff(edges) < 0):
        raise ValueError("variogram bin edges must be non-decreasing")
    return dim, n, f, edges, pos


def unstructured(f, bin_edges, pos, estimator_type="m", distance_type="e",
                 num_threads=None):
    """Omnidirectional variogram of unstructured points: (variogram, counts)."""
    dim, n, f, edges, pos = _pairs_inputs(f, bin_edges, pos)
    nb = max(edges.size - 1, 0)
    dev = device()
    vario = torch.zeros(nb, dtype=torch.float64, device=dev)
    counts = torch.zeros(nb, dtype=torch.int64, device=dev)
    df, de, dp = _dev(f, dev), _dev(edges, dev), _dev(pos, dev)
    dt = str(distance_type)
    if dt not in ("e", "h"):
        raise ValueError(f"unknown distance type {distance_type!r}")
    _native.call("gst_vario_unstructured", dim, n, f.shape[0], _p(df), nb, _p(de),
                 _p(dp), _est(estimator_type), ord(dt), _p(vario), _p(counts),
                 _stream(dev))
    return vario.cpu().numpy(), counts.cpu().numpy()


def directional(f, bin_edges, pos, direction, angles_tol=np.pi / 8.0,
                bandwidth=-1.0, separate_dirs=False, estimator_type="m",
                num_threads=None):
    """Directional variograms: (variogram, counts), each (directions, bins)."""
    dim, n, f, edges, pos = _pairs_inputs(f, bin_edges, pos)
    dirs = np.atleast_2d(np.asarray(direction, dtype=np.float64)).reshape(-1, dim)
    nb = max(edges.size - 1, 0)
    dev = device()
    vario = torch.zeros((dirs.shape[0], nb), dtype=torch.float64, device=dev)
    counts = torch.zeros((dirs.shape[0], nb), dtype=torch.int64, device=dev)
    df, de, dp, dd = _dev(f, dev), _dev(edges, dev), _dev(pos, dev), _dev(dirs, dev)
    _native.call("gst_vario_directional", dim, n, f.shape[0], _p(df), nb, _p(de),
                 _p(dp), dirs.shape[0], _p(dd), float(angles_tol),
                 float(bandwidth), int(bool(separate_dirs)), _est(estimator_type),
                 _p(vario), _p(counts), _stream(dev))
    return vario.cpu().numpy(), counts.cpu().numpy()


def _structured(f, mask, estimator_type):
    f = np.asarray(f, dtype=np.float64)
    n0 = f.shape[0] if f.ndim else 1
    f = f.reshape(n0, -1)
    dev = device()
    vario = torch.zeros(n0, dtype=torch.float64, device=dev)
    df = _dev(f, dev)
    dm = None
    if mask is not None:
        m = np.ascontiguousarray(np.asarray(mask, dtype=bool).reshape(n0, -1),
                                 dtype=np.uint8)
        dm = torch.from_numpy(m).to(dev)
    _native.call("gst_vario_structured", n0, f.shape[1], _p(df),
                 _p(dm) if dm is not None else ctypes.c_void_p(0),
                 _est(estimator_type), _p(vario), _stream(dev))
    return vario.cpu().numpy()


def structured(f, estimator_type="m", num_threads=None):
    """Variogram along axis 0 of ``f`` (lags 0 .. len - 1)."""
    return _structured(f, None, estimator_type)


def ma_structured(f, mask, estimator_type="m", num_threads=None):
    """Masked variogram along axis 0 of ``f`` (``mask`` True = missing)."""
    return _structured(f, mask, estimator_type)
