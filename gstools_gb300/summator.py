"""Drop-in summators with the reference's call signature.

``summate(cov_samples, z_1, z_2, pos, num_threads=None)`` and
``summate_incompr(...)`` replace ``gstools_cython.field.summate`` /
``summate_incompr`` (imported at src/gstools/field/generator.py:22-24 and
called through ``_summate`` / ``_summate_incompr`` at :42-64, :266-268,
:554-560); ``summate_fourier`` replaces ``gstools_cython.field.summate_fourier``
(:23, :67-75, :682-689).

Arguments may be numpy arrays (host; the result is a new numpy array, as the
reference returns) or torch tensors (any device; the result is a CUDA tensor
and no host copy is made).  Computation always runs on the current CUDA
device through ``libgstools_gb300.so``; without a device these functions
raise.

``summate_grid`` / ``summate_incompr_grid`` evaluate the same sums on a
structured grid given by its axis arrays without materialising the meshgrid:
the caller passes wave vectors already mapped by the transpose of the
isometrize matrix (``<k, M x> = <M^T k, x>``).
"""

import ctypes
import threading

import numpy as np
import torch

from . import _native, config

__all__ = [
    "summate",
    "summate_incompr",
    "summate_fourier",
    "summate_grid",
    "summate_incompr_grid",
    "summate_fourier_grid",
    "summate_structured",
    "structured_supported",
    "device",
]


def device():
    """The CUDA device the summators run on (raises without one)."""
    if not torch.cuda.is_available():
        raise RuntimeError(
            "gstools_gb300 needs a CUDA device; there is no CPU fallback"
        )
    return torch.device("cuda", torch.cuda.current_device())


def _stream(dev):
    return ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _p(t):
    return ctypes.c_void_p(t.data_ptr() if t.numel() else 0)


def _on_device(a, dev):
    if isinstance(a, torch.Tensor):
        return a.to(device=dev, dtype=torch.float64).contiguous()
    arr = np.ascontiguousarray(a, dtype=np.float64)
    return torch.from_numpy(arr).to(dev)


def _is_torch(*arrays):
    return any(isinstance(a, torch.Tensor) for a in arrays)


def _upload_host(arrays, dev):
    """Host arrays as float64 device tensors, each by one copy straight from
    its (pageable) memory: on this platform the copy engine reads pageable
    host memory at ~170 GB/s, so staging through a page-locked block (a
    host memcpy first, ~15 GB/s per core) only adds time (measured: 0.079
    against 0.179 ms for a 100 000-point 2-D call's inputs).  Returns the
    tensors and None (nothing for the caller to keep alive)."""
    flat = [np.ascontiguousarray(a, dtype=np.float64) for a in arrays]
    return [torch.from_numpy(f).to(dev) for f in flat], None


def _prepare(cov_samples, z_1, z_2, pos):
    """Validated float64 device tensors of the inputs, and an object the
    caller keeps referenced until the result is synchronised (the staging
    block of host inputs, or None)."""
    dev = device()
    keep = None
    if _is_torch(cov_samples, z_1, z_2, pos):
        cov, z1, z2, x = (_on_device(a, dev) for a in (cov_samples, z_1, z_2, pos))
    else:
        (cov, z1, z2, x), keep = _upload_host((cov_samples, z_1, z_2, pos), dev)
    if cov.dim() == 1:
        cov = cov.reshape(1, -1)
    if cov.dim() != 2:
        raise ValueError("cov_samples must have shape (dim, N)")
    dim, n_modes = cov.shape
    z1 = z1.reshape(-1)
    z2 = z2.reshape(-1)
    if z1.numel() != n_modes or z2.numel() != n_modes:
        raise ValueError("z_1 and z_2 must have N = cov_samples.shape[1] values")
    if x.numel() % max(dim, 1):
        raise ValueError("pos must have shape (dim, n)")
    x = x.reshape(dim, -1)
    return dev, cov, z1, z2, x, keep


_PINNED_MIN_BYTES = 1 << 20
_PINNED_POOL_BYTES = 2 << 30   # released page-locked blocks kept for reuse


def _output(shape, dtype, dev, as_torch):
    """Device output buffer of a summation (numpy results are copied to the
    host by ``_finish``; measured on GB300, the copy engine moves the field
    faster than the kernels' own stores into pinned host memory)."""
    return torch.empty(shape, dtype=dtype, device=dev)


class _PinnedBlock:
    """Owner of a pooled pinned host buffer exposed to numpy.

    A numpy array built from it keeps it alive; when the array is released
    the buffer goes back to the pool for the next result of that size, so
    large results skip both the pinned allocation (~0.3 ms for 64 MiB) and
    the page faults of fresh pageable memory (~10x slower copies).
    """

    _pool = {}
    _lock = threading.Lock()

    def __init__(self, nbytes):
        with self._lock:
            free = self._pool.get(nbytes)
            tensor = free.pop() if free else None
        if tensor is None:
            tensor = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        self.tensor = tensor
        self.nbytes = nbytes

    def array(self, shape, np_dtype):
        iface = {"shape": tuple(shape), "typestr": np.dtype(np_dtype).str,
                 "data": (self.tensor.data_ptr(), False), "version": 3}
        self.__array_interface__ = iface
        return np.asarray(self)

    def __del__(self):
        with self._lock:
            pooled = sum(n * len(v) for n, v in self._pool.items())
            if pooled + self.nbytes <= _PINNED_POOL_BYTES:
                self._pool.setdefault(self.nbytes, []).append(self.tensor)


_NP_DTYPE = {torch.float64: np.float64, torch.float32: np.float32}


def _finish(out, as_torch):
    """Return the device result, or copy it to a new host array.

    Large results are copied by the copy engine into a pooled pinned buffer
    (192 GB/s measured on GB300 for 64 MiB) that the returned array owns.
    """
    if as_torch:
        return out
    nbytes = out.numel() * out.element_size()
    if nbytes < _PINNED_MIN_BYTES or out.dtype not in _NP_DTYPE:
        return out.cpu().numpy()
    block = _PinnedBlock(nbytes)
    host = block.tensor.view(out.dtype).view(out.shape)
    host.copy_(out, non_blocking=True)
    torch.cuda.current_stream(out.device).synchronize()
    return block.array(out.shape, _NP_DTYPE[out.dtype])


def _out_type(dtype):
    if dtype in (None, np.float64, torch.float64, "float64", "f64"):
        return _native.GST_OUT_F64, torch.float64
    if dtype in (np.float32, torch.float32, "float32", "f32"):
        return _native.GST_OUT_F32, torch.float32
    raise ValueError(f"unsupported output dtype {dtype!r}")


def summate(cov_samples, z_1, z_2, pos, num_threads=None, *, precision=None,
            out_dtype=None):
    """Randomization-method sum (generator.py:193-199).

    ``out[i] = sum_j z_1[j] cos(<k_j, x_i>) + z_2[j] sin(<k_j, x_i>)`` with
    ``k_j = cov_samples[:, j]`` and ``x_i = pos[:, i]``.
    """
    prec = config.check_precision(precision)
    as_torch = _is_torch(cov_samples, z_1, z_2, pos)
    dev, cov, z1, z2, x, keep = _prepare(cov_samples, z_1, z_2, pos)
    dim, n_modes = cov.shape
    n_pts = x.shape[1]
    stream = _stream(dev)
    if prec == "f64":
        if out_dtype not in (None, np.float64, torch.float64, "float64", "f64"):
            raise ValueError("precision 'f64' produces float64 output")
        out = _output((n_pts,), torch.float64, dev, as_torch)
        _native.call("gst_summate_f64", dim, n_modes, n_pts, _p(cov), _p(z1),
                     _p(z2), _p(x), _p(out), stream)
    else:
        code, tdtype = _out_type(out_dtype)
        out = _output((n_pts,), tdtype, dev, as_torch)
        _native.call("gst_summate_mixed", dim, n_modes, n_pts, _p(cov),
                     _p(z1), _p(z2), _p(x), _p(out), code, stream)
    result = _finish(out, as_torch)
    del keep   # the staged inputs are no longer read
    return result


def summate_incompr(cov_samples, z_1, z_2, pos, num_threads=None, *,
                    precision=None, out_dtype=None):
    """Incompressible randomization-method sum (generator.py:479-495).

    ``out[c, i] = sum_j (delta_c0 - k_cj k_0j / |k_j|^2)
    (z_1[j] cos(<k_j, x_i>) + z_2[j] sin(<k_j, x_i>))``; dim 2 or 3.
    """
    prec = config.check_precision(precision)
    as_torch = _is_torch(cov_samples, z_1, z_2, pos)
    dev, cov, z1, z2, x, keep = _prepare(cov_samples, z_1, z_2, pos)
    dim, n_modes = cov.shape
    n_pts = x.shape[1]
    stream = _stream(dev)
    if prec == "f64":
        out = torch.empty((dim, n_pts), dtype=torch.float64, device=dev)
        _native.call("gst_summate_incompr_f64", dim, n_modes, n_pts, _p(cov),
                     _p(z1), _p(z2), _p(x), _p(out), stream)
    else:
        code, tdtype = _out_type(out_dtype)
        out = torch.empty((dim, n_pts), dtype=tdtype, device=dev)
        _native.call("gst_summate_incompr_mixed", dim, n_modes, n_pts,
                     _p(cov), _p(z1), _p(z2), _p(x), _p(out), code, stream)
    result = _finish(out, as_torch)
    del keep   # the staged inputs are no longer read
    return result


def summate_fourier(spectrum_factor, modes, z_1, z_2, pos, num_threads=None):
    """Fourier-method sum (generator.py:682-689), FP64.

    ``out[i] = sum_j f[j] (z_1[j] cos(<k_j, x_i>) + z_2[j] sin(<k_j, x_i>))``.
    """
    as_torch = _is_torch(spectrum_factor, modes, z_1, z_2, pos)
    dev, kk, z1, z2, x, keep = _prepare(modes, z_1, z_2, pos)
    fac = _on_device(spectrum_factor, dev).reshape(-1)
    dim, n_modes = kk.shape
    if fac.numel() != n_modes:
        raise ValueError("spectrum_factor must have one value per mode")
    n_pts = x.shape[1]
    out = torch.empty(n_pts, dtype=torch.float64, device=dev)
    _native.call("gst_summate_fourier_f64", dim, n_modes, n_pts, _p(fac),
                 _p(kk), _p(z1), _p(z2), _p(x), _p(out), _stream(dev))
    result = _finish(out, as_torch)
    del keep   # the staged inputs are no longer read
    return result


def _prepare_grid(cov_samples, z_1, z_2, axes):
    dev = device()
    cov = _on_device(cov_samples, dev)
    if cov.dim() == 1:
        cov = cov.reshape(1, -1)
    dim, n_modes = cov.shape
    if len(axes) != dim:
        raise ValueError("need one axis array per dimension")
    z1 = _on_device(z_1, dev).reshape(-1)
    z2 = _on_device(z_2, dev).reshape(-1)
    if z1.numel() != n_modes or z2.numel() != n_modes:
        raise ValueError("z_1 and z_2 must have N = cov_samples.shape[1] values")
    ax = [_on_device(a, dev).reshape(-1) for a in axes]
    lens = (ctypes.c_int64 * 4)(*([a.numel() for a in ax] + [1] * (4 - dim)))
    flat = torch.cat(ax) if ax else torch.empty(0, dtype=torch.float64,
                                                device=dev)
    shape = tuple(a.numel() for a in ax)
    return dev, cov, z1, z2, flat, lens, shape


def _prepare_grid_host(cov_samples, z_1, z_2, axes):
    """Validated contiguous float64 host copies of the grid inputs."""
    cov = np.ascontiguousarray(cov_samples, dtype=np.float64)
    if cov.ndim == 1:
        cov = cov.reshape(1, -1)
    if cov.ndim != 2:
        raise ValueError("cov_samples must have shape (dim, N)")
    dim, n_modes = cov.shape
    if len(axes) != dim:
        raise ValueError("need one axis array per dimension")
    z1 = np.ascontiguousarray(z_1, dtype=np.float64).reshape(-1)
    z2 = np.ascontiguousarray(z_2, dtype=np.float64).reshape(-1)
    if z1.size != n_modes or z2.size != n_modes:
        raise ValueError("z_1 and z_2 must have N = cov_samples.shape[1] values")
    ax = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in axes]
    lens = (ctypes.c_int64 * 4)(*([a.size for a in ax] + [1] * (4 - dim)))
    flat = np.concatenate(ax) if ax else np.empty(0)
    return cov, z1, z2, flat, lens, tuple(a.size for a in ax)


def _np_p(a):
    return ctypes.c_void_p(a.ctypes.data if a.size else 0)


def _grid_host_call(entry, dim, n_modes, lens, arrays, shape, out_dtype,
                    scale):
    """Run a ``*_grid_tc_host`` entry point: host inputs, host result.

    The library pipelines the device work with the copies (each finished
    slab of the field moves to the host while the next one computes); the
    result lands in a pooled page-locked buffer owned by the returned array.
    """
    dev = device()
    code, tdtype = _out_type(out_dtype)
    np_dtype = _NP_DTYPE[tdtype]
    nbytes = int(np.prod(shape)) * np.dtype(np_dtype).itemsize
    if nbytes >= _PINNED_MIN_BYTES:
        block = _PinnedBlock(nbytes)
        out = block.array(shape, np_dtype)
    else:
        block, out = None, np.empty(shape, dtype=np_dtype)
    with torch.cuda.device(dev):
        _native.call(entry, dim, n_modes, lens, *[_np_p(a) for a in arrays],
                     _np_p(out), code, float(scale), _stream(dev))
        torch.cuda.current_stream(dev).synchronize()
    return out


def _grid_dim(cov_samples):
    shape = np.shape(cov_samples)
    return 1 if len(shape) == 1 else shape[0]


def summate_grid(cov_samples, z_1, z_2, axes, *, precision=None,
                 out_dtype=None, scale=1.0, method="auto"):
    """``summate`` on the structured grid spanned by ``axes`` ("ij" order).

    ``cov_samples`` must already be multiplied by ``M^T`` when the reference
    would isometrize the grid with ``M``.  Returns an array of shape
    ``tuple(len(a) for a in axes)``; ``scale`` multiplies the result.

    ``method`` picks the kernel:

    * ``"pointwise"`` -- per-point phases (FP64 or mixed, per ``precision``);
    * ``"tensor"``    -- the separable tensor-core contraction (three-product
      FP16 split by default, 3xTF32 selectable; 2-D and 3-D grids, requires
      ``precision="mixed"``);
    * ``"auto"``      -- ``"tensor"`` for mixed precision on 2-D / 3-D grids,
      ``"pointwise"`` otherwise.
    """
    prec = config.check_precision(precision)
    if method not in ("auto", "pointwise", "tensor"):
        raise ValueError(f"unknown method {method!r}")
    as_torch = _is_torch(cov_samples, z_1, z_2, *axes)
    if method == "auto":
        method = ("tensor" if (prec == "mixed" and _grid_dim(cov_samples) in (2, 3))
                  else "pointwise")
    if method == "tensor" and not as_torch:
        cov, z1, z2, flat, lens, shape = _prepare_grid_host(cov_samples, z_1,
                                                            z_2, axes)
        dim, n_modes = cov.shape
        if prec != "mixed":
            raise ValueError("the tensor-core grid path is mixed precision")
        if dim not in (2, 3):
            raise ValueError("the tensor-core grid path needs a 2-D or 3-D grid")
        return _grid_host_call("gst_summate_grid_tc_host", dim, n_modes, lens,
                               [flat, cov, z1, z2], shape, out_dtype, scale)
    dev, cov, z1, z2, flat, lens, shape = _prepare_grid(cov_samples, z_1,
                                                        z_2, axes)
    dim, n_modes = cov.shape
    stream = _stream(dev)
    if method == "tensor":
        if prec != "mixed":
            raise ValueError("the tensor-core grid path is mixed precision")
        if dim not in (2, 3):
            raise ValueError("the tensor-core grid path needs a 2-D or 3-D grid")
        code, tdtype = _out_type(out_dtype)
        out = _output(shape, tdtype, dev, as_torch)
        _native.call("gst_summate_grid_tc", dim, n_modes, lens, _p(flat),
                     _p(cov), _p(z1), _p(z2), _p(out), code, float(scale),
                     stream)
    elif prec == "f64":
        out = torch.empty(shape, dtype=torch.float64, device=dev)
        _native.call("gst_summate_grid_f64", dim, n_modes, lens, _p(flat),
                     _p(cov), _p(z1), _p(z2), _p(out), stream)
        if scale != 1.0:
            out.mul_(scale)
    else:
        code, tdtype = _out_type(out_dtype)
        out = torch.empty(shape, dtype=tdtype, device=dev)
        _native.call("gst_summate_grid_mixed", dim, n_modes, lens, _p(flat),
                     _p(cov), _p(z1), _p(z2), _p(out), code, float(scale),
                     stream)
    return _finish(out, as_torch)


def summate_incompr_grid(cov_samples, z_1, z_2, axes, *, precision=None,
                         out_dtype=None, scale=1.0, method="auto",
                         proj_cov=None):
    """``summate_incompr`` on a structured grid; output (dim, *shape).

    ``cov_samples`` drive the phases (multiply by ``M^T`` when the reference
    would isometrize the grid with ``M``); the projector
    ``p(k) = e_1 - k k_1 / |k|^2`` uses ``proj_cov`` (the unmapped wave
    vectors; default ``cov_samples``).  ``method``: "pointwise", "tensor"
    (mixed precision, 2-D / 3-D) or "auto" (tensor for mixed precision).
    The pointwise kernels take the projector from ``cov_samples``, so they
    need ``proj_cov`` to be absent or equal.
    """
    prec = config.check_precision(precision)
    if method not in ("auto", "pointwise", "tensor"):
        raise ValueError(f"unknown method {method!r}")
    as_torch = _is_torch(cov_samples, z_1, z_2, proj_cov, *axes)
    if method == "auto":
        method = ("tensor" if (prec == "mixed" and _grid_dim(cov_samples) in (2, 3))
                  else "pointwise")
    if method == "tensor" and not as_torch:
        cov, z1, z2, flat, lens, shape = _prepare_grid_host(cov_samples, z_1,
                                                            z_2, axes)
        dim, n_modes = cov.shape
        if prec != "mixed":
            raise ValueError("the tensor-core grid path is mixed precision")
        if dim not in (2, 3):
            raise ValueError("the tensor-core grid path needs a 2-D or 3-D grid")
        pc = cov if proj_cov is None else np.ascontiguousarray(
            proj_cov, dtype=np.float64).reshape(dim, n_modes)
        return _grid_host_call("gst_summate_incompr_grid_tc_host", dim,
                               n_modes, lens, [flat, cov, pc, z1, z2],
                               (dim,) + shape, out_dtype, scale)
    dev, cov, z1, z2, flat, lens, shape = _prepare_grid(cov_samples, z_1,
                                                        z_2, axes)
    dim, n_modes = cov.shape
    stream = _stream(dev)
    if method == "tensor":
        if prec != "mixed":
            raise ValueError("the tensor-core grid path is mixed precision")
        pc = cov if proj_cov is None else _on_device(proj_cov, dev).reshape(
            dim, n_modes)
        code, tdtype = _out_type(out_dtype)
        out = _output((dim,) + shape, tdtype, dev, as_torch)
        _native.call("gst_summate_incompr_grid_tc", dim, n_modes, lens,
                     _p(flat), _p(cov), _p(pc), _p(z1), _p(z2), _p(out), code,
                     float(scale), stream)
        return _finish(out, as_torch)
    if proj_cov is not None:
        raise ValueError("the pointwise grid kernels take the projector from "
                         "cov_samples; use method='tensor' for proj_cov")
    if prec == "f64":
        out = torch.empty((dim,) + shape, dtype=torch.float64, device=dev)
        _native.call("gst_summate_incompr_grid_f64", dim, n_modes, lens,
                     _p(flat), _p(cov), _p(z1), _p(z2), _p(out), stream)
        if scale != 1.0:
            out.mul_(scale)
    else:
        code, tdtype = _out_type(out_dtype)
        out = torch.empty((dim,) + shape, dtype=tdtype, device=dev)
        _native.call("gst_summate_incompr_grid_mixed", dim, n_modes, lens,
                     _p(flat), _p(cov), _p(z1), _p(z2), _p(out), code,
                     float(scale), stream)
    return _finish(out, as_torch)


def summate_fourier_grid(spectrum_factor, modes, z_1, z_2, axes, *,
                         out_dtype=None, scale=1.0):
    """``summate_fourier`` on a structured grid (tensor-core path, mixed
    precision, 2-D / 3-D); output of shape ``tuple(len(a) for a in axes)``."""
    as_torch = _is_torch(spectrum_factor, modes, z_1, z_2, *axes)
    if not as_torch:
        kk, z1, z2, flat, lens, shape = _prepare_grid_host(modes, z_1, z_2,
                                                           axes)
        dim, n_modes = kk.shape
        if dim not in (2, 3):
            raise ValueError("the tensor-core grid path needs a 2-D or 3-D grid")
        fac = np.ascontiguousarray(spectrum_factor, dtype=np.float64).reshape(-1)
        if fac.size != n_modes:
            raise ValueError("spectrum_factor must have one value per mode")
        return _grid_host_call("gst_summate_fourier_grid_tc_host", dim, n_modes,
                               lens, [flat, fac, kk, z1, z2], shape, out_dtype,
                               scale)
    dev, kk, z1, z2, flat, lens, shape = _prepare_grid(modes, z_1, z_2, axes)
    dim, n_modes = kk.shape
    if dim not in (2, 3):
        raise ValueError("the tensor-core grid path needs a 2-D or 3-D grid")
    fac = _on_device(spectrum_factor, dev).reshape(-1)
    if fac.numel() != n_modes:
        raise ValueError("spectrum_factor must have one value per mode")
    code, tdtype = _out_type(out_dtype)
    out = torch.empty(shape, dtype=tdtype, device=dev)
    _native.call("gst_summate_fourier_grid_tc", dim, n_modes, lens, _p(flat),
                 _p(fac), _p(kk), _p(z1), _p(z2), _p(out), code, float(scale),
                 _stream(dev))
    return _finish(out, as_torch)


_KINDS = ("scalar", "incompr", "fourier")


def _iso_matrix(iso, dim):
    if iso is None:
        return np.eye(dim)
    m = np.asarray(iso, dtype=np.float64)
    if m.shape != (dim, dim):
        raise ValueError(f"iso must be a ({dim}, {dim}) matrix")
    return m


def structured_supported(kind, dim, precision=None, iso=None):
    """Whether :func:`summate_structured` evaluates this case on the grid
    kernels: scalar sums in any precision (dim 1-3); incompressible sums in
    mixed precision (dim 2-3, tensor cores) or in FP64 when the isometrize
    map is the identity (the FP64 grid kernel takes the projector from the
    phase wave vectors); Fourier sums in mixed precision (dim 2-3)."""
    prec = config.check_precision(precision)
    if kind not in _KINDS:
        raise ValueError(f"kind must be one of {_KINDS}")
    if not 1 <= dim <= 3:
        return False
    if kind == "scalar":
        return True
    if dim not in (2, 3):
        return False
    if kind == "incompr":
        return prec == "mixed" or iso is None or np.array_equal(
            np.asarray(iso, dtype=np.float64), np.eye(dim))
    return prec == "mixed"


def summate_structured(cov_samples, z_1, z_2, axes, iso=None, *,
                       kind="scalar", spectrum_factor=None, precision=None):
    """The reference summators on a structured grid, with their flat result.

    Returns what ``summate`` / ``summate_incompr`` / ``summate_fourier``
    return for ``pos = iso @ generate_grid(axes)`` -- the grid the
    reference's ``Field.pre_pos`` builds for a structured mesh and
    isometrizes (src/gstools/field/base.py:289-297,
    src/gstools/tools/geometric.py:340-356, src/gstools/covmodel/base.py:
    572-582) -- a float64 array of shape (n,) (scalar, Fourier) or (d, n)
    (incompressible) in meshgrid "ij" order, without building that grid:
    the wave vectors are mapped instead (``<k, M x> = <M^T k, x>``) and the
    separable grid kernels run on the axis arrays.

    * ``precision="f64"``: the FP64 grid kernel (reference operation order
      per point, with the mapped wave vectors);
    * ``precision="mixed"``: the tensor-core contraction on 2-D / 3-D grids
      (the mixed pointwise grid kernel in 1-D).

    ``cov_samples`` holds the wave vectors (the Fourier generator's
    ``modes`` for ``kind="fourier"``, with ``spectrum_factor``).  Cases
    :func:`structured_supported` rejects raise ``ValueError``.
    """
    prec = config.check_precision(precision)
    cov = np.ascontiguousarray(cov_samples, dtype=np.float64)
    if cov.ndim == 1:
        cov = cov.reshape(1, -1)
    dim = cov.shape[0]
    if not structured_supported(kind, dim, prec, iso):
        raise ValueError(f"no grid kernel for a {dim}-D {kind} sum in "
                         f"{prec} with this isometrize map")
    m = _iso_matrix(iso, dim)
    kmap = np.ascontiguousarray(m.T @ cov)
    axes = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in axes]
    n = int(np.prod([a.size for a in axes]))
    if kind == "scalar":
        if prec == "f64":
            out = summate_grid(kmap, z_1, z_2, axes, precision="f64",
                               method="pointwise")
        else:
            out = summate_grid(kmap, z_1, z_2, axes, precision="mixed",
                               method="auto", out_dtype=np.float64)
        return out.reshape(n)
    if kind == "incompr":
        if prec == "f64":
            out = summate_incompr_grid(cov, z_1, z_2, axes, precision="f64",
                                       method="pointwise")
        else:
            out = summate_incompr_grid(kmap, z_1, z_2, axes, precision="mixed",
                                       method="tensor", out_dtype=np.float64,
                                       proj_cov=cov)
        return out.reshape(dim, n)
    if spectrum_factor is None:
        raise ValueError("kind='fourier' needs spectrum_factor")
    out = summate_fourier_grid(spectrum_factor, kmap, z_1, z_2, axes,
                               out_dtype=np.float64)
    return out.reshape(n)
