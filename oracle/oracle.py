"""Loader for the C oracle and the numpy witness (test infrastructure only).

Every function here restates the reference's formulas:

* summate          -- src/gstools/field/generator.py:193-199
* summate_incompr  -- src/gstools/field/generator.py:479-495
* summate_fourier  -- src/gstools/field/generator.py:682-689
* krige            -- calc_field_krige(_and_variance) of gstools-cython, called
                      by src/gstools/krige/base.py:42-60, 307-320
* vario_*          -- the variogram estimators of gstools-cython (unstructured,
                      directional, structured, ma_structured), called by
                      src/gstools/variogram/variogram.py:48-124
* sample_modes     -- the device spectral sampler of
                      gstools_gb300/csrc/gst_sampling.cu (Philox4x64-10
                      stream, sphere formulas of src/gstools/random/rng.py:
                      142-193, the models' analytic radial laws)

Inputs follow the reference's array layouts: ``cov_samples`` (dim, N),
``z_1``/``z_2`` (N,), ``pos`` (dim, n), all float64.
"""

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_NAME = "liboracle_summate.so"
_lib = None
_lock = threading.Lock()


def library_path():
    """Path of the compiled C oracle."""
    return os.path.join(_HERE, _LIB_NAME)


def build(force=False):
    """Compile the C oracle with its Makefile (gcc, OpenMP)."""
    srcs = [os.path.join(_HERE, f)
            for f in ("summate_oracle.c", "sample_oracle.c", "krige_oracle.c",
                      "vario_oracle.c")]
    out = library_path()
    if (
        not force
        and os.path.exists(out)
        and os.path.getmtime(out) >= max(os.path.getmtime(f) for f in srcs)
    ):
        return out
    subprocess.run(["make", "-s", "-C", _HERE, "-B"], check=True)
    return out


def _load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = ctypes.CDLL(library_path())
            dp = ctypes.POINTER(ctypes.c_double)
            i64 = ctypes.c_int64
            for name in ("oracle_summate", "oracle_summate_incompr"):
                fn = getattr(lib, name)
                fn.restype = ctypes.c_int
                fn.argtypes = [ctypes.c_int, i64, i64, dp, dp, dp, dp, dp,
                               ctypes.c_int]
            fn = lib.oracle_summate_fourier
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.c_int, i64, i64, dp, dp, dp, dp, dp, dp,
                           ctypes.c_int]
            lib.oracle_num_threads.restype = ctypes.c_int
            lib.oracle_num_threads.argtypes = []
            u64 = ctypes.c_uint64
            lib.oracle_philox4x64.restype = None
            lib.oracle_philox4x64.argtypes = [u64] * 6 + [ctypes.POINTER(u64)]
            ip = ctypes.POINTER(i64)
            ch = ctypes.c_char
            lib.oracle_vario_unstructured.restype = ctypes.c_int
            lib.oracle_vario_unstructured.argtypes = [
                ctypes.c_int, i64, i64, dp, i64, dp, dp, ch, ch, dp, ip]
            lib.oracle_vario_directional.restype = ctypes.c_int
            lib.oracle_vario_directional.argtypes = [
                ctypes.c_int, i64, i64, dp, i64, dp, dp, i64, dp, ctypes.c_double,
                ctypes.c_double, ctypes.c_int, ch, dp, ip]
            lib.oracle_vario_structured.restype = ctypes.c_int
            lib.oracle_vario_structured.argtypes = [
                i64, i64, dp, ctypes.POINTER(ctypes.c_ubyte), ch, dp]
            lib.oracle_krige.restype = ctypes.c_int
            lib.oracle_krige.argtypes = [i64, i64, dp, dp, dp, dp, dp]
            lib.oracle_sample_modes.restype = ctypes.c_int
            lib.oracle_sample_modes.argtypes = [
                ctypes.c_int, i64, i64, ctypes.POINTER(i64), ctypes.c_int,
                ctypes.c_double, ctypes.POINTER(u64), dp, dp, dp, dp]
            _lib = lib
    return _lib


def num_threads():
    """OpenMP threads the C oracle uses by default."""
    return _load().oracle_num_threads()


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check(cov, z_1, z_2, pos):
    cov, z_1, z_2, pos = _f64(cov), _f64(z_1), _f64(z_2), _f64(pos)
    cov = np.atleast_2d(cov)
    pos = pos.reshape(cov.shape[0], -1)
    if z_1.shape != (cov.shape[1],) or z_2.shape != (cov.shape[1],):
        raise ValueError("oracle: z_1/z_2 must have shape (N,)")
    return cov, z_1, z_2, pos


def c_summate(cov_samples, z_1, z_2, pos, num_threads=0):
    """C oracle of ``summate`` (generator.py:193-199)."""
    cov, z_1, z_2, pos = _check(cov_samples, z_1, z_2, pos)
    dim, n_modes = cov.shape
    n_pts = pos.shape[1]
    out = np.empty(n_pts, dtype=np.float64)
    rc = _load().oracle_summate(dim, n_modes, n_pts, _ptr(cov), _ptr(z_1),
                                _ptr(z_2), _ptr(pos), _ptr(out),
                                int(num_threads or 0))
    if rc:
        raise ValueError(f"oracle_summate failed with code {rc}")
    return out


def c_summate_incompr(cov_samples, z_1, z_2, pos, num_threads=0):
    """C oracle of ``summate_incompr`` (generator.py:479-495)."""
    cov, z_1, z_2, pos = _check(cov_samples, z_1, z_2, pos)
    dim, n_modes = cov.shape
    n_pts = pos.shape[1]
    out = np.empty((dim, n_pts), dtype=np.float64)
    rc = _load().oracle_summate_incompr(dim, n_modes, n_pts, _ptr(cov),
                                        _ptr(z_1), _ptr(z_2), _ptr(pos),
                                        _ptr(out), int(num_threads or 0))
    if rc:
        raise ValueError(f"oracle_summate_incompr failed with code {rc}")
    return out


def c_summate_fourier(spectrum_factor, modes, z_1, z_2, pos, num_threads=0):
    """C oracle of ``summate_fourier`` (generator.py:682-689)."""
    modes, z_1, z_2, pos = _check(modes, z_1, z_2, pos)
    fac = _f64(spectrum_factor)
    dim, n_modes = modes.shape
    n_pts = pos.shape[1]
    out = np.empty(n_pts, dtype=np.float64)
    rc = _load().oracle_summate_fourier(dim, n_modes, n_pts, _ptr(fac),
                                        _ptr(modes), _ptr(z_1), _ptr(z_2),
                                        _ptr(pos), _ptr(out),
                                        int(num_threads or 0))
    if rc:
        raise ValueError(f"oracle_summate_fourier failed with code {rc}")
    return out


def _phase_chunks(cov, pos, chunk):
    for start in range(0, pos.shape[1], chunk):
        stop = min(start + chunk, pos.shape[1])
        # phase[j, i] = sum_d k[d, j] x[d, i], accumulated over d in order
        phase = np.zeros((cov.shape[1], stop - start))
        for d in range(cov.shape[0]):
            phase += np.outer(cov[d], pos[d, start:stop])
        yield start, stop, phase


def np_summate(cov_samples, z_1, z_2, pos, chunk=4096):
    """numpy witness of ``summate`` (generator.py:193-199)."""
    cov, z_1, z_2, pos = _check(cov_samples, z_1, z_2, pos)
    out = np.empty(pos.shape[1])
    for start, stop, phase in _phase_chunks(cov, pos, chunk):
        out[start:stop] = z_1 @ np.cos(phase) + z_2 @ np.sin(phase)
    return out


def np_summate_incompr(cov_samples, z_1, z_2, pos, chunk=4096):
    """numpy witness of ``summate_incompr`` (generator.py:479-495)."""
    cov, z_1, z_2, pos = _check(cov_samples, z_1, z_2, pos)
    dim = cov.shape[0]
    k2 = np.sum(cov**2, axis=0)
    e1 = np.zeros(dim)
    e1[0] = 1.0
    proj = e1[:, None] - cov * cov[0] / k2  # (dim, N)
    out = np.empty((dim, pos.shape[1]))
    for start, stop, phase in _phase_chunks(cov, pos, chunk):
        amp = z_1[:, None] * np.cos(phase) + z_2[:, None] * np.sin(phase)
        out[:, start:stop] = proj @ amp
    return out


def np_summate_fourier(spectrum_factor, modes, z_1, z_2, pos, chunk=4096):
    """numpy witness of ``summate_fourier`` (generator.py:682-689)."""
    modes, z_1, z_2, pos = _check(modes, z_1, z_2, pos)
    fac = _f64(spectrum_factor)
    out = np.empty(pos.shape[1])
    for start, stop, phase in _phase_chunks(modes, pos, chunk):
        out[start:stop] = (fac * z_1) @ np.cos(phase) + (fac * z_2) @ np.sin(
            phase
        )
    return out


MODEL_KINDS = {"Gaussian": 0, "Exponential": 1, "Matern": 2}


def c_philox4x64(counter, key):
    """Philox4x64-10 of one 256-bit counter under a 128-bit key."""
    out = (ctypes.c_uint64 * 4)()
    _load().oracle_philox4x64(*[int(c) for c in counter], *[int(k) for k in key],
                              out)
    return np.array(list(out), dtype=np.uint64)


def c_sample_modes(dim, mode_counts, model, nu, seeds, len_rescaled):
    """CPU restatement of gst_batch_sample_modes: (cov (dim, M), z1, z2)."""
    counts = np.ascontiguousarray(mode_counts, dtype=np.int64)
    off = np.ascontiguousarray(np.concatenate(([0], np.cumsum(counts))),
                               dtype=np.int64)
    total = int(off[-1])
    seeds = np.ascontiguousarray(seeds, dtype=np.uint64)
    ls = _f64(len_rescaled)
    cov = np.zeros((dim, total))
    z1 = np.zeros(total)
    z2 = np.zeros(total)
    rc = _load().oracle_sample_modes(
        dim, len(counts), total, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
        MODEL_KINDS[model] if isinstance(model, str) else int(model), float(nu),
        seeds.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), _ptr(ls),
        _ptr(cov), _ptr(z1), _ptr(z2))
    if rc:
        raise ValueError(f"oracle_sample_modes failed with code {rc}")
    return cov, z1, z2


def c_krige(krig_mat, krig_vecs, cond, with_error=True):
    """C restatement of gstools-cython's calc_field_krige(_and_variance):
    (field, error) or field for M (K, K), V (K, n), cond (K,)."""
    mat = _f64(np.atleast_2d(krig_mat))
    vecs = _f64(np.atleast_2d(krig_vecs))
    cnd = _f64(cond).reshape(-1)
    k, n = vecs.shape
    if mat.shape != (k, k) or cnd.size != k:
        raise ValueError("oracle_krige: M (K, K), V (K, n), cond (K,)")
    field = np.empty(n)
    error = np.empty(n) if with_error else None
    rc = _load().oracle_krige(k, n, _ptr(mat), _ptr(vecs), _ptr(cnd), _ptr(field),
                              _ptr(error) if with_error else None)
    if rc:
        raise ValueError(f"oracle_krige failed with code {rc}")
    return (field, error) if with_error else field


def np_krige(krig_mat, krig_vecs, cond):
    """numpy witness: (field, error, scale) per target point, with
    scale = sum_i (|c_i| + |v_i|) (|M| |v|)_i, the magnitude that rounding
    errors of both nested sums scale with (kriging matrices of smooth
    covariances are ill-conditioned, so the sums cancel)."""
    m = np.asarray(krig_mat)
    v = np.asarray(krig_vecs)
    mv = m @ v
    c = np.asarray(cond).reshape(-1, 1)
    amv = np.abs(m) @ np.abs(v)
    return ((c * mv).sum(axis=0), (v * mv).sum(axis=0),
            ((np.abs(c) + np.abs(v)) * amv).sum(axis=0))


def _est(estimator_type):
    e = str(estimator_type)
    if e not in ("m", "c"):
        raise ValueError(f"unknown estimator type {estimator_type!r}")
    return e.encode()


def c_vario_unstructured(f, bin_edges, pos, estimator_type="m",
                         distance_type="e", num_threads=None):
    """gstools-cython's ``variogram.unstructured``: (variogram, counts)."""
    pos = _f64(np.atleast_2d(pos))
    dim, n = pos.shape
    f = _f64(np.atleast_2d(f)).reshape(-1, n)
    edges = _f64(bin_edges).reshape(-1)
    nb = max(edges.size - 1, 0)
    vario = np.zeros(nb)
    counts = np.zeros(nb, dtype=np.int64)
    dist = str(distance_type)
    if dist not in ("e", "h"):
        raise ValueError(f"unknown distance type {distance_type!r}")
    rc = _load().oracle_vario_unstructured(
        dim, n, f.shape[0], _ptr(f), nb, _ptr(edges), _ptr(pos), _est(estimator_type),
        dist.encode(), _ptr(vario), counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    if rc:
        raise ValueError(f"oracle_vario_unstructured failed with code {rc}")
    return vario, counts


def c_vario_directional(f, bin_edges, pos, direction, angles_tol=np.pi / 8.0,
                        bandwidth=-1.0, separate_dirs=False, estimator_type="m",
                        num_threads=None):
    """gstools-cython's ``variogram.directional``: (variogram, counts),
    each (directions, bins)."""
    pos = _f64(np.atleast_2d(pos))
    dim, n = pos.shape
    f = _f64(np.atleast_2d(f)).reshape(-1, n)
    edges = _f64(bin_edges).reshape(-1)
    dirs = _f64(np.atleast_2d(direction)).reshape(-1, dim)
    nb = max(edges.size - 1, 0)
    vario = np.zeros((dirs.shape[0], nb))
    counts = np.zeros((dirs.shape[0], nb), dtype=np.int64)
    rc = _load().oracle_vario_directional(
        dim, n, f.shape[0], _ptr(f), nb, _ptr(edges), _ptr(pos), dirs.shape[0],
        _ptr(dirs), float(angles_tol), float(bandwidth), int(bool(separate_dirs)),
        _est(estimator_type), _ptr(vario),
        counts.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    if rc:
        raise ValueError(f"oracle_vario_directional failed with code {rc}")
    return vario, counts


def c_vario_structured(f, estimator_type="m", num_threads=None, mask=None):
    """gstools-cython's ``variogram.structured`` / ``ma_structured``:
    the variogram along axis 0 of f (n0, ...), lags 0 .. n0 - 1."""
    f = _f64(f)
    n0 = f.shape[0] if f.ndim else 1
    f = f.reshape(n0, -1)
    m = None
    if mask is not None:
        m = np.ascontiguousarray(np.asarray(mask, dtype=bool).reshape(n0, -1),
                                 dtype=np.uint8)
    vario = np.zeros(n0)
    rc = _load().oracle_vario_structured(
        n0, f.shape[1], _ptr(f),
        m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)) if m is not None else None,
        _est(estimator_type), _ptr(vario))
    if rc:
        raise ValueError(f"oracle_vario_structured failed with code {rc}")
    return vario
