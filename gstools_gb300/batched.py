"""Ensembles of realizations in one persistent launch.

The reference draws an ensemble by calling ``SRF`` once per seed, each call
re-sampling the modes on the host and making one native ``summate`` call
(src/gstools/field/srf.py:109-163; examples/01_random_field/
01_srf_ensemble.py).  :class:`BatchedSummator` sums a whole ensemble --
realizations with their own modes, variances and point sets of uneven size --
in a single persistent kernel over a queue of (realization, point tile) work
items (``gst_batch_*`` in include/gstools_gb300.h), replayed from a CUDA
graph.

The kernel shape -- points per work tile, modes per shared-memory stage and
CTAs per SM, six compiled variants (``VARIANT_SHAPES``) -- is chosen per
ensemble shape by timing every variant on the loaded data
(:meth:`BatchedSummator.tune`); the choice and the timings are cached per
shape for the process.

The modes can also be drawn on the device (:meth:`BatchedSummator.sample`):
all realizations' amplitudes, directions and radii in one launch from a
counter-based Philox stream per realization seed, instead of the reference's
host loop over ``RandMeth.reset_seed`` (src/gstools/field/generator.py:
346-387).  That stream is not the reference's MT19937 stream; the
distributions are the models' spectral laws.
"""

import ctypes
import hashlib
import os
import threading

import numpy as np
import torch

from . import _native
from .summator import _finish, device

__all__ = ["BatchedSummator", "VARIANTS"]

# (points per work tile, modes per stage, CTAs per SM) of each compiled
# variant of the persistent kernel (gst_batched.cu)
VARIANT_SHAPES = {
    0: (512, 256, 2),
    1: (1024, 256, 2),
    2: (512, 256, 3),
    3: (512, 128, 3),
    4: (256, 256, 4),
    5: (1024, 128, 2),
}
VARIANTS = tuple(VARIANT_SHAPES)

_tune_cache = {}
_tune_lock = threading.Lock()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr() if t is not None and t.numel() else 0)


class BatchedSummator:
    """Sum an ensemble of realizations on the GPU in one launch.

    Parameters
    ----------
    dim : int
        Spatial dimension (1, 2 or 3).
    mode_counts, point_counts : sequence of int
        Modes and evaluation points of every realization.
    out_dtype : "float32" or "float64"
        Element type of the output field.
    graph : bool
        Replay the run step from a captured CUDA graph.
    """

    def __init__(self, dim, mode_counts, point_counts, *, out_dtype="float32",
                 graph=True):
        if dim not in (1, 2, 3):
            raise ValueError("dim must be 1, 2 or 3")
        if len(mode_counts) != len(point_counts):
            raise ValueError("one mode count and one point count per item")
        self.dim = int(dim)
        self.dev = device()
        self.modes = np.ascontiguousarray(mode_counts, dtype=np.int64)
        self.points = np.ascontiguousarray(point_counts, dtype=np.int64)
        if np.any(self.modes < 0) or np.any(self.points < 0):
            raise ValueError("counts must be non-negative")
        self.n_items = len(self.modes)
        self.mode_off = np.concatenate(([0], np.cumsum(self.modes)))
        self.point_off = np.concatenate(([0], np.cumsum(self.points)))
        self.total_modes = int(self.mode_off[-1])
        self.total_points = int(self.point_off[-1])
        if out_dtype in ("float32", np.float32, torch.float32):
            self.out_code, tdtype = _native.GST_OUT_F32, torch.float32
        elif out_dtype in ("float64", np.float64, torch.float64):
            self.out_code, tdtype = _native.GST_OUT_F64, torch.float64
        else:
            raise ValueError(f"unsupported out_dtype {out_dtype!r}")
        f64 = dict(dtype=torch.float64, device=self.dev)
        self.cov = torch.zeros((self.dim, self.total_modes), **f64)
        self.z1 = torch.zeros(self.total_modes, **f64)
        self.z2 = torch.zeros(self.total_modes, **f64)
        self.pos = torch.zeros((self.dim, self.total_points), **f64)
        self.scales = torch.ones(max(self.n_items, 1), **f64)
        self.out = torch.zeros(self.total_points, dtype=tdtype, device=self.dev)
        self._modes_c = self.modes.ctypes.data_as(ctypes.c_void_p)
        self._points_c = self.points.ctypes.data_as(ctypes.c_void_p)
        self.use_graph = bool(graph)
        self.variant = None
        self.timings = {}
        self._stage = {}      # page-locked host staging buffers of load()
        self._staged = None   # event: the last uploads from them are done
        self.workspace = None
        self.ws_bytes = ctypes.c_size_t(0)
        self._graph = None
        self.key = (self.dim, hashlib.sha1(self.modes.tobytes()
                                           + self.points.tobytes()).hexdigest())

    # -- data -------------------------------------------------------------
    def _staging(self, name, shape):
        """A page-locked host buffer of this summator (allocated once), free
        to overwrite: the copies issued from it by the previous load have
        completed."""
        if self._staged is not None:
            self._staged.synchronize()
            self._staged = None
        buf = self._stage.get(name)
        if buf is None:
            buf = torch.empty(shape, dtype=torch.float64, pin_memory=True)
            self._stage[name] = buf
        return buf

    def _upload(self, pairs):
        """Asynchronous copies host staging -> device, then an event that
        the next load waits for before it refills the staging buffers."""
        stream = torch.cuda.current_stream(self.dev)
        for dst, src in pairs:
            dst.copy_(src, non_blocking=True)
        self._staged = torch.cuda.Event()
        self._staged.record(stream)

    def _as_items(self, arrays, counts, what, flat=False):
        """The per-realization arrays as C-contiguous float64 (dim, n) (or
        (n,)) arrays, checked against the plan's sizes."""
        out = []
        for r, a in enumerate(arrays):
            if not (isinstance(a, np.ndarray) and a.dtype == np.float64
                    and a.flags.c_contiguous):
                a = np.ascontiguousarray(a, dtype=np.float64)
            a = a.reshape(-1) if flat else a.reshape(self.dim, -1)
            if a.shape[-1] != counts[r]:
                raise ValueError(f"realization {r}: {what} sizes do not match the plan")
            out.append(a)
        return out

    @staticmethod
    def _gather(dst, items, cols):
        """``dst[...] = np.concatenate(items, axis=-1)`` by the library's
        host gather (plain memcpy on the host's threads)."""
        ptrs = np.fromiter((a.__array_interface__["data"][0] for a in items),
                           dtype=np.uint64, count=len(items))
        cols = np.ascontiguousarray(cols, dtype=np.int64)
        rows = 1 if dst.ndim == 1 else dst.shape[0]
        _native.call("gst_host_gather", len(items), ptrs.ctypes.data,
                     cols.ctypes.data, rows, dst.ctypes.data, dst.shape[-1],
                     min(16, os.cpu_count() or 1))

    def _fill_points(self, pos, xx, jobs=None):
        """Copy the point sets (and the copies in `jobs`: (dst, items,
        counts)) into the staging buffers."""
        jobs = [] if jobs is None else jobs
        jobs.append((xx, self._as_items(pos, self.points, "point"), self.points))
        for dst, items, counts in jobs:
            self._gather(dst, items, counts)

    def load_points(self, pos):
        """Copy the per-realization point sets (already isometrized, the
        reference's (dim, n) layout) into the device buffer."""
        if len(pos) != self.n_items:
            raise ValueError("one point set per realization expected")
        xx = self._staging("pos", (self.dim, self.total_points))
        self._fill_points(pos, xx.numpy())
        self._upload([(self.pos, xx)])

    def sample(self, model, seeds, len_scales=None, variances=None):
        """Draw every realization's modes on the device (asynchronous).

        ``model`` (Gaussian, Exponential or Matern with nu <= 20) gives the
        spectral law; ``seeds`` one uint64 per realization; ``len_scales``
        and ``variances`` override the model's per realization.  Sets the
        scales to ``sqrt(var_r / N_r)`` (RandMeth's normalisation).
        """
        kinds = {"Gaussian": _native.GST_MODEL_GAUSSIAN,
                 "Exponential": _native.GST_MODEL_EXPONENTIAL,
                 "Matern": _native.GST_MODEL_MATERN}
        name = type(model).__name__
        if name not in kinds:
            raise ValueError(f"device sampling supports {sorted(kinds)}, "
                             f"not {name}")
        if model.dim != self.dim:
            raise ValueError("model dimension does not match the plan")
        nu = float(getattr(model, "nu", 0.0)) if name == "Matern" else 0.0
        if name == "Matern" and not 0.0 < nu <= 20.0:
            raise ValueError("device sampling of Matern needs 0 < nu <= 20")
        seeds = np.array(seeds, dtype=np.uint64).reshape(-1)
        if seeds.size != self.n_items:
            raise ValueError("one seed per realization expected")
        ls = (np.full(self.n_items, model.len_scale) if len_scales is None
              else np.asarray(len_scales, dtype=np.float64).reshape(-1))
        var = (np.full(self.n_items, model.var) if variances is None
               else np.asarray(variances, dtype=np.float64).reshape(-1))
        if ls.size != self.n_items or var.size != self.n_items:
            raise ValueError("one len_scale / variance per realization expected")
        if getattr(self, "_mode_off_dev", None) is None:
            self._mode_off_dev = torch.from_numpy(
                self.mode_off.astype(np.int64)).to(self.dev)
        params = np.concatenate((seeds.view(np.float64), ls / model.rescale))
        self._sample_params = torch.from_numpy(params).to(self.dev)
        off = self._mode_off_dev
        sd = self._sample_params[: self.n_items]
        lsr = self._sample_params[self.n_items:]
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        _native.call("gst_batch_sample_modes", self.dim, self.n_items,
                     self.total_modes, _ptr(off), kinds[name], nu, _ptr(sd),
                     _ptr(lsr), _ptr(self.cov), _ptr(self.z1), _ptr(self.z2),
                     stream)
        counts = np.maximum(self.modes, 1)
        self.scales[: self.n_items].copy_(
            torch.from_numpy(np.sqrt(var / counts)))

    def load(self, cov_samples, z_1, z_2, pos, scales=None):
        """Copy one ensemble's inputs (lists of per-realization arrays, the
        reference's layouts) into the device buffers."""
        if not (len(cov_samples) == len(z_1) == len(z_2) == len(pos)
                == self.n_items):
            raise ValueError("one array per realization expected")
        cov_h = self._staging("cov", (self.dim, self.total_modes))
        z1_h = self._staging("z1", (self.total_modes,))
        z2_h = self._staging("z2", (self.total_modes,))
        xx_h = self._staging("pos", (self.dim, self.total_points))
        jobs = [(cov_h.numpy(), self._as_items(cov_samples, self.modes, "mode"),
                 self.modes),
                (z1_h.numpy(), self._as_items(z_1, self.modes, "z_1", flat=True),
                 self.modes),
                (z2_h.numpy(), self._as_items(z_2, self.modes, "z_2", flat=True),
                 self.modes)]
        uploads = [(self.cov, cov_h), (self.z1, z1_h), (self.z2, z2_h),
                   (self.pos, xx_h)]
        if scales is not None:
            s = np.asarray(scales, dtype=np.float64).reshape(-1)
            if s.size != self.n_items:
                raise ValueError("one scale per realization expected")
            s_h = self._staging("scales", (self.n_items,))
            s_h.numpy()[:] = s
            uploads.append((self.scales[: self.n_items], s_h))
        else:
            self.scales.fill_(1.0)
        self._fill_points(pos, xx_h.numpy(), jobs)
        self._upload(uploads)

    def split(self, out=None):
        """Per-realization numpy views of a host copy of ``out`` (a pooled
        page-locked buffer that the returned arrays keep alive)."""
        src = self.out if out is None else out
        host = _finish(src, False)
        return [host[self.point_off[r]:self.point_off[r + 1]]
                for r in range(self.n_items)]

    # -- planning ---------------------------------------------------------
    def _prepare(self, variant):
        nbytes = ctypes.c_size_t(0)
        _native.call("gst_batch_workspace_size", self.dim, self.n_items,
                     self._modes_c, self._points_c, variant,
                     ctypes.byref(nbytes))
        ws = torch.empty(max(nbytes.value, 256), dtype=torch.uint8,
                         device=self.dev)
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        _native.call("gst_batch_prepare", self.dim, self.n_items,
                     self._modes_c, self._points_c, variant, _ptr(ws),
                     nbytes, stream)
        return ws, nbytes

    def _launch(self, variant, ws, nbytes):
        stream = ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)
        _native.call("gst_batch_run", self.dim, self.n_items, self._modes_c,
                     self._points_c, variant, _ptr(self.cov), _ptr(self.z1),
                     _ptr(self.z2), _ptr(self.pos), _ptr(self.scales),
                     _ptr(self.out), self.out_code, _ptr(ws), nbytes, stream)

    def tune(self, repeats=3, variants=None):
        """Time every kernel variant on the loaded data (best of ``repeats``
        runs after one warm-up, CUDA events) and keep the fastest; returns
        ``{variant: ms}`` (the cached timings when this ensemble shape was
        tuned before in this process)."""
        with _tune_lock:
            cached = _tune_cache.get(self.key)
        if cached is None:
            timings = {}
            stream = torch.cuda.current_stream(self.dev)
            for v in (VARIANTS if variants is None else variants):
                ws, nbytes = self._prepare(v)
                self._launch(v, ws, nbytes)  # warm-up
                best = float("inf")
                for _ in range(repeats):
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    self._launch(v, ws, nbytes)
                    e1.record(stream)
                    e1.synchronize()
                    best = min(best, e0.elapsed_time(e1))
                timings[v] = best
                del ws
            cached = (min(timings, key=timings.get), timings)
            with _tune_lock:
                _tune_cache[self.key] = cached
        self.variant, timings = cached
        self.timings = dict(timings)
        self.workspace, self.ws_bytes = self._prepare(self.variant)
        self._graph = None
        return dict(timings)

    def _capture(self):
        side = torch.cuda.Stream(self.dev)
        side.wait_stream(torch.cuda.current_stream(self.dev))
        with torch.cuda.stream(side):
            self._launch(self.variant, self.workspace, self.ws_bytes)
        torch.cuda.current_stream(self.dev).wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            self._launch(self.variant, self.workspace, self.ws_bytes)
        self._graph = graph

    # -- execution --------------------------------------------------------
    def run(self):
        """Sum the loaded ensemble into ``self.out`` (asynchronous)."""
        if self.variant is None:
            self.tune()
        if self.use_graph:
            if self._graph is None:
                self._capture()
            self._graph.replay()
        else:
            self._launch(self.variant, self.workspace, self.ws_bytes)
        return self.out

    def __call__(self, cov_samples, z_1, z_2, pos, scales=None):
        """Load, run and return the per-realization fields (numpy)."""
        self.load(cov_samples, z_1, z_2, pos, scales)
        self.run()
        return self.split()
