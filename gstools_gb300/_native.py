"""ctypes binding of ``libgstools_gb300.so`` (C ABI: include/gstools_gb300.h).

The library is the only compute path of this package.  If it has not been
built, or no CUDA device is present, every entry point raises -- there is no
CPU fallback.
"""

import ctypes
import os
import threading

from . import build as _build

GST_OK = 0
GST_ERR_INVALID_ARGUMENT = 1
GST_ERR_UNSUPPORTED_DIM = 2
GST_ERR_CUDA = 3
GST_ERR_ALIGNMENT = 4
GST_ERR_NO_DEVICE = 5
GST_ERR_DEVICE_TIMEOUT = 6
GST_ERR_TOO_LARGE = 7

GST_OUT_F64 = 0
GST_OUT_F32 = 1
GST_TC_TF32 = 0
GST_TC_F16 = 1
GST_MODEL_GAUSSIAN = 0
GST_MODEL_EXPONENTIAL = 1
GST_MODEL_MATERN = 2

_c_int = ctypes.c_int
_i64 = ctypes.c_int64
_u32 = ctypes.c_uint32
_ptr = ctypes.c_void_p
_dbl = ctypes.c_double

# name -> (restype, argtypes); mirrors include/gstools_gb300.h
SIGNATURES = {
    "gst_version": (_c_int, []),
    "gst_status_string": (ctypes.c_char_p, [_c_int]),
    "gst_last_cuda_error": (_c_int, []),
    "gst_read_device_error": (_c_int, [_ptr, ctypes.POINTER(_u32)]),
    "gst_host_gather": (_c_int, [_i64, _ptr, _ptr, _i64, _ptr, _i64, _c_int]),
    "gst_summate_f64": (_c_int, [_c_int, _i64, _i64, _ptr, _ptr, _ptr, _ptr,
                                 _ptr, _ptr]),
    "gst_summate_f64_noalloc": (_c_int, [_c_int, _i64, _i64, _ptr, _ptr,
                                         _ptr, _ptr, _ptr, _ptr]),
    "gst_summate_incompr_f64": (_c_int, [_c_int, _i64, _i64, _ptr, _ptr,
                                         _ptr, _ptr, _ptr, _ptr]),
    "gst_summate_fourier_f64": (_c_int, [_c_int, _i64, _i64, _ptr, _ptr,
                                         _ptr, _ptr, _ptr, _ptr, _ptr]),
    "gst_summate_mixed": (_c_int, [_c_int, _i64, _i64, _ptr, _ptr, _ptr,
                                   _ptr, _ptr, _c_int, _ptr]),
    "gst_summate_incompr_mixed": (_c_int, [_c_int, _i64, _i64, _ptr, _ptr,
                                           _ptr, _ptr, _ptr, _c_int, _ptr]),
    "gst_summate_grid_f64": (_c_int, [_c_int, _i64, _ptr, _ptr, _ptr, _ptr,
                                      _ptr, _ptr, _ptr]),
    "gst_summate_grid_mixed": (_c_int, [_c_int, _i64, _ptr, _ptr, _ptr, _ptr,
                                        _ptr, _ptr, _c_int, _dbl, _ptr]),
    "gst_summate_incompr_grid_f64": (_c_int, [_c_int, _i64, _ptr, _ptr, _ptr,
                                              _ptr, _ptr, _ptr, _ptr]),
    "gst_summate_incompr_grid_mixed": (_c_int, [_c_int, _i64, _ptr, _ptr,
                                                _ptr, _ptr, _ptr, _ptr, _c_int,
                                                _dbl, _ptr]),
    "gst_summate_grid_tc": (_c_int, [_c_int, _i64, _ptr, _ptr, _ptr, _ptr,
                                     _ptr, _ptr, _c_int, _dbl, _ptr]),
    "gst_summate_incompr_grid_tc": (_c_int, [_c_int, _i64, _ptr, _ptr, _ptr,
                                             _ptr, _ptr, _ptr, _ptr, _c_int,
                                             _dbl, _ptr]),
    "gst_summate_fourier_grid_tc": (_c_int, [_c_int, _i64, _ptr, _ptr, _ptr,
                                             _ptr, _ptr, _ptr, _ptr, _c_int,
                                             _dbl, _ptr]),
    "gst_grid_tc_workspace_size": (_c_int, [_c_int, _i64, _ptr,
                                            ctypes.POINTER(ctypes.c_size_t)]),
    "gst_grid_tc_tile_cols": (_c_int, [_i64]),
    "gst_grid_tc_tables": (_c_int, [_c_int, _i64, _ptr, _ptr, _ptr, _ptr,
                                    _ptr, _ptr, ctypes.c_size_t, _ptr]),
    "gst_grid_tc_contract": (_c_int, [_c_int, _i64, _ptr, _ptr,
                                      ctypes.c_size_t, _ptr, _c_int, _dbl,
                                      _ptr]),
    "gst_batch_variants": (_c_int, []),
    "gst_batch_workspace_size": (_c_int, [_c_int, _i64, _ptr, _ptr, _c_int,
                                          ctypes.POINTER(ctypes.c_size_t)]),
    "gst_batch_prepare": (_c_int, [_c_int, _i64, _ptr, _ptr, _c_int, _ptr,
                                   ctypes.c_size_t, _ptr]),
    "gst_batch_run": (_c_int, [_c_int, _i64, _ptr, _ptr, _c_int, _ptr, _ptr,
                               _ptr, _ptr, _ptr, _ptr, _c_int, _ptr,
                               ctypes.c_size_t, _ptr]),
    "gst_summate_vjp_modes_f64": (_c_int, [_c_int, _i64, _i64] + [_ptr] * 9),
    "gst_summate_vjp_modes_mixed": (_c_int, [_c_int, _i64, _i64] + [_ptr] * 9),
    "gst_summate_vjp_pos_f64": (_c_int, [_c_int, _i64, _i64] + [_ptr] * 6),
    "gst_summate_vjp_pos_mixed": (_c_int, [_c_int, _i64, _i64] + [_ptr] * 6),
    "gst_gather_points": (_c_int, [_c_int, _ptr, _ptr, _i64, _ptr, _i64] + [_ptr] * 5),
    "gst_mode_map": (_c_int, [_c_int, _ptr, _dbl, _ptr, _ptr, _ptr]),
    "gst_grid_tc_contract_rows": (_c_int, [_c_int, _i64, _ptr, _ptr,
                                           ctypes.c_size_t, _ptr, _c_int, _dbl,
                                           _i64, _i64, _ptr]),
    "gst_summate_grid_tc_host": (_c_int, [_c_int, _i64, _ptr, _ptr, _ptr, _ptr,
                                          _ptr, _ptr, _c_int, _dbl, _ptr]),
    "gst_summate_incompr_grid_tc_host": (_c_int, [_c_int, _i64, _ptr, _ptr, _ptr,
                                                  _ptr, _ptr, _ptr, _ptr, _c_int,
                                                  _dbl, _ptr]),
    "gst_summate_fourier_grid_tc_host": (_c_int, [_c_int, _i64, _ptr, _ptr, _ptr,
                                                  _ptr, _ptr, _ptr, _ptr, _c_int,
                                                  _dbl, _ptr]),
    "gst_grid_tc_set_operands": (_c_int, [_c_int]),
    "gst_batch_sample_modes": (_c_int, [_c_int, _i64, _i64, _ptr, _c_int, _dbl,
                                        _ptr, _ptr, _ptr, _ptr, _ptr, _ptr]),
    "gst_calc_field_krige": (_c_int, [_i64, _i64, _ptr, _ptr, _ptr, _ptr, _ptr,
                                      _ptr]),
    "gst_vario_unstructured": (_c_int, [_c_int, _i64, _i64, _ptr, _i64, _ptr, _ptr,
                                        _c_int, _c_int, _ptr, _ptr, _ptr]),
    "gst_vario_angle_boundary": (_c_int, [_dbl, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double)]),
    "gst_vario_directional": (_c_int, [_c_int, _i64, _i64, _ptr, _i64, _ptr, _ptr,
                                       _i64, _ptr, _dbl, _dbl, _c_int, _c_int,
                                       _ptr, _ptr, _ptr]),
    "gst_vario_structured": (_c_int, [_i64, _i64, _ptr, _ptr, _c_int, _ptr, _ptr]),
    "gst_philox4x64_fill": (_c_int, [ctypes.c_uint64, ctypes.c_uint64, _i64,
                                     ctypes.c_uint64, _ptr, _ptr]),
    "gst_peak_probe": (_c_int, [_c_int, _i64, _ptr, ctypes.POINTER(_dbl),
                                _ptr]),
}

_lib = None
_lock = threading.Lock()


class NativeError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, func, code, detail=""):
        self.func = func
        self.code = code
        super().__init__(f"{func} failed: {status_string(code)} ({code})"
                         + (f"; {detail}" if detail else ""))


def library_path():
    return _build.LIB_PATH


def load():
    """Load the native library (raises if it is missing)."""
    global _lib
    with _lock:
        if _lib is None:
            path = library_path()
            if not os.path.exists(path):
                raise RuntimeError(
                    f"gstools_gb300: native library {path} is not built; run "
                    "`python -m gstools_gb300.build` (no CPU fallback exists)"
                )
            lib = ctypes.CDLL(path)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def status_string(code):
    try:
        return load().gst_status_string(int(code)).decode()
    except Exception:  # pragma: no cover - library missing
        return "unknown status"


def call(name, *args):
    """Call a C-ABI entry point and map non-zero status to an exception."""
    rc = getattr(load(), name)(*args)
    if rc != GST_OK:
        if rc in (GST_ERR_INVALID_ARGUMENT, GST_ERR_UNSUPPORTED_DIM,
                  GST_ERR_TOO_LARGE, GST_ERR_ALIGNMENT):
            raise ValueError(f"{name}: {status_string(rc)} ({rc})")
        detail = ""
        if rc == GST_ERR_CUDA:
            detail = f"cudaError {load().gst_last_cuda_error()}"
        raise NativeError(name, rc, detail)
    return rc


_TC_KINDS = {"tf32": GST_TC_TF32, "f16": GST_TC_F16}


def set_tc_operands(kind):
    """Select the operand format of the tensor-core grid path ("f16", the
    default, or "tf32"; process-wide) and return the previous one."""
    if kind not in _TC_KINDS:
        raise ValueError(f"unknown operand kind {kind!r}; use 'f16' or 'tf32'")
    prev = load().gst_grid_tc_set_operands(_TC_KINDS[kind])
    return {v: k for k, v in _TC_KINDS.items()}[prev]


def grid_tile_cols(nz):
    """z tile width (MMA N) of the tensor-core grid path for nz points."""
    return load().gst_grid_tc_tile_cols(int(nz))


def read_device_error(stream=0):
    """Read and clear the device error word (synchronises ``stream``)."""
    word = _u32(0)
    call("gst_read_device_error", ctypes.c_void_p(stream), ctypes.byref(word))
    return int(word.value)
