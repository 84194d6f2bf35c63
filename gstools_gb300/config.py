"""Runtime switches, in the spirit of the reference's ``gstools.config``
(src/gstools/config.py:8-17: ``NUM_THREADS`` and ``USE_GSTOOLS_CORE`` are
module globals read at call time).

PRECISION
    Arithmetic of ``summate`` / ``summate_incompr`` when called with the
    reference's signature:

    * ``"f64"`` (default) -- the plain FP64 kernels, matching the reference's
      FP64 ``summate`` to <= 1e-12 relative (max|diff| / max|ref|);
    * ``"mixed"`` -- exact turn reduction + FP32/SFU sin/cos with FP64 block
      accumulation (field RMS error ~1e-7 sigma, see the parity tests).

NUM_THREADS
    Accepted for signature compatibility with the reference and ignored: the
    work runs on the current CUDA device.
"""

PRECISION = "f64"
NUM_THREADS = None

PRECISIONS = ("f64", "mixed")


def check_precision(precision):
    """Return a validated precision name (``None`` -> ``PRECISION``)."""
    prec = PRECISION if precision is None else precision
    if prec not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}, got {prec!r}")
    return prec
