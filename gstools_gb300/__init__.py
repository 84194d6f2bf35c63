"""gstools_gb300 -- the randomization-method summation of GSTools on GB300.

Drop-in for the native summators behind ``gstools.field.generator.RandMeth``
and ``IncomprRandMeth`` (src/gstools/field/generator.py:22-24, 42-64):

* :func:`summate`, :func:`summate_incompr`, :func:`summate_fourier` -- the
  reference's signatures ``(cov_samples, z_1, z_2, pos, num_threads=None)``;
* :func:`install` -- rebinds ``gstools.field.generator._summate`` /
  ``_summate_incompr`` / ``_summate_fourier`` so an unmodified
  ``gstools.SRF(model, generator="RandMeth", mode_no=...)`` runs on the GPU,
  and sends structured SRF / CondSRF evaluations to the separable grid
  kernels (:func:`summate_structured`) without building the meshgrid;
* :class:`RandMeth`, :class:`IncomprRandMeth`, :class:`SRF` and the models
  :class:`Gaussian`, :class:`Exponential`, :class:`Matern` -- a standalone
  mirror of the reference's generator stack with the same seeds and streams.

All compute runs in ``libgstools_gb300.so`` (hand-written sm_103a CUDA behind
a C ABI, include/gstools_gb300.h); there is no CPU fallback.
"""

from . import config
from .batched import BatchedSummator
from .covmodel import CovModel, Exponential, Gaussian, Matern
from .generator import Fourier, IncomprRandMeth, RandMeth
from .hook import install, uninstall
from .krige import calc_field_krige, calc_field_krige_and_variance
from .rng import RNG, MasterRNG
from .srf import SRF
from .summator import (
    summate,
    summate_fourier,
    summate_fourier_grid,
    summate_grid,
    summate_incompr,
    summate_incompr_grid,
    summate_structured,
)

__version__ = "0.1.0"

__all__ = [
    "config",
    "BatchedSummator",
    "Fourier",
    "calc_field_krige",
    "calc_field_krige_and_variance",
    "CovModel",
    "Gaussian",
    "Exponential",
    "Matern",
    "RandMeth",
    "IncomprRandMeth",
    "SRF",
    "RNG",
    "MasterRNG",
    "summate",
    "summate_incompr",
    "summate_fourier",
    "summate_grid",
    "summate_incompr_grid",
    "summate_fourier_grid",
    "summate_structured",
    "install",
    "uninstall",
]
