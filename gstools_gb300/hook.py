"""Install the GB300 summators into an imported reference GSTools.

The reference resolves its summators per call through module globals:
``RandMeth.__call__`` calls ``_summate(...)`` (src/gstools/field/generator.py:
266-268), ``IncomprRandMeth.__call__`` calls ``_summate_incompr(...)``
(:554-560) and ``Fourier.__call__`` calls ``_summate_fourier(...)``
(:682-689).  Rebinding those three names routes every ``SRF`` / ``CondSRF`` /
generator call of that process through this package, with no other change
to the reference.
"""

import sys

from . import config
from .summator import summate, summate_fourier, summate_incompr

_saved = {}

_NAMES = ("_summate", "_summate_incompr", "_summate_fourier")


def _generator_module(module=None):
    if module is not None:
        return module
    mod = sys.modules.get("gstools.field.generator")
    if mod is None:
        import gstools.field.generator as mod  # noqa: F811
    return mod


def install(module=None, precision=None):
    """Route the reference's summation calls to the GPU kernels.

    ``module`` defaults to ``gstools.field.generator``; ``precision``
    ("f64" or "mixed") is fixed for the installed wrappers (``None`` follows
    ``gstools_gb300.config.PRECISION`` at call time).  Returns the module.
    """
    mod = _generator_module(module)
    if precision is not None:
        config.check_precision(precision)
    if id(mod) not in _saved:
        _saved[id(mod)] = {n: getattr(mod, n) for n in _NAMES}

    def _summate(cov_samples, z_1, z_2, pos, num_threads=None):
        return summate(cov_samples, z_1, z_2, pos, num_threads,
                       precision=precision)

    def _summate_incompr(cov_samples, z_1, z_2, pos, num_threads=None):
        return summate_incompr(cov_samples, z_1, z_2, pos, num_threads,
                               precision=precision)

    def _summate_fourier(spectrum_factor, modes, z_1, z_2, pos,
                         num_threads=None):
        return summate_fourier(spectrum_factor, modes, z_1, z_2, pos,
                               num_threads)

    mod._summate = _summate
    mod._summate_incompr = _summate_incompr
    mod._summate_fourier = _summate_fourier
    return mod


def uninstall(module=None):
    """Restore the summators that :func:`install` replaced."""
    mod = _generator_module(module)
    saved = _saved.pop(id(mod), None)
    if saved:
        for name, fct in saved.items():
            setattr(mod, name, fct)
    return mod
