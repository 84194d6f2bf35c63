"""Install the GB300 summators into an imported reference GSTools.

The reference resolves its summators per call through module globals:
``RandMeth.__call__`` calls ``_summate(...)`` (src/gstools/field/generator.py:
266-268), ``IncomprRandMeth.__call__`` calls ``_summate_incompr(...)``
(:554-560) and ``Fourier.__call__`` calls ``_summate_fourier(...)``
(:682-689).  Rebinding those three names routes every ``SRF`` / ``CondSRF`` /
generator call of that process through this package, with no other change
to the reference.  Kriging is routed the same way: ``Krige._summate``
(src/gstools/krige/base.py:307-320) calls the module globals
``_calc_field_krige`` / ``_calc_field_krige_and_variance`` (:42-60), which
:func:`install` rebinds in ``gstools.krige.base`` when that module is
importable, and the variogram estimators likewise: ``vario_estimate`` /
``vario_estimate_axis`` call ``_unstructured``, ``_directional``,
``_structured`` and ``_ma_structured`` (src/gstools/variogram/
variogram.py:48-124) in ``gstools.variogram.variogram``.
"""

import sys

from . import config
from . import variogram as _vario
from .krige import calc_field_krige, calc_field_krige_and_variance
from .summator import summate, summate_fourier, summate_incompr

_saved = {}

_NAMES = ("_summate", "_summate_incompr", "_summate_fourier")
_KRIGE_NAMES = ("_calc_field_krige", "_calc_field_krige_and_variance")
_VARIO_NAMES = ("_unstructured", "_directional", "_structured", "_ma_structured")


def _generator_module(module=None):
    if module is not None:
        return module
    mod = sys.modules.get("gstools.field.generator")
    if mod is None:
        import gstools.field.generator as mod  # noqa: F811
    return mod


def _krige_module(module=None):
    if module is not None:
        return module
    mod = sys.modules.get("gstools.krige.base")
    if mod is None:
        try:
            import gstools.krige.base as mod  # noqa: F811
        except ImportError:
            return None
    return mod


def _vario_module(module=None):
    if module is not None:
        return module
    mod = sys.modules.get("gstools.variogram.variogram")
    if mod is None:
        try:
            import gstools.variogram.variogram as mod  # noqa: F811
        except ImportError:
            return None
    return mod


def install(module=None, precision=None, krige_module=None, vario_module=None):
    """Route the reference's summation and kriging calls to the GPU kernels.

    ``module`` defaults to ``gstools.field.generator`` and ``krige_module``
    to ``gstools.krige.base`` (skipped when it cannot be imported);
    ``precision`` ("f64" or "mixed") is fixed for the installed summators
    (``None`` follows ``gstools_gb300.config.PRECISION`` at call time).
    Kriging always runs in FP64.  Returns the generator module.
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

    kmod = _krige_module(krige_module)
    if kmod is not None:
        if id(kmod) not in _saved:
            _saved[id(kmod)] = {n: getattr(kmod, n) for n in _KRIGE_NAMES}

        def _calc_field_krige(krig_mat, krig_vecs, cond, num_threads=None):
            return calc_field_krige(krig_mat, krig_vecs, cond, num_threads)

        def _calc_field_krige_and_variance(krig_mat, krig_vecs, cond,
                                           num_threads=None):
            return calc_field_krige_and_variance(krig_mat, krig_vecs, cond,
                                                 num_threads)

        kmod._calc_field_krige = _calc_field_krige
        kmod._calc_field_krige_and_variance = _calc_field_krige_and_variance

    vmod = _vario_module(vario_module)
    if vmod is not None:
        if id(vmod) not in _saved:
            _saved[id(vmod)] = {n: getattr(vmod, n) for n in _VARIO_NAMES}

        def _unstructured(field, bin_edges, pos, estimator_type="m",
                          distance_type="e", num_threads=None):
            return _vario.unstructured(field, bin_edges, pos, estimator_type,
                                       distance_type, num_threads)

        def _directional(field, bin_edges, pos, direction,
                         angles_tol=3.141592653589793 / 8.0, bandwidth=-1.0,
                         separate_dirs=False, estimator_type="m",
                         num_threads=None):
            return _vario.directional(field, bin_edges, pos, direction,
                                      angles_tol, bandwidth, separate_dirs,
                                      estimator_type, num_threads)

        def _structured(field, estimator_type="m", num_threads=None):
            return _vario.structured(field, estimator_type, num_threads)

        def _ma_structured(field, mask, estimator_type="m", num_threads=None):
            return _vario.ma_structured(field, mask, estimator_type, num_threads)

        vmod._unstructured = _unstructured
        vmod._directional = _directional
        vmod._structured = _structured
        vmod._ma_structured = _ma_structured
    return mod


def uninstall(module=None, krige_module=None, vario_module=None):
    """Restore the functions that :func:`install` replaced."""
    mod = _generator_module(module)
    for m in (mod, _krige_module(krige_module), _vario_module(vario_module)):
        if m is None:
            continue
        saved = _saved.pop(id(m), None)
        if saved:
            for name, fct in saved.items():
                setattr(m, name, fct)
    return mod
