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

Structured fields.  ``SRF.__call__`` and ``CondSRF.__call__``
(src/gstools/field/srf.py:150-163, cond_srf.py:115-121) get their positions
from ``Field.pre_pos`` (src/gstools/field/base.py:254-297), which builds the
full meshgrid of a structured mesh and isometrizes it before the generator
hands it to the summator.  With ``structured=True`` :func:`install` wraps
those two ``__call__`` methods and ``pre_pos``: for a structured mesh of a
non-latlon model whose generator is the reference's ``RandMeth``,
``IncomprRandMeth`` or ``Fourier``, ``pre_pos`` stores the positions as the
reference does (``set_pos``) but returns a read-only placeholder of the
grid's shape that occupies no memory; the generator's own ``__call__``
(scaling, nugget, mean velocity) runs unchanged and passes the placeholder
to the installed summator, which recognises it and evaluates the sum on the
axis arrays with the separable grid kernels (:func:`summate_structured`,
wave vectors mapped by the transpose of the isometrize matrix).  The field
then goes through the reference's own reshape and ``post_field``.  Cases the
grid kernels do not cover (latlon models, other generators, FP64
incompressible or Fourier sums under a non-identity isometrize map) take the
reference's meshgrid path.
"""

import sys
import threading

import numpy as np

from . import config
from . import variogram as _vario
from .krige import calc_field_krige, calc_field_krige_and_variance
from .summator import (
    structured_supported,
    summate,
    summate_fourier,
    summate_incompr,
    summate_structured,
)

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


# ------------------------------------------------------ structured fields --

_route = threading.local()


class GridPlaceholder:
    """A structured evaluation the installed summators run on the grid
    kernels: the axis arrays, the isometrize matrix and the generator kind.
    ``token`` is the read-only zero-stride array of shape (dim, n) that
    stands in for the isometrized meshgrid."""

    __slots__ = ("token", "axes", "iso", "kind", "precision")

    def __init__(self, axes, iso, kind, precision):
        self.axes = [np.asarray(a, dtype=np.float64).reshape(-1) for a in axes]
        self.iso = np.asarray(iso, dtype=np.float64)
        self.kind = kind
        self.precision = precision
        n = int(np.prod([a.size for a in self.axes]))
        self.token = np.broadcast_to(np.zeros((1, 1)), (len(self.axes), n))

    def register(self):
        grids = getattr(_route, "grids", None)
        if grids is None:
            grids = _route.grids = {}
        grids[id(self.token)] = self
        return self.token

    def release(self):
        grids = getattr(_route, "grids", None)
        if grids is not None:
            grids.pop(id(self.token), None)


def grid_of(pos):
    """The :class:`GridPlaceholder` whose token is ``pos``, or None."""
    grids = getattr(_route, "grids", None)
    if not grids:
        return None
    grid = grids.get(id(pos))
    return grid if grid is not None and grid.token is pos else None


def _run_grid(grid, cov, z_1, z_2, spectrum_factor=None):
    return summate_structured(cov, z_1, z_2, grid.axes, grid.iso,
                              kind=grid.kind, spectrum_factor=spectrum_factor,
                              precision=grid.precision)


def _generator_kind(gen_mod, generator):
    """"scalar" / "incompr" / "fourier" when the generator's ``__call__`` is
    the reference's own (so positions only pass through to the summator),
    else None."""
    call = getattr(type(generator), "__call__", None)
    kinds = (("RandMeth", "scalar"), ("IncomprRandMeth", "incompr"),
             ("Fourier", "fourier"))
    for name, kind in kinds:
        cls = getattr(gen_mod, name, None)
        if cls is not None and call is cls.__call__:
            return kind
    return None


def _structured_route(field, pos, mesh_type, gen_mod, precision):
    """A placeholder for a structured evaluation of ``field`` the grid
    kernels cover, or None (the reference's meshgrid path runs)."""
    mtype = field.mesh_type if pos is None else mesh_type
    if mtype == "unstructured" or (pos is None and field.pos is None):
        return None
    model = getattr(field, "model", None)
    if model is None or getattr(model, "latlon", False):
        return None
    kind = _generator_kind(gen_mod, getattr(field, "generator", None))
    if kind is None:
        return None
    prec = config.check_precision(precision)
    dim = int(model.dim)
    iso = np.asarray(model.isometrize(np.eye(dim)), dtype=np.float64)
    if iso.shape != (dim, dim) or not structured_supported(kind, dim, prec, iso):
        return None
    return kind, prec, iso


def _wrap_call(orig):
    def __call__(self, *args, **kwargs):
        prev = (getattr(_route, "field", None), getattr(_route, "created", None))
        _route.field, _route.created = self, []
        try:
            return orig(self, *args, **kwargs)
        finally:
            for grid in _route.created:
                grid.release()
            _route.field, _route.created = prev
    __call__.__wrapped__ = orig
    __call__.__doc__ = orig.__doc__
    return __call__


def _wrap_pre_pos(orig, gen_mod, precision):
    def pre_pos(self, pos=None, mesh_type="unstructured", info=False):
        if getattr(_route, "field", None) is not self:
            return orig(self, pos, mesh_type, info)
        route = _structured_route(self, pos, mesh_type, gen_mod, precision)
        if route is None:
            return orig(self, pos, mesh_type, info)
        # the reference's pre_pos, minus generate_grid + isometrize
        info_ret = {"deleted": False}
        if pos is not None:
            info_ret = self.set_pos(pos, mesh_type, info=True)
        kind, prec, iso = route
        grid = GridPlaceholder(self.pos, iso, kind, prec)
        token = grid.register()
        _route.created.append(grid)
        return (token, self.field_shape) + info * (info_ret,)
    pre_pos.__wrapped__ = orig
    pre_pos.__doc__ = orig.__doc__
    return pre_pos


def _field_classes():
    """(Field, SRF, CondSRF) of the imported reference, or None."""
    try:
        base = sys.modules.get("gstools.field.base")
        srf = sys.modules.get("gstools.field.srf")
        cond = sys.modules.get("gstools.field.cond_srf")
        if base is None or srf is None or cond is None:
            import gstools.field.base as base  # noqa: F811
            import gstools.field.cond_srf as cond  # noqa: F811
            import gstools.field.srf as srf  # noqa: F811
        return base.Field, srf.SRF, cond.CondSRF
    except ImportError:
        return None


def _install_structured(gen_mod, precision):
    classes = _field_classes()
    if classes is None:
        return
    field_cls, srf_cls, cond_cls = classes
    if "structured" not in _saved:
        _saved["structured"] = {
            (field_cls, "pre_pos"): field_cls.__dict__["pre_pos"],
            (srf_cls, "__call__"): srf_cls.__dict__["__call__"],
            (cond_cls, "__call__"): cond_cls.__dict__["__call__"],
        }
    saved = _saved["structured"]
    field_cls.pre_pos = _wrap_pre_pos(saved[(field_cls, "pre_pos")], gen_mod,
                                      precision)
    srf_cls.__call__ = _wrap_call(saved[(srf_cls, "__call__")])
    cond_cls.__call__ = _wrap_call(saved[(cond_cls, "__call__")])


def _uninstall_structured():
    saved = _saved.pop("structured", None)
    if saved:
        for (cls, name), fct in saved.items():
            setattr(cls, name, fct)


# ----------------------------------------------------------------- install --

def install(module=None, precision=None, krige_module=None, vario_module=None,
            structured=True):
    """Route the reference's summation and kriging calls to the GPU kernels.

    ``module`` defaults to ``gstools.field.generator`` and ``krige_module``
    to ``gstools.krige.base`` (skipped when it cannot be imported);
    ``precision`` ("f64" or "mixed") is fixed for the installed summators
    (``None`` follows ``gstools_gb300.config.PRECISION`` at call time).
    Kriging always runs in FP64.  ``structured`` (default True; needs the
    reference's ``gstools.field`` classes, skipped when ``module`` is given)
    sends structured ``SRF`` / ``CondSRF`` evaluations to the separable grid
    kernels without building the meshgrid.  Returns the generator module.
    """
    mod = _generator_module(module)
    if precision is not None:
        config.check_precision(precision)
    if id(mod) not in _saved:
        _saved[id(mod)] = {n: getattr(mod, n) for n in _NAMES}

    def _summate(cov_samples, z_1, z_2, pos, num_threads=None):
        grid = grid_of(pos)
        if grid is not None:
            return _run_grid(grid, cov_samples, z_1, z_2)
        return summate(cov_samples, z_1, z_2, pos, num_threads,
                       precision=precision)

    def _summate_incompr(cov_samples, z_1, z_2, pos, num_threads=None):
        grid = grid_of(pos)
        if grid is not None:
            return _run_grid(grid, cov_samples, z_1, z_2)
        return summate_incompr(cov_samples, z_1, z_2, pos, num_threads,
                               precision=precision)

    def _summate_fourier(spectrum_factor, modes, z_1, z_2, pos,
                         num_threads=None):
        grid = grid_of(pos)
        if grid is not None:
            return _run_grid(grid, modes, z_1, z_2, spectrum_factor)
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
    if structured and module is None:
        _install_structured(mod, precision)
    return mod


def uninstall(module=None, krige_module=None, vario_module=None):
    """Restore the functions that :func:`install` replaced."""
    mod = _generator_module(module)
    if module is None:
        _uninstall_structured()
    for m in (mod, _krige_module(krige_module), _vario_module(vario_module)):
        if m is None:
            continue
        saved = _saved.pop(id(m), None)
        if saved:
            for name, fct in saved.items():
                setattr(m, name, fct)
    return mod
