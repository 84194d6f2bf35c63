"""Randomization-method generators driving the GB300 summators.

``RandMeth`` and ``IncomprRandMeth`` mirror the reference's generators
(src/gstools/field/generator.py:165-446 and :449-592): the same constructor
arguments, ``update`` / ``reset_seed`` / ``seed`` / ``mode_no`` / ``model``
semantics and random streams, so the same seed gives the same
``cov_samples``, ``z_1`` and ``z_2`` (bit for bit on the inversion path), and
``__call__(pos)`` returns ``sqrt(var / N) * summate(...) + nugget``
(:266-270) or ``mean_u e1 + mean_u sqrt(var / N) summate_incompr(...) +
nugget`` (:554-567).

Differences, all additive:

* ``precision`` ("f64" or "mixed") selects the kernel family;
* ``structured(axes)`` evaluates a structured grid without materialising the
  meshgrid, mapping the wave vectors by the transpose of the isometrize
  matrix instead;
* radii of models without a ppf are drawn by the model's exact analytic
  sampler (the reference's MCMC path needs emcee, which is not used here);
  ``sampling="inversion"`` still reproduces the reference's scipy inversion.
"""

import warnings
from copy import deepcopy

import numpy as np

from . import config
from .covmodel import CovModel
from .rng import RNG
from .geometric import generate_grid
from .summator import (
    summate,
    summate_fourier,
    summate_fourier_grid,
    summate_grid,
    summate_incompr,
    summate_incompr_grid,
)

__all__ = ["RandMeth", "IncomprRandMeth", "Fourier"]

SAMPLING = ["auto", "inversion", "mcmc", "analytic"]


class RandMeth:
    """Randomization method for isotropic random fields.

    ``u(x) = sqrt(var / N) sum_i Z1_i cos(<k_i, x>) + Z2_i sin(<k_i, x>)``
    """

    def __init__(self, model, *, mode_no=1000, seed=None, sampling="auto",
                 precision=None, **kwargs):
        if kwargs:
            warnings.warn("gstools_gb300.RandMeth: **kwargs are ignored")
        self._mode_no = int(mode_no)
        self._model = None
        self._seed = None
        self._rng = None
        self._z_1 = None
        self._z_2 = None
        self._cov_sample = None
        self._value_type = "scalar"
        self._sampling = None
        self.sampling = sampling
        self.precision = config.check_precision(precision)
        self.update(model, seed)

    # -- evaluation --------------------------------------------------------
    def __call__(self, pos, add_nugget=True):
        """Field values at the (already isometrized) positions ``pos``."""
        pos = np.asarray(pos, dtype=np.double)
        if self.zero_var:
            shp = pos.shape[1:]
            return self.get_nugget(shp) if add_nugget else np.full(shp, 0.0)
        summed = summate(self._cov_sample, self._z_1, self._z_2, pos,
                         config.NUM_THREADS, precision=self.precision)
        nugget = self.get_nugget(summed.shape) if add_nugget else 0.0
        return np.sqrt(self.model.var / self._mode_no) * summed + nugget

    def structured(self, axes, add_nugget=True, out_dtype=None):
        """Field on the structured grid spanned by ``axes`` (physical
        coordinates; the model's isometrize map is applied to the modes)."""
        axes = [np.asarray(a, dtype=np.double).reshape(-1) for a in axes]
        shape = tuple(len(a) for a in axes)
        if self.zero_var:
            return self.get_nugget(shape) if add_nugget else np.full(shape, 0.0)
        cov = self.model.isometrize_matrix.T @ self._cov_sample
        scale = float(np.sqrt(self.model.var / self._mode_no))
        field = summate_grid(cov, self._z_1, self._z_2, axes,
                             precision=self.precision, out_dtype=out_dtype,
                             scale=scale)
        if add_nugget and self.model.nugget > 0:
            field = field + self.get_nugget(shape)
        return field

    def get_nugget(self, shape):
        """Normal nugget noise (generator.py:272-292)."""
        if self.model.nugget > 0:
            return np.sqrt(self.model.nugget) * self._rng.random.normal(
                size=shape)
        return np.full(shape, 0.0) if self.zero_var else 0.0

    # -- state -----------------------------------------------------------
    def update(self, model=None, seed=np.nan):
        """Update model and/or seed (generator.py:294-344)."""
        if isinstance(model, CovModel):
            if self.model != model:
                self._model = deepcopy(model)
                if seed is None or not np.isnan(seed):
                    self.reset_seed(seed)
                else:
                    self.reset_seed(self._seed)
            elif seed is None or not np.isnan(seed):
                self.seed = seed
        elif model is None and (seed is None or not np.isnan(seed)):
            if isinstance(self._model, CovModel):
                self.seed = seed
            else:
                raise ValueError(f"{self.name}: no 'model' given")
        elif model is None and np.isnan(seed):
            if not (isinstance(self._model, CovModel)
                    and self._z_1 is not None and self._z_2 is not None
                    and self._cov_sample is not None):
                raise ValueError(f"{self.name}: neither 'model' nor 'seed' "
                                 "given!")
        else:
            raise ValueError(f"{self.name}: 'model' is not a CovModel")

    def reset_seed(self, seed=np.nan):
        """Redraw amplitudes and wave vectors (generator.py:346-387)."""
        if seed is None or not np.isnan(seed):
            self._seed = seed
        self._rng = RNG(self._seed)
        self._z_1 = self._rng.random.normal(size=self._mode_no)
        self._z_2 = self._rng.random.normal(size=self._mode_no)
        if self.zero_var:
            self._cov_sample = np.full((self.model.dim, self._mode_no), 0.0)
            return
        sph = self._rng.sample_sphere(self.model.dim, self._mode_no)
        if self.sampling == "inversion" or (
                self.sampling == "auto" and self.model.has_ppf):
            pdf, cdf, ppf = self.model.dist_func
            rad = self._rng.sample_dist(size=self._mode_no, pdf=pdf, cdf=cdf,
                                        ppf=ppf, a=0)
        else:
            rad = self.model.sample_radius(self._rng.random, self._mode_no)
        self._cov_sample = rad * sph

    # -- properties ----------------------------------------------------------
    @property
    def sampling(self):
        return self._sampling

    @sampling.setter
    def sampling(self, sampling):
        if sampling not in SAMPLING:
            raise ValueError(f"{self.name}: sampling not in {SAMPLING}.")
        if sampling == "mcmc":
            warnings.warn(f"{self.name}: MCMC sampling (emcee) is not "
                          "available; using the exact analytic sampler")
        self._sampling = sampling

    @property
    def seed(self):
        return self._seed

    @seed.setter
    def seed(self, new_seed):
        if new_seed is not self._seed:
            self.reset_seed(new_seed)

    @property
    def model(self):
        return self._model

    @model.setter
    def model(self, model):
        self.update(model)

    @property
    def mode_no(self):
        return self._mode_no

    @mode_no.setter
    def mode_no(self, mode_no):
        if int(mode_no) != self._mode_no:
            self._mode_no = int(mode_no)
            self.reset_seed(self._seed)

    @property
    def zero_var(self):
        return bool(np.isclose(self.model.var, 0))

    @property
    def value_type(self):
        return self._value_type

    @property
    def name(self):
        return self.__class__.__name__

    @property
    def cov_samples(self):
        return self._cov_sample

    @property
    def z_1(self):
        return self._z_1

    @property
    def z_2(self):
        return self._z_2

    def __repr__(self):
        return (f"{self.name}(model={self.model}, mode_no={self._mode_no}, "
                f"seed={self.seed})")


class IncomprRandMeth(RandMeth):
    """Randomization method for incompressible vector fields (2-D / 3-D).

    ``u_i(x) = mean_u delta_i1 + mean_u sqrt(var / N) sum_j p_i(k_j)
    (Z1_j cos(<k_j, x>) + Z2_j sin(<k_j, x>))`` with the projector
    ``p(k) = e_1 - k k_1 / |k|^2``.
    """

    def __init__(self, model, *, mean_velocity=1.0, mode_no=1000, seed=None,
                 sampling="auto", precision=None, **kwargs):
        if model.dim < 2 or model.dim > 3:
            raise ValueError(
                "Only 2D and 3D incompressible fields can be generated.")
        super().__init__(model=model, mode_no=mode_no, seed=seed,
                         sampling=sampling, precision=precision, **kwargs)
        self.mean_u = mean_velocity
        self._value_type = "vector"

    def _unit_vector(self, ndim):
        shape = np.ones(ndim, dtype=int)
        shape[0] = self.model.dim
        e1 = np.zeros(shape)
        e1[0] = 1.0
        return e1

    def __call__(self, pos, add_nugget=True):
        pos = np.asarray(pos, dtype=np.double)
        nugget = self.get_nugget(pos.shape) if add_nugget else 0.0
        e1 = self._unit_vector(pos.ndim)
        if self.zero_var:
            return self.mean_u * e1 + nugget
        summed = summate_incompr(self._cov_sample, self._z_1, self._z_2, pos,
                                 config.NUM_THREADS, precision=self.precision)
        return (self.mean_u * e1
                + self.mean_u * np.sqrt(self.model.var / self._mode_no) * summed
                + nugget)

    def structured(self, axes, add_nugget=True, out_dtype=None):
        axes = [np.asarray(a, dtype=np.double).reshape(-1) for a in axes]
        shape = (self.model.dim,) + tuple(len(a) for a in axes)
        nugget = self.get_nugget(shape) if add_nugget else 0.0
        e1 = self._unit_vector(len(shape))
        if self.zero_var:
            return self.mean_u * e1 + nugget
        scale = float(self.mean_u * np.sqrt(self.model.var / self._mode_no))
        if self.precision == "mixed" and self.model.dim in (2, 3):
            # tensor-core path: phases from M^T k, projector from k
            cov = self.model.isometrize_matrix.T @ self._cov_sample
            summed = summate_incompr_grid(
                cov, self._z_1, self._z_2, axes, precision="mixed",
                out_dtype=out_dtype, scale=scale, method="tensor",
                proj_cov=self._cov_sample)
            return self.mean_u * e1 + summed + nugget
        if self.model.is_isotropic:
            summed = summate_incompr_grid(
                self._cov_sample, self._z_1, self._z_2, axes,
                precision=self.precision, out_dtype=out_dtype, scale=scale,
                method="pointwise")
            return self.mean_u * e1 + summed + nugget
        # The projector needs the unmapped wave vectors: evaluate pointwise on
        # the isometrized grid.
        from .geometric import generate_grid

        iso = self.model.isometrize(generate_grid(axes))
        summed = summate_incompr(self._cov_sample, self._z_1, self._z_2, iso,
                                 precision=self.precision)
        return (self.mean_u * e1 + scale * np.reshape(summed, shape) + nugget)


class Fourier:
    """Fourier method for periodic random fields (generator.py:595-919).

    ``u(x) = sum_i sqrt(2 S(k_i) dk) (Z1_i cos(<k_i, x>) + Z2_i sin(<k_i, x>))``
    on the equidistant wave-vector grid ``k`` of ``mode_no`` points per
    dimension with spacing ``dk = 2 pi / period * (1, anis)``.  Same
    constructor, ``update`` / ``reset_seed`` semantics and random streams as
    the reference, so the same seed gives the same ``z_1``, ``z_2`` and
    spectrum factors.  ``__call__`` sums with the FP64 ``summate_fourier``
    kernel; ``structured(axes)`` evaluates grids without the meshgrid (FP64
    kernel on the isometrized points, or the tensor-core grid path for
    ``precision="mixed"`` on 2-D / 3-D grids).
    """

    def __init__(self, model, period, mode_no=32, seed=None, precision=None,
                 **kwargs):
        if kwargs:
            warnings.warn("gstools_gb300.Fourier: **kwargs are ignored")
        self._modes = None
        self._period = None
        self._mode_no = None
        self._delta_k = None
        self._model = None
        self._seed = None
        self._rng = None
        self._z_1 = None
        self._z_2 = None
        self._spectrum_factor = None
        self._value_type = "scalar"
        self.precision = config.check_precision(precision)
        self.update(model, seed, period, mode_no)

    # -- evaluation --------------------------------------------------------
    def __call__(self, pos, add_nugget=True):
        """Field at the (already isometrized) positions ``pos`` (:657-688)."""
        pos = np.asarray(pos, dtype=np.double)
        if self.zero_var:
            shp = pos.shape[1:]
            return self.get_nugget(shp) if add_nugget else np.full(shp, 0.0)
        summed = summate_fourier(self._spectrum_factor, self._modes, self._z_1,
                                 self._z_2, pos, config.NUM_THREADS)
        nugget = self.get_nugget(summed.shape) if add_nugget else 0.0
        return summed + nugget

    def structured(self, axes, add_nugget=True, out_dtype=None):
        """Field on the structured grid spanned by ``axes`` (physical
        coordinates, "ij" order)."""
        axes = [np.asarray(a, dtype=np.double).reshape(-1) for a in axes]
        shape = tuple(len(a) for a in axes)
        if self.zero_var:
            return self.get_nugget(shape) if add_nugget else np.full(shape, 0.0)
        m = self.model.isometrize_matrix
        if self.precision == "mixed" and len(axes) in (2, 3):
            field = summate_fourier_grid(self._spectrum_factor,
                                         m.T @ self._modes, self._z_1,
                                         self._z_2, axes, out_dtype=out_dtype)
        else:
            iso = m @ generate_grid(axes)
            field = summate_fourier(self._spectrum_factor, self._modes,
                                    self._z_1, self._z_2, iso).reshape(shape)
        if add_nugget and self.model.nugget > 0:
            field = field + self.get_nugget(shape)
        return field

    def get_nugget(self, shape):
        """Normal nugget noise (:690-711)."""
        if self.model.nugget > 0:
            return np.sqrt(self.model.nugget) * self._rng.random.normal(
                size=shape)
        return np.full(shape, 0.0) if self.zero_var else 0.0

    # -- state -------------------------------------------------------------
    def update(self, model=None, seed=np.nan, period=None, mode_no=None):
        """Update model, seed, period and/or mode numbers (:713-797)."""
        tmp_model = model if model is not None else self._model
        dim = tmp_model.dim
        if period is not None:
            self._period = self._fill_to_dim(period, dim)
            anis = np.insert(tmp_model.anis.copy(), 0, 1.0)
            self._delta_k = 2.0 * np.pi / self._period * anis
            if mode_no is None:
                self._set_modes(self._mode_no, dim)
        if mode_no is not None:
            mode_no = self._fill_to_dim(mode_no, dim)
            if (np.asarray([m % 2 for m in mode_no]) != 0).any():
                raise ValueError("Fourier: Odd mode_no not supported.")
            self._set_modes(mode_no, dim)

        if isinstance(model, CovModel):
            if self.model != model:
                self._model = deepcopy(model)
                if seed is None or not np.isnan(seed):
                    self.reset_seed(seed)
                else:
                    self.reset_seed(self._seed)
            elif seed is None or not np.isnan(seed):
                self.seed = seed
        elif model is None and (seed is None or not np.isnan(seed)):
            if isinstance(self._model, CovModel):
                self.seed = seed
            else:
                raise ValueError("gstools_gb300.Fourier: no 'model' given")
        elif mode_no is not None or period is not None:
            if seed is None or not np.isnan(seed):
                self.reset_seed(seed)
            else:
                self.reset_seed(self._seed)
        elif model is None and np.isnan(seed):
            if (isinstance(self._model, CovModel) and self._z_1 is not None
                    and self._z_2 is not None
                    and self._spectrum_factor is not None):
                raise ValueError("gstools_gb300.Fourier: neither 'model' nor "
                                 "'seed' given!")
        else:
            raise ValueError("gstools_gb300.Fourier: 'model' is not a "
                             "CovModel")

    def reset_seed(self, seed=np.nan):
        """Redraw the amplitudes and the spectrum factors (:799-828)."""
        if seed is None or not np.isnan(seed):
            self._seed = seed
        self._rng = RNG(self._seed)
        n = int(np.prod(self._mode_no))
        self._z_1 = self._rng.random.normal(size=n)
        self._z_2 = self._rng.random.normal(size=n)
        if self.zero_var:
            self._spectrum_factor = np.full(n, 0.0)
        else:
            k_norm = np.linalg.norm(self._modes, axis=0)
            self._spectrum_factor = np.sqrt(
                self._model.spectrum(k_norm) * np.prod(self._delta_k))

    @staticmethod
    def _fill_to_dim(values, dim, dtype=float, default_value=None):
        """Pad ``values`` with its last entry to length ``dim`` (:830-845)."""
        r = np.atleast_1d(values)
        if values is None:
            if default_value is None:
                raise ValueError("Fourier: Value has to be provided")
            r = default_value
        r = np.atleast_1d(np.array(r, dtype=dtype))[:dim]
        if len(r) < dim:
            r = np.pad(r, (0, dim - len(r)), "edge")
        return r

    def _set_modes(self, mode_no, dim):
        """Equidistant wave-vector grid (:847-870)."""
        modes = [np.arange(-mode_no[d] / 2.0 * self._delta_k[d],
                           mode_no[d] / 2.0 * self._delta_k[d],
                           self._delta_k[d]) for d in range(dim)]
        self._modes = generate_grid(modes)
        self._mode_no = [len(m) for m in modes]

    # -- properties ----------------------------------------------------------
    @property
    def seed(self):
        return self._seed

    @seed.setter
    def seed(self, new_seed):
        if new_seed is not self._seed:
            self.reset_seed(new_seed)

    @property
    def model(self):
        return self._model

    @model.setter
    def model(self, model):
        self.update(model)

    @property
    def modes(self):
        return self._modes

    @property
    def mode_no(self):
        return self._mode_no

    @mode_no.setter
    def mode_no(self, mode_no):
        self.update(mode_no=mode_no)

    @property
    def period(self):
        return self._period

    @period.setter
    def period(self, period):
        self.update(period=period)

    @property
    def spectrum_factor(self):
        return self._spectrum_factor

    @property
    def z_1(self):
        return self._z_1

    @property
    def z_2(self):
        return self._z_2

    @property
    def zero_var(self):
        return bool(np.isclose(self.model.var, 0))

    @property
    def value_type(self):
        return self._value_type

    @property
    def name(self):
        return self.__class__.__name__

    def __repr__(self):
        return f"{self.name}(model={self.model}, seed={self.seed})"
