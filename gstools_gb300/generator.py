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
from .summator import summate, summate_grid, summate_incompr, summate_incompr_grid

__all__ = ["RandMeth", "IncomprRandMeth"]

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
