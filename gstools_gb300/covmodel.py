"""Covariance models as far as the randomization method needs them.

The randomization method consumes a model through four things: its
variance / nugget, the isometrize map applied to positions
(src/gstools/covmodel/base.py:572-582), the rescaled length scale
(base.py:985-988) and the radial law of the wave numbers, i.e. the spectral
density S(k) turned into a radial pdf (covmodel/tools.py:374-405) with an
optional cdf / ppf (base.py:1054-1077).  This module implements exactly those
for the models of the hot path:

* ``Gaussian``    -- models.py:118-190 (rescale sqrt(pi)/2; cdf 1-3 D,
  ppf 1-2 D)
* ``Exponential`` -- models.py:192-273 (cdf 1-3 D, ppf 1-2 D)
* ``Matern``      -- models.py:351-458 (density only)

Where the reference has no ppf it samples radii by MCMC (emcee,
random/rng.py:38-104), which is not part of this package.  Instead each
model offers an exact analytic sampler of its spectral law, derived from the
densities above:

* Gaussian:    k ~ N(0, (2 / l^2) I)                (radius sqrt(2)/l * chi_d)
* Exponential: k ~ multivariate t, 1 dof, scale 1/l
* Matern nu:   k ~ multivariate t, 2 nu dof, scale 1/(sqrt(2) l)

(l = len_rescaled).  Fitting, plotting, spatio-temporal and lat/lon models
are outside the summation path and are not provided.
"""

import numpy as np
import scipy.special as sps

from .geometric import matrix_isometrize, no_of_angles, set_angles, set_anis

__all__ = ["CovModel", "Gaussian", "Exponential", "Matern", "rad_fac"]


def rad_fac(dim, r):
    """Surface factor of the radial integral in ``dim`` dimensions."""
    if dim == 1:
        return 2.0
    if dim == 2:
        return 2 * np.pi * r
    if dim == 3:
        return 4 * np.pi * r**2
    return dim * r ** (dim - 1) * np.sqrt(np.pi) ** dim / sps.gamma(dim / 2 + 1)


def _set_len_anis(dim, len_scale, anis):
    """Main length scale and anisotropies (covmodel/tools.py:186-245)."""
    ls = np.atleast_1d(np.array(len_scale, dtype=np.double))[:dim]
    main = ls[0]
    if len(ls) == 1:
        out_anis = set_anis(dim, anis)
    else:
        if len(ls) < dim:
            ls = np.pad(ls, (0, dim - len(ls)), "edge")
        out_anis = ls[1:] / ls[0]
    if np.any(~(out_anis > 0.0)):
        raise ValueError(f"anisotropy-ratios needs to be > 0, got: {out_anis}")
    return float(main), np.asarray(out_anis, dtype=np.double)


class CovModel:
    """Base class: variance, length scale, anisotropy and rotation."""

    def __init__(self, dim=3, var=1.0, len_scale=1.0, nugget=0.0, anis=1.0,
                 angles=0.0, rescale=None, **opt_arg):
        if int(dim) < 1:
            raise ValueError("dim must be >= 1")
        self._dim = int(dim)
        self._opt = dict(self.default_opt_arg())
        unknown = set(opt_arg) - set(self._opt)
        if unknown:
            raise ValueError(f"{self.name}: unknown arguments {sorted(unknown)}")
        self._opt.update({k: float(v) for k, v in opt_arg.items()})
        self.var = var
        self.nugget = nugget
        self._len_scale, self._anis = _set_len_anis(self._dim, len_scale, anis)
        self._angles = set_angles(self._dim, angles)
        self.rescale = rescale

    # -- parameters ---------------------------------------------------
    def default_opt_arg(self):
        return {}

    def default_rescale(self):
        return 1.0

    def __getattr__(self, name):
        opt = self.__dict__.get("_opt", {})
        if name in opt:
            return opt[name]
        raise AttributeError(name)

    @property
    def name(self):
        return self.__class__.__name__

    @property
    def dim(self):
        return self._dim

    @dim.setter
    def dim(self, dim):
        self._dim = int(dim)
        self._len_scale, self._anis = _set_len_anis(self._dim, self._len_scale,
                                                    self._anis)
        self._angles = set_angles(self._dim, self._angles)

    @property
    def var(self):
        return self._var

    @var.setter
    def var(self, var):
        self._var = float(var)

    @property
    def nugget(self):
        return self._nugget

    @nugget.setter
    def nugget(self, nugget):
        self._nugget = float(nugget)

    @property
    def sill(self):
        return self.var + self.nugget

    @property
    def len_scale(self):
        return self._len_scale

    @len_scale.setter
    def len_scale(self, len_scale):
        self._len_scale, self._anis = _set_len_anis(self._dim, len_scale,
                                                    self._anis)

    @property
    def anis(self):
        return self._anis

    @anis.setter
    def anis(self, anis):
        self._len_scale, self._anis = _set_len_anis(self._dim, self._len_scale,
                                                    anis)

    @property
    def angles(self):
        return self._angles

    @angles.setter
    def angles(self, angles):
        self._angles = set_angles(self._dim, angles)

    @property
    def rescale(self):
        return self._rescale

    @rescale.setter
    def rescale(self, rescale):
        rescale = self.default_rescale() if rescale is None else rescale
        self._rescale = abs(float(rescale))

    @property
    def len_rescaled(self):
        """Length scale divided by the rescale factor (base.py:985-988)."""
        return self.len_scale / self.rescale

    def __eq__(self, other):
        if not isinstance(other, CovModel) or type(self) is not type(other):
            return False
        return (self.dim == other.dim
                and np.isclose(self.var, other.var)
                and np.isclose(self.nugget, other.nugget)
                and np.isclose(self.len_scale, other.len_scale)
                and np.allclose(self.anis, other.anis)
                and np.allclose(self.angles, other.angles)
                and np.isclose(self.rescale, other.rescale)
                and self._opt.keys() == other._opt.keys()
                and all(np.isclose(self._opt[k], other._opt[k])
                        for k in self._opt))

    def __ne__(self, other):
        return not self.__eq__(other)

    __hash__ = None

    # -- geometry ----------------------------------------------------------
    @property
    def isometrize_matrix(self):
        """The linear map M of ``isometrize``: derotate, then stretch."""
        return matrix_isometrize(self.dim, self.angles, self.anis)

    def isometrize(self, pos):
        """Positions in the isotropic frame: ``M @ pos`` (base.py:572-582)."""
        pos = np.asarray(pos, dtype=np.double).reshape((self.dim, -1))
        return np.dot(self.isometrize_matrix, pos)

    @property
    def is_isotropic(self):
        return (np.allclose(self.anis, 1.0)
                and np.allclose(self.angles, 0.0))

    # -- spectral law --------------------------------------------------------
    def spectral_density(self, k):  # pragma: no cover - abstract
        raise NotImplementedError

    def spectrum(self, k):
        """Spectrum ``var * spectral_density(k)`` (covmodel/base.py:511-533)."""
        return self.spectral_density(k) * self.var

    def spectral_rad_pdf(self, r):
        """Radial spectral pdf (covmodel/tools.py:374-405)."""
        r = np.asarray(np.abs(r), dtype=np.double)
        if self.dim > 1:
            pos = np.logical_not(np.isclose(r, 0))
            res = np.zeros_like(r, dtype=np.double)
            res[pos] = rad_fac(self.dim, r[pos]) * np.abs(
                self.spectral_density(r[pos]))
        else:
            res = rad_fac(self.dim, r) * np.abs(self.spectral_density(r))
        res = np.atleast_1d(res)
        res[np.logical_not(np.isfinite(res))] = 0.0
        return np.maximum(res, 0.0)

    def ln_spectral_rad_pdf(self, r):
        with np.errstate(divide="ignore"):
            return np.log(self.spectral_rad_pdf(r))

    def _has_cdf(self):
        return hasattr(self, "spectral_rad_cdf")

    def _has_ppf(self):
        return hasattr(self, "spectral_rad_ppf")

    @property
    def has_cdf(self):
        return self._has_cdf()

    @property
    def has_ppf(self):
        return self._has_ppf()

    @property
    def dist_func(self):
        """pdf, cdf and ppf of the radial law (cdf/ppf may be None)."""
        cdf = self.spectral_rad_cdf if self.has_cdf else None
        ppf = self.spectral_rad_ppf if self.has_ppf else None
        return self.spectral_rad_pdf, cdf, ppf

    def sample_radius(self, random_state, size):
        """Exact analytic draw of ``size`` wave-number radii."""
        raise NotImplementedError(f"{self.name}: no analytic radial sampler")

    def __repr__(self):
        opt = "".join(f", {k}={v:.4g}" for k, v in self._opt.items())
        return (f"{self.name}(dim={self.dim}, var={self.var:.4g}, "
                f"len_scale={self.len_scale:.4g}, nugget={self.nugget:.4g}, "
                f"anis={list(self.anis)}, angles={list(self.angles)}{opt})")


def _chi(random_state, dof, size):
    """Norm of a ``dof``-dimensional standard normal vector."""
    return np.sqrt(random_state.chisquare(dof, size))


class Gaussian(CovModel):
    """Gaussian model, cor(h) = exp(-h^2) (models.py:118-190)."""

    def default_rescale(self):
        return np.sqrt(np.pi) / 2.0

    def spectral_density(self, k):
        k = np.asarray(k, dtype=np.double)
        ls = self.len_rescaled
        return (ls / 2.0 / np.sqrt(np.pi)) ** self.dim * np.exp(
            -((k * ls / 2.0) ** 2))

    def spectral_rad_cdf(self, r):
        r = np.asarray(r, dtype=np.double)
        ls = self.len_rescaled
        if self.dim == 1:
            return sps.erf(r * ls / 2.0)
        if self.dim == 2:
            return 1.0 - np.exp(-((r * ls / 2.0) ** 2))
        if self.dim == 3:
            return sps.erf(r * ls / 2.0) - r * ls / np.sqrt(np.pi) * np.exp(
                -((r * ls / 2.0) ** 2))
        return None

    def spectral_rad_ppf(self, u):
        u = np.asarray(u, dtype=np.double)
        if self.dim == 1:
            return 2.0 / self.len_rescaled * sps.erfinv(u)
        if self.dim == 2:
            return 2.0 / self.len_rescaled * np.sqrt(-np.log(1.0 - u))
        return None

    def _has_cdf(self):
        return self.dim in (1, 2, 3)

    def _has_ppf(self):
        return self.dim in (1, 2)

    def sample_radius(self, random_state, size):
        return np.sqrt(2.0) / self.len_rescaled * _chi(random_state, self.dim,
                                                       size)


class Exponential(CovModel):
    """Exponential model, cor(h) = exp(-h) (models.py:192-273)."""

    def spectral_density(self, k):
        k = np.asarray(k, dtype=np.double)
        ls = self.len_rescaled
        return (ls**self.dim * sps.gamma((self.dim + 1) / 2.0)
                / (np.pi * (1.0 + (k * ls) ** 2)) ** ((self.dim + 1) / 2.0))

    def spectral_rad_cdf(self, r):
        r = np.asarray(r, dtype=np.double)
        ls = self.len_rescaled
        if self.dim == 1:
            return np.arctan(r * ls) * 2.0 / np.pi
        if self.dim == 2:
            return 1.0 - 1.0 / np.sqrt(1.0 + (r * ls) ** 2)
        if self.dim == 3:
            return (np.arctan(r * ls) - r * ls / (1.0 + (r * ls) ** 2)) \
                * 2.0 / np.pi
        return None

    def spectral_rad_ppf(self, u):
        u = np.asarray(u, dtype=np.double)
        if self.dim == 1:
            return np.tan(np.pi / 2 * u) / self.len_rescaled
        if self.dim == 2:
            u_power = np.divide(1, u**2, out=np.full_like(u, np.inf),
                                where=np.logical_not(np.isclose(u, 0)))
            return np.sqrt(u_power - 1.0) / self.len_rescaled
        return None

    def _has_cdf(self):
        return self.dim in (1, 2, 3)

    def _has_ppf(self):
        return self.dim in (1, 2)

    def sample_radius(self, random_state, size):
        g = _chi(random_state, self.dim, size)
        t = np.abs(random_state.standard_normal(size))
        return g / t / self.len_rescaled


class Matern(CovModel):
    """Matern model with shape ``nu`` (models.py:351-458)."""

    def default_opt_arg(self):
        return {"nu": 1.0}

    def spectral_density(self, k):
        k = np.asarray(k, dtype=np.double)
        ls = self.len_rescaled
        x = (k * ls) ** 2
        nu = self.nu
        if nu > 20.0:
            return ((ls / np.sqrt(np.pi)) ** self.dim * np.exp(-x)
                    * (1 + 0.5 * x**2 / nu) * np.sqrt(1 + x / nu) ** (-self.dim))
        return (ls / np.sqrt(np.pi)) ** self.dim * np.exp(
            -(nu + self.dim / 2.0) * np.log(1.0 + x / nu)
            + sps.loggamma(nu + self.dim / 2.0)
            - sps.loggamma(nu)
            - self.dim * np.log(np.sqrt(nu)))

    def sample_radius(self, random_state, size):
        if self.nu > 20.0:
            raise NotImplementedError(
                "Matern nu > 20 uses the reference's Gaussian-limit density; "
                "use sampling='inversion'")
        dof = 2.0 * self.nu
        g = _chi(random_state, self.dim, size)
        w = np.sqrt(random_state.chisquare(dof, size) / dof)
        return g / w / (np.sqrt(2.0) * self.len_rescaled)
