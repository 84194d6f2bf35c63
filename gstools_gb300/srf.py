"""Spatial random field front end for the randomization-method generators.

A reduced mirror of the reference's ``SRF`` (src/gstools/field/srf.py:25-186)
and of the position handling of ``Field.pre_pos`` / ``post_field``
(src/gstools/field/base.py:254-349), covering what the summation path needs:
generator selection by name ("RandMeth", "IncomprRandMeth", "VectorField",
"VelocityField", "Fourier") or class, ``update(model, seed)``, isometrized unstructured
positions, structured grids and a constant (scalar or per-component) mean.
Normalizers, trends, upscaling and plotting are not part of this package.

Structured grids never materialise the meshgrid: the generator's
``structured`` method evaluates them from the axis arrays.
"""

import numpy as np

from .generator import Fourier, IncomprRandMeth, RandMeth

__all__ = ["SRF", "GENERATOR"]

GENERATOR = {
    "RandMeth": RandMeth,
    "IncomprRandMeth": IncomprRandMeth,
    "VectorField": IncomprRandMeth,
    "VelocityField": IncomprRandMeth,
    "Fourier": Fourier,
}


class SRF:
    """Spatial random field from a covariance model."""

    def __init__(self, model, mean=0.0, generator="RandMeth",
                 **generator_kwargs):
        self.model = model
        self.mean = mean
        self.field = None
        self.pos = None
        self.mesh_type = None
        gen = GENERATOR[generator] if generator in GENERATOR else generator
        if not (isinstance(gen, type) and issubclass(gen, (RandMeth, Fourier))):
            raise ValueError(f"SRF: unknown or wrong generator: {generator}")
        self.generator = gen(model, **generator_kwargs)
        self.value_type = self.generator.value_type

    def __call__(self, pos=None, seed=np.nan, mesh_type="unstructured",
                 store=True):
        """Generate the field at ``pos`` (a tuple of coordinate arrays)."""
        if pos is None:
            pos, mesh_type = self.pos, self.mesh_type
        if pos is None:
            raise ValueError("SRF: no position tuple 'pos' present")
        self.generator.update(self.model, seed)
        if mesh_type == "structured":
            axes = [np.asarray(a, dtype=np.double).reshape(-1) for a in pos]
            field = self.generator.structured(axes)
        else:
            pts = np.asarray(pos, dtype=np.double).reshape(self.model.dim, -1)
            iso = self.model.isometrize(pts)
            field = self.generator(iso)
        field = self._apply_mean(np.asarray(field))
        if store:
            self.pos, self.mesh_type, self.field = pos, mesh_type, field
        return field

    def structured(self, pos, **kwargs):
        return self(pos, mesh_type="structured", **kwargs)

    def unstructured(self, pos, **kwargs):
        return self(pos, mesh_type="unstructured", **kwargs)

    def _apply_mean(self, field):
        mean = self.mean
        if mean is None:
            return field
        if self.value_type == "vector" and np.size(mean) > 1:
            m = np.asarray(mean, dtype=np.double).reshape(
                (-1,) + (1,) * (field.ndim - 1))
            return field + m
        return field + mean
