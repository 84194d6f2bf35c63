"""Coordinate maps of the hot path (host side, FP64 numpy).

Same conventions as the reference's src/gstools/tools/geometric.py:
rotation planes and Givens rotations (:141-182), derotation with alternating
Tait-Bryan signs (:208-234), the isotropifying stretch diag(1, 1/anis)
(:237-254), their product ``matrix_isometrize`` (:275-294) and the "ij"
meshgrid of ``generate_grid`` (:340-356).  The grid kernels never call
``generate_grid``; they take the axis arrays directly.
"""

import numpy as np

__all__ = [
    "no_of_angles",
    "set_angles",
    "set_anis",
    "rotation_planes",
    "givens_rotation",
    "matrix_rotate",
    "matrix_derotate",
    "matrix_isotropify",
    "matrix_isometrize",
    "generate_grid",
]


def no_of_angles(dim):
    """Number of rotation angles in ``dim`` dimensions."""
    return (dim * (dim - 1)) // 2


def set_angles(dim, angles):
    """Angles cut or zero-padded to ``no_of_angles(dim)`` values."""
    out = np.atleast_1d(np.asarray(angles, dtype=np.double))[: no_of_angles(dim)]
    return np.pad(out, (0, no_of_angles(dim) - len(out)), "constant",
                  constant_values=0.0)


def set_anis(dim, anis):
    """Anisotropy ratios cut or front-padded with ones to ``dim - 1`` values."""
    out = np.atleast_1d(np.asarray(anis, dtype=np.double))[: dim - 1]
    if len(out) < dim - 1:
        out = np.pad(out, (dim - len(out) - 1, 0), "constant",
                     constant_values=1.0)
    return out


def rotation_planes(dim):
    """All coordinate planes (i, j), i < j, ordered by j then i."""
    return [(i, j) for j in range(1, dim) for i in range(j)]


def givens_rotation(dim, plane, angle):
    """Rotation by ``angle`` in the coordinate plane ``plane``."""
    rot = np.eye(dim, dtype=np.double)
    c, s = np.cos(angle), np.sin(angle)
    rot[plane[0], plane[0]] = c
    rot[plane[1], plane[1]] = c
    rot[plane[0], plane[1]] = -s
    rot[plane[1], plane[0]] = s
    return rot


def matrix_rotate(dim, angles):
    """Rotation into the target coordinate system."""
    angles = set_angles(dim, angles)
    res = np.eye(dim, dtype=np.double)
    for i, (ang, plane) in enumerate(zip(angles, rotation_planes(dim))):
        res = np.matmul(givens_rotation(dim, plane, (-1) ** i * ang), res)
    return res


def matrix_derotate(dim, angles):
    """Inverse of :func:`matrix_rotate`."""
    angles = -set_angles(dim, angles)
    res = np.eye(dim, dtype=np.double)
    for i, (ang, plane) in enumerate(zip(angles, rotation_planes(dim))):
        res = np.matmul(res, givens_rotation(dim, plane, (-1) ** i * ang))
    return res


def matrix_isotropify(dim, anis):
    """Stretch diag(1, 1/anis_1, ...)."""
    return np.diag(np.concatenate(([1.0], 1.0 / set_anis(dim, anis))))


def matrix_isometrize(dim, angles, anis):
    """Derotate, then make isotropic: the map applied to positions."""
    return np.matmul(matrix_isotropify(dim, anis), matrix_derotate(dim, angles))


def generate_grid(pos):
    """Materialised "ij" meshgrid of the axis arrays, shape (dim, n)."""
    return np.asarray(np.meshgrid(*pos, indexing="ij"),
                      dtype=np.double).reshape((len(pos), -1))
