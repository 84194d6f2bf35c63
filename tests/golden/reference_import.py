"""Import the reference GSTools Python package with stand-ins for its
missing third-party modules.

Used only where the reference tree is present (fixture generation and the
CPU-side drop-in test); nothing in the GPU tests, the smoke check or the
benchmark imports this.

The reference's summation kernels live in the external ``gstools_cython``
package (src/gstools/field/generator.py:22-24), which is absent.  The
stand-in ``gstools_cython.field`` routes to the FP64 C oracle so that the
reference's own RNG, covariance models and SRF/RandMeth code drive the oracle.
``emcee`` (MCMC sampling, src/gstools/random/rng.py:12-15), ``hankel``,
``meshio`` and ``pyevtk`` are absent too; their stand-ins raise if used.
"""

import os
import sys
import types

REFERENCE_SRC = os.environ.get(
    "GSTOOLS_REFERENCE_SRC", "/root/reference/src"
)


def available():
    """Whether the reference tree can be imported on this machine."""
    return os.path.isdir(os.path.join(REFERENCE_SRC, "gstools"))


def _unavailable(name):
    def fct(*args, **kwargs):
        raise NotImplementedError(f"{name} is not available here")

    return fct


def _install_stubs():
    import oracle

    if "gstools_cython" not in sys.modules:
        pkg = types.ModuleType("gstools_cython")
        field = types.ModuleType("gstools_cython.field")
        field.summate = lambda c, z1, z2, p, num_threads=None: (
            oracle.c_summate(c, z1, z2, p)
        )
        field.summate_incompr = lambda c, z1, z2, p, num_threads=None: (
            oracle.c_summate_incompr(c, z1, z2, p)
        )
        field.summate_fourier = lambda f, m, z1, z2, p, num_threads=None: (
            oracle.c_summate_fourier(f, m, z1, z2, p)
        )
        vario = types.ModuleType("gstools_cython.variogram")
        for name in ("directional", "ma_structured", "structured",
                     "unstructured"):
            setattr(vario, name, _unavailable(f"variogram.{name}"))
        krige = types.ModuleType("gstools_cython.krige")
        krige.calc_field_krige = lambda m, v, c, num_threads=None: (
            oracle.c_krige(m, v, c, with_error=False)
        )
        krige.calc_field_krige_and_variance = (
            lambda m, v, c, num_threads=None: oracle.c_krige(m, v, c)
        )
        pkg.field, pkg.variogram, pkg.krige = field, vario, krige
        sys.modules.update({
            "gstools_cython": pkg,
            "gstools_cython.field": field,
            "gstools_cython.variogram": vario,
            "gstools_cython.krige": krige,
        })
    if "emcee" not in sys.modules:
        emcee = types.ModuleType("emcee")
        state = types.ModuleType("emcee.state")

        class _Missing:
            def __init__(self, *args, **kwargs):
                raise NotImplementedError(
                    "emcee is not available: MCMC spectral sampling cannot "
                    "run here; use sampling='inversion'"
                )

        emcee.EnsembleSampler = _Missing
        state.State = _Missing
        emcee.state = state
        sys.modules.update({"emcee": emcee, "emcee.state": state})
    if "hankel" not in sys.modules:
        hankel = types.ModuleType("hankel")

        class SymmetricFourierTransform:
            def __init__(self, *args, **kwargs):
                pass

            def transform(self, *args, **kwargs):
                raise NotImplementedError("hankel is not available here")

        hankel.SymmetricFourierTransform = SymmetricFourierTransform
        sys.modules["hankel"] = hankel
    if "meshio" not in sys.modules:
        sys.modules["meshio"] = types.ModuleType("meshio")
    if "pyevtk" not in sys.modules:
        pyevtk = types.ModuleType("pyevtk")
        hl = types.ModuleType("pyevtk.hl")
        hl.gridToVTK = _unavailable("pyevtk.gridToVTK")
        hl.pointsToVTK = _unavailable("pyevtk.pointsToVTK")
        pyevtk.hl = hl
        sys.modules.update({"pyevtk": pyevtk, "pyevtk.hl": hl})


def import_gstools():
    """Import and return the reference ``gstools`` package."""
    if not available():
        raise ImportError("reference GSTools tree not found")
    sys.dont_write_bytecode = True
    _install_stubs()
    if REFERENCE_SRC not in sys.path:
        sys.path.insert(0, REFERENCE_SRC)
    import gstools

    return gstools
