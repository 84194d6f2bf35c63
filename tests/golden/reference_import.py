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

import numpy as np
import sys
import types

# The reference's ``src`` directory: $GSTOOLS_REFERENCE_SRC, else a checkout
# named ``reference`` beside this repository.
_REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REFERENCE_SRC = os.environ.get(
    "GSTOOLS_REFERENCE_SRC",
    os.path.join(os.path.dirname(_REPO), "reference", "src"),
)


REF_TESTS = os.path.join(os.path.dirname(REFERENCE_SRC), "tests")


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
        vario.unstructured = oracle.c_vario_unstructured
        vario.directional = oracle.c_vario_directional
        vario.structured = (lambda f, estimator_type="m", num_threads=None:
                            oracle.c_vario_structured(f, estimator_type))
        vario.ma_structured = (
            lambda f, mask, estimator_type="m", num_threads=None:
            oracle.c_vario_structured(f, estimator_type, mask=mask))
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
        # emcee is absent: a small stand-in with the same interface and the
        # affine-invariant stretch move (Goodman and Weare, Comm. App. Math.
        # Comp. Sci. 5(1), 2010), so the reference's MCMC radius sampling
        # (src/gstools/random/rng.py:38-103) runs.  Its random stream is not
        # emcee's: samples follow the right law, but literal values drawn
        # through MCMC differ from the reference's.
        emcee = types.ModuleType("emcee")
        state = types.ModuleType("emcee.state")

        class State:
            def __init__(self, coords, copy=False):
                src = coords.coords if isinstance(coords, State) else coords
                self.coords = np.array(src, dtype=float, copy=True)
                self.random_state = getattr(coords, "random_state", None)

        class EnsembleSampler:
            def __init__(self, nwalkers, ndim, log_prob_fn, vectorize=False,
                         a=2.0):
                self.nwalkers, self.ndim, self.a = nwalkers, ndim, a
                self.log_prob = log_prob_fn
                self.vectorize = vectorize
                self._chain = []

            def _lp(self, x):
                if self.vectorize:
                    return np.asarray(self.log_prob(x), dtype=float).reshape(-1)
                return np.array([self.log_prob(v) for v in x], dtype=float)

            def run_mcmc(self, initial_state, nsteps, **kwargs):
                st = initial_state if isinstance(initial_state, State) else \
                    State(initial_state)
                rng = np.random.RandomState()
                if st.random_state is not None:
                    rng.set_state(st.random_state)
                x = st.coords.reshape(self.nwalkers, self.ndim).copy()
                lp = self._lp(x)
                half = self.nwalkers // 2
                groups = (np.arange(half), np.arange(half, self.nwalkers))
                for _ in range(int(nsteps)):
                    for g in (0, 1):
                        s_idx, c_idx = groups[g], groups[1 - g]
                        z = ((self.a - 1.0) * rng.rand(len(s_idx)) + 1.0) ** 2 / self.a
                        c = x[c_idx[rng.randint(len(c_idx), size=len(s_idx))]]
                        prop = c + z[:, None] * (x[s_idx] - c)
                        lp_new = self._lp(prop)
                        ln_ratio = (self.ndim - 1.0) * np.log(z) + lp_new - lp[s_idx]
                        acc = np.log(rng.rand(len(s_idx))) < ln_ratio
                        x[s_idx[acc]] = prop[acc]
                        lp[s_idx[acc]] = lp_new[acc]
                    self._chain.append(x.copy())
                out = State(x)
                out.random_state = rng.get_state()
                return out

            def reset(self):
                self._chain = []

            def get_chain(self, flat=False, **kwargs):
                chain = np.array(self._chain)
                return chain.reshape(-1, self.ndim) if flat else chain

        emcee.EnsembleSampler = EnsembleSampler
        state.State = State
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
