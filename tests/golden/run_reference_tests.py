"""Run the reference's own test files with the C oracle as gstools-cython.

Run from the repository root, where the reference tree is available:

    python tests/golden/run_reference_tests.py [test file names ...]

``reference_import`` installs the oracle as ``gstools_cython.field``,
``.krige`` and ``.variogram`` (and stand-ins for the absent emcee, hankel,
meshio, pyevtk); the reference's test files then run unchanged under pytest.
Passing tests pin the oracle's restatement of the absent gstools-cython
kernels to the reference's own assertions.  Tests that need modules absent
here (emcee's MCMC sampler, plotting, VTK export) fail or are skipped and are
reported as such.
"""

import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import pytest  # noqa: E402

from reference_import import REF_TESTS, import_gstools  # noqa: E402

DEFAULT = [
    "test_variogram_unstructured.py", "test_variogram_structured.py",
    "test_krige.py", "test_condition.py", "test_randmeth.py",
    "test_incomprrandmeth.py", "test_fouriergen.py", "test_rng.py",
]


def main(argv):
    """Arguments: reference test file names (default: DEFAULT); anything
    else (``--deselect <node id>`` ...) is passed on to pytest."""
    import_gstools()
    files, extra = [], []
    it = iter(argv)
    for a in it:
        if a.startswith("-"):
            extra.append(a)
            if a in ("--deselect", "-k", "-m"):
                extra.append(next(it))
        else:
            files.append(a)
    paths = [os.path.join(REF_TESTS, f) for f in (files or DEFAULT)]
    return pytest.main(["-q", "-p", "no:cacheprovider", "-o",
                        "python_files=test_*.py", "--rootdir", ROOT, *extra,
                        *paths])


if __name__ == "__main__":
    sys.exit(main(sys.argv[1:]))
