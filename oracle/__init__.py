"""FP64 CPU oracle for the randomization-method summation.

TEST INFRASTRUCTURE ONLY.  This package is the checker: tests/, the smoke
check in __graft_entry__ and the CPU-baseline leg of bench.py import it.  The
gstools_gb300 product never imports it, and the product path has no CPU
fallback that could route here.

Two independent restatements of the reference formulas
(src/gstools/field/generator.py:193-199 for ``summate``, :479-495 for
``summate_incompr``, :682-689 for ``summate_fourier``):

* ``c_summate`` / ``c_summate_incompr`` / ``c_summate_fourier``: the C/OpenMP
  library built from ``summate_oracle.c`` (the primary oracle and the timed CPU
  baseline);
* ``np_summate`` / ``np_summate_incompr`` / ``np_summate_fourier``: a chunked
  numpy witness used to cross-check the C oracle;
* ``c_krige`` / ``np_krige``: the kriging kernels of gstools-cython
  (``krige_oracle.c``) and a numpy witness;
* ``c_vario_unstructured`` / ``c_vario_directional`` / ``c_vario_structured``:
  the variogram estimators of gstools-cython (``vario_oracle.c``);
* ``c_sample_modes`` / ``c_philox4x64``: the C restatement of the device
  spectral sampler (``sample_oracle.c``), its Philox stream pinned to numpy's
  Philox bit generator by the tests.
"""

from .oracle import (  # noqa: F401
    MODEL_KINDS,
    build,
    c_krige,
    c_philox4x64,
    c_sample_modes,
    c_summate,
    c_summate_fourier,
    c_summate_incompr,
    c_vario_directional,
    c_vario_structured,
    c_vario_unstructured,
    library_path,
    num_threads,
    np_krige,
    np_summate,
    np_summate_fourier,
    np_summate_incompr,
)
