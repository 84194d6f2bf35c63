"""The drop-in hook into an unmodified GSTools (CPU side).

``gstools_gb300.install()`` must rebind the three module globals the
reference resolves at call time (src/gstools/field/generator.py:42-75,
266, 554, 682) and ``uninstall()`` must restore them.  Without a GPU the
installed summators must raise instead of falling back to a CPU path.
"""

import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import reference_import  # noqa: E402

import gstools_gb300 as gg  # noqa: E402


@pytest.fixture(scope="module")
def gen_module():
    if not reference_import.available():
        pytest.skip("reference tree not present")
    gs = reference_import.import_gstools()
    import gstools.field.generator as gen

    assert gs is not None
    return gen


def test_install_rebinds_and_uninstall_restores(gen_module):
    before = {n: getattr(gen_module, n) for n in
              ("_summate", "_summate_incompr", "_summate_fourier")}
    gg.install(gen_module)
    try:
        for name, fct in before.items():
            assert getattr(gen_module, name) is not fct
            assert getattr(gen_module, name).__module__ == "gstools_gb300.hook"
    finally:
        gg.uninstall(gen_module)
    for name, fct in before.items():
        assert getattr(gen_module, name) is fct


def test_installed_srf_has_no_cpu_fallback(gen_module):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    import gstools

    gg.install(gen_module)
    try:
        srf = gstools.SRF(gstools.Gaussian(dim=2, var=1.0, len_scale=4.0),
                          mode_no=50)
        with pytest.raises(RuntimeError):
            srf((np.arange(5.0), np.arange(5.0)), seed=3)
    finally:
        gg.uninstall(gen_module)


def test_install_rejects_unknown_precision(gen_module):
    with pytest.raises(ValueError):
        gg.install(gen_module, precision="fp16")
