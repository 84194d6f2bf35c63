"""The C-ABI library: it loads and exports every entry point the header
declares.  Only non-compute calls are made here (no GPU needed)."""

import ctypes
import os
import re

import pytest

from gstools_gb300 import _native, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include",
                      "gstools_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gst_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _native.load()


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("gst_summate_f64", "gst_summate_incompr_f64",
                     "gst_summate_mixed", "gst_summate_grid_f64"):
        assert required in names


def test_every_declared_symbol_is_exported(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_binding_table_matches_header():
    assert set(declared_functions()) == set(_native.SIGNATURES)


def test_version_and_status_strings(lib):
    assert lib.gst_version() >= 100
    assert _native.status_string(0) == "ok"
    assert "argument" in _native.status_string(_native.GST_ERR_INVALID_ARGUMENT)
    assert _native.status_string(12345) == "unknown status"


def test_library_is_the_in_tree_build(lib):
    assert os.path.dirname(_native.library_path()) == os.path.dirname(
        os.path.abspath(_native.__file__))
    assert isinstance(lib, ctypes.CDLL)


def test_tc_operand_kind_switch(lib):
    """The operand switch needs no device: it returns the previous kind and
    rejects unknown kinds without changing the setting."""
    from gstools_gb300 import _native

    assert lib.gst_grid_tc_set_operands(7) == -1
    prev = _native.set_tc_operands("tf32")
    assert prev == "f16"
    assert _native.set_tc_operands("f16") == "tf32"
    with pytest.raises(ValueError):
        _native.set_tc_operands("bf16")


def test_tc_tile_width_choice(lib):
    """The tensor-core grid path's z tile (MMA N) for a last axis of nz
    points: fewest tile-times, then least padding, then the wider tile (host
    code, no device needed)."""
    expect = {1: 128, 40: 128, 128: 128, 129: 192, 192: 192, 193: 256, 256: 256,
              320: 192, 384: 192, 640: 256, 1000: 256, 4096: 256}
    for nz, nt in expect.items():
        assert lib.gst_grid_tc_tile_cols(nz) == nt, nz
    assert lib.gst_grid_tc_tile_cols(-1) == -1
    # never more padded columns than the 256-wide tile
    for nz in range(1, 2000, 7):
        nt = lib.gst_grid_tc_tile_cols(nz)
        assert -(-nz // nt) * nt <= -(-nz // 256) * 256 or nt == 256, nz


def test_host_gather_matches_concatenate(lib):
    """gst_host_gather (host memcpy on threads, no device work) writes what
    np.concatenate(axis=-1) writes: 2-D and 1-D, empty members, one thread
    and many, above and below its threading threshold."""
    import numpy as np

    rng = np.random.RandomState(6)
    for rows, scale in ((2, 1), (2, 3000), (1, 3000), (3, 7)):
        cols = list(rng.randint(0, 50 * scale, size=33)) + [0, 5]
        items = [np.ascontiguousarray(rng.normal(size=(rows, c))) for c in cols]
        dst = np.zeros((rows, sum(cols)))
        ptrs = np.array([a.__array_interface__["data"][0] for a in items],
                        dtype=np.uint64)
        cc = np.array(cols, dtype=np.int64)
        for threads in (1, 7):
            dst[...] = 0.0
            rc = lib.gst_host_gather(len(items), ptrs.ctypes.data, cc.ctypes.data,
                                     rows, dst.ctypes.data, dst.shape[1], threads)
            assert rc == 0
            np.testing.assert_array_equal(dst, np.concatenate(items, axis=-1))
    # column counts that do not add up to the destination are refused
    cc = np.array([3, 4], dtype=np.int64)
    ptrs = np.array([1, 1], dtype=np.uint64)
    assert lib.gst_host_gather(2, ptrs.ctypes.data, cc.ctypes.data, 1,
                               dst.ctypes.data, 8, 1) == _native.GST_ERR_INVALID_ARGUMENT
