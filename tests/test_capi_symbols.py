"""The C-ABI library loads and exports every entry point of include/*.h.

Runs without a GPU: only host-side entry points (version, scratch sizing,
argument validation that fails before any CUDA call) are called.
"""
import ctypes
import glob
import os
import re

import pytest

from distance3d_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(d3d_\w+)\s*\(", text))
    return names


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def test_header_declares_entry_points():
    names = declared_symbols()
    assert {"d3d_gjk_distance", "d3d_gjk_intersection", "d3d_epa", "d3d_store_pack"} <= names


def test_every_declared_symbol_is_exported(lib):
    for name in sorted(declared_symbols()):
        assert hasattr(lib, name), f"{name} not exported by {build.LIB}"


def test_binding_covers_header():
    bound = {s[0] for s in _lib.SIGNATURES}
    assert declared_symbols() <= bound


def test_abi_version(lib):
    assert lib.d3d_abi_version() == 3


def test_epa_scratch_sizing(lib):
    opt = _lib.EpaOptions(64, 32, 64, 0, 1e-8)
    assert lib.d3d_epa_scratch_bytes(0, ctypes.byref(opt)) == 0
    one = lib.d3d_epa_scratch_bytes(1, ctypes.byref(opt))
    assert one >= (64 * 12 + 32 * 6) * 8
    bad = _lib.EpaOptions(64, 32, 3, 0, 1e-8)
    assert lib.d3d_epa_scratch_bytes(10, ctypes.byref(bad)) == 0


def test_invalid_arguments_rejected_on_host(lib):
    opt = _lib.GjkOptions(1e-10, 1e5, 1e-8, 100, 0)
    rc = lib.d3d_gjk_distance(None, None, None, 1, ctypes.byref(opt), None, None, None, None, None, None,
                              None, None)
    assert rc == _lib.D3D_ERR_INVALID
    assert b"invalid d3d_store" in lib.d3d_last_error()
    st = _lib.D3DStore(0, 0, 8, 8, 8, 0, 0, 0, 0)  # dummy non-null pointers, never dereferenced
    bad = _lib.GjkOptions(1e-10, 1e5, 1e-8, 0, 0)
    rc = lib.d3d_gjk_distance(ctypes.byref(st), None, None, 1, ctypes.byref(bad), None, None, None, None,
                              None, None, None, None)
    assert rc == _lib.D3D_ERR_INVALID
    assert b"max_iterations" in lib.d3d_last_error()
    eo = _lib.EpaOptions(64, 32, 2, 0, 1e-8)
    rc = lib.d3d_epa(ctypes.byref(st), None, None, 1, None, ctypes.byref(eo), None, None, None, None, None, 0,
                     None)
    assert rc == _lib.D3D_ERR_INVALID
