"""The C-ABI library loads and exports what include/wstack_gb300.h declares.

No compute call is made here: these run without a GPU.
"""
import ctypes
import os
import re
import subprocess

import pytest

from lofar_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "wstack_gb300.h")


def declared_symbols():
    text = "\n".join(ln for ln in open(HEADER).read().splitlines()
                     if not ln.lstrip().startswith("#"))
    return sorted(set(re.findall(r"WSG_API\s+[\w\s\*]*?\b(\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from lofar_gb300 import build
        build.build()
    return _lib.load()


def test_header_declares_reference_entry_points():
    syms = declared_symbols()
    for name in ("wstack", "phase_correction", "test", "wstack_fft_planes"):
        assert name in syms


def test_every_declared_symbol_is_exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if " T " in ln}
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    # and nothing internal leaks out
    assert all(s in declared_symbols() for s in exported)


def test_ctypes_signatures_cover_header(lib):
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_reference_test_function(lib):
    assert lib.test(41) == 42


def test_argument_errors_need_no_gpu(lib):
    h = ctypes.c_void_p()
    assert lib.wsg_plan_create(ctypes.byref(h), 64, 64, 4, 17, 1 / 64, 1 / 4, 1, None) == \
        _lib.WSG_ERR_UNSUPPORTED
    assert b"w_support" in lib.wstack_gb300_last_error_string()
    assert lib.wsg_plan_create(ctypes.byref(h), 0, 64, 4, 7, 1 / 64, 1 / 4, 1, None) == _lib.WSG_ERR_ARG
    assert lib.wsg_plan_create(ctypes.byref(h), 64, 64, 4, 7, 1 / 64, 1 / 4, 9, None) == _lib.WSG_ERR_ARG
    assert lib.wsg_plan_create(ctypes.byref(h), 64, 64, 4, 7, -1.0, 1 / 4, 1, None) == _lib.WSG_ERR_ARG
    assert lib.wsg_bin(None, 1, 1, 1, None, None, None, None, None, None) == _lib.WSG_ERR_ARG
    assert lib.wstack_gb300_set_precision(7) == -1


def test_status_codes_match_header():
    text = open(HEADER).read()
    for name, val in re.findall(r"(WSG_\w+)\s*=\s*(\d+)", text):
        assert getattr(_lib, name) == int(val), name
