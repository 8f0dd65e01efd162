"""The C-ABI library loads and exports what include/wstack_gb300.h declares.

No compute call is made here: these run without a GPU.
"""
import ctypes
import glob
import os
import re
import subprocess

import pytest

from lofar_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "wstack_gb300.h")
HEADERS = sorted(glob.glob(os.path.join(ROOT, "include", "*.h")))


def declared_symbols():
    text = "\n".join(ln for h in HEADERS for ln in open(h).read().splitlines()
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


def _compile_c(tmp_path, src, link=False):
    c = tmp_path / "probe.c"
    c.write_text(src)
    exe = tmp_path / "probe"
    cmd = ["gcc", "-std=c99", "-Wall", "-Werror", f"-I{os.path.join(ROOT, 'include')}", str(c),
           "-o", str(exe)]
    if link:
        d = os.path.dirname(_lib.LIB_PATH)
        cmd += [f"-L{d}", "-lwstack_gb300", f"-Wl,-rpath,{d}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout


def test_struct_layouts_match_ctypes(tmp_path):
    out = _compile_c(tmp_path, """
#include <stdio.h>
#include <stddef.h>
#include "wstack_gb300.h"
int main(void) {
    printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(wsg_stats), sizeof(wsg_tuning),
           sizeof(wsg_channel), offsetof(wsg_channel, weight), offsetof(wsg_tuning, ms),
           offsetof(wsg_stats, ctas));
    return 0;
}
""")
    got = [int(x) for x in out.split()]
    want = [ctypes.sizeof(_lib.Stats), ctypes.sizeof(_lib.Tuning), ctypes.sizeof(_lib.Channel),
            _lib.Channel.weight.offset, _lib.Tuning.ms.offset, _lib.Stats.ctas.offset]
    assert got == want


def test_plain_c_program_links_the_library(lib, tmp_path):
    """The reference is C: a C translation unit that includes the header and
    links the library (as a patched reference build would) builds and runs."""
    out = _compile_c(tmp_path, """
#include <stdio.h>
#include "wstack_gb300.h"
int main(void) {
    wsg_batch *b = 0;
    int st = wsg_batch_create(&b, 300, 256, 4, 7, 1.0 / 300, 0.25, 2, 4, 0);
    printf("%d %d %d\\n", test(41), st, wstack_gb300_last_error() == WSG_OK);
    return 0;
}
""", link=True)
    assert out.split() == ["42", str(_lib.WSG_ERR_UNSUPPORTED), "0"]


def test_batch_argument_errors_need_no_gpu(lib):
    h = ctypes.c_void_p()
    assert lib.wsg_batch_create(ctypes.byref(h), 256, 256, 4, 7, 1 / 256, 1 / 4, 0, 4, None) == \
        _lib.WSG_ERR_ARG
    assert lib.wsg_batch_create(ctypes.byref(h), 256, 256, 4, 7, 1 / 256, 1 / 4, 4, 0, None) == \
        _lib.WSG_ERR_ARG
    assert lib.wsg_batch_create(ctypes.byref(h), 300, 256, 4, 7, 1 / 300, 1 / 4, 4, 4, None) == \
        _lib.WSG_ERR_UNSUPPORTED
    assert lib.wsg_batch_create(ctypes.byref(h), 256, 256, 4, 7, 1 / 256, 1 / 4, 5000, 1, None) == \
        _lib.WSG_ERR_UNSUPPORTED
    assert lib.wsg_batch_create(ctypes.byref(h), 256, 256, 128, 7, 1 / 256, 1 / 128, 256, 4,
                                None) == _lib.WSG_ERR_UNSUPPORTED   # 131072 cube planes
    assert b"65535" in lib.wstack_gb300_last_error_string()
    assert lib.wsg_batch_forward(None, None, 1) == _lib.WSG_ERR_ARG
    assert lib.wsg_batch_vis_offset(None, 0) == -1
    assert lib.wsg_plan_autotune(None, 0, 1, 1, None, None, None, None, None, None, None, 1,
                                 None, None, 0, None) == _lib.WSG_ERR_ARG
