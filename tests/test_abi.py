"""The C-ABI library loads and exports every function include/nmg.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(nmg_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "nmg_mixture_sample" in names and "nmg_last_error" in names


def test_library_exports_every_declared_symbol(nmg):
    lib = nmg.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings(nmg):
    lib = nmg.lib()
    assert lib.nmg_status_string(0) == b"ok"
    assert lib.nmg_status_string(7).startswith(b"size")


def test_invalid_arguments_are_rejected_without_a_device(nmg):
    lib = nmg.lib()
    o = nmg.mixture_opts(5, 32)  # K=5 not compiled
    rc = lib.nmg_mixture_sample(ctypes.byref(o), None, None, None, 16, None, None, None, None)
    assert rc == 1 and b"n_lobes" in lib.nmg_last_error()
    o = nmg.mixture_opts(8, 30)  # stride not a multiple of 4
    assert lib.nmg_mixture_pdf(ctypes.byref(o), None, None, None, 16, None, None) == 1
    o = nmg.mixture_opts(8, 32)
    assert lib.nmg_mixture_sample(ctypes.byref(o), None, None, None, 0, None, None, None, None) == 0  # empty batch
    assert lib.nmg_mixture_sample(ctypes.byref(o), None, None, None, -1, None, None, None, None) == 1
