"""The C-ABI library builds for sm_103a, loads, and exports every symbol the public header
declares. No GPU needed (no compute calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "ferrite_gb300.h")


def header_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fe_[a-z_0-9]+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = header_symbols()
    for s in ["fe_create", "fe_assemble", "fe_destroy", "fe_last_error", "fe_get_index_map"]:
        assert s in syms


def test_library_exports_every_declared_symbol(fg):
    fg.build()
    L = ctypes.CDLL(fg.LIB_PATH)
    missing = [s for s in header_symbols() if not hasattr(L, s)]
    assert not missing, missing
    assert set(fg.EXPORTED) <= set(header_symbols())


def test_abi_version(fg):
    assert fg.lib().fe_abi_version() == 1


def test_build_targets_sm103a(fg):
    """The build recipe compiles device code for sm_103a only."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_b", os.path.join(ROOT, "ferrite.jl_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
