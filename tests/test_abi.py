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


def test_python_constants_match_header(fg):
    """Every flag, precision, physics, cell-type and status constant of the Python binding has
    the value the header defines."""
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(FE_[A-Z0-9_]+)\s+(\d+)u?\b", txt)}
    pairs = {"FE_FILLZERO": fg.FILLZERO, "FE_NO_K": fg.NO_K, "FE_NO_F": fg.NO_F, "FE_ASYNC": fg.ASYNC,
             "FE_PROFILE": fg.PROFILE, "FE_COMPENSATED": fg.COMPENSATED, "FE_TWO_PHASE": fg.TWO_PHASE,
             "FE_FUSED": fg.FUSED, "FE_NO_TENSOR": fg.NO_TENSOR, "FE_STAGED_OUTPUT": fg.STAGED_OUTPUT, "FE_FP32_SUM": fg.FP32_SUM,
             "FE_PREC_MIXED": fg.PREC_MIXED, "FE_PREC_FP64": fg.PREC_FP64, "FE_HEAT": fg.HEAT,
             "FE_LINEAR_ELASTIC": fg.LINEAR_ELASTIC, "FE_NEO_HOOKE": fg.NEO_HOOKE, "FE_TRIANGLE": fg.TRIANGLE,
             "FE_QUADRILATERAL": fg.QUADRILATERAL, "FE_TETRAHEDRON": fg.TETRAHEDRON, "FE_HEXAHEDRON": fg.HEXAHEDRON,
             "FE_WEDGE": fg.WEDGE, "FE_OK": fg.FE_OK, "FE_ERR_ARG": fg.FE_ERR_ARG, "FE_ERR_BOUNDS": fg.FE_ERR_BOUNDS,
             "FE_ERR_DETJ": fg.FE_ERR_DETJ, "FE_ERR_PATTERN_MISSING": fg.FE_ERR_PATTERN_MISSING}
    for name, value in pairs.items():
        assert defs.get(name) == value, (name, defs.get(name), value)
    for code, name in fg.ERROR_NAMES.items():
        assert defs.get("FE_OK" if name == "OK" else "FE_ERR_" + name) == code, name
    flag_names = ("FE_FILLZERO", "FE_NO_K", "FE_NO_F", "FE_ASYNC", "FE_PROFILE", "FE_COMPENSATED", "FE_TWO_PHASE",
                  "FE_FUSED", "FE_NO_TENSOR", "FE_STAGED_OUTPUT", "FE_FP32_SUM")
    flags = [defs[k] for k in flag_names]
    assert len(set(flags)) == len(flags) and all(f & (f - 1) == 0 for f in flags)  # distinct single bits
