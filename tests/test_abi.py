"""The C ABI: the library builds, loads without a GPU, and exports every symbol
the public header declares.  CPU only (no compute calls)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "spnngp_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(nngp_[A-Za-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for must in ("nngp_mkNNIndxCB", "nngp_mkNNIndx", "nngp_mkUIndx", "nngp_updateBF", "nngp_updateConjBF",
                 "nngp_Q", "nngp_rNNGP", "nngp_cNNGP", "nngp_rNNGPPredict", "nngp_rNNGPReplicated"):
        assert must in syms


def test_library_exports_every_declared_symbol():
    from spnngp_gb300.build import build

    path = build()
    lib = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, f"declared but not exported: {missing}"


def test_package_import_does_not_touch_gpu():
    import spnngp_gb300

    assert spnngp_gb300.COV_MODELS == ("exponential", "spherical", "matern", "gaussian")


def test_missing_library_fails_loudly(tmp_path):
    from spnngp_gb300 import _lib

    with pytest.raises(ImportError):
        _lib._Lib(str(tmp_path / "nope.so"))


def declared_arity():
    text = open(HEADER).read()
    out = {}
    for m in re.finditer(r"\b(nngp_[A-Za-z0-9_]+)\s*\(([^;{]*?)\)\s*;", text, re.S):
        args = m.group(2).strip()
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_python_bindings_match_header():
    """Every ctypes signature names a declared entry point with the declared number of arguments."""
    from spnngp_gb300._lib import _SIGNATURES

    arity = declared_arity()
    for name, (_, argtypes) in _SIGNATURES.items():
        assert name in arity, name
        assert len(argtypes) == arity[name], (name, len(argtypes), arity[name])
