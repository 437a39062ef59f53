"""The C-ABI library builds for sm_103a, loads, and exports every function
include/kpm.h declares (no compute call: this runs without a GPU)."""
import ctypes
import os
import re

from conftest import ROOT
from minijclsquant_gb300 import _build, _capi

HEADER = os.path.join(ROOT, "include", "kpm.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*([A-Za-z_][A-Za-z0-9_]*)\s*\(", text, re.M)
    return sorted(set(n for n in names if n not in ("if", "defined")))


def test_header_declarations_found():
    names = declared_functions()
    assert "kpm_cheb_moments" in names and "rec_A_tab" in names
    assert len(names) >= 14


def test_library_exports_every_declared_symbol():
    path = _build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    assert set(declared_functions()) == set(_capi.SIGNATURES)


def test_strerror_and_version_without_gpu():
    lib = _capi.load(build_if_missing=True)
    assert lib.kpm_strerror(0) == b"ok"
    assert lib.kpm_strerror(_capi.KPM_ERR_INDEX) == b"ELL column index out of range"
    assert lib.kpm_version() >= 100
