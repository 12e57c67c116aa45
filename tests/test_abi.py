"""The C-ABI library loads and exports every entry point declared in
include/cem.h (no device calls)."""

import ctypes
import os
import re

from casmcode_clexmonte_gb300 import build as B
from casmcode_clexmonte_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    txt = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(cem_\w+)\s*\(", txt, re.M)))


def test_library_exports_header_symbols():
    path = B.build()
    lib = ctypes.CDLL(path)
    names = declared("cem.h")
    assert len(names) >= 24
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) <= set(_lib.EXPORTS) | set(names)
    assert set(_lib.EXPORTS) <= set(names)
