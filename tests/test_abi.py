"""The C-ABI library loads without a GPU and exports every entry point that
include/*.h declares (CPU only; no compute call is made)."""
import ctypes
import re

from conftest import ROOT

import kcoregpu_gb300 as kc
from kcoregpu_gb300 import _lib


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"\b(kc_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing
    assert len(declared_symbols()) >= 25


def test_python_binding_covers_the_header():
    assert set(declared_symbols()) <= set(_lib.SIGNATURES) | {"kc_last_error"}


def test_strerror_names_every_code():
    lib = kc.lib()
    for code in range(0, -12, -1):
        assert lib.kc_strerror(code) and lib.kc_strerror(code) != b"unknown error"


def test_product_library_does_not_link_the_oracle():
    data = _lib.LIB_PATH.read_bytes()
    assert b"kco_bz" not in data and b"libkc_oracle" not in data
