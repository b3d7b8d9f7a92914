"""The C-ABI library builds, loads without a GPU and exports every function
include/imsrg_gb300.h declares (no compute calls)."""
import ctypes
import os
import re

import imsrg_gb300 as ig
from imsrg_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "imsrg_gb300.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(imsrg_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_functions():
    names = declared_functions()
    assert "imsrg_comm222_phss" in names and "imsrg_bch_transform" in names
    assert len(names) >= 35


def test_library_exports_every_declared_symbol():
    L = ctypes.CDLL(ig.library_path())
    for name in declared_functions():
        assert hasattr(L, name), name


def test_binding_covers_every_declared_symbol():
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_errors_are_codes_not_exits():
    L = _lib.lib()
    assert L.imsrg_space_create_reference(-1, 16, 8, None) == _lib.ERR_ARG
    assert b"bad" in L.imsrg_last_error()
    assert L.imsrg_set_term(b"no_such_term", 1) == _lib.ERR_ARG
    assert L.imsrg_set_default_precision(7) == _lib.ERR_ARG


def test_term_switch_roundtrip():
    ig.Commutator.TurnOffTerm("comm122ss")
    assert not ig.Commutator.IsTermOn("comm122ss")
    ig.Commutator.TurnOnTerm("comm122ss")
    assert ig.Commutator.IsTermOn("comm122ss")
