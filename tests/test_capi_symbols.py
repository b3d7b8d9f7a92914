"""The C-ABI library builds, loads without a GPU and exports every function
include/imsrg_gb300.h declares (no compute calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

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


def test_tensor_layout_matches_reference_rules():
    # the C ABI's tensor arena layout equals the one the reference harness
    # reads (TwoBodyME::Allocate order, 32-double alignment)
    from modelspace_ref import RefModelSpace
    for emax in (2, 3):
        ms = ig.ModelSpace(emax, "O16", "O16")
        r = RefModelSpace(emax)
        for rank in ((2, 0, 0), (1, 0, 1), (1, 1, 0), (0, 0, 0), (3, 1, 1)):
            blocks, offs, total = r.tensor_layout(*rank)
            mine = ms.tensor_layout(*rank)
            assert list(mine) == blocks and list(mine.values()) == offs
            assert ms.tensor_size(*rank) == total


def test_ninej_vs_exact():
    # the 9j of the scalar-tensor kernels (a sum of three tabulated 6j) against
    # SymPy's exact Racah-formula 9j, on argument sets that satisfy the triads
    sympy = pytest.importorskip("sympy")
    from sympy.physics.wigner import wigner_9j
    R = sympy.Rational
    ms = ig.ModelSpace(4, "O16", "O16")

    def tri(a, b, c):  # doubled
        return (a + b + c) % 2 == 0 and abs(a - b) <= c <= a + b

    rng = np.random.default_rng(7)
    n = 0
    while n < 300:
        ja, jb, jc, jd = (int(x) for x in rng.choice([1, 3, 5, 7, 9], 4))
        lam = int(rng.integers(0, 4))
        J1 = int(rng.integers(0, 10)); J2 = int(rng.integers(0, 10))
        Jb = int(rng.integers(0, 10)); Jk = int(rng.integers(0, 10))
        if not (tri(ja, jd, 2 * J1) and tri(jb, jc, 2 * J2) and tri(2 * Jb, 2 * Jk, 2 * lam) and tri(ja, jb, 2 * Jb)
                and tri(jd, jc, 2 * Jk) and tri(2 * J1, 2 * J2, 2 * lam)):
            continue
        n += 1
        v = ms.GetNineJ(ja / 2, jd / 2, J1, jb / 2, jc / 2, J2, Jb, Jk, lam)
        ref = float(wigner_9j(R(ja, 2), R(jd, 2), J1, R(jb, 2), R(jc, 2), J2, Jb, Jk, lam, prec=None))
        assert abs(v - ref) < 1e-14, (ja, jd, J1, jb, jc, J2, Jb, Jk, lam, v, ref)
