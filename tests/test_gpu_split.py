"""Split-precision form (Ozaki-style BF16 digit products on tcgen05) through
the C ABI, against the reference's golden outputs and the C oracle.

Tolerance: relative Frobenius error per body rank <= 1e-10 (the split-form
target; the digit expansion keeps about 36 bits per operand)."""
import numpy as np
import pytest

import imsrg_gb300 as ig
from helpers import CASES, load_golden, rel_errors, ref_space
from oracle import Oracle

pytestmark = pytest.mark.gpu

TOL_SPLIT = 1e-10


def full(ms, A, B, hA, hB, prec):
    with ig.DeviceOperator(ms, hA) as dA, ig.DeviceOperator(ms, hB) as dB, ig.DeviceOperator(ms, 1) as dZ:
        dA.upload(A)
        dB.upload(B)
        ig.Commutator.device_commutator(dA, dB, dZ, prec)
        return dZ.download()


def term(ms, name, A, B, hA, hB, prec):
    hZ = -1 if hA == hB else 1
    with ig.DeviceOperator(ms, hA) as dA, ig.DeviceOperator(ms, hB) as dB, ig.DeviceOperator(ms, hZ) as dZ:
        dA.upload(A)
        dB.upload(B)
        ig.Commutator.device_term(name, dA, dB, dZ, prec)
        return dZ.download()


@pytest.mark.parametrize("emax", [2, 3])
def test_split_full_vs_reference(emax):
    g = load_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    ops = {"X": g["X"], "Y": g["Y"], "W": g["W"]}
    for cs, (a, b, ha, hb) in CASES.items():
        if cs + "_full" not in g:
            continue
        Z = full(ms, ops[a], ops[b], ha, hb, "split")
        errs = rel_errors(r, Z, g[cs + "_full"])
        assert max(errs) < TOL_SPLIT, (cs, errs)


@pytest.mark.parametrize("emax", [2, 3])
@pytest.mark.parametrize("name", ["comm222_pp_hhss", "comm222_phss"])
def test_split_gemm_terms_vs_reference(emax, name):
    g = load_golden(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    r = ref_space(emax)
    ops = {"X": g["X"], "Y": g["Y"], "W": g["W"]}
    for cs, (a, b, ha, hb) in CASES.items():
        if cs + "_full" not in g:
            continue
        Z = term(ms, name, ops[a], ops[b], ha, hb, "split")
        errs = rel_errors(r, Z, g[cs + "_" + name])
        assert max(errs) < TOL_SPLIT, (cs, name, errs)


@pytest.mark.parametrize("emax", [4, 6])
def test_split_full_vs_oracle(emax):
    o = Oracle(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    X = o.ms.random_operator(31 + emax, True)
    Y = o.ms.random_operator(41 + emax, False)
    R = o.commutator(X, Y, 1, -1)
    Z = full(ms, X, Y, 1, -1, "split")
    errs = rel_errors(o.ms, Z, R)
    assert max(errs) < TOL_SPLIT, errs


@pytest.mark.parametrize("emax", [7, 8])
def test_split_full_antihermitian_z_vs_oracle(emax):
    # two hermitian operators: Z anti-hermitian, so the inverse Pandya blocks
    # skip diagonal elements; at these sizes some blocks are split into runs
    # of j rows to fit shared memory
    o = Oracle(emax)
    ms = ig.ModelSpace(emax, "O16", "O16")
    X = o.ms.random_operator(51 + emax, True)
    W = o.ms.random_operator(61 + emax, True)
    R = o.commutator(X, W, 1, 1)
    Z = full(ms, X, W, 1, 1, "split")
    errs = rel_errors(o.ms, Z, R)
    assert max(errs) < TOL_SPLIT, errs


def test_split_bch_vs_reference():
    g = load_golden(3)
    ms = ig.ModelSpace(3, "O16", "O16")
    r = ref_space(3)
    X = ig.Operator(ms, arena=g["X"], hermitian=True)
    Y = ig.Operator(ms, arena=g["Y"], hermitian=False)
    Om = Y * (0.25 / Y.Norm())
    Hs = ig.BCH.BCH_Transform(X, Om, precision="split")
    errs = rel_errors(r, Hs.arena, g["bch"])
    assert max(errs) < TOL_SPLIT, errs
